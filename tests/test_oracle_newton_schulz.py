"""CPU checks of the oracle's Newton-Schulz restatement (matrix_blas_lapack.rs:1710-1932).

The reference's own test of this routine (matrix_blas_lapack.rs:1520-1600)
prints its results without asserting, so the restatement is pinned against
the mathematics: S^-1/2 from a symmetric eigendecomposition, and X S X = I.
"""
import numpy as np
import pytest

import oracle


def spd(n, lo=1.0, hi=2.5, seed=0):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    S = (Q * rng.uniform(lo, hi, n)) @ Q.T
    return 0.5 * (S + S.T)


def inv_sqrt(S):
    w, V = np.linalg.eigh(S)
    return (V * w ** -0.5) @ V.T


@pytest.mark.parametrize("n", [1, 7, 50])
def test_reference_parameters_converge_to_the_inverse_square_root(n):
    # the parameters of the reference's own call (matrix_blas_lapack.rs:1585)
    S = spd(n, seed=n)
    X, n_singular, conv, evals = oracle.newton_schulz_inverse_square_root_v02(S, 1e-8, 1.0, 100, [0.0])
    assert conv and n_singular == 0 and evals >= 1
    assert np.abs(X - inv_sqrt(S)).max() <= 1e-12 * np.abs(inv_sqrt(S)).max()
    assert np.abs(X @ S @ X - np.eye(n)).max() <= 1e-12


def test_level_shift_stages_end_at_the_last_shift():
    S = spd(40, seed=3)
    X, _, conv, _ = oracle.newton_schulz_inverse_square_root_v02(S, 1e-10, 0.3, 200, [1e-3, 1e-4, 0.0])
    assert conv
    assert np.abs(X - inv_sqrt(S)).max() <= 1e-12 * np.abs(inv_sqrt(S)).max()
    # a single stage with a shift converges to the shifted normalised matrix's inverse square root
    norm = np.sqrt(np.sum(S ** 2))
    X1, _, conv1, _ = oracle.newton_schulz_inverse_square_root_v02(S, 1e-10, 1.0, 200, [1e-3])
    want = inv_sqrt(S / norm + 1e-3 * np.eye(40)) * norm ** -0.5
    assert conv1 and np.abs(X1 - want).max() <= 1e-12 * np.abs(want).max()


def test_failed_stage_retries_six_times_with_halved_mixing():
    S = spd(20, seed=4)
    # one iteration cannot reach 1e-14: the stage fails, is retried with mix/2, /4, ... six times, then stops
    _, _, conv, evals = oracle.newton_schulz_inverse_square_root_v02(S, 1e-14, 1.0, 1, [0.0, 1.0])
    assert not conv
    assert evals == 7 * 2  # 7 calls of the stage loop, 2 evaluations each; the second shift never runs


def test_empty_level_shift_is_rejected():
    with pytest.raises(ValueError):
        oracle.newton_schulz_inverse_square_root_v02(spd(3), 1e-8, 1.0, 10, [])


def test_reference_sqrt_inverse_matrix_is_out_of_reach_of_the_iteration():
    # The SPD matrix of the reference's test_sqrt_inverse (matrix_blas_lapack.rs:1398-1405), which the
    # reference inverts with lapack_power.  Its condition number is ~6600; the uncoupled iteration
    # X <- 0.5 X (3I - A X X) reaches ||dX|| / n^2 ~ 3e-5 and then amplifies rounding, so the reference's
    # algorithm never converges: the stage and its six halved-mixing retries each run all 101 evaluations.
    A = np.array([[4.0, 12.0, -16.0], [12.0, 37.0, -43.0], [-16.0, -43.0, 98.0]])
    assert np.linalg.cond(A) > 6000
    _, _, conv, evals = oracle.newton_schulz_inverse_square_root_v02(A, 1e-10, 1.0, 100, [0.0])
    assert not conv
    assert evals == 7 * 101
