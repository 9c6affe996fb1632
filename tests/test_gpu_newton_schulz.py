"""GPU parity of the Newton-Schulz inverse square root (rt_newton_schulz_inv_sqrt) against the oracle.

Tolerances (written here): float64 form 1e-12 relative to max|oracle| with
the same convergence flag and evaluation count; split form (7 BF16 digits)
1e-11 relative, converged.
"""
import ctypes

import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RT_ERR_INVALID_ARG = 1


def spd(n, lo=1.0, hi=2.5, seed=0):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    S = (Q * rng.uniform(lo, hi, n)) @ Q.T
    return np.asfortranarray(0.5 * (S + S.T))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).cuda()


def relerr(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


CASES = [
    # n, threshold, mix, num_iter, level_shift
    (1, 1e-8, 1.0, 100, [0.0]),
    (7, 1e-8, 1.0, 100, [0.0]),
    (50, 1e-8, 1.0, 100, [0.0]),
    (200, 1e-10, 0.3, 200, [1e-3, 1e-4, 0.0]),
    (333, 1e-10, 0.7, 200, [0.0]),
    (20, 1e-14, 1.0, 1, [0.0, 1.0]),  # every stage fails: six retries with halved mixing, then stop
]


@pytest.mark.parametrize("case", CASES)
def test_fp64_matches_oracle(case):
    n, thr, mix, it, shifts = case
    S = spd(n, seed=n)
    want, _, conv_w, evals_w = oracle.newton_schulz_inverse_square_root_v02(S, thr, mix, it, shifts)
    X, n_singular, conv, evals = rt.newton_schulz_inverse_square_root_v02(dev(S), n, thr, mix, it, shifts)
    got = X.cpu().numpy().reshape(n, n, order="F")
    assert n_singular == 0 and conv == conv_w and evals == evals_w
    assert relerr(got, want) <= 1e-12


@pytest.mark.parametrize("n", [64, 300])
def test_split_form_converges_to_the_same_matrix(n):
    S = spd(n, seed=10 + n)
    want, _, _, _ = oracle.newton_schulz_inverse_square_root_v02(S, 1e-10, 1.0, 100, [0.0])
    X, _, conv, _ = rt.newton_schulz_inverse_square_root_v02(dev(S), n, 1e-10, 1.0, 100, [0.0], form="split")
    got = X.cpu().numpy().reshape(n, n, order="F")
    assert conv
    assert relerr(got, want) <= 1e-11


def test_scalar_case_is_exact():
    # the first evaluation already converges; the reference's loop still runs once (evals 2)
    X, _, conv, evals = rt.newton_schulz_inverse_square_root_v02(dev(np.array([[4.0]])), 1, 1e-8, 1.0, 10, [0.0])
    assert conv and evals == 2 and float(X[0]) == 0.5
    _, _, conv_w, evals_w = oracle.newton_schulz_inverse_square_root_v02(np.array([[4.0]]), 1e-8, 1.0, 10, [0.0])
    assert conv_w and evals_w == 2


def test_bad_arguments_are_rejected():
    S = dev(spd(4))
    out = torch.empty(16, dtype=torch.float64, device="cuda")
    L = rt.lib()
    shifts = (ctypes.c_double * 1)(0.0)
    st = L.rt_newton_schulz_inv_sqrt(S.data_ptr(), 4, 1e-8, 1.0, 10, shifts, 0, 0, 7, out.data_ptr(), None, None,
                                     torch.cuda.current_stream().cuda_stream)
    assert st == RT_ERR_INVALID_ARG
    st = L.rt_newton_schulz_inv_sqrt(S.data_ptr(), 4, 1e-8, 1.0, 10, shifts, 1, 1, 2, out.data_ptr(), None, None,
                                     torch.cuda.current_stream().cuda_stream)
    assert st == RT_ERR_INVALID_ARG
    with pytest.raises(ValueError):
        rt.newton_schulz_inverse_square_root_v02(S, 4, 1e-8, 1.0, 10, [])
    zero = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(rt.RTError):
        rt.newton_schulz_inverse_square_root_v02(zero, 4, 1e-8, 1.0, 10, [0.0])
