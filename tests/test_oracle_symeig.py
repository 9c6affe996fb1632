"""The oracle's lapack_power and lapack_dspgvx restatements, pinned on the CPU.

The reference's tests of lapack_power (matrix_blas_lapack.rs:1398-1406 and
lib.rs:171-186) print without asserting, so their inputs (read as text into
tests/golden/reference_doctests.json) are checked here against the
mathematics: S^p = V diag(ev^p) V^T over the eigenvalues >= threshold, from
numpy's eigh.  dspgvx is checked against scipy's generalised eigh.
"""
import json
import os

import numpy as np
import pytest

import oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_doctests.json")))


def power_ref(S, p, threshold):
    w, V = np.linalg.eigh(S)
    keep = w >= threshold
    f = np.where(keep, np.sqrt(np.where(keep, w, 1.0)) ** p, 0.0)
    return (V * f) @ (V * f).T, int(keep.sum())


@pytest.mark.parametrize("name", ["lapack_power_3x3", "lapack_power_8x8"])
def test_lapack_power_on_the_reference_test_inputs(name):
    c = next(x for x in GOLD["cases"] if x["name"] == name)
    n = c["n"]
    S = np.array(c["matrix"]).reshape(n, n, order="F")
    out, kept = oracle.lapack_power(S, c["p"], c["threshold"])
    ref, kept_ref = power_ref(S, c["p"], c["threshold"])
    assert kept == kept_ref
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 1e-10
    if kept == n and c["p"] == -0.5:  # S^-1/2 S S^-1/2 = I where nothing is dropped
        assert np.max(np.abs(out @ S @ out - np.eye(n))) < 1e-8


# Eigenvalues 1e-6 .. 5e-4 beside O(1): negative powers of kept tiny eigenvalues amplify any
# eigensolver's rounding by their condition, so the thresholds drop the smallest ones there.
@pytest.mark.parametrize("p,threshold", [(-0.5, 2e-4), (0.5, 0.0), (-1.0, 1e-3), (2.0, -1.0)])
def test_lapack_power_random(p, threshold):
    rng = np.random.default_rng(7)
    n = 40
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.concatenate([rng.uniform(0.5, 3.0, n - 4), [1e-6, 2e-5, 1e-4, 5e-4]])
    S = (Q * ev) @ Q.T
    S = 0.5 * (S + S.T)
    out, kept = oracle.lapack_power(S, p, threshold)
    ref, kept_ref = power_ref(S, p, threshold)
    assert kept == kept_ref
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 1e-11


def test_dspgvx_matches_scipy_generalised_eigh():
    sl = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(3)
    n, k = 60, 12
    A = rng.standard_normal((n, n))
    A = A + A.T
    M = rng.standard_normal((n, n))
    B = M @ M.T / n + np.eye(n)
    z, w, m = oracle.dspgvx(oracle.full_to_upper_packed(A), oracle.full_to_upper_packed(B), n, k)
    lam, X = sl.eigh(A, B)
    assert m == k and not w[k:].any()
    assert np.max(np.abs(w[:k] - lam[:k])) < 1e-12 * np.max(np.abs(lam))
    assert np.max(np.abs(z.T @ B @ z - np.eye(k))) < 1e-12
    for j in range(k):  # eigenvectors up to sign
        s = np.sign(z[:, j] @ B @ X[:, j])
        assert np.max(np.abs(s * z[:, j] - X[:, j])) < 1e-10
