"""CPU checks of the Davidson subspace eigensolver (rt_debug_symeig): Householder
tridiagonalisation + implicit QR with Wilkinson shifts, host code in the native library.

It stands in for the reference's packed LAPACK dspevx (matrix_blas_lapack.rs:1075-1095)
on matrices of the Davidson subspace's size.  Tolerances: eigenvalues within
1e-13 * ||A|| of numpy's eigh, residuals ||A z - w z|| and ||Z^T Z - I|| within 1e-12 * n.
"""
import ctypes

import numpy as np
import pytest

import rest_tensors_gb300 as rt


def symeig(a):
    n = a.shape[0]
    a = np.asfortranarray(a, dtype=np.float64)
    w = np.zeros(n)
    z = np.zeros((n, n), order="F")
    dp = ctypes.POINTER(ctypes.c_double)
    L = rt.lib()
    L.rt_debug_symeig.restype = ctypes.c_int
    st = L.rt_debug_symeig(n, a.ctypes.data_as(dp), w.ctypes.data_as(dp), z.ctypes.data_as(dp))
    assert st == 0, L.rt_last_error()
    return w, z


def cases():
    rng = np.random.default_rng(7)
    out = []
    for n in (1, 2, 3, 5, 8, 17, 40, 69):
        m = rng.standard_normal((n, n))
        out.append(("random", 0.5 * (m + m.T)))
    # clustered spectrum, like converging Ritz values
    Q, _ = np.linalg.qr(rng.standard_normal((48, 48)))
    d = np.concatenate([0.547 + 1e-4 * np.arange(8), np.linspace(1, 5, 40)])
    out.append(("clustered", (Q * d) @ Q.T))
    out.append(("diagonal", np.diag(rng.standard_normal(12))))
    out.append(("degenerate", np.eye(10) * 2.0 + np.outer(np.ones(10), np.ones(10))))
    out.append(("tridiagonal", np.diag(np.arange(20.0)) + np.diag(np.ones(19), 1) + np.diag(np.ones(19), -1)))
    return out


@pytest.mark.parametrize("name,a", cases(), ids=[c[0] + str(c[1].shape[0]) for c in cases()])
def test_symeig_matches_numpy(name, a):
    a = 0.5 * (a + a.T)
    n = a.shape[0]
    w, z = symeig(a)
    scale = max(1.0, np.abs(a).max() * n)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - np.linalg.eigvalsh(a)).max() <= 1e-13 * scale
    assert np.abs(a @ z - z * w).max() <= 1e-12 * scale
    assert np.abs(z.T @ z - np.eye(n)).max() <= 1e-12 * n
    for k in range(n):  # sign convention: largest-magnitude component positive
        assert z[np.argmax(np.abs(z[:, k])), k] > 0
