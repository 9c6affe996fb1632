"""The device eigensolver and the SCF-side routines on it, through the C ABI.

* rt_dsyev (lapack_dsyev, matrix_blas_lapack.rs:775-797) against numpy's eigh:
  eigenvalues within 1e-12 of max|eigenvalue| (times a size factor for n in
  the hundreds), residual ||A V - V diag(w)|| and orthonormality at the same
  level, on random, degenerate, diagonal and tridiagonal matrices; only the
  lower triangle is read; bitwise repeatable.
* rt_lapack_power (matrix_blas_lapack.rs:1004-1064) against the oracle's
  restatement over OpenBLAS, on the reference's own test inputs and on
  well-conditioned random matrices up to n = 600: 1e-12 relative (float64
  product), 1e-11 (split product); with small eigenvalues kept under negative
  powers (ill-conditioned by construction): 1e-10.
* rt_dspgvx (matrix_blas_lapack.rs:1096-1147) against the oracle's dspgvx:
  eigenvalues 1e-12 relative, eigenvectors up to sign 1e-10, B-orthonormal.
"""
import json
import os

import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_doctests.json")))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))).cuda()


def host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


def sym(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n))
    return 0.5 * (A + A.T)


def with_spectrum(ev, seed):
    n = len(ev)
    Q, _ = np.linalg.qr(np.random.default_rng(seed).standard_normal((n, n)))
    A = (Q * np.asarray(ev, dtype=np.float64)) @ Q.T
    return 0.5 * (A + A.T)


def check_eigh(A, tol):
    n = A.shape[0]
    dA = dev(A)
    w = rt.dsyev(dA, n)
    rt.sync_status()
    wv, V = w.cpu().numpy(), host(dA, (n, n))
    ref = np.linalg.eigvalsh(A)
    scale = max(1.0, np.max(np.abs(ref)))
    assert np.max(np.abs(wv - ref)) <= tol * scale
    assert np.max(np.abs(A @ V - V * wv)) <= tol * scale
    assert np.max(np.abs(V.T @ V - np.eye(n))) <= tol
    return wv, V


@pytest.mark.parametrize("n", [1, 2, 3, 4, 17, 64, 200, 777])
def test_dsyev_random(n):
    check_eigh(sym(n, n), 1e-12 * max(1.0, n / 64))


def test_dsyev_degenerate_diagonal_and_tridiagonal():
    check_eigh(with_spectrum([1.0] * 5 + [2.0] * 7 + [3.0] * 3 + [-1.0] * 9, 1), 1e-12)
    check_eigh(np.diag(np.arange(10.0, 0.0, -1.0)), 1e-13)
    T = np.diag(np.full(50, 2.0)) + np.diag(np.full(49, -1.0), 1) + np.diag(np.full(49, -1.0), -1)
    check_eigh(T, 1e-12)
    check_eigh(with_spectrum(np.concatenate([[1e-9, 2e-9], np.linspace(1, 2, 60)]), 4), 1e-12)


def test_dsyev_reads_only_the_lower_triangle_and_repeats_bitwise():
    n = 90
    A = sym(n, 5)
    junk = A.copy()
    junk[np.triu_indices(n, 1)] = 1e300
    dA = dev(junk)
    w = rt.dsyev(dA, n)
    ref = np.linalg.eigvalsh(A)
    assert np.max(np.abs(w.cpu().numpy() - ref)) < 1e-12 * np.max(np.abs(ref))
    dB = dev(junk)
    w2 = rt.dsyev(dB, n)
    assert torch.equal(w, w2) and torch.equal(dA, dB)


@pytest.mark.parametrize("name", ["lapack_power_3x3", "lapack_power_8x8"])
@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("split", 1e-11)])
def test_lapack_power_on_the_reference_test_inputs(name, form, tol):
    c = next(x for x in GOLD["cases"] if x["name"] == name)
    n = c["n"]
    S = np.array(c["matrix"]).reshape(n, n, order="F")
    ref, kept_ref = oracle.lapack_power(S, c["p"], c["threshold"])
    out, kept = rt.lapack_power(dev(S), n, c["p"], c["threshold"], form=form)
    rt.sync_status()
    assert kept == kept_ref
    assert np.max(np.abs(host(out, (n, n)) - ref)) / np.max(np.abs(ref)) < tol * (10 if name.endswith("3x3") else 1)


@pytest.mark.parametrize("n,p", [(64, -0.5), (600, -0.5), (600, 0.5), (300, -1.0), (300, 2.0)])
@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("split", 1e-11)])
def test_lapack_power_matches_oracle(n, p, form, tol):
    # Eigenvalues in [0.5, 3] (a metric-like, well-conditioned matrix): two correct eigensolvers agree
    # to a few ulps of the result.
    ev = np.random.default_rng(n).uniform(0.5, 3.0, n)
    S = with_spectrum(ev, n + 1)
    ref, kept_ref = oracle.lapack_power(S, p, 1e-10)
    out, kept = rt.lapack_power(dev(S), n, p, 1e-10, form=form)
    rt.sync_status()
    assert kept == kept_ref == n
    assert np.max(np.abs(host(out, (n, n)) - ref)) / np.max(np.abs(ref)) < tol


@pytest.mark.parametrize("n,p,threshold", [(40, -0.5, 2e-4), (120, 0.5, 0.0), (300, -1.0, 1e-3), (64, 2.0, -1.0)])
@pytest.mark.parametrize("form", ["fp64", "split"])
def test_lapack_power_threshold_matches_oracle(n, p, threshold, form):
    # Four eigenvalues in 1e-6 .. 5e-4 beside [0.5, 3]: the threshold drops some of them, as the
    # reference zeroes their columns.  A kept eigenvalue ev under a negative power amplifies any
    # eigensolver's rounding by about ev^(p-1) / gap, so the tolerance here is 1e-10.
    rng = np.random.default_rng(n)
    ev = np.concatenate([rng.uniform(0.5, 3.0, n - 4), [1e-6, 2e-5, 1e-4, 5e-4]])
    S = with_spectrum(ev, n + 1)
    ref, kept_ref = oracle.lapack_power(S, p, threshold)
    out, kept = rt.lapack_power(dev(S), n, p, threshold, form=form)
    rt.sync_status()
    assert kept == kept_ref
    assert np.max(np.abs(host(out, (n, n)) - ref)) / np.max(np.abs(ref)) < 1e-10


@pytest.mark.parametrize("n,k", [(60, 12), (200, 50), (5, 5)])
@pytest.mark.parametrize("form", ["fp64", "split"])
def test_dspgvx_matches_oracle(n, k, form):
    rng = np.random.default_rng(n + k)
    A = sym(n, n)
    M = rng.standard_normal((n, n))
    B = M @ M.T / n + np.eye(n)
    ap, bp = oracle.full_to_upper_packed(A), oracle.full_to_upper_packed(B)
    z_ref, w_ref, _ = oracle.dspgvx(ap, bp, n, k)
    z, w = rt.dspgvx(dev(ap), dev(bp), n, k, form=form)
    rt.sync_status()
    z, w = host(z, (n, k)), w.cpu().numpy()
    scale = np.max(np.abs(w_ref[:k]))
    tol = 1e-12 if form == "fp64" else 1e-11
    assert np.max(np.abs(w[:k] - w_ref[:k])) <= tol * scale * max(1.0, n / 64)
    assert not w[k:].any()
    assert np.max(np.abs(z.T @ B @ z - np.eye(k))) < 100 * tol
    for j in range(k):
        s = np.sign(z[:, j] @ B @ z_ref[:, j])
        assert np.max(np.abs(s * z[:, j] - z_ref[:, j])) < 1e-9


def test_dspgvx_rejects_an_indefinite_overlap():
    n = 6
    A = sym(n, 1)
    B = np.diag([1.0, 2.0, -1.0, 1.0, 1.0, 1.0])
    with pytest.raises(rt.RTError, match="positive definite"):
        rt.dspgvx(dev(oracle.full_to_upper_packed(A)), dev(oracle.full_to_upper_packed(B)), n, 2)
    with pytest.raises(rt.RTError):
        rt.dspgvx(dev(oracle.full_to_upper_packed(A)), dev(oracle.full_to_upper_packed(np.eye(n))), n, 7)
