"""Davidson, the RI response operator and the (ia|jb) block on the GPU,
checked against the CPU oracle (a line-by-line restatement of
src/davidson.rs) and against dense eigensolves.

Tolerances: float64 products 1e-12 relative; split products 1e-11 relative
(7 BF16 digits); eigenvalues of runs converged to `tol` agree with the oracle's
Davidson to 1e-9 and with a dense eigensolve to 10*tol.
"""
import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))).cuda()


def ri_ov_block(nb, naux, nocc, seed):
    C = oracle.synth_coef(seed, nb)
    B = oracle.synth_ri3ao(seed, nb, naux)
    ov, _ = oracle.ri_ov_k(C, B, nocc)
    nov = nocc * (nb - nocc)
    return np.asfortranarray(ov.reshape(nov, naux, order="F"))


@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("split", 1e-11)])
def test_response_matvec_matches_oracle(form, tol):
    Bov = ri_ov_block(40, 30, 6, seed=1)
    nov, naux = Bov.shape
    d = oracle.synth_delta(1, nov)
    X = np.asfortranarray(np.random.default_rng(0).standard_normal((nov, 5)))
    ref = oracle.response_matvec(Bov, d, X)
    got = rt.ri_response_matvec(dev(Bov), dev(d), nov, naux, dev(X), 5, form=form, nslices=7)
    got = got.cpu().numpy().reshape(nov, 5, order="F")
    assert np.max(np.abs(got - ref)) < tol * np.max(np.abs(ref))


@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("split", 1e-11)])
def test_iajb_matches_oracle(form, tol):
    Bov = ri_ov_block(36, 25, 5, seed=2)
    nov, naux = Bov.shape
    ref = oracle.iajb(Bov)
    got = rt.ri_iajb(dev(Bov), nov, naux, form=form, nslices=7).cpu().numpy().reshape(nov, nov, order="F")
    assert np.max(np.abs(got - ref)) < tol * np.max(np.abs(ref))
    assert np.array_equal(got, got.T)


def test_davidson_dense_operator_matches_reference_restatement():
    rng = np.random.default_rng(7)
    n = 300
    R = rng.standard_normal((n, n)) * 0.02
    A = np.diag(np.linspace(0.5, 6.0, n)) + (R + R.T)
    hdiag = np.diag(A).copy()
    x0 = np.zeros(n)
    x0[0] = 1.0
    p = oracle.DavidsonParams(tol=1e-10, maxcyc=60, maxspace=16, nroots=3)
    conv_ref, e_ref, x_ref = oracle.davidson_solve(lambda x: A @ x, x0, hdiag, p)
    dA = torch.from_numpy(A).cuda()
    conv, e, x, its = rt.davidson_solve(lambda X: X @ dA, dev(x0), dev(hdiag),
                                        rt.DavidsonParams(tol=1e-10, maxcyc=60, maxspace=16, nroots=3))
    assert conv == conv_ref and all(conv)
    assert np.allclose(e, e_ref, atol=1e-9)
    assert np.allclose(e, np.linalg.eigvalsh(A)[:3], atol=1e-9)
    for k in range(3):
        overlap = abs(float(np.dot(x[k].cpu().numpy(), x_ref[k])))
        assert abs(overlap - 1.0) < 1e-6


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_davidson_ri_response(form):
    # Couplings scaled to a diagonally dominant response matrix (diag(B B^T) ~ 0.1-0.2
    # against delta in [0.5, 3]), the regime the diagonal preconditioner is made for.
    Bov = np.asfortranarray(0.05 * ri_ov_block(60, 200, 10, seed=3))
    nov, naux = Bov.shape
    d = oracle.synth_delta(3, nov)
    A = np.diag(d) + Bov @ Bov.T
    hd = np.diag(A).copy()
    exact = np.linalg.eigvalsh(A)[:4]
    x0 = np.zeros(nov)
    x0[np.argmin(hd)] = 1.0
    tol = 1e-10
    p = oracle.DavidsonParams(tol=tol, maxcyc=80, maxspace=20, nroots=4)
    conv_ref, e_ref, _ = oracle.davidson_solve(lambda x: oracle.response_matvec(Bov, d, x[:, None])[:, 0], x0, hd, p)
    conv, e, x, its = rt.davidson_ri_response(dev(Bov), dev(d), nov, naux, dev(x0),
                                              rt.DavidsonParams(tol=tol, maxcyc=80, maxspace=20, nroots=4),
                                              form=form, nslices=7)
    assert all(conv) and all(conv_ref)
    assert np.allclose(e, e_ref, atol=1e-9)
    assert np.allclose(e, exact, atol=10 * tol)
    # Ritz vectors are eigenvectors: residual norm below sqrt(tol)
    X = x.cpu().numpy()
    for k in range(4):
        r = A @ X[k] - e[k] * X[k]
        assert np.linalg.norm(r) < np.sqrt(tol) * 1.5


def test_davidson_rejects_too_many_roots():
    n = 5
    x0 = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(rt.RTError):
        rt.davidson_solve(lambda X: X, x0, x0, rt.DavidsonParams(nroots=3))
