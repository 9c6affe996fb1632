"""The CPU oracle, pinned to the reference's own known answers and to numpy."""
import json
import os

import numpy as np
import pytest

import oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_doctests.json")))


def _case(name):
    return next(c for c in GOLD["cases"] if c["name"] == name)


def _mat_1_9():
    return np.asfortranarray(np.arange(1, 10, dtype=np.float64).reshape(3, 3, order="F"))


@pytest.mark.parametrize("name", ["general_dgemm_f", "_dgemm_0", "_dgemm_1", "_dgemm_2"])
def test_gemm_seam_doctests(name):
    c = _case(name)
    a = _mat_1_9()
    b = a + 5.0
    out = np.full((3, 3), c["c_init"], order="F")
    oracle.general_dgemm_f(a, c["rows_a"], c["cols_a"], c["opa"], b, c["rows_b"], c["cols_b"], c["opb"],
                           out, c["rows_c"], c["cols_c"], c["alpha"], c["beta"])
    r0, r1 = c["check_rows"]
    c0, c1 = c["check_cols"]
    got = out[r0:r1, c0:c1].flatten(order="F")
    assert got.tolist() == c["expected"]


def test_dsyev_doctest_and_dspevx_agree():
    c = _case("_dsyev")
    full = np.zeros((3, 3), order="F")
    idx = 0
    for j in range(3):
        for i in range(j + 1):
            full[i, j] = full[j, i] = c["packed_upper"][idx]
            idx += 1
    vec, w = oracle.dsyev(full, "V")
    assert np.sum((w - np.array(c["eigval"])) ** 2) < c["tol_sq"]
    assert np.sum((vec.flatten(order="F") - np.array(c["eigvec"])) ** 2) < c["tol_sq"]
    z, w2, nf = oracle.dspevx_packed(np.array(c["packed_upper"]))
    assert nf == 3
    assert np.allclose(w2, c["eigval"], atol=1e-12)
    # eigenvectors agree up to sign
    for k in range(3):
        assert abs(abs(np.dot(z[:, k], vec[:, k])) - 1.0) < 1e-12


def test_bench_ao2mo_known_answer():
    c = _case("bench_ao2mo")
    nb, _, naux = c["ri3fn_size"]
    B = np.full((nb, nb, naux), c["ri3fn_fill"], order="F")
    C = np.full(tuple(c["eigenvector_size"]), c["eigenvector_fill"], order="F")
    out = oracle.ri_ao2mo(C, B)
    assert out.shape == (naux, C.shape[1], C.shape[1])
    assert np.all(out == c["expected_every_element"])


def _inputs(nb, naux, seed=0):
    return oracle.synth_coef(seed, nb), oracle.synth_ri3ao(seed, nb, naux)


def test_synth_symmetry_and_orthogonality():
    C, B = _inputs(17, 5)
    assert np.array_equal(B, B.transpose(1, 0, 2))
    assert np.allclose(C.T @ C, np.eye(17), atol=1e-13)


def test_ri_ao2mo_matches_einsum():
    C, B = _inputs(24, 9, seed=3)
    ref = np.einsum("mp,mnP,nq->Ppq", C, B, C)
    out = oracle.ri_ao2mo(C, B)
    assert np.max(np.abs(out - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))


def test_ri_ao2mo_identity_and_norm():
    _, B = _inputs(16, 4, seed=5)
    out = oracle.ri_ao2mo(np.eye(16, order="F"), B)
    assert np.array_equal(out, B.transpose(2, 0, 1))
    C, _ = _inputs(16, 4, seed=6)
    out = oracle.ri_ao2mo(C, B)
    for P in range(4):
        assert abs(np.sum(out[P] ** 2) - np.sum(B[:, :, P] ** 2)) < 1e-11 * np.sum(B[:, :, P] ** 2)


def test_ri_ov_k_j_exchange():
    nb, naux, nocc = 20, 12, 4
    C, B = _inputs(nb, naux, seed=7)
    ov, K = oracle.ri_ov_k(C, B, nocc)
    Co, Cv = C[:, :nocc], C[:, nocc:]
    ov_ref = np.einsum("mi,mnP,na->iaP", Co, B, Cv)
    X = np.einsum("mnP,ni->miP", B, Co)
    K_ref = np.einsum("miP,niP->mn", X, X)
    assert np.max(np.abs(ov - ov_ref)) < 1e-12
    assert np.max(np.abs(K - K_ref)) < 1e-11
    assert np.max(np.abs(K - K.T)) < 1e-12
    D = Co @ Co.T
    ex = oracle.exchange_energy(D, K)
    full = oracle.ri_ao2mo(C, B)
    ex_ref = -np.sum(full[:, :nocc, :nocc] ** 2)
    assert abs(ex - ex_ref) < 1e-11 * abs(ex_ref)
    w, J = oracle.ri_j(B, D)
    assert np.allclose(w, np.einsum("mnP,mn->P", B, D), atol=1e-12)
    assert np.allclose(J, np.einsum("mnP,P->mn", B, w), atol=1e-11)


def test_iajb_and_matvec():
    rng = np.random.default_rng(1)
    Bov = np.asfortranarray(rng.standard_normal((30, 7)))
    M = oracle.iajb(Bov)
    assert np.allclose(M, Bov @ Bov.T, atol=1e-12)
    d = oracle.synth_delta(0, 30)
    assert d.min() >= 0.5 and d.max() <= 3.0
    X = np.asfortranarray(rng.standard_normal((30, 3)))
    AX = oracle.response_matvec(Bov, d, X)
    assert np.allclose(AX, d[:, None] * X + Bov @ (Bov.T @ X), atol=1e-12)


def test_davidson_oracle_lowest_roots():
    rng = np.random.default_rng(2)
    n, naux = 60, 6
    Bov = rng.standard_normal((n, naux)) * 0.3
    d = oracle.synth_delta(4, n)
    A = np.diag(d) + Bov @ Bov.T
    p = oracle.DavidsonParams(tol=1e-10, maxcyc=100, maxspace=20, nroots=3)
    x0 = np.zeros(n)
    x0[np.argmin(d)] = 1.0
    conv, e, xs = oracle.davidson_solve(lambda x: A @ x, x0, d.copy(), p)
    ref = np.linalg.eigvalsh(A)[:3]
    assert all(conv)
    assert np.allclose(e, ref, atol=1e-8)
