"""The large-system flow (split RI transform + RI-K, then Davidson on the
implicit response matrix) at a scaled-down size, against the CPU oracle.

The full-size run (nbas=1200, naux=4800, nocc=120, 55 GB of ri3ao) is in
bench.py; here nbas=160, naux=640, nocc=16 keep the oracle to seconds.
Tolerances: split ov within 1e-10 absolute, K within 1e-11 relative, E_x
within 1e-9 Eh.  Davidson follows the reference's convergence test (eigenvalue
change below tol and residual norm below sqrt(tol)); with tol = 1e-8 the eight
roots agree with a dense eigensolve to 1e-6 and every residual norm is below
1.5 sqrt(tol).
"""
import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

NB, NAUX, NOCC = 160, 640, 16


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))).cuda()


def test_synth_delta_matches_oracle():
    for nov in (1, 257, 14400):
        assert np.array_equal(rt.synth_delta(5, nov).cpu().numpy(), oracle.synth_delta(5, nov))


@pytest.fixture(scope="module")
def system():
    C = oracle.synth_coef(9, NB)
    B = oracle.synth_ri3ao(9, NB, NAUX)
    return C, B


def test_split_rik_and_exchange_energy(system):
    C, B = system
    nvir = NB - NOCC
    ov_ref, K_ref = oracle.ri_ov_k(C, B, NOCC)
    Cocc = C[:, :NOCC]
    D = Cocc @ Cocc.T
    ex_ref = oracle.exchange_energy(D, K_ref)
    ov, K = rt.ri_ov_k(dev(C), dev(B), NB, NAUX, NOCC, nvir, form="split", nslices=7)
    rt.sync_status()
    assert np.max(np.abs(ov.cpu().numpy().reshape(NOCC, nvir, NAUX, order="F") - ov_ref)) < 1e-10
    Kh = K.cpu().numpy().reshape(NB, NB, order="F")
    assert np.max(np.abs(Kh - K_ref)) < 1e-11 * np.max(np.abs(K_ref))
    ex = rt.exchange_energy(dev(D), K, NB).item()
    assert abs(ex - ex_ref) < 1e-9


@pytest.mark.parametrize("nv", [NOCC, NB - NOCC])
def test_davidson_eight_roots(system, nv):
    C, B = system
    nov = NOCC * nv
    ov_ref, _ = oracle.ri_ov_k(C[:, :NOCC + nv], B, NOCC)
    Bov = np.asfortranarray(ov_ref.reshape(nov, NAUX, order="F"))
    gamma = 0.3 / np.sqrt(np.mean(np.sum(Bov * Bov, axis=1)))
    Bov *= gamma
    d = oracle.synth_delta(4, nov)
    A = np.diag(d) + Bov @ Bov.T
    exact = np.linalg.eigvalsh(A)[:8]
    hd = np.diag(A)
    x0 = np.zeros(nov)
    x0[np.argmin(hd)] = 1.0
    conv, e, x, its = rt.davidson_ri_response(dev(Bov), rt.synth_delta(4, nov), nov, NAUX, dev(x0),
                                              rt.DavidsonParams(tol=1e-8, maxcyc=100, maxspace=24, nroots=8),
                                              form="split", nslices=7)
    assert all(conv)
    assert np.max(np.abs(np.array(e) - exact)) < 1e-6
    X = x.cpu().numpy()
    for k in range(8):
        assert np.linalg.norm(A @ X[k] - e[k] * X[k]) < 1.5e-4
