"""ri3ao prepared once for repeated split-form ov + RI-K (rt_ri3ao_prepare,
rt_ri_ov_k_prepared), as in an SCF loop where ri3fn stays fixed while the
orbitals change.

The half-transform never splits its contraction, so each element is computed
the same way whether ri3ao is sliced per call or once beforehand: the
prepared results must equal rt_ri_ov_k's split form bit for bit, for several
orbital sets in a row and for shapes whose half-transform rows cross slab and
tile boundaries.  They are also checked against the oracle (1e-10 absolute on
ov, 1e-11 relative on K).
"""
import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nb,naux,nocc,S", [(100, 40, 20, 7), (33, 9, 5, 6), (600, 96, 60, 7)])
def test_prepared_equals_the_split_entry_bitwise(nb, naux, nocc, S):
    nvir = nb - nocc
    B = rt.synth_ri3ao(11, nb, naux)
    prep = rt.Ri3aoPrepared(B, nb, naux, nslices=S)
    assert prep.nbytes() >= 2 * S * nb * nb * naux
    for seed in (1, 2, 3):  # new orbitals each "iteration"
        C = rt.synth_coef(seed, nb)
        ov_ref, K_ref = rt.ri_ov_k(C, B, nb, naux, nocc, nvir, form="split", nslices=S)
        ov, K = prep.ri_ov_k(C, nocc, nvir)
        rt.sync_status()
        assert torch.equal(ov, ov_ref) and torch.equal(K, K_ref)
    prep.release()
    prep.release()  # idempotent


def test_prepared_matches_oracle_and_single_outputs():
    nb, naux, nocc = 64, 30, 9
    nvir = nb - nocc
    B = rt.synth_ri3ao(5, nb, naux)
    C = rt.synth_coef(5, nb)
    ov_ref, K_ref = oracle.ri_ov_k(C.cpu().numpy().reshape(nb, nb, order="F"),
                                   B.view(naux, nb, nb).cpu().numpy().transpose(2, 1, 0), nocc)
    prep = rt.Ri3aoPrepared(B, nb, naux)
    ov, _ = prep.ri_ov_k(C, nocc, nvir, want_k=False)
    _, K = prep.ri_ov_k(C, nocc, nvir, want_ov=False)
    rt.sync_status()
    assert np.max(np.abs(ov.cpu().numpy().reshape(nocc, nvir, naux, order="F") - ov_ref)) < 1e-10
    Kh = K.cpu().numpy().reshape(nb, nb, order="F")
    assert np.max(np.abs(Kh - K_ref)) / np.max(np.abs(K_ref)) < 1e-11
    _, K0 = prep.ri_ov_k(C, 0, nb, want_ov=False)  # no occupied orbitals: K = 0
    assert torch.count_nonzero(K0).item() == 0


def test_prepare_rejects_bad_arguments():
    B = rt.synth_ri3ao(0, 8, 2)
    with pytest.raises(rt.RTError):
        rt.Ri3aoPrepared(B, 8, 2, nslices=9)
    with pytest.raises(ValueError):
        rt.Ri3aoPrepared(B, 8, 4)  # B holds 2 slabs, not 4
    prep = rt.Ri3aoPrepared(B, 8, 2)
    prep.release()
    with pytest.raises(ValueError):
        prep.ri_ov_k(rt.synth_coef(0, 8), 2, 6)
