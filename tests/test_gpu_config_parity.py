"""Oracle parity at the measured workloads' own sizes.

The other parity tests run small and odd shapes.  These run the shapes the
bench measures, on the same synthetic inputs: ri3ao and C are generated on the
device, copied to the host and handed to the oracle, so both sides see the
same bits.

  * nbas=600, naux=2400, nocc=60 (the headline workload) in both forms;
  * a batch of uneven molecules (nbas uniform in [40, 400], naux = 4 nbas,
    nocc = round(nbas / 10)) through the grouped entry point;
  * nbas=1200, nocc=120 on a slab subset (the whole 55 GB tensor does not
    belong in a test).

Tolerances: float64 form 1e-12 relative to max|oracle|; split form 1e-10
absolute on ov (values O(0.1-1)), 1e-11 relative on K, 1e-9 Eh on E_x.
"""
import os

import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def to_host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b))))


def density(C, nocc):
    Co = C[:, :nocc]
    return np.asfortranarray(Co @ Co.T)


def check(nb, naux, nocc, B, C, ov_ref, K_ref, ex_ref, forms=("fp64", "split")):
    nvir = nb - nocc
    Ch = to_host(C, (nb, nb))
    D = rt_dev(density(Ch, nocc))
    for form in forms:
        ov, K = rt.ri_ov_k(C, B, nb, naux, nocc, nvir, form=form)
        ex = rt.exchange_energy(D, K, nb).item()
        rt.sync_status()
        ov_h, K_h = to_host(ov, (nocc, nvir, naux)), to_host(K, (nb, nb))
        if form == "fp64":
            assert relerr(ov_h, ov_ref) < 1e-12
            assert relerr(K_h, K_ref) < 1e-12
            assert abs(ex - ex_ref) / abs(ex_ref) < 1e-12
        else:
            assert np.max(np.abs(ov_h - ov_ref)) < 1e-10
            assert relerr(K_h, K_ref) < 1e-11
            assert abs(ex - ex_ref) < 1e-9


def rt_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).cuda()


def test_headline_workload_matches_oracle():
    nb, naux, nocc = 600, 2400, 60
    B = rt.synth_ri3ao(0, nb, naux)
    C = rt.synth_coef(0, nb)
    Bh = B.view(naux, nb, nb).cpu().numpy().transpose(2, 1, 0)  # Fortran-ordered [nb, nb, naux] view
    Ch = to_host(C, (nb, nb))
    oracle.set_threads(os.cpu_count() or 1)
    ov_ref, K_ref = oracle.ri_ov_k(Ch, Bh, nocc)
    ex_ref = oracle.exchange_energy(density(Ch, nocc), K_ref)
    del Bh
    check(nb, naux, nocc, B, C, ov_ref, K_ref, ex_ref)


def test_uneven_batch_matches_oracle_per_molecule():
    rng = np.random.default_rng(0)
    shapes = [(int(nb), 4 * int(nb), int(round(nb / 10))) for nb in rng.integers(40, 401, size=8)]
    probs, refs = [], []
    oracle.set_threads(os.cpu_count() or 1)
    for k, (nb, naux, nocc) in enumerate(shapes):
        nvir = nb - nocc
        B = rt.synth_ri3ao(k, nb, naux)
        C = rt.synth_coef(k, nb)
        Ch = to_host(C, (nb, nb))
        ov_ref, K_ref = oracle.ri_ov_k(Ch, B.view(naux, nb, nb).cpu().numpy().transpose(2, 1, 0), nocc)
        refs.append((ov_ref, K_ref))
        probs.append(dict(C=C, B=B, nb=nb, naux=naux, nocc=nocc, nvir=nvir,
                          ov=torch.empty(nocc * nvir * naux, dtype=torch.float64, device="cuda"),
                          K=torch.empty(nb * nb, dtype=torch.float64, device="cuda")))
    for form in ("fp64", "split"):
        rt.ri_ov_k_batched(probs, form=form)
        rt.sync_status()
        for q, (ov_ref, K_ref) in zip(probs, refs):
            ov_h = to_host(q["ov"], (q["nocc"], q["nvir"], q["naux"]))
            K_h = to_host(q["K"], (q["nb"], q["nb"]))
            if form == "fp64":
                assert relerr(ov_h, ov_ref) < 1e-12 and relerr(K_h, K_ref) < 1e-12
            else:
                assert np.max(np.abs(ov_h - ov_ref)) < 1e-10 and relerr(K_h, K_ref) < 1e-11


def test_large_system_slab_subset_matches_oracle():
    nb, nocc, nsub = 1200, 120, 48
    # slabs 1000..1047 of the naux=4800 tensor: the generator is keyed on the slab index
    B = rt.synth_ri3ao(0, nb, nsub, P0=1000)
    C = rt.synth_coef(0, nb)
    Ch = to_host(C, (nb, nb))
    oracle.set_threads(os.cpu_count() or 1)
    ov_ref, K_ref = oracle.ri_ov_k(Ch, B.view(nsub, nb, nb).cpu().numpy().transpose(2, 1, 0), nocc)
    ex_ref = oracle.exchange_energy(density(Ch, nocc), K_ref)
    check(nb, nsub, nocc, B, C, ov_ref, K_ref, ex_ref)
