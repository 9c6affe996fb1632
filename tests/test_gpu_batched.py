"""Batched uneven-molecule ov transform + RI-K (rt_ri_ov_k_batched) on the GPU.

A batch of molecules of different sizes runs as one grouped launch per product
(X = B C_occ, ov, K).  Checked against the CPU oracle per molecule with the
tolerances of the single-molecule parity tests (float64 form 1e-12 relative;
split form ov within 1e-10 absolute and K within 1e-11 relative), against the
single-molecule entry point, for every tuning candidate, and replayed from a
CUDA graph.
"""
import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt
from rest_tensors_gb300 import autotune

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# (nb, naux, nocc): uneven sizes, a molecule with no virtuals, one with no
# occupied orbitals, a multi-chunk contraction (nb > 640) and tiny ones.
SHAPES = [(40, 60, 5), (72, 100, 9), (24, 30, 3), (130, 200, 12), (64, 16, 64), (20, 12, 0), (700, 3, 6),
          (9, 5, 2)]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))).cuda()


def host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b))))


def make_batch(shapes, seed0=0):
    probs, refs = [], []
    for i, (nb, naux, nocc) in enumerate(shapes):
        C = oracle.synth_coef(seed0 + i, nb)
        B = oracle.synth_ri3ao(seed0 + i, nb, naux)
        nvir = nb - nocc
        probs.append(dict(C=dev(C), B=dev(B), nb=nb, naux=naux, nocc=nocc, nvir=nvir,
                          ov=torch.full((max(1, nocc * nvir * naux),), float("nan"), dtype=torch.float64,
                                        device="cuda"),
                          K=torch.full((nb * nb,), float("nan"), dtype=torch.float64, device="cuda")))
        refs.append(oracle.ri_ov_k(C, B, nocc) if nocc > 0 else (None, np.zeros((nb, nb))))
    return probs, refs


def check(probs, refs, form):
    for q, (ov_ref, K_ref) in zip(probs, refs):
        nb, naux, nocc, nvir = q["nb"], q["naux"], q["nocc"], q["nvir"]
        K = host(q["K"], (nb, nb))
        if nocc == 0:
            assert np.count_nonzero(K) == 0
            continue
        if form == "fp64":
            assert relerr(K, K_ref) < 1e-12
            if nvir:
                assert relerr(host(q["ov"][:nocc * nvir * naux], (nocc, nvir, naux)), ov_ref) < 1e-12
        else:
            assert relerr(K, K_ref) < 1e-11
            assert np.array_equal(K, K.T)
            if nvir:
                assert np.max(np.abs(host(q["ov"][:nocc * nvir * naux], (nocc, nvir, naux)) - ov_ref)) < 1e-10


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_batched_matches_oracle(form):
    probs, refs = make_batch(SHAPES)
    rt.ri_ov_k_batched(probs, form=form, nslices=7)
    rt.sync_status()
    check(probs, refs, form)


@pytest.mark.parametrize("tuning", autotune.CANDIDATES)
def test_every_tuning_candidate_is_correct(tuning):
    probs, refs = make_batch(SHAPES[:5], seed0=10)
    rt.ri_ov_k_batched(probs, form="split", nslices=7, tuning=tuning)
    rt.sync_status()
    check(probs, refs, "split")


def test_batched_agrees_with_single_molecule_entry():
    probs, _ = make_batch(SHAPES[:4], seed0=20)
    rt.ri_ov_k_batched(probs, form="split", nslices=7)
    for q in probs:
        ov, K = rt.ri_ov_k(q["C"], q["B"], q["nb"], q["naux"], q["nocc"], q["nvir"], form="split", nslices=7)
        n = q["nocc"] * q["nvir"] * q["naux"]
        assert float((q["ov"][:n] - ov).abs().max()) <= 1e-13 * float(ov.abs().max())
        assert float((q["K"] - K).abs().max()) <= 1e-13 * float(K.abs().max())


def test_more_molecules_than_one_launch_holds():
    # 60 molecules: the split form needs two grouped launches per product (48 + 12).
    shapes = [(16 + 4 * (i % 9), 8 + i % 5, 2 + i % 3) for i in range(60)]
    probs, refs = make_batch(shapes, seed0=100)
    rt.ri_ov_k_batched(probs, form="split", nslices=7)
    rt.ri_ov_k_batched([dict(q) for q in probs], form="split", nslices=7)
    rt.sync_status()
    check(probs, refs, "split")


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_batched_cuda_graph_replay(form):
    probs, refs = make_batch(SHAPES[:4], seed0=30)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        rt.ri_ov_k_batched(probs, form=form, nslices=7, tuning=(0, 0), stream=s)   # sets kernel attributes
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    for q in probs:
        q["K"].fill_(float("nan"))
    with torch.cuda.graph(g):
        rt.ri_ov_k_batched(probs, form=form, nslices=7, tuning=(0, 0))
    torch.cuda.synchronize()
    # New coefficients copied into the captured input buffers, then replay.
    new_refs = []
    for i, q in enumerate(probs):
        C = oracle.synth_coef(500 + i, q["nb"])
        q["C"].copy_(dev(C))
        Bh = oracle.synth_ri3ao(30 + i, q["nb"], q["naux"])
        new_refs.append(oracle.ri_ov_k(C, Bh, q["nocc"]))
    g.replay()
    torch.cuda.synchronize()
    rt.sync_status()
    check(probs, new_refs, form)
    g.replay()
    torch.cuda.synchronize()
    check(probs, new_refs, form)


def test_autotune_lookup_tunes_once_and_persists(tmp_path, monkeypatch):
    monkeypatch.setenv("RT_TUNE_TABLE", str(tmp_path / "tune.json"))
    autotune.reset_cache()
    probs, refs = make_batch(SHAPES[:3], seed0=40)
    rt.ri_ov_k_batched(probs, form="split", nslices=7, tuning="auto")
    check(probs, refs, "split")
    assert (tmp_path / "tune.json").exists()
    key = autotune.shape_key(probs, "split", 7)
    autotune.reset_cache()
    t = autotune.lookup(probs, "split", 7, tune_on_miss=False)
    assert t is not None and (t.fuse, t.chunks_per_item) in autotune.CANDIDATES
    assert key in open(tmp_path / "tune.json").read()
    autotune.reset_cache()


def test_batched_rejects_bad_arguments():
    probs, _ = make_batch(SHAPES[:2])
    with pytest.raises(rt.RTError):
        rt.ri_ov_k_batched(probs, form="split", nslices=9)
    bad = [dict(probs[0], nb=-1)]
    with pytest.raises(rt.RTError):
        rt.ri_ov_k_batched(bad, form="fp64")
    rt.ri_ov_k_batched([], form="split")
