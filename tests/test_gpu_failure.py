"""Failure detection without a GPU fault.

* Scratch exhaustion: an allocator hook makes the n-th scratch allocation of a
  call fail; the call returns RT_ERR_NO_MEMORY (no abort, no partial output
  trusted), releases what it holds, and the next call succeeds and matches the
  oracle.
* Bounded waits: every pipeline wait in the library has a clock64 budget and
  records a timeout in the device error word instead of spinning forever.  A
  one-thread kernel runs that path out on purpose (a barrier nothing arrives
  at, ~1 ms budget); rt_sync_status reports RT_ERR_TIMEOUT, clears the word,
  and the context keeps working.
"""
import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RT_ERR_NO_MEMORY, RT_ERR_TIMEOUT = 3, 6


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))).cuda()


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_injected_allocation_failure_is_reported_and_recovers(form):
    nb, naux, nocc = 40, 30, 6
    nvir = nb - nocc
    C, B = oracle.synth_coef(2, nb), oracle.synth_ri3ao(2, nb, naux)
    dC, dB = dev(C), dev(B)
    for n in ((0,) if form == "fp64" else (0, 1, 2, 3)):
        rt.debug_fail_alloc_after(n)
        try:
            with pytest.raises(rt.RTError) as ei:
                rt.ri_ov_k(dC, dB, nb, naux, nocc, nvir, form=form, nslices=7)
            assert ei.value.status == RT_ERR_NO_MEMORY
            assert "injected" in str(ei.value)
        finally:
            rt.debug_fail_alloc_after(-1)
    torch.cuda.synchronize()
    rt.sync_status()
    ov, K = rt.ri_ov_k(dC, dB, nb, naux, nocc, nvir, form=form, nslices=7)
    ov_ref, K_ref = oracle.ri_ov_k(C, B, nocc)
    assert np.max(np.abs(ov.cpu().numpy().reshape(nocc, nvir, naux, order="F") - ov_ref)) < 1e-10
    Kh = K.cpu().numpy().reshape(nb, nb, order="F")
    assert np.max(np.abs(Kh - K_ref)) < 1e-11 * np.max(np.abs(K_ref))


def test_injected_allocation_failure_in_batched_entry():
    nb, naux, nocc = 24, 20, 4
    C, B = oracle.synth_coef(3, nb), oracle.synth_ri3ao(3, nb, naux)
    probs = [dict(C=dev(C), B=dev(B), nb=nb, naux=naux, nocc=nocc, nvir=nb - nocc,
                  ov=torch.zeros(nocc * (nb - nocc) * naux, dtype=torch.float64, device="cuda"),
                  K=torch.zeros(nb * nb, dtype=torch.float64, device="cuda"))]
    rt.debug_fail_alloc_after(0)
    try:
        with pytest.raises(rt.RTError) as ei:
            rt.ri_ov_k_batched(probs, form="split", nslices=7, tuning=(0, 0))
        assert ei.value.status == RT_ERR_NO_MEMORY
    finally:
        rt.debug_fail_alloc_after(-1)
    rt.ri_ov_k_batched(probs, form="split", nslices=7, tuning=(0, 0))
    rt.sync_status()
    _, K_ref = oracle.ri_ov_k(C, B, nocc)
    assert np.max(np.abs(probs[0]["K"].cpu().numpy().reshape(nb, nb, order="F") - K_ref)) < 1e-11 * np.abs(K_ref).max()


def test_bounded_wait_runs_out_and_context_survives():
    torch.cuda.synchronize()
    rt.sync_status()
    rt.debug_wait_timeout(2_000_000)  # about 1 ms at 2 GHz
    with pytest.raises(rt.RTError) as ei:
        rt.sync_status()
    assert ei.value.status == RT_ERR_TIMEOUT
    rt.sync_status()  # the word was cleared
    A = torch.randn(70, 50, dtype=torch.float64, device="cuda")
    Bm = torch.randn(50, 40, dtype=torch.float64, device="cuda")
    Cm = torch.empty(40, 70, dtype=torch.float64, device="cuda")  # column-major 70 x 40
    rt.dgemm("N", "N", 70, 40, 50, 1.0, A.t().contiguous(), 70, Bm.t().contiguous(), 50, 0.0, Cm, 70)
    rt.sync_status()
    assert torch.allclose(Cm.t(), A @ Bm, rtol=1e-12, atol=1e-12)


def test_wait_budget_is_validated():
    with pytest.raises(rt.RTError):
        rt.debug_wait_timeout(-1)
    with pytest.raises(rt.RTError):
        rt.debug_wait_timeout(3_000_000_000)


def test_wrappers_refuse_undersized_or_host_tensors():
    # An undersized output is refused in Python, before any kernel could write past its end.
    nb, naux, nocc, nvir = 16, 4, 3, 13
    C = rt.synth_coef(0, nb)
    B = rt.synth_ri3ao(0, nb, naux)
    K = torch.empty(nb * nb - 1, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="K"):
        rt.ri_ov_k(C, B, nb, naux, nocc, nvir, K=K)
    with pytest.raises(ValueError, match="B"):
        rt.ri_j(B[:-1], torch.zeros(nb * nb, dtype=torch.float64, device="cuda"), nb, naux)
    with pytest.raises(TypeError):
        rt.ri_ov_k(C.cpu(), B, nb, naux, nocc, nvir)
