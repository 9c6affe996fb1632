"""The allocation-free float64 ov transform + RI-K entry point.

Some callers cannot allocate device memory while they run: a host that hands
all GPU memory to a fixed arena owned by another runtime, or a serving loop
where cudaMalloc/cudaFree (and their implicit synchronisation) are not
allowed.  For them,
rt_ri_ov_k_fp64_noalloc keeps its half-transform in a fixed 32 MiB device
array and streams the aux slabs through it.  These tests call it through the
C ABI twice in a row (the array keeps the previous call's contents) and
compare with rt_ri_ov_k in the float64 form, to the float64 tolerance used
by the other parity tests (1e-12 relative to the largest element).

This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _entry():
    L = rt.lib()
    f = L.rt_ri_ov_k_fp64_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return L, f


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("nb,naux,nocc", [(600, 300, 60), (33, 7, 5)])
def test_noalloc_matches_fp64_entry_on_two_calls(nb, naux, nocc):
    # nb=600, nocc=60: 116 slabs fit the fixed array, so 300 slabs take three blocks.
    L, f = _entry()
    nvir = nb - nocc
    B = rt.synth_ri3ao(4, nb, naux)
    C = rt.synth_coef(4, nb)
    ov_ref, K_ref = rt.ri_ov_k(C, B, nb, naux, nocc, nvir, form="fp64")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        ov = torch.full((nocc * nvir * naux,), float("nan"), dtype=torch.float64, device="cuda")
        K = torch.full((nb * nb,), float("nan"), dtype=torch.float64, device="cuda")
        st = f(C.data_ptr(), B.data_ptr(), nb, naux, nocc, nvir, ov.data_ptr(), K.data_ptr(), stream)
        assert st == 0, L.rt_last_error()
        torch.cuda.synchronize()
        assert _rel(ov, ov_ref) < 1e-12
        assert _rel(K, K_ref) < 1e-12


def test_noalloc_rejects_sizes_beyond_its_array():
    L, f = _entry()
    # nb * nocc = 4.5M doubles > 4,194,304 (32 MiB): refused before any device work.
    st = f(None, None, 3000, 4, 1500, 10, None, None, None)
    assert st == 1
    assert b"exceeds the fixed scratch" in L.rt_last_error()


def _call(f, C, B, nb, naux, nocc, nvir, ov, K):
    stream = torch.cuda.current_stream().cuda_stream
    p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    return f(p(C), p(B), nb, naux, nocc, nvir, p(ov), p(K), stream)


@pytest.mark.parametrize("nocc,naux", [(0, 6), (5, 0)])
def test_noalloc_empty_contraction_zeroes_k(nocc, naux):
    # No occupied orbitals or no aux slabs: K is zero and ov has no elements, as in rt_ri_ov_k.
    L, f = _entry()
    nb, nvir = 20, 15
    C = rt.synth_coef(1, nb)
    B = rt.synth_ri3ao(1, nb, max(naux, 1))
    K = torch.full((nb * nb,), float("nan"), dtype=torch.float64, device="cuda")
    ov = torch.empty(max(nocc * nvir * naux, 1), dtype=torch.float64, device="cuda")
    assert _call(f, C, B, nb, naux, nocc, nvir, ov, K) == 0, L.rt_last_error()
    torch.cuda.synchronize()
    assert bool((K == 0).all())


def test_noalloc_single_outputs_and_no_virtuals():
    # ov only, K only, and nvir = 0 (K only, nothing to write in ov), each twice in a row.
    L, f = _entry()
    nb, naux, nocc = 40, 9, 6
    nvir = nb - nocc
    B = rt.synth_ri3ao(2, nb, naux)
    C = rt.synth_coef(2, nb)
    ov_ref, K_ref = rt.ri_ov_k(C, B, nb, naux, nocc, nvir, form="fp64")
    _, K0_ref = rt.ri_ov_k(C[: nb * nocc], B, nb, naux, nocc, 0, form="fp64", want_ov=False)
    for _ in range(2):
        ov = torch.full((nocc * nvir * naux,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(f, C, B, nb, naux, nocc, nvir, ov, None) == 0, L.rt_last_error()
        K = torch.full((nb * nb,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(f, C, B, nb, naux, nocc, nvir, None, K) == 0, L.rt_last_error()
        K0 = torch.full((nb * nb,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(f, C[: nb * nocc], B, nb, naux, nocc, 0, None, K0) == 0, L.rt_last_error()
        torch.cuda.synchronize()
        assert _rel(ov, ov_ref) < 1e-12
        assert _rel(K, K_ref) < 1e-12
        assert _rel(K0, K0_ref) < 1e-12
