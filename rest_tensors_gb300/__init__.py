"""GB300 (sm_103a) implementation of rest_tensors' dense RI contraction path.

The compute lives in ``librest_tensors_gb300.so`` (CUDA C++, C ABI declared
in ``include/rest_tensors_gb300.h``).  This module is the host-side mirror of
the reference's Rust interface for the path, with the same names, argument
meaning and error behaviour:

* ``RIFull`` / ``MatrixFull``: column-major containers (src/ri.rs:19-40,
  src/matrix/mod.rs:473-480) with ``RIFull.ao2mo`` (src/ri.rs:356-408) running
  through the drop-in ``ri_ao2mo_f_`` symbol;
* ``general_dgemm_f`` and ``_dgemm`` (src/external_libs/mod.rs:60-83,
  src/matrix/matrix_blas_lapack.rs:122-178) through ``general_dgemm_f_``;
* device-tensor entry points (``ri_ov_k``, ``ri_ao2mo``, ``ri_j``,
  ``exchange_energy``, ``dgemm``) taking torch CUDA tensors, for callers that
  keep data resident in HBM.

There is no CPU fallback: if the native library cannot be loaded, every call
raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librest_tensors_gb300.so")

RT_OK = 0
RT_FORM_FP64 = 0
RT_FORM_SPLIT = 1
DEFAULT_NSLICES = 7

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


class _DavidsonParamsC(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("maxcyc", ctypes.c_int), ("maxspace", ctypes.c_int),
                ("lindep", ctypes.c_double), ("nroots", ctypes.c_int)]


MATVEC_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong,
                             ctypes.c_void_p, ctypes.c_void_p)


class RiProblem(ctypes.Structure):
    """One molecule of a batch (``rt_ri_problem``): device addresses and sizes."""
    _fields_ = [("C", ctypes.c_void_p), ("B", ctypes.c_void_p), ("ov", ctypes.c_void_p), ("K", ctypes.c_void_p),
                ("nb", ctypes.c_int), ("naux", ctypes.c_int), ("nocc", ctypes.c_int), ("nvir", ctypes.c_int)]


class Tuning(ctypes.Structure):
    """Launch options of the split form (``rt_tuning``)."""
    _fields_ = [("fuse", ctypes.c_int), ("chunks_per_item", ctypes.c_int)]


class RTError(RuntimeError):
    """A non-zero rt_status from the native library."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"rt_status {status}: {msg}")
        self.status = status


def lib() -> ctypes.CDLL:
    """Load the native library (building it in-tree if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build

        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    c_int, c_dbl, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    L.rt_version.restype = c_int
    L.rt_status_string.restype = ctypes.c_char_p
    L.rt_status_string.argtypes = [c_int]
    L.rt_last_error.restype = ctypes.c_char_p
    L.rt_last_status.restype = c_int
    L.rt_sync_status.restype = c_int
    L.rt_sync_status.argtypes = [vp]
    L.rt_dgemm.restype = c_int
    L.rt_dgemm.argtypes = [ctypes.c_char, ctypes.c_char, c_int, c_int, c_int, c_dbl, vp, c_int, vp, c_int, c_dbl, vp,
                           c_int, vp]
    L.rt_dgemm_split.restype = c_int
    L.rt_dgemm_split.argtypes = [ctypes.c_char, ctypes.c_char, c_int, c_int, c_int, vp, c_int, vp, c_int, vp, c_int,
                                 c_int, vp]
    L.rt_ri_ao2mo.restype = c_int
    L.rt_ri_ao2mo.argtypes = [vp, vp, vp, c_int, c_int, c_int, c_int, c_int, vp]
    L.rt_ri_ov_k.restype = c_int
    L.rt_ri_ov_k.argtypes = [vp, vp, c_int, c_int, c_int, c_int, vp, vp, c_int, c_int, vp]
    L.rt_ri_ov_k_batched.restype = c_int
    L.rt_ri_ov_k_batched.argtypes = [ctypes.POINTER(RiProblem), c_int, c_int, c_int, ctypes.POINTER(Tuning), vp]
    L.rt_ri_ov_k_host.restype = c_int
    L.rt_ri_ov_k_host.argtypes = [vp, vp, c_int, c_int, c_int, c_int, vp, vp, c_int, c_int, vp]
    L.rt_ri_ao2mo_host.restype = c_int
    L.rt_ri_ao2mo_host.argtypes = [vp, vp, vp, c_int, c_int, c_int, c_int, c_int, vp]
    L.rt_ri_ov_k_host_symmetric.restype = c_int
    L.rt_ri_ov_k_host_symmetric.argtypes = [vp, vp, c_int, c_int, c_int, c_int, vp, vp, c_int, c_int, vp]
    L.rt_ri_ov_k_fp64_noalloc.restype = c_int
    L.rt_ri_ov_k_fp64_noalloc.argtypes = [vp, vp, c_int, c_int, c_int, c_int, vp, vp, vp]
    L.rt_ri3ao_prepare.restype = c_int
    L.rt_ri3ao_prepare.argtypes = [vp, c_int, c_int, c_int, ctypes.POINTER(vp), vp]
    L.rt_ri3ao_prepared_bytes.restype = c_int
    L.rt_ri3ao_prepared_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    L.rt_ri_ov_k_prepared.restype = c_int
    L.rt_ri_ov_k_prepared.argtypes = [vp, vp, c_int, c_int, vp, vp, vp]
    L.rt_ri3ao_release.restype = c_int
    L.rt_ri3ao_release.argtypes = [vp]
    L.rt_ri_j.restype = c_int
    L.rt_ri_j.argtypes = [vp, vp, c_int, c_int, vp, vp, vp]
    L.rt_ri_j_symmetric.restype = c_int
    L.rt_ri_j_symmetric.argtypes = [vp, vp, c_int, c_int, vp, vp, vp]
    L.rt_ri_exchange_energy.restype = c_int
    L.rt_ri_exchange_energy.argtypes = [vp, vp, c_int, vp, vp]
    L.rt_synth_ri3ao.restype = c_int
    L.rt_synth_ri3ao.argtypes = [ctypes.c_uint64, c_int, c_int, c_int, vp, vp]
    L.rt_synth_delta.restype = c_int
    L.rt_synth_delta.argtypes = [ctypes.c_uint64, ctypes.c_longlong, vp, vp]
    L.rt_synth_coef_seed.restype = c_int
    L.rt_synth_coef_seed.argtypes = [ctypes.c_uint64, c_int, vp, vp]
    L.rt_launch_count.restype = ctypes.c_longlong
    L.rt_profile_enable.restype = None
    L.rt_profile_enable.argtypes = [c_int]
    L.rt_profile_get.restype = c_int
    L.rt_profile_get.argtypes = [c_int, ctypes.POINTER(c_dbl), ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(c_dbl)]
    L.rt_ri_iajb.restype = c_int
    L.rt_ri_iajb.argtypes = [vp, ctypes.c_longlong, c_int, vp, c_int, c_int, vp]
    L.rt_ri_response_matvec.restype = c_int
    L.rt_ri_response_matvec.argtypes = [vp, vp, ctypes.c_longlong, c_int, vp, vp, c_int, c_int, c_int, vp]
    L.rt_davidson_solve.restype = c_int
    L.rt_davidson_solve.argtypes = [MATVEC_FN, vp, vp, vp, ctypes.c_longlong, ctypes.POINTER(_DavidsonParamsC), c_int,
                                    ctypes.POINTER(c_int), ctypes.POINTER(c_dbl), vp, ctypes.POINTER(c_int), vp]
    L.rt_davidson_ri_response.restype = c_int
    L.rt_davidson_ri_response.argtypes = [vp, vp, ctypes.c_longlong, c_int, c_int, c_int, vp,
                                          ctypes.POINTER(_DavidsonParamsC), c_int, ctypes.POINTER(c_int),
                                          ctypes.POINTER(c_dbl), vp, ctypes.POINTER(c_int), vp]
    L.rt_debug_fail_alloc_after.restype = c_int
    L.rt_debug_fail_alloc_after.argtypes = [ctypes.c_longlong]
    L.rt_debug_wait_timeout.restype = c_int
    L.rt_debug_wait_timeout.argtypes = [ctypes.c_longlong, vp]
    L.rt_debug_chunk_bytes.restype = c_int
    L.rt_debug_chunk_bytes.argtypes = [ctypes.c_longlong]
    L.rt_special_dgemm_01.restype = c_int
    L.rt_special_dgemm_01.argtypes = [vp] + [c_int] * 7 + [vp] + [c_int] * 6 + [c_dbl, c_dbl, c_int, c_int, vp]
    L.rt_copy_mm.restype = c_int
    L.rt_copy_mm.argtypes = [c_int, c_int, vp, c_int, c_int, c_int, c_int, vp, c_int, c_int, c_int, c_int, vp]
    L.rt_copy_mr.restype = c_int
    L.rt_copy_mr.argtypes = [c_int, c_int, vp, c_int, c_int, c_int, c_int, vp] + [c_int] * 7 + [vp]
    L.rt_copy_rm.restype = c_int
    L.rt_copy_rm.argtypes = [c_int, c_int, vp] + [c_int] * 7 + [vp, c_int, c_int, c_int, c_int, vp]
    L.rt_copy_rr.restype = c_int
    L.rt_copy_rr.argtypes = [c_int] * 3 + [vp] + [c_int] * 6 + [vp] + [c_int] * 6 + [vp]
    L.rt_ri_transpose.restype = c_int
    L.rt_ri_transpose.argtypes = [vp, c_int, c_int, c_int, ctypes.c_char_p, vp, vp]
    L.rt_ri_pack_symm.restype = c_int
    L.rt_ri_pack_symm.argtypes = [vp, c_int, c_int, vp, vp]
    L.special_dgemm_f_01_.restype = None
    L.rt_newton_schulz_inv_sqrt.restype = c_int
    L.rt_newton_schulz_inv_sqrt.argtypes = [vp, c_int, c_dbl, c_dbl, c_int, ctypes.POINTER(c_dbl), c_int, c_int, c_int,
                                            vp, ctypes.POINTER(c_int), ctypes.POINTER(c_int), vp]
    L.rt_dsyev.restype = c_int
    L.rt_dsyev.argtypes = [c_int, vp, vp, vp]
    L.rt_lapack_power.restype = c_int
    L.rt_lapack_power.argtypes = [vp, c_int, c_dbl, c_dbl, vp, ctypes.POINTER(c_int), c_int, c_int, vp]
    L.rt_dspgvx.restype = c_int
    L.rt_dspgvx.argtypes = [vp, vp, c_int, c_int, vp, vp, c_int, c_int, vp]
    L.ri_ao2mo_f_.restype = None
    L.general_dgemm_f_.restype = None
    _lib = L
    return L


def _check(status: int) -> None:
    if status != RT_OK:
        L = lib()
        raise RTError(status, L.rt_last_error().decode(errors="replace"))


def last_status() -> int:
    return int(lib().rt_last_status())


# --------------------------------------------------------------------------
# Reference containers
# --------------------------------------------------------------------------
class MatrixFull:
    """Column-major rank-2 tensor (src/matrix/mod.rs:473-480): ``size=[rows, cols]``, ``indicing=[1, rows]``."""

    def __init__(self, size: Sequence[int], data: np.ndarray):
        self.size = [int(size[0]), int(size[1])]
        self.indicing = [1, self.size[0]]
        self.data = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1))
        if self.data.size < self.size[0] * self.size[1]:
            raise ValueError("MatrixFull::from_vec: vector shorter than the requested shape")

    @classmethod
    def new(cls, size, value: float = 0.0) -> "MatrixFull":
        return cls(size, np.full(size[0] * size[1], value, dtype=np.float64))

    @classmethod
    def from_vec(cls, size, vec) -> "MatrixFull":
        return cls(size, np.asarray(vec, dtype=np.float64))

    def to_numpy(self) -> np.ndarray:
        return self.data[: self.size[0] * self.size[1]].reshape(self.size, order="F")


class RIFull:
    """Column-major rank-3 tensor (src/ri.rs:19-40): element [x, y, z] at x + y*X + z*X*Y."""

    def __init__(self, size: Sequence[int], data: np.ndarray):
        self.size = [int(s) for s in size]
        self.indicing = [1, self.size[0], self.size[0] * self.size[1]]
        self.data = np.ascontiguousarray(np.asarray(data, dtype=np.float64).reshape(-1))
        if self.data.size < int(np.prod(self.size)):
            raise ValueError("RIFull::from_vec: vector shorter than the requested shape")

    @classmethod
    def new(cls, size, value: float = 0.0) -> "RIFull":
        return cls(size, np.full(int(np.prod(size)), value, dtype=np.float64))

    @classmethod
    def from_vec(cls, size, vec) -> "RIFull":
        return cls(size, np.asarray(vec, dtype=np.float64))

    def get_reducing_matrix(self, i_reduced: int) -> np.ndarray:
        """The i-th [x, y] slab (src/ri.rs:92-100), as a column-major view."""
        n = self.indicing[2]
        return self.data[n * i_reduced: n * (i_reduced + 1)].reshape(self.size[:2], order="F")

    def to_numpy(self) -> np.ndarray:
        return self.data[: int(np.prod(self.size))].reshape(self.size, order="F")

    def ao2mo(self, eigenvector: MatrixFull) -> "RIFull":
        """ao2mo_v02 (src/ri.rs:382-408): [nb, nb, naux] -> [naux, ns, ns] through ri_ao2mo_f_."""
        nb, ns = eigenvector.size
        naux = self.size[2]
        out = RIFull.new([naux, ns, ns], 0.0)
        ri_ao2mo_f(eigenvector.data, self.data, out.data, ns, nb, naux)
        return out


# --------------------------------------------------------------------------
# Fortran seam (host pointers)
# --------------------------------------------------------------------------
def _hp(a: np.ndarray):
    if a.dtype != np.float64 or not (a.flags.c_contiguous or a.flags.f_contiguous):
        raise TypeError("expected a contiguous float64 numpy array")
    return a.ctypes.data_as(_dp)


def ri_ao2mo_f(eigenvector: np.ndarray, ri3fn: np.ndarray, ri3mo: np.ndarray, num_states: int, num_basis: int,
               num_auxbas: int) -> None:
    """src/external_libs/mod.rs:6-22 -> ri_ao2mo_f_ (every argument by reference)."""
    L = lib()
    i = ctypes.c_int
    L.ri_ao2mo_f_(_hp(eigenvector), _hp(ri3fn), _hp(ri3mo), ctypes.byref(i(num_states)), ctypes.byref(i(num_basis)),
                  ctypes.byref(i(num_auxbas)))
    _check(last_status())


def general_dgemm_f(matr_a: np.ndarray, size_a, range_row_a, range_column_a, opa: str,
                    matr_b: np.ndarray, size_b, range_row_b, range_column_b, opb: str,
                    matr_c: np.ndarray, size_c, range_row_c, range_column_c, alpha: float, beta: float) -> None:
    """src/external_libs/mod.rs:60-83: ranges are Python ``range`` objects (start, stop)."""
    L = lib()
    i = ctypes.c_int
    r = ctypes.byref

    def blk(rg):
        return r(i(rg.start)), r(i(len(rg)))

    ra, la = blk(range_row_a)
    ca, lca = blk(range_column_a)
    rb, lb = blk(range_row_b)
    cb, lcb = blk(range_column_b)
    rc, lc = blk(range_row_c)
    cc, lcc = blk(range_column_c)
    L.general_dgemm_f_(_hp(matr_a), r(i(size_a[0])), r(i(size_a[1])), ra, la, ca, lca, r(ctypes.c_char(opa.encode())),
                       _hp(matr_b), r(i(size_b[0])), r(i(size_b[1])), rb, lb, cb, lcb, r(ctypes.c_char(opb.encode())),
                       _hp(matr_c), r(i(size_c[0])), r(i(size_c[1])), rc, lc, cc, lcc,
                       r(ctypes.c_double(alpha)), r(ctypes.c_double(beta)))
    _check(last_status())


def special_dgemm_f_01(ten3_a: np.ndarray, size_a, range_x_a: range, i_y: int, range_z_a: range,
                       matr_b: np.ndarray, size_b, range_row_b: range, range_column_b: range, alpha: float,
                       beta: float) -> None:
    """src/external_libs/mod.rs:85-99 -> special_dgemm_f_01_: in place on the host tensor ten3_a[size_a],
    every y-slice block times matr_b[range_row_b, range_column_b] (see restmatr.f90:111-154)."""
    L = lib()
    i = ctypes.c_int
    r = ctypes.byref
    L.special_dgemm_f_01_(_hp(ten3_a), r(i(size_a[0])), r(i(size_a[1])), r(i(size_a[2])), r(i(range_x_a.start)),
                          r(i(len(range_x_a))), r(i(i_y)), r(i(range_z_a.start)), r(i(len(range_z_a))),
                          _hp(matr_b), r(i(size_b[0])), r(i(size_b[1])), r(i(range_row_b.start)),
                          r(i(len(range_row_b))), r(i(range_column_b.start)), r(i(len(range_column_b))),
                          r(ctypes.c_double(alpha)), r(ctypes.c_double(beta)))
    _check(last_status())


def _dgemm(matr_a: MatrixFull, sub_a: Tuple[range, range], opa: str,
           matr_b: MatrixFull, sub_b: Tuple[range, range], opb: str,
           matr_c: MatrixFull, sub_c: Tuple[range, range], alpha: float, beta: float) -> None:
    """src/matrix/matrix_blas_lapack.rs:122-178, including its shape and bounds checks
    (the reference panics; this raises ValueError)."""
    la0, la1 = len(sub_a[0]), len(sub_a[1])
    lb0, lb1 = len(sub_b[0]), len(sub_b[1])
    lc0, lc1 = len(sub_c[0]), len(sub_c[1])
    ok = {
        ("N", "N"): la1 == lb0 and la0 == lc0 and lb1 == lc1,
        ("T", "N"): la0 == lb0 and la1 == lc0 and lb1 == lc1,
        ("N", "T"): la1 == lb1 and la0 == lc0 and lb0 == lc1,
        ("T", "T"): la0 == lb1 and la1 == lc0 and lb0 == lc1,
    }.get((opa, opb), False)
    if not ok:
        raise ValueError(f"ERROR:: Matr_A[{la0},{la1},{opa}] * Matr_B[{lb0},{lb1},{opb}] -> Matr_C[{lc0},{lc1}]")
    within = (sub_a[0].stop <= matr_a.size[0] and sub_a[1].stop <= matr_a.size[1]
              and sub_b[0].stop <= matr_b.size[0] and sub_b[1].stop <= matr_b.size[1]
              and sub_c[0].stop <= matr_c.size[0] and sub_c[1].stop <= matr_c.size[1])
    if not within:
        raise ValueError("ERROR:: sub-matrix block outside the matrix")
    general_dgemm_f(matr_a.data, matr_a.size, sub_a[0], sub_a[1], opa, matr_b.data, matr_b.size, sub_b[0], sub_b[1],
                    opb, matr_c.data, matr_c.size, sub_c[0], sub_c[1], alpha, beta)


# --------------------------------------------------------------------------
# Device-tensor API (torch CUDA tensors, float64)
# --------------------------------------------------------------------------
def _dptr(t, need: int = 0, name: str = "tensor") -> int:
    """Device address of a contiguous float64 CUDA tensor on the current device holding at least
    ``need`` elements (the extent the native call will touch); raw integer addresses pass unchecked."""
    import torch

    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise TypeError(f"{name}: expected a contiguous float64 CUDA tensor")
    if t.device.index != torch.cuda.current_device():
        raise ValueError(f"{name}: tensor on cuda:{t.device.index}, current device is cuda:{torch.cuda.current_device()}")
    if t.numel() < need:
        raise ValueError(f"{name}: {t.numel()} elements, the call needs {need}")
    return t.data_ptr()


def _mat_extent(ld: int, rows: int, cols: int) -> int:
    """Elements a column-major rows x cols block with leading dimension ld spans."""
    return 0 if rows <= 0 or cols <= 0 else (cols - 1) * ld + rows


def _gemm_extents(opa: str, opb: str, m: int, n: int, k: int, lda: int, ldb: int, ldc: int):
    """Elements of A, B and C that C = op(A) op(B) reads and writes (column-major, leading dimensions)."""
    a = _mat_extent(lda, m, k) if opa in "Nn" else _mat_extent(lda, k, m)
    b = _mat_extent(ldb, k, n) if opb in "Nn" else _mat_extent(ldb, n, k)
    return (a if n > 0 else 0), (b if m > 0 else 0), _mat_extent(ldc, m, n)


def _stream(stream) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _form(form: str) -> int:
    if form == "fp64":
        return RT_FORM_FP64
    if form == "split":
        return RT_FORM_SPLIT
    raise ValueError("form must be 'fp64' or 'split'")


def dgemm(opa, opb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream=None) -> None:
    ea, eb, ec = _gemm_extents(opa, opb, m, n, k, lda, ldb, ldc)
    _check(lib().rt_dgemm(opa.encode(), opb.encode(), m, n, k, alpha, _dptr(A, ea, "A"), lda, _dptr(B, eb, "B"), ldb,
                          beta, _dptr(C, ec, "C"), ldc, _stream(stream)))


def dgemm_split(opa, opb, m, n, k, A, lda, B, ldb, C, ldc, nslices: int = DEFAULT_NSLICES, stream=None) -> None:
    """C = op(A) op(B) in the split-precision form (float64 in and out)."""
    ea, eb, ec = _gemm_extents(opa, opb, m, n, k, lda, ldb, ldc)
    _check(lib().rt_dgemm_split(opa.encode(), opb.encode(), m, n, k, _dptr(A, ea, "A"), lda, _dptr(B, eb, "B"), ldb,
                                _dptr(C, ec, "C"), ldc, nslices, _stream(stream)))


def ri_ao2mo(C, B, nb: int, ns: int, naux: int, out=None, form: str = "fp64", nslices: int = DEFAULT_NSLICES,
             stream=None):
    """Device ri3mo [naux, ns, ns] (P fastest) from device C [nb, ns] and B [nb, nb, naux] (flat tensors)."""
    import torch

    if out is None:
        out = torch.empty(naux * ns * ns, dtype=torch.float64, device=C.device)
    _check(lib().rt_ri_ao2mo(_dptr(C, nb * ns, "C"), _dptr(B, nb * nb * naux, "B"), _dptr(out, naux * ns * ns, "out"),
                             nb, ns, naux, _form(form), nslices, _stream(stream)))
    return out


def ri_ov_k(C, B, nb: int, naux: int, nocc: int, nvir: int, ov=None, K=None, form: str = "split",
            nslices: int = DEFAULT_NSLICES, stream=None, want_ov: bool = True, want_k: bool = True):
    """ov (i,a,P) and K [nb, nb] on the device."""
    import torch

    if want_ov and ov is None:
        ov = torch.empty(nocc * nvir * naux, dtype=torch.float64, device=C.device)
    if want_k and K is None:
        K = torch.empty(nb * nb, dtype=torch.float64, device=C.device)
    _check(lib().rt_ri_ov_k(_dptr(C, nb * (nocc + nvir), "C"), _dptr(B, nb * nb * naux, "B"), nb, naux, nocc, nvir,
                            _dptr(ov, nocc * nvir * naux, "ov") if want_ov else None,
                            _dptr(K, nb * nb, "K") if want_k else None, _form(form), nslices, _stream(stream)))
    return ov, K


def ri_ov_k_fp64_noalloc(C, B, nb: int, naux: int, nocc: int, nvir: int, ov=None, K=None, stream=None):
    """Float64 ov and K without any device allocation by the library (rt_ri_ov_k_fp64_noalloc): its scratch is
    a fixed 32 MiB device array, so nb * nocc <= 4,194,304.  Outputs must be passed in (or None to skip)."""
    _check(lib().rt_ri_ov_k_fp64_noalloc(_dptr(C, nb * (nocc + nvir), "C"), _dptr(B, nb * nb * naux, "B"), nb, naux,
                                         nocc, nvir, _dptr(ov, nocc * nvir * naux, "ov"), _dptr(K, nb * nb, "K"),
                                         _stream(stream)))
    return ov, K


class Ri3aoPrepared:
    """ri3ao sliced once into split-form digit planes (rt_ri3ao_prepare) for repeated ov + RI-K with new
    orbitals, as in an SCF loop where ri3fn is fixed while C changes.  Holds about 2 nslices nb^2 naux bytes of
    device memory until release() (or garbage collection)."""

    def __init__(self, B, nb: int, naux: int, nslices: int = DEFAULT_NSLICES, stream=None):
        self.h = None
        h = ctypes.c_void_p()
        _check(lib().rt_ri3ao_prepare(_dptr(B, nb * nb * naux, "B"), nb, naux, nslices, ctypes.byref(h),
                                      _stream(stream)))
        self.h, self.nb, self.naux, self.nslices = h, nb, naux, nslices

    def nbytes(self) -> int:
        b = ctypes.c_longlong()
        _check(lib().rt_ri3ao_prepared_bytes(self.h, ctypes.byref(b)))
        return b.value

    def ri_ov_k(self, C, nocc: int, nvir: int, ov=None, K=None, stream=None, want_ov: bool = True,
                want_k: bool = True):
        """ov (i,a,P) and K [nb, nb] for orbitals C, from the prepared digit planes."""
        import torch

        if self.h is None:
            raise ValueError("Ri3aoPrepared: already released")
        nb, naux = self.nb, self.naux
        if want_ov and ov is None:
            ov = torch.empty(max(nocc * nvir * naux, 1), dtype=torch.float64, device=C.device)
        if want_k and K is None:
            K = torch.empty(nb * nb, dtype=torch.float64, device=C.device)
        _check(lib().rt_ri_ov_k_prepared(self.h, _dptr(C, nb * (nocc + nvir), "C"), nocc, nvir,
                                         _dptr(ov, nocc * nvir * naux, "ov") if want_ov else None,
                                         _dptr(K, nb * nb, "K") if want_k else None, _stream(stream)))
        return ov, K

    def release(self) -> None:
        if getattr(self, "h", None) is not None:
            lib().rt_ri3ao_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def ri_ov_k_batched(problems, form: str = "split", nslices: int = DEFAULT_NSLICES, tuning=None, stream=None):
    """rt_ri_ov_k over a batch of molecules of uneven sizes, one grouped launch per product.

    ``problems`` is a sequence of dicts with keys C, B, ov, K (torch CUDA float64
    tensors or None for ov/K) and nb, naux, nocc, nvir.  ``tuning`` is a
    ``Tuning``, a ``(fuse, chunks_per_item)`` pair, ``"auto"`` (look the batch
    up in the autotuned table, tuning it on a miss) or None (defaults).
    """
    arr = (RiProblem * max(len(problems), 1))()
    for i, q in enumerate(problems):
        nb, naux, nocc, nvir = q["nb"], q["naux"], q["nocc"], q["nvir"]
        arr[i] = RiProblem(_dptr(q["C"], nb * (nocc + nvir), f"problem {i} C"),
                           _dptr(q["B"], nb * nb * naux, f"problem {i} B"),
                           _dptr(q.get("ov"), nocc * nvir * naux, f"problem {i} ov"),
                           _dptr(q.get("K"), nb * nb, f"problem {i} K"), nb, naux, nocc, nvir)
    if isinstance(tuning, str) and tuning == "auto":
        from . import autotune

        tuning = autotune.lookup(problems, form, nslices, stream=stream)
    if tuning is not None and not isinstance(tuning, Tuning):
        tuning = Tuning(int(tuning[0]), int(tuning[1]))
    _check(lib().rt_ri_ov_k_batched(arr, len(problems), _form(form), nslices,
                                    ctypes.byref(tuning) if tuning is not None else None, _stream(stream)))


def ri_ov_k_host(C: np.ndarray, B: np.ndarray, nb: int, naux: int, nocc: int, nvir: int, ov: np.ndarray,
                 K: np.ndarray, form: str = "split", nslices: int = DEFAULT_NSLICES, stream=None,
                 symmetric: bool = False) -> None:
    """Host-buffer form (numpy or pinned memory addresses): copies in, runs, copies out.

    symmetric=True reads only the upper triangle of each ri3ao slab from the host
    (rt_ri_ov_k_host_symmetric); the slabs must be symmetric."""
    def hp(a):
        return a.ctypes.data if isinstance(a, np.ndarray) else int(a)

    fn = lib().rt_ri_ov_k_host_symmetric if symmetric else lib().rt_ri_ov_k_host
    _check(fn(hp(C), hp(B), nb, naux, nocc, nvir, hp(ov), hp(K), _form(form), nslices, _stream(stream)))


def ri_ao2mo_host(C: np.ndarray, B: np.ndarray, ri3mo: np.ndarray, nb: int, ns: int, naux: int,
                  form: str = "fp64", nslices: int = DEFAULT_NSLICES, stream=None) -> None:
    """Host-buffer full transform (rt_ri_ao2mo_host): C [nb, ns], B [nb, nb, naux] -> ri3mo [naux, ns, ns],
    pipelined over the host link.  Arguments are numpy arrays or raw host addresses."""
    def hp(a, need, name):
        if isinstance(a, np.ndarray):
            if a.dtype != np.float64 or not (a.flags.c_contiguous or a.flags.f_contiguous):
                raise TypeError(f"{name}: expected a contiguous float64 array")
            if a.size < need:
                raise ValueError(f"{name}: {a.size} elements, the call needs {need}")
            return a.ctypes.data
        return int(a)

    _check(lib().rt_ri_ao2mo_host(hp(C, nb * ns, "C"), hp(B, nb * nb * naux, "B"), hp(ri3mo, naux * ns * ns, "ri3mo"),
                                  nb, ns, naux, _form(form), nslices, _stream(stream)))


def special_dgemm_01(ten3, size_a, range_x_a: range, range_z_a: range, matr_b, size_b, range_row_b: range,
                     range_column_b: range, alpha: float = 1.0, beta: float = 0.0, form: str = "fp64",
                     nslices: int = DEFAULT_NSLICES, stream=None) -> None:
    """special_dgemm_f_01 on device tensors (flat, column-major), in place on ``ten3``."""
    _check(lib().rt_special_dgemm_01(
        _dptr(ten3, size_a[0] * size_a[1] * size_a[2], "ten3_a"), size_a[0], size_a[1], size_a[2], range_x_a.start,
        len(range_x_a), range_z_a.start, len(range_z_a), _dptr(matr_b, size_b[0] * size_b[1], "matr_b"), size_b[0],
        size_b[1], range_row_b.start, len(range_row_b),
        range_column_b.start, len(range_column_b), alpha, beta, _form(form), nslices, _stream(stream)))


def copy_mm(x_len: int, y_len: int, f_matr, f_size, f_start, t_matr, t_size, t_start, stream=None) -> None:
    """restmatr.f90:197-212 on device matrices: t[ts.., ..] = f[fs.., ..] for an x_len x y_len block."""
    _check(lib().rt_copy_mm(x_len, y_len, _dptr(f_matr, f_size[0] * f_size[1], "f_matr"), f_size[0], f_size[1],
                            f_start[0], f_start[1], _dptr(t_matr, t_size[0] * t_size[1], "t_matr"), t_size[0],
                            t_size[1], t_start[0], t_start[1], _stream(stream)))


def copy_mr(x1_len: int, x2_len: int, f_matr, f_size, f_start, t_ri, t_size, t_start, t_x3: int, mode: int,
            stream=None) -> None:
    """restmatr.f90:215-238 on device data: a matrix block into a rank-3 tensor (mode 0, 1 or 2)."""
    _check(lib().rt_copy_mr(x1_len, x2_len, _dptr(f_matr, f_size[0] * f_size[1], "f_matr"), f_size[0], f_size[1],
                            f_start[0], f_start[1], _dptr(t_ri, t_size[0] * t_size[1] * t_size[2], "t_ri"),
                            t_size[0], t_size[1], t_size[2], t_start[0], t_start[1], t_x3, mode, _stream(stream)))


def copy_rm(x1_len: int, x2_len: int, f_ri, f_size, f_start, f_x3: int, mode: int, t_matr, t_size, t_start,
            stream=None) -> None:
    """restmatr.f90:241-264 on device data: a rank-3 tensor block into a matrix (mode 0, 1 or 2)."""
    _check(lib().rt_copy_rm(x1_len, x2_len, _dptr(f_ri, f_size[0] * f_size[1] * f_size[2], "f_ri"), f_size[0],
                            f_size[1], f_size[2], f_start[0], f_start[1], f_x3, mode,
                            _dptr(t_matr, t_size[0] * t_size[1], "t_matr"), t_size[0], t_size[1], t_start[0],
                            t_start[1], _stream(stream)))


def copy_rr(lens, f_ri, f_size, f_start, t_ri, t_size, t_start, stream=None) -> None:
    """restmatr.f90:266-285 on device data: a block between rank-3 tensors."""
    _check(lib().rt_copy_rr(lens[0], lens[1], lens[2], _dptr(f_ri, f_size[0] * f_size[1] * f_size[2], "f_ri"),
                            f_size[0], f_size[1], f_size[2], f_start[0], f_start[1], f_start[2],
                            _dptr(t_ri, t_size[0] * t_size[1] * t_size[2], "t_ri"), t_size[0], t_size[1], t_size[2],
                            t_start[0], t_start[1], t_start[2], _stream(stream)))


def ri_transpose(ri, size, order: str, out=None, stream=None):
    """RIFull transpose_<order> (src/ri.rs:226-294) of a device [i, j, k] tensor, e.g. order="jki"."""
    import torch

    if out is None:
        out = torch.empty(int(size[0]) * int(size[1]) * int(size[2]), dtype=torch.float64, device=ri.device)
    nel = int(size[0]) * int(size[1]) * int(size[2])
    _check(lib().rt_ri_transpose(_dptr(ri, nel, "ri"), size[0], size[1], size[2], order.encode(), _dptr(out, nel, "out"),
                                 _stream(stream)))
    return out


def ri_pack_symm(ri, nao: int, naux: int, out=None, stream=None):
    """rifull_to_matfull_symm (src/ri.rs:296-307): [nao, nao, naux] -> [nao (nao + 1) / 2, naux]."""
    import torch

    if out is None:
        out = torch.empty(max(nao * (nao + 1) // 2 * naux, 1), dtype=torch.float64, device=ri.device)
    _check(lib().rt_ri_pack_symm(_dptr(ri, nao * nao * naux, "ri"), nao, naux,
                                 _dptr(out, nao * (nao + 1) // 2 * naux, "out"), _stream(stream)))
    return out[: nao * (nao + 1) // 2 * naux]


def newton_schulz_inverse_square_root_v02(S, n: int, threshold: float, mix_parameter: float, num_iter: int,
                                          level_shift, form: str = "fp64", nslices: int = DEFAULT_NSLICES,
                                          out=None, stream=None):
    """_newton_schulz_inverse_square_root_v02 (src/matrix/matrix_blas_lapack.rs:1710-1778) on a device
    [n, n] matrix.  Returns (matrix, n_singular = 0, converged) like the reference, plus the number of
    X_next evaluations (three n x n products each)."""
    import torch

    if len(level_shift) == 0:
        raise ValueError("level_shift must not be empty")
    if out is None:
        out = torch.empty(n * n, dtype=torch.float64, device=S.device)
    shifts = (ctypes.c_double * len(level_shift))(*[float(x) for x in level_shift])
    conv, steps = ctypes.c_int(0), ctypes.c_int(0)
    _check(lib().rt_newton_schulz_inv_sqrt(_dptr(S, n * n, "S"), n, threshold, mix_parameter, num_iter, shifts,
                                           len(level_shift), _form(form), nslices, _dptr(out, n * n, "out"),
                                           ctypes.byref(conv),
                                           ctypes.byref(steps), _stream(stream)))
    return out, 0, bool(conv.value), int(steps.value)


def dsyev(A, n: int, w=None, stream=None):
    """lapack_dsyev (src/matrix/matrix_blas_lapack.rs:775-797) on a device [n, n] matrix (lower triangle read):
    eigenvalues ascending into w (returned), eigenvectors into A's columns, in place."""
    import torch

    if w is None:
        w = torch.empty(max(n, 1), dtype=torch.float64, device=A.device)
    _check(lib().rt_dsyev(n, _dptr(A, n * n, "A"), _dptr(w, n, "w"), _stream(stream)))
    return w[:n]


def lapack_power(S, n: int, p: float, threshold: float, out=None, form: str = "fp64",
                 nslices: int = DEFAULT_NSLICES, stream=None):
    """lapack_power (src/matrix/matrix_blas_lapack.rs:1004-1064): S^p over the eigenvalues >= threshold.
    Returns (out [n*n], number of eigenvalues kept)."""
    import torch

    if out is None:
        out = torch.empty(max(n * n, 1), dtype=torch.float64, device=S.device)
    kept = ctypes.c_int(0)
    _check(lib().rt_lapack_power(_dptr(S, n * n, "S"), n, p, threshold, _dptr(out, n * n, "out"), ctypes.byref(kept),
                                 _form(form), nslices, _stream(stream)))
    return out, kept.value


def dspgvx(ap, bp, n: int, num_orb: int, eigvec=None, w=None, form: str = "fp64", nslices: int = DEFAULT_NSLICES,
           stream=None):
    """lapack_dspgvx (src/matrix/matrix_blas_lapack.rs:1096-1147) on packed upper device matrices A and B:
    the lowest num_orb eigenpairs of A x = lambda B x.  Returns (eigvec [n * num_orb], w [n])."""
    import torch

    npk = n * (n + 1) // 2
    if eigvec is None:
        eigvec = torch.empty(max(n * num_orb, 1), dtype=torch.float64, device=ap.device)
    if w is None:
        w = torch.empty(max(n, 1), dtype=torch.float64, device=ap.device)
    _check(lib().rt_dspgvx(_dptr(ap, npk, "ap"), _dptr(bp, npk, "bp"), n, num_orb, _dptr(eigvec, n * num_orb, "eigvec"),
                           _dptr(w, n, "w"), _form(form), nslices, _stream(stream)))
    return eigvec, w


def ri_j(B, D, nb: int, naux: int, w=None, J=None, stream=None, symmetric: bool = False):
    """RI-J (w, J).  symmetric=True calls rt_ri_j_symmetric: every slab of B and
    D must be symmetric; only their entries mu <= nu are read."""
    import torch

    if w is None:
        w = torch.empty(naux, dtype=torch.float64, device=B.device)
    if J is None:
        J = torch.empty(nb * nb, dtype=torch.float64, device=B.device)
    fn = lib().rt_ri_j_symmetric if symmetric else lib().rt_ri_j
    _check(fn(_dptr(B, nb * nb * naux, "B"), _dptr(D, nb * nb, "D"), nb, naux, _dptr(w, naux, "w"),
              _dptr(J, nb * nb, "J"), _stream(stream)))
    return w, J


def exchange_energy(D, K, nb: int, out=None, stream=None):
    import torch

    if out is None:
        out = torch.empty(1, dtype=torch.float64, device=D.device)
    _check(lib().rt_ri_exchange_energy(_dptr(D, nb * nb, "D"), _dptr(K, nb * nb, "K"), nb, _dptr(out, 1, "out"),
                                       _stream(stream)))
    return out


def synth_ri3ao(seed: int, nb: int, naux: int, P0: int = 0, out=None, stream=None):
    import torch

    if out is None:
        out = torch.empty(nb * nb * naux, dtype=torch.float64, device="cuda")
    _check(lib().rt_synth_ri3ao(seed, nb, P0, naux, _dptr(out, nb * nb * naux, "out"), _stream(stream)))
    return out


def synth_delta(seed: int, nov: int, stream=None):
    """Device copy of the synthetic orbital-energy-difference diagonal (uniform in [0.5, 3.0])."""
    import torch

    d = torch.empty(max(nov, 1), dtype=torch.float64, device="cuda")
    _check(lib().rt_synth_delta(seed, nov, _dptr(d), _stream(stream)))
    return d[:nov]


def synth_coef(seed: int, nb: int, stream=None):
    """Synthetic orbital coefficients: Q of the Householder QR of the seeded N(0,1) matrix.

    The seed matrix is generated on the device; the QR factorisation (input
    preparation only) runs on the host through numpy's LAPACK.
    """
    import torch

    M = torch.empty(nb * nb, dtype=torch.float64, device="cuda")
    _check(lib().rt_synth_coef_seed(seed, nb, _dptr(M), _stream(stream)))
    Mh = M.cpu().numpy().reshape(nb, nb, order="F")
    Q, _ = np.linalg.qr(Mh)
    return torch.from_numpy(np.ascontiguousarray(Q.reshape(-1, order="F"))).to(M.device)


PROF_OZ_GEMM, PROF_OZ_SLICE, PROF_DGEMM, PROF_RIJ = 0, 1, 2, 3


def launch_count() -> int:
    return int(lib().rt_launch_count())


def profile_enable(on: bool) -> None:
    lib().rt_profile_enable(1 if on else 0)


def profile_get(kind: int):
    """(total event milliseconds, launches, algorithmic work) recorded for a kernel kind."""
    ms, n, w = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
    _check(lib().rt_profile_get(kind, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(w)))
    return ms.value, n.value, w.value


# --------------------------------------------------------------------------
# Response operator and Davidson
# --------------------------------------------------------------------------
class DavidsonParams:
    """DavidsonParams (src/davidson.rs:28-46), same field names and defaults."""

    def __init__(self, tol=1e-5, maxcyc=50, maxspace=12, lindep=1e-14, nroots=3):
        self.tol, self.maxcyc, self.maxspace, self.lindep, self.nroots = tol, maxcyc, maxspace, lindep, nroots

    def _c(self):
        return _DavidsonParamsC(self.tol, self.maxcyc, self.maxspace, self.lindep, self.nroots)


def _device_view(ptr: int, nvec: int, n: int):
    """A torch view [nvec, n] of a column-major device block [n, nvec]."""
    import torch

    class _Arr:
        pass

    o = _Arr()
    o.__cuda_array_interface__ = {"shape": (nvec, n), "typestr": "<f8", "data": (int(ptr), False), "version": 3,
                                  "strides": None}
    return torch.as_tensor(o, device="cuda")


def ri_iajb(Bov, nov: int, naux: int, M=None, form: str = "split", nslices: int = DEFAULT_NSLICES, stream=None):
    import torch

    if M is None:
        M = torch.empty(nov * nov, dtype=torch.float64, device=Bov.device)
    _check(lib().rt_ri_iajb(_dptr(Bov, nov * naux, "Bov"), nov, naux, _dptr(M, nov * nov, "M"), _form(form), nslices,
                            _stream(stream)))
    return M


def ri_response_matvec(Bov, delta, nov: int, naux: int, X, nvec: int, AX=None, form: str = "split",
                       nslices: int = DEFAULT_NSLICES, stream=None):
    import torch

    if AX is None:
        AX = torch.empty(nov * nvec, dtype=torch.float64, device=Bov.device)
    _check(lib().rt_ri_response_matvec(_dptr(Bov, nov * naux, "Bov"), _dptr(delta, nov, "delta"), nov, naux,
                                       _dptr(X, nov * nvec, "X"), _dptr(AX, nov * nvec, "AX"), nvec, _form(form),
                                       nslices, _stream(stream)))
    return AX


def davidson_solve(a_x, x0_1d, hdiag, params: DavidsonParams = None, print_level: int = 0, stream=None):
    """davidson_solve (src/davidson.rs:48-266) with vectors on the device.

    a_x(X) receives a torch view [nvec, n] (row v = vector v) and returns A X in
    the same shape; it plays the role of the reference's `a_x` closure.
    Returns (conv: list[bool], e: list[float], x: torch [nroots, n]).
    """
    import torch

    params = params or DavidsonParams()
    n = int(x0_1d.numel())

    def cb(xp, axp, nvec, nn, ctx, st):
        try:
            X = _device_view(xp, nvec, nn)
            AX = _device_view(axp, nvec, nn)
            AX.copy_(a_x(X))
            return 0
        except Exception as ex:  # reported to the native side as a failed callback
            print("davidson a_x callback failed:", ex)
            return 1

    cfn = MATVEC_FN(cb)
    nr = params.nroots
    conv = (ctypes.c_int * nr)()
    e = (ctypes.c_double * nr)()
    its = ctypes.c_int(0)
    x = torch.zeros(nr * n, dtype=torch.float64, device=x0_1d.device)
    pc = params._c()
    _check(lib().rt_davidson_solve(cfn, None, _dptr(x0_1d, n, "x0"), _dptr(hdiag, n, "hdiag"), n, ctypes.byref(pc),
                                   print_level, conv, e, _dptr(x, nr * n, "x"), ctypes.byref(its), _stream(stream)))
    return [bool(c) for c in conv], list(e), x.view(nr, n), its.value


def davidson_ri_response(Bov, delta, nov: int, naux: int, x0_1d, params: DavidsonParams = None, form: str = "split",
                         nslices: int = DEFAULT_NSLICES, print_level: int = 0, stream=None):
    """Lowest roots of diag(delta) + B_ov B_ov^T by the native Davidson driver."""
    import torch

    params = params or DavidsonParams()
    nr = params.nroots
    conv = (ctypes.c_int * nr)()
    e = (ctypes.c_double * nr)()
    its = ctypes.c_int(0)
    x = torch.zeros(nr * nov, dtype=torch.float64, device=Bov.device)
    pc = params._c()
    _check(lib().rt_davidson_ri_response(_dptr(Bov, nov * naux, "Bov"), _dptr(delta, nov, "delta"), nov, naux,
                                         _form(form), nslices, _dptr(x0_1d, nov, "x0"),
                                         ctypes.byref(pc), print_level, conv, e, _dptr(x), ctypes.byref(its),
                                         _stream(stream)))
    return [bool(c) for c in conv], list(e), x.view(nr, nov), its.value


def debug_fail_alloc_after(n: int) -> None:
    """Testing hook: the next n scratch allocations succeed, the one after fails (n < 0: off)."""
    _check(lib().rt_debug_fail_alloc_after(n))


def debug_chunk_bytes(nbytes: int) -> None:
    """Testing hook: scratch bound of one staged chunk in special_dgemm_01 (<= 0 restores 8 GB)."""
    _check(lib().rt_debug_chunk_bytes(int(nbytes)))


def debug_wait_timeout(cycles: int, stream=None) -> None:
    """Testing hook: run the bounded-wait path out on purpose (see rt_debug_wait_timeout)."""
    _check(lib().rt_debug_wait_timeout(cycles, _stream(stream)))


def sync_status(stream=None) -> None:
    _check(lib().rt_sync_status(_stream(stream)))
