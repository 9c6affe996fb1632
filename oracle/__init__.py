"""CPU oracle for the dense RI contraction path -- TEST INFRASTRUCTURE ONLY.

This package is the checker used by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py``.  The product library never imports it.

It wraps ``oracle.c`` (a C restatement of ``src/external_libs/restmatr.f90``
and the composed RI-J/RI-K/exchange contractions over OpenBLAS) and
``davidson_ref.py`` (a line-by-line restatement of ``src/davidson.rs``).
All arrays are numpy float64 in column-major (Fortran) order, matching the
reference's ``MatrixFull``/``RIFull`` storage.
"""
from __future__ import annotations

import ctypes
import glob
import os

import numpy as np

from . import build as _build

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


def openblas_path() -> str:
    import scipy

    libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs", "libscipy_openblas*.so"))
    if not libs:
        raise RuntimeError("scipy's bundled OpenBLAS was not found")
    return os.path.realpath(sorted(libs)[0])


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        rc = L.oracle_init(openblas_path().encode())
        if rc != 0:
            raise RuntimeError(f"oracle_init failed ({rc})")
        L.oracle_exchange_energy.restype = ctypes.c_double
        L.oracle_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64
    return a.ctypes.data_as(_dp)


def _f(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def get_threads() -> int:
    return int(lib().oracle_get_threads())


# --------------------------------------------------------------------------
# GEMM seam
# --------------------------------------------------------------------------
def general_dgemm_f(a, rng_ra, rng_ca, opa, b, rng_rb, rng_cb, opb, c, rng_rc, rng_cc, alpha, beta):
    """restmatr.f90:63-107 on column-major numpy matrices; ranges are (start, stop)."""
    a, b = _f(a), _f(b)
    assert c.flags.f_contiguous and c.dtype == np.float64
    L = lib()
    i = ctypes.c_int
    L.oracle_general_dgemm_f(
        _p(a), i(a.shape[0]), i(a.shape[1]), i(rng_ra[0]), i(rng_ra[1] - rng_ra[0]), i(rng_ca[0]),
        i(rng_ca[1] - rng_ca[0]), ctypes.c_char(opa.encode()),
        _p(b), i(b.shape[0]), i(b.shape[1]), i(rng_rb[0]), i(rng_rb[1] - rng_rb[0]), i(rng_cb[0]),
        i(rng_cb[1] - rng_cb[0]), ctypes.c_char(opb.encode()),
        _p(c), i(c.shape[0]), i(c.shape[1]), i(rng_rc[0]), i(rng_rc[1] - rng_rc[0]), i(rng_cc[0]),
        i(rng_cc[1] - rng_cc[0]), ctypes.c_double(alpha), ctypes.c_double(beta))
    return c


def dgemm(opa, opb, a, b, alpha=1.0, beta=0.0, c=None):
    """lapack_dgemm semantics (matrix_blas_lapack.rs:739-774)."""
    a, b = _f(a), _f(b)
    m = a.shape[0] if opa == "N" else a.shape[1]
    k = a.shape[1] if opa == "N" else a.shape[0]
    n = b.shape[1] if opb == "N" else b.shape[0]
    if c is None:
        c = np.zeros((m, n), order="F")
    lib().oracle_dgemm(ctypes.c_char(opa.encode()), ctypes.c_char(opb.encode()), m, n, k, ctypes.c_double(alpha),
                       _p(a), max(a.shape[0], 1), _p(b), max(b.shape[0], 1), ctypes.c_double(beta), _p(c), max(m, 1))
    return c


# --------------------------------------------------------------------------
# RI path
# --------------------------------------------------------------------------
def ri_ao2mo(eigenvector, ri3fn, P0=0, P1=None):
    """ri_ao2mo_f: eigenvector [nb, ns], ri3fn [nb, nb, naux] -> ri3mo [naux, ns, ns]."""
    C, B = _f(eigenvector), _f(ri3fn)
    nb, ns = C.shape
    naux = B.shape[2]
    P1 = naux if P1 is None else P1
    out = np.zeros((naux, ns, ns), order="F")
    lib().oracle_ri_ao2mo_range(_p(C), _p(B), _p(out), ns, nb, naux, int(P0), int(P1))
    return out


def ri_ov_k(C, B, nocc, P0=0, P1=None):
    """Occupied-virtual block (i,a,P) and RI-K over slabs P0..P1."""
    C, B = _f(C), _f(B)
    nb, ns = C.shape
    naux = B.shape[2]
    nvir = ns - nocc
    P1 = naux if P1 is None else P1
    ov = np.zeros((nocc, nvir, naux), order="F")
    K = np.zeros((nb, nb), order="F")
    lib().oracle_ri_ov_k_range(_p(C), _p(B), nb, naux, nocc, nvir, _p(ov), _p(K), int(P0), int(P1))
    return ov, K


def ri_j(B, D):
    B, D = _f(B), _f(D)
    nb, naux = B.shape[0], B.shape[2]
    w = np.zeros(naux)
    J = np.zeros((nb, nb), order="F")
    lib().oracle_ri_j(_p(B), _p(D), nb, naux, _p(w), _p(J))
    return w, J


def exchange_energy(D, K) -> float:
    D, K = _f(D), _f(K)
    return float(lib().oracle_exchange_energy(_p(D), _p(K), D.shape[0]))


def iajb(Bov2d):
    Bov2d = _f(Bov2d)
    nov, naux = Bov2d.shape
    M = np.zeros((nov, nov), order="F")
    lib().oracle_iajb(_p(Bov2d), nov, naux, _p(M))
    return M


def response_matvec(Bov2d, delta, X):
    Bov2d, X = _f(Bov2d), _f(X)
    delta = np.ascontiguousarray(delta, dtype=np.float64)
    nov, naux = Bov2d.shape
    nvec = X.shape[1]
    AX = np.zeros((nov, nvec), order="F")
    lib().oracle_response_matvec(_p(Bov2d), _p(delta), nov, naux, _p(X), _p(AX), nvec)
    return AX


# --------------------------------------------------------------------------
# LAPACK seam
# --------------------------------------------------------------------------
def dspevx_packed(ap):
    """lapack_dspevx (matrix_blas_lapack.rs:1075-1095).  Returns (eigvec [n,n], eigval, n_found).

    n is recovered from the packed length through an f32 square root, as the
    reference does at :1077.
    """
    ap = np.array(ap, dtype=np.float64)
    n = int(np.sqrt(np.float32(8.0 * np.float32(ap.size) + 1.0)) / np.float32(2.0))
    w = np.zeros(max(n, 1))
    z = np.zeros((max(n, 1), max(n, 1)), order="F")
    nf = ctypes.c_int(0)
    info = lib().oracle_dspevx_packed(n, _p(ap), _p(w), _p(z), ctypes.byref(nf))
    if info != 0:
        raise RuntimeError(f"dspevx info={info}")
    return z[:n, :n], w[:n], nf.value


def dsyev(a, jobz="V"):
    a = np.array(_f(a), order="F")
    n = a.shape[0]
    w = np.zeros(n)
    info = lib().oracle_dsyev(ctypes.c_char(jobz.encode()), n, _p(a), _p(w))
    if info != 0:
        raise RuntimeError(f"dsyev info={info}")
    return (a if jobz == "V" else None), w


def lapack_power(S, p: float, threshold: float):
    """lapack_power (matrix_blas_lapack.rs:1004-1064) through oracle.c over OpenBLAS dsyev.
    Returns (S^p restricted to eigenvalues >= threshold, number of such eigenvalues)."""
    S = _f(S)
    n = S.shape[0]
    out = np.zeros((n, n), order="F")
    kept = ctypes.c_int(0)
    info = lib().oracle_lapack_power(n, _p(S), ctypes.c_double(p), ctypes.c_double(threshold), _p(out),
                                     ctypes.byref(kept))
    if info != 0:
        raise RuntimeError(f"dsyev info={info}")
    return out, kept.value


def dspgvx(ap, bp, n: int, num_orb: int):
    """lapack_dspgvx (matrix_blas_lapack.rs:1096-1147): packed upper A and B -> (eigenvectors [n, num_orb],
    w [n] with the num_orb eigenvalues first, m).  Raises like the reference when info != 0 or m != num_orb."""
    ap = np.ascontiguousarray(ap, dtype=np.float64)
    bp = np.ascontiguousarray(bp, dtype=np.float64)
    z = np.zeros((n, num_orb), order="F")
    w = np.zeros(n)
    m = ctypes.c_int(0)
    info = lib().oracle_dspgvx(n, _p(ap), _p(bp), num_orb, _p(z), _p(w), ctypes.byref(m))
    if info != 0:
        raise RuntimeError(f"dspgvx info={info}")
    if m.value != num_orb:
        raise RuntimeError(f"dspgvx returned {m.value} eigenvectors, expected {num_orb}")
    return z, w, m.value


def full_to_upper_packed(m) -> np.ndarray:
    """MatrixFull::to_matrixupper: column j keeps rows 0..=j (packed 'U')."""
    m = _f(m)
    n = m.shape[0]
    return np.concatenate([m[: j + 1, j] for j in range(n)]) if n else np.zeros(0)


# --------------------------------------------------------------------------
# ri3fn preparation and layout utilities
# --------------------------------------------------------------------------
def special_dgemm_f_01(ten3, size_a, range_x_a, range_z_a, matr_b, size_b, range_row_b, range_column_b,
                       alpha, beta):
    """restmatr.f90:111-154 (through oracle.c) on flat column-major data; ranges are (start, stop).

    Returns the updated tensor as a new flat array; ``ten3`` is not modified.
    """
    t = np.array(np.asarray(ten3, dtype=np.float64).reshape(-1), copy=True)
    b = np.ascontiguousarray(np.asarray(matr_b, dtype=np.float64).reshape(-1))
    i = ctypes.c_int
    lib().oracle_special_dgemm_f_01(
        _p(t), i(size_a[0]), i(size_a[1]), i(size_a[2]), i(range_x_a[0]), i(range_x_a[1] - range_x_a[0]),
        i(range_z_a[0]), i(range_z_a[1] - range_z_a[0]), _p(b), i(size_b[0]), i(size_b[1]), i(range_row_b[0]),
        i(range_row_b[1] - range_row_b[0]), i(range_column_b[0]), i(range_column_b[1] - range_column_b[0]),
        ctypes.c_double(alpha), ctypes.c_double(beta))
    return t


def _fview(flat, size):
    return np.asarray(flat).reshape(tuple(size), order="F")


def copy_mm(x_len, y_len, f, f_size, f_start, t, t_size, t_start):
    """restmatr.f90:197-212: t[tx:tx+x_len, ty:ty+y_len] = f[fx:fx+x_len, fy:fy+y_len] (flat arrays; t updated)."""
    F, T = _fview(f, f_size), _fview(t, t_size)
    T[t_start[0]:t_start[0] + x_len, t_start[1]:t_start[1] + y_len] = \
        F[f_start[0]:f_start[0] + x_len, f_start[1]:f_start[1] + y_len].copy()
    return t


def _ri_block(R, a0, alen, b0, blen, fix, mode):
    if mode == 0:
        return (slice(a0, a0 + alen), slice(b0, b0 + blen), fix)
    if mode == 1:
        return (slice(a0, a0 + alen), fix, slice(b0, b0 + blen))
    if mode == 2:
        return (fix, slice(a0, a0 + alen), slice(b0, b0 + blen))
    return None


def copy_mr(x1_len, x2_len, f, f_size, f_start, t, t_size, t_start, t_x3, mode):
    """restmatr.f90:215-238: a matrix block into rank-3 t by mode 0/1/2 (other modes copy nothing)."""
    F, T = _fview(f, f_size), _fview(t, t_size)
    idx = _ri_block(T, t_start[0], x1_len, t_start[1], x2_len, t_x3, mode)
    if idx is not None:
        T[idx] = F[f_start[0]:f_start[0] + x1_len, f_start[1]:f_start[1] + x2_len].copy()
    return t


def copy_rm(x1_len, x2_len, f, f_size, f_start, f_x3, mode, t, t_size, t_start):
    """restmatr.f90:241-264: the reverse of copy_mr."""
    F, T = _fview(f, f_size), _fview(t, t_size)
    idx = _ri_block(F, f_start[0], x1_len, f_start[1], x2_len, f_x3, mode)
    if idx is not None:
        T[t_start[0]:t_start[0] + x1_len, t_start[1]:t_start[1] + x2_len] = F[idx].copy()
    return t


def copy_rr(lens, f, f_size, f_start, t, t_size, t_start):
    """restmatr.f90:266-285: a [x1, x2, x3] block between rank-3 tensors."""
    F, T = _fview(f, f_size), _fview(t, t_size)
    T[tuple(slice(t_start[d], t_start[d] + lens[d]) for d in range(3))] = \
        F[tuple(slice(f_start[d], f_start[d] + lens[d]) for d in range(3))].copy()
    return t


# The RIFull transposes restated with the reference's own enumeration
# (src/ri.rs:226-294), in pure Python: small tensors only.
def transpose_jik(data, size):
    """ri.rs:226-238: each [i, j] chunk of the slab order is transposed."""
    i, j, k = size
    out = []
    for z in range(k):
        chunk = data[z * i * j:(z + 1) * i * j]
        out.extend(chunk[r + c * i] for r in range(i) for c in range(j))
    return out


def transpose_jki(data, size):
    """ri.rs:240-256: for each ii, the elements whose flat index is congruent to ii mod i, in order."""
    i, j, k = size
    out = []
    for ii in range(i):
        out.extend(v for idx, v in enumerate(data) if abs(idx - ii) % i == 0)
    return out


def transpose_kji(data, size):
    """ri.rs:258-275: transpose_jik, then for each ij the elements congruent to ij mod i*j."""
    i, j, k = size
    t = transpose_jik(data, size)
    out = []
    for ij in range(i * j):
        out.extend(v for idx, v in enumerate(t) if abs(idx - ij) % (i * j) == 0)
    return out


def transpose_ikj(data, size):
    """ri.rs:277-294: for each jj, column jj of every [i, j] slab."""
    i, j, k = size
    out = []
    for jj in range(j):
        for z in range(k):
            chunk = data[z * i * j:(z + 1) * i * j]
            out.extend(chunk[jj * i:(jj + 1) * i])
    return out


def rifull_to_matfull_symm(data, nao, naux):
    """ri.rs:296-307 with richunk_reduce_by_symm (ri.rs:330-341): rows 0..=c of column c, per slab."""
    out = []
    for P in range(naux):
        chunk = data[P * nao * nao:(P + 1) * nao * nao]
        for c in range(nao):
            out.extend(chunk[c * nao:c * nao + c + 1])
    return out


# --------------------------------------------------------------------------
# Newton-Schulz inverse square root (src/matrix/matrix_blas_lapack.rs:1710-1932)
# --------------------------------------------------------------------------
def newton_schulz_lf(input_matr, initial_guess, threshold, mix_parameter, level_shift, num_iter):
    """_newton_schulz_inverse_square_root_lf (matrix_blas_lapack.rs:1780-1932), step by step.

    X_next = 0.5 X (3I - A X X); the mixing branches, the level shift on
    diagonal elements above the threshold and the returned iterate (the last
    X_next, not the mixed X) follow the reference.  Returns
    (matrix, n_singular = 0, converged, evals), where evals counts the X_next
    evaluations (three products each).
    """
    a = np.array(input_matr, dtype=np.float64, order="F")
    n = a.shape[0]
    num_elems = a.size
    unit = 3.0 * np.eye(n)
    matr = a.copy(order="F")
    d = np.diag(matr).copy()
    d = np.where(d > threshold, d + level_shift, 0.0)
    matr[np.arange(n), np.arange(n)] = d
    trace_1 = float(np.sum(np.diag(matr))) / n
    initial_a = 1.0 / np.sqrt(trace_1)
    if initial_guess is not None:
        x = np.array(initial_guess, dtype=np.float64, order="F")
    else:
        x = np.zeros((n, n), order="F")
        x[np.arange(n), np.arange(n)] = np.where(np.abs(np.diag(matr)) < threshold, 0.0, initial_a)

    def step(x):
        t = matr @ x
        w = t @ x
        u = unit + w * -1.0
        return 0.5 * (x @ u)

    nxt = step(x)
    evals = 1
    norm = np.sqrt(np.sum((x - nxt) ** 2)) / num_elems
    prev_norm = norm
    x = nxt.copy()
    converged = bool(norm <= threshold)
    count_unchanged = 0
    for _ in range(num_iter):
        nxt = step(x)
        evals += 1
        norm = np.sqrt(np.sum((x - nxt) ** 2)) / num_elems
        converged = bool(norm <= threshold)
        change_norm = norm - prev_norm
        prev_norm = norm
        prev = x.copy()
        if converged:
            break
        if norm <= threshold * 10.0:
            x = mix_parameter * nxt + (1.0 - mix_parameter) * x
            x = mix_parameter * prev + (1.0 - mix_parameter) * x
            count_unchanged = 0
        elif change_norm > threshold:
            count_unchanged = 0
            x = mix_parameter * nxt + (1.0 - mix_parameter) * x
            tmp = np.sqrt(np.sum(x ** 2))
            if tmp >= 100.0:
                x = x / tmp
                x = x / tmp
                x[np.arange(n), np.arange(n)] *= tmp
        elif abs(change_norm) <= threshold:
            if count_unchanged < 5:
                x = mix_parameter * nxt + (1.0 - mix_parameter) * x
                count_unchanged += 1
            else:
                x[np.arange(n), np.arange(n)] = initial_a
                count_unchanged = 0
        else:
            x = nxt.copy()
            count_unchanged = 0
    return np.asfortranarray(nxt), 0, converged, evals


def newton_schulz_inverse_square_root_v02(original_matr, threshold, mix_parameter, num_iter, level_shift):
    """_newton_schulz_inverse_square_root_v02 (matrix_blas_lapack.rs:1710-1778): normalise by the
    Frobenius norm, run the level-shift sequence (halving the mixing parameter up to six times when a
    stage fails, then stopping), rescale by norm^-1/2.  Returns (matrix, 0, converged, total_evals)."""
    if len(level_shift) == 0:
        raise ValueError("level_shift must not be empty (the reference unwraps a None guess)")
    a = np.array(original_matr, dtype=np.float64, order="F")
    original_norm = float(np.sqrt(np.sum(a ** 2)))
    matr_0 = a / original_norm
    guess = None
    converged = False
    total = 0
    for shift in level_shift:
        out, _, lf_conv, steps = newton_schulz_lf(matr_0, guess, threshold, mix_parameter, shift, num_iter)
        total += steps
        fine_mix = mix_parameter
        if not lf_conv:
            lf2 = lf_conv
            cur = 0
            while not lf2:
                fine_mix = fine_mix / 2.0
                cur += 1
                out, _, lf2, steps = newton_schulz_lf(matr_0, guess, threshold, fine_mix, shift, num_iter)
                total += steps
                if cur > 5:
                    break
            guess = out
            converged = lf2
            break
        converged = lf_conv
        guess = out
    res = guess * original_norm ** -0.5
    return np.asfortranarray(res), 0, converged, total


# --------------------------------------------------------------------------
# Synthetic inputs
# --------------------------------------------------------------------------
def synth_ri3ao(seed, nb, naux, P0=0, P1=None):
    P1 = naux if P1 is None else P1
    B = np.zeros((nb, nb, P1 - P0), order="F")
    lib().oracle_synth_ri3ao(ctypes.c_uint64(seed), nb, naux, int(P0), int(P1), _p(B))
    return B


def synth_coef(seed, nb):
    """C = Q of the Householder QR of an nb x nb N(0,1) matrix (LAPACK dgeqrf/dorgqr via numpy)."""
    M = np.zeros((nb, nb), order="F")
    lib().oracle_synth_coef_seed(ctypes.c_uint64(seed), nb, _p(M))
    Q, _ = np.linalg.qr(M)
    return np.asfortranarray(Q)


def synth_delta(seed, nov):
    d = np.zeros(nov)
    lib().oracle_synth_delta(ctypes.c_uint64(seed), ctypes.c_int64(nov), _p(d))
    return d


from .davidson_ref import DavidsonParams, davidson_solve  # noqa: E402,F401
