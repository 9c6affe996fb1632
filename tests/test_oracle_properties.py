"""Property-based checks of the oracle's layout and ri3fn restatements (CPU only).

Random shapes, blocks and modes: the reference-enumeration restatements must
agree with independent numpy formulations.  Skipped where hypothesis is not
installed.
"""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings  # noqa: E402
from hypothesis import strategies as st  # noqa: E402

import oracle  # noqa: E402

PERMS = {"jik": (1, 0, 2), "jki": (1, 2, 0), "kji": (2, 1, 0), "ikj": (0, 2, 1)}
dims = st.integers(min_value=1, max_value=6)


@settings(max_examples=60, deadline=None)
@given(i=dims, j=dims, k=dims, order=st.sampled_from(sorted(PERMS)))
def test_transposes_are_axis_permutations(i, j, k, order):
    a = np.arange(i * j * k, dtype=np.float64)
    got = np.array(getattr(oracle, "transpose_" + order)(list(a), [i, j, k]))
    want = np.transpose(a.reshape((i, j, k), order="F"), PERMS[order]).reshape(-1, order="F")
    assert np.array_equal(got, want)


@settings(max_examples=40, deadline=None)
@given(nao=st.integers(1, 9), naux=st.integers(1, 4))
def test_pack_symm_is_the_column_major_upper_triangle(nao, naux):
    a = np.arange(nao * nao * naux, dtype=np.float64)
    got = np.array(oracle.rifull_to_matfull_symm(list(a), nao, naux)).reshape((-1, naux), order="F")
    R = a.reshape((nao, nao, naux), order="F")
    want = np.concatenate([R[: c + 1, c, :] for c in range(nao)], axis=0)
    assert np.array_equal(got, want)


@st.composite
def blocks(draw):
    X, Y, Z = draw(st.integers(1, 6)), draw(st.integers(1, 4)), draw(st.integers(1, 7))
    sx = draw(st.integers(0, X - 1))
    lx = draw(st.integers(1, X - sx))
    sz = draw(st.integers(0, Z - 1))
    lz = draw(st.integers(1, Z - sz))
    rows = draw(st.integers(lz, lz + 3))
    cols = draw(st.integers(lz, lz + 3))
    rb = draw(st.integers(0, rows - lz))
    cb = draw(st.integers(0, cols - lz))
    alpha = draw(st.sampled_from([1.0, 0.5, -2.0, 0.0]))
    beta = draw(st.sampled_from([0.0, 1.0, -0.25]))
    return (X, Y, Z), (sx, sx + lx), (sz, sz + lz), (rows, cols), (rb, rb + lz), (cb, cb + lz), alpha, beta


@settings(max_examples=60, deadline=None)
@given(case=blocks(), seed=st.integers(0, 2 ** 16))
def test_special_dgemm_restatement_matches_numpy(case, seed):
    size_a, rx, rz, size_b, rrb, rcb, alpha, beta = case
    rng = np.random.default_rng(seed)
    t = rng.standard_normal(int(np.prod(size_a)))
    b = rng.standard_normal(size_b[0] * size_b[1])
    got = oracle.special_dgemm_f_01(t, size_a, rx, rz, b, size_b, rrb, rcb, alpha, beta).reshape(size_a, order="F")
    T = t.reshape(size_a, order="F").copy()
    B = b.reshape(size_b, order="F")[rrb[0]:rrb[1], rcb[0]:rcb[1]]
    for y in range(size_a[1]):
        blk = T[rx[0]:rx[1], y, rz[0]:rz[1]].copy()
        T[rx[0]:rx[1], y, rz[0]:rz[1]] = alpha * (blk @ B) + beta * blk
    np.testing.assert_allclose(got, T, rtol=0, atol=1e-12 * max(1.0, np.abs(T).max()))


@settings(max_examples=40, deadline=None)
@given(mode=st.sampled_from([0, 1, 2]), seed=st.integers(0, 2 ** 16))
def test_copy_mr_then_rm_round_trips(mode, seed):
    rng = np.random.default_rng(seed)
    X, Y, Z = 5, 6, 7
    full = (X, Y, Z)
    a_axis = {0: 0, 1: 0, 2: 1}[mode]
    b_axis = {0: 1, 1: 2, 2: 2}[mode]
    f_axis = {0: 2, 1: 1, 2: 0}[mode]
    la = int(rng.integers(1, full[a_axis] + 1))
    lb = int(rng.integers(1, full[b_axis] + 1))
    sa = int(rng.integers(0, full[a_axis] - la + 1))
    sb = int(rng.integers(0, full[b_axis] - lb + 1))
    fix = int(rng.integers(0, full[f_axis]))
    m = rng.standard_normal(la * lb)
    R = np.zeros(X * Y * Z)
    oracle.copy_mr(la, lb, m, (la, lb), (0, 0), R, (X, Y, Z), (sa, sb), fix, mode)
    back = np.zeros(la * lb)
    oracle.copy_rm(la, lb, R, (X, Y, Z), (sa, sb), fix, mode, back, (la, lb), (0, 0))
    assert np.array_equal(back, m)
    assert np.count_nonzero(R) == np.count_nonzero(m)
