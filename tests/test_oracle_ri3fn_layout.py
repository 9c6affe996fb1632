"""CPU checks of the oracle for the ri3fn metric step and the layout utilities.

The reference has no asserting test for either: its transpose tests
(src/ri.rs:436-476) print their results.  The oracle therefore restates the
reference's own enumeration (ri.rs:226-341, restmatr.f90:111-285), and these
tests pin that restatement against independent numpy formulations, including
on the reference tests' own input tensors.
"""
import numpy as np
import pytest

import oracle


def fview(flat, size):
    return np.asarray(flat).reshape(tuple(size), order="F")


# ----------------------------------------------------- special_dgemm_f_01 --
@pytest.mark.parametrize("case", [
    # size_a, range_x, range_z, size_b, range_row_b, range_col_b, alpha, beta
    ((6, 4, 9), (0, 6), (0, 9), (9, 9), (0, 9), (0, 9), 1.0, 0.0),
    ((7, 5, 12), (2, 6), (3, 10), (11, 13), (1, 8), (4, 11), 0.7, -0.3),
    ((1, 3, 5), (0, 1), (1, 4), (3, 3), (0, 3), (0, 3), -2.0, 1.0),
])
def test_special_dgemm_oracle_matches_per_slice_numpy(case):
    size_a, rx, rz, size_b, rrb, rcb, alpha, beta = case
    rng = np.random.default_rng(1)
    t = rng.standard_normal(int(np.prod(size_a)))
    b = rng.standard_normal(size_b[0] * size_b[1])
    got = fview(oracle.special_dgemm_f_01(t, size_a, rx, rz, b, size_b, rrb, rcb, alpha, beta), size_a)
    T = fview(t, size_a).copy()
    B = fview(b, size_b)[rrb[0]:rrb[1], rcb[0]:rcb[1]]
    for y in range(size_a[1]):
        blk = T[rx[0]:rx[1], y, rz[0]:rz[1]]
        T[rx[0]:rx[1], y, rz[0]:rz[1]] = alpha * blk @ B + beta * blk
    np.testing.assert_allclose(got, T, rtol=0, atol=1e-13 * max(1.0, np.abs(T).max()))
    # elements outside the block are untouched
    mask = np.ones(size_a, bool)
    mask[rx[0]:rx[1], :, rz[0]:rz[1]] = False
    assert np.array_equal(got[mask], fview(t, size_a)[mask])


# ------------------------------------------------------------- transposes --
PERMS = {"jik": (1, 0, 2), "jki": (1, 2, 0), "kji": (2, 1, 0), "ikj": (0, 2, 1)}


@pytest.mark.parametrize("size", [(3, 2, 2), (9, 3, 2), (3, 2, 3), (5, 4, 3), (1, 6, 2)])
@pytest.mark.parametrize("order", sorted(PERMS))
def test_transpose_restatement_matches_numpy(size, order):
    # (3, 2, 2) holds 0..12 as in ri.rs:437-449; (9, 3, 2) and (3, 2, 3) are ri.rs:452-459's tensors.
    data = list(np.arange(int(np.prod(size)), dtype=np.float64))
    got = np.array(getattr(oracle, "transpose_" + order)(data, list(size)))
    want = np.transpose(fview(np.array(data), size), PERMS[order]).reshape(-1, order="F")
    assert np.array_equal(got, want)


@pytest.mark.parametrize("nao,naux", [(1, 1), (3, 2), (7, 3)])
def test_pack_symm_restatement_keeps_upper_triangle(nao, naux):
    data = np.arange(nao * nao * naux, dtype=np.float64)
    got = np.array(oracle.rifull_to_matfull_symm(list(data), nao, naux)).reshape((-1, naux), order="F")
    R = fview(data, (nao, nao, naux))
    r, c = np.triu_indices(nao)
    order = np.lexsort((r, c))  # column-major over the upper triangle
    want = R[r[order], c[order], :]
    assert got.shape == (nao * (nao + 1) // 2, naux)
    assert np.array_equal(got, want)


# ------------------------------------------------------------- block copies --
def test_copy_oracles_follow_fortran_sections():
    rng = np.random.default_rng(2)
    f = rng.standard_normal(6 * 5)
    t = np.zeros(7 * 8)
    oracle.copy_mm(3, 2, f, (6, 5), (1, 2), t, (7, 8), (4, 5))
    assert np.array_equal(fview(t, (7, 8))[4:7, 5:7], fview(f, (6, 5))[1:4, 2:4])
    assert np.count_nonzero(t) == 6

    R = np.zeros(4 * 5 * 6)
    oracle.copy_mr(3, 2, f, (6, 5), (1, 2), R, (4, 5, 6), (1, 3), 2, 1)  # mode 1: (a, x3, b)
    assert np.array_equal(fview(R, (4, 5, 6))[1:4, 2, 3:5], fview(f, (6, 5))[1:4, 2:4])
    back = np.zeros(6 * 5)
    oracle.copy_rm(3, 2, R, (4, 5, 6), (1, 3), 2, 1, back, (6, 5), (1, 2))
    assert np.array_equal(fview(back, (6, 5))[1:4, 2:4], fview(f, (6, 5))[1:4, 2:4])
    untouched = R.copy()
    oracle.copy_mr(3, 2, f, (6, 5), (1, 2), R, (4, 5, 6), (1, 3), 2, 7)  # unknown mode: nothing
    assert np.array_equal(R, untouched)

    a = rng.standard_normal(4 * 5 * 6)
    b = np.zeros(5 * 6 * 7)
    oracle.copy_rr((2, 3, 4), a, (4, 5, 6), (1, 2, 2), b, (5, 6, 7), (3, 0, 1))
    assert np.array_equal(fview(b, (5, 6, 7))[3:5, 0:3, 1:5], fview(a, (4, 5, 6))[1:3, 2:5, 2:6])
