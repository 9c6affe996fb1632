"""GPU parity of the ri3fn metric step and the layout utilities, through the C ABI.

special_dgemm_f_01 (restmatr.f90:111-154) and its device form against the
oracle's restatement over OpenBLAS; the block copies, transposes and symmetric
packing (restmatr.f90:197-285, src/ri.rs:226-341) against the oracle's
restatements of the reference's enumeration.

Tolerances (written here):
  * float64 form: 1e-12 relative to max|oracle| (different summation order);
  * split form (7 BF16 digits): 1e-11 relative to max|oracle|;
  * copies, transposes and packing move bytes: bit-exact.
"""
import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RT_ERR_INVALID_ARG = 1


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))).cuda()


def host(t):
    return t.cpu().numpy()


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b))))


# ----------------------------------------------------- special_dgemm_f_01 --
CASES = [
    # size_a, range_x, range_z, size_b, range_row_b, range_col_b, alpha, beta
    ((6, 4, 9), (0, 6), (0, 9), (9, 9), (0, 9), (0, 9), 1.0, 0.0),
    ((7, 5, 12), (2, 6), (3, 10), (11, 13), (1, 8), (4, 11), 0.7, -0.3),
    ((1, 3, 5), (0, 1), (1, 4), (3, 3), (0, 3), (0, 3), -2.0, 1.0),
    ((40, 30, 96), (3, 37), (5, 85), (100, 100), (10, 90), (2, 82), 0.5, 0.25),
    ((120, 120, 480), (0, 120), (0, 480), (480, 480), (0, 480), (0, 480), 1.0, 0.0),
]


def make_case(size_a, size_b, seed=3):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(int(np.prod(size_a))), rng.standard_normal(size_b[0] * size_b[1])


def run_device(t, b, case, form, stream=None):
    size_a, rx, rz, size_b, rrb, rcb, alpha, beta = case
    T, B = dev(t), dev(b)
    rt.special_dgemm_01(T, size_a, range(*rx), range(*rz), B, size_b, range(*rrb), range(*rcb), alpha, beta,
                        form=form)
    torch.cuda.synchronize()
    return host(T)


@pytest.mark.parametrize("form,tol", [("fp64", 1e-12), ("split", 1e-11)])
@pytest.mark.parametrize("ci", range(len(CASES)))
def test_special_dgemm_device_matches_oracle(ci, form, tol):
    case = CASES[ci]
    size_a, rx, rz, size_b, rrb, rcb, alpha, beta = case
    t, b = make_case(size_a, size_b)
    want = oracle.special_dgemm_f_01(t, size_a, rx, rz, b, size_b, rrb, rcb, alpha, beta)
    got = run_device(t, b, case, form)
    assert relerr(got, want) <= tol
    mask = np.ones(size_a, bool)
    mask[rx[0]:rx[1], :, rz[0]:rz[1]] = False
    mask = mask.reshape(-1, order="F")
    assert np.array_equal(got[mask], t[mask])  # outside the block: untouched, bit for bit


@pytest.mark.parametrize("form", ["fp64", "split"])
@pytest.mark.parametrize("slices_per_chunk", [1, 7])
def test_special_dgemm_in_several_chunks_equals_one_chunk(form, slices_per_chunk):
    case = CASES[3]
    size_a, rx, rz, size_b, rrb, rcb, alpha, beta = case
    t, b = make_case(size_a, size_b)
    whole = run_device(t, b, case, form)
    per_y = (rx[1] - rx[0]) * (rz[1] - rz[0]) * 8
    rt.debug_chunk_bytes(per_y * slices_per_chunk)
    try:
        chunked = run_device(t, b, case, form)
    finally:
        rt.debug_chunk_bytes(0)
    # Each output element depends only on its own row of the block, so chunking over y changes nothing.
    assert np.array_equal(chunked, whole)


def test_special_dgemm_host_dropin_matches_oracle():
    case = CASES[1]
    size_a, rx, rz, size_b, rrb, rcb, alpha, beta = case
    t, b = make_case(size_a, size_b)
    want = oracle.special_dgemm_f_01(t, size_a, rx, rz, b, size_b, rrb, rcb, alpha, beta)
    got = t.copy()
    # i_y is ignored, as in the Fortran, which loops over every y-slice
    rt.special_dgemm_f_01(got, size_a, range(*rx), 3, range(*rz), b, size_b, range(*rrb), range(*rcb), alpha, beta)
    assert relerr(got, want) <= 1e-12


def test_special_dgemm_rejects_bad_blocks_and_leaves_data_unchanged():
    size_a, size_b = (7, 5, 12), (11, 13)
    t, b = make_case(size_a, size_b)
    T, B = dev(t), dev(b)
    with pytest.raises(rt.RTError) as e:  # matr_b block 7 x 6, len_z_a 7
        rt.special_dgemm_01(T, size_a, range(2, 6), range(3, 10), B, size_b, range(1, 8), range(4, 10))
    assert e.value.status == RT_ERR_INVALID_ARG
    with pytest.raises(rt.RTError):  # block of ten3_a outside the tensor
        rt.special_dgemm_01(T, size_a, range(2, 8), range(3, 10), B, size_b, range(1, 8), range(4, 11))
    torch.cuda.synchronize()
    assert np.array_equal(host(T), t)
    h = t.copy()
    with pytest.raises(rt.RTError):
        rt.special_dgemm_f_01(h, size_a, range(2, 6), 0, range(3, 10), b, size_b, range(1, 8), range(4, 10), 1.0, 0.0)
    assert np.array_equal(h, t)


# ------------------------------------------------------------ block copies --
def test_copy_mm_matches_oracle():
    rng = np.random.default_rng(5)
    f = rng.standard_normal(37 * 29)
    t = rng.standard_normal(41 * 33)
    want = oracle.copy_mm(20, 11, f, (37, 29), (5, 7), t.copy(), (41, 33), (19, 20))
    T = dev(t)
    rt.copy_mm(20, 11, dev(f), (37, 29), (5, 7), T, (41, 33), (19, 20))
    assert np.array_equal(host(T), want)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_copy_mr_and_rm_match_oracle(mode):
    rng = np.random.default_rng(6 + mode)
    X, Y, Z = 13, 17, 19
    f = rng.standard_normal(23 * 21)
    r = rng.standard_normal(X * Y * Z)
    lens = {0: (9, 11), 1: (9, 14), 2: (12, 14)}[mode]
    start = (2, 3)
    x3 = {0: 18, 1: 16, 2: 12}[mode]
    want = oracle.copy_mr(lens[0], lens[1], f, (23, 21), (4, 6), r.copy(), (X, Y, Z), start, x3, mode)
    R = dev(r)
    rt.copy_mr(lens[0], lens[1], dev(f), (23, 21), (4, 6), R, (X, Y, Z), start, x3, mode)
    assert np.array_equal(host(R), want)

    m = rng.standard_normal(23 * 21)
    want = oracle.copy_rm(lens[0], lens[1], r, (X, Y, Z), start, x3, mode, m.copy(), (23, 21), (4, 6))
    M = dev(m)
    rt.copy_rm(lens[0], lens[1], dev(r), (X, Y, Z), start, x3, mode, M, (23, 21), (4, 6))
    assert np.array_equal(host(M), want)


def test_copy_rr_matches_oracle_and_handles_overlap():
    rng = np.random.default_rng(9)
    a = rng.standard_normal(31 * 27 * 11)
    b = rng.standard_normal(33 * 29 * 13)
    want = oracle.copy_rr((20, 21, 9), a, (31, 27, 11), (3, 5, 1), b.copy(), (33, 29, 13), (13, 2, 4))
    Bd = dev(b)
    rt.copy_rr((20, 21, 9), dev(a), (31, 27, 11), (3, 5, 1), Bd, (33, 29, 13), (13, 2, 4))
    assert np.array_equal(host(Bd), want)
    # source and target blocks inside one tensor, overlapping: the whole source is read first
    want = oracle.copy_rr((20, 20, 8), a, (31, 27, 11), (3, 5, 1), a.copy(), (31, 27, 11), (5, 6, 2))
    Ad = dev(a)
    rt.copy_rr((20, 20, 8), Ad, (31, 27, 11), (3, 5, 1), Ad, (31, 27, 11), (5, 6, 2))
    assert np.array_equal(host(Ad), want)


def test_copy_rejects_bad_mode_and_ranges_and_accepts_empty_blocks():
    r = dev(np.zeros(4 * 5 * 6))
    f = dev(np.ones(6 * 5))
    with pytest.raises(rt.RTError) as e:
        rt.copy_mr(2, 2, f, (6, 5), (0, 0), r, (4, 5, 6), (0, 0), 0, 3)
    assert e.value.status == RT_ERR_INVALID_ARG
    with pytest.raises(rt.RTError):
        rt.copy_mr(4, 2, f, (6, 5), (0, 0), r, (4, 5, 6), (1, 0), 0, 0)  # rows 1..5 of a 4-row tensor
    rt.copy_mr(0, 2, f, (6, 5), (0, 0), r, (4, 5, 6), (0, 0), 0, 0)
    torch.cuda.synchronize()
    assert float(r.abs().sum()) == 0.0


# -------------------------------------------------------------- transposes --
PERMS = {"ijk": (0, 1, 2), "jik": (1, 0, 2), "jki": (1, 2, 0), "kji": (2, 1, 0), "ikj": (0, 2, 1), "kij": (2, 0, 1)}


@pytest.mark.parametrize("order", ["jik", "jki", "kji", "ikj"])
@pytest.mark.parametrize("size", [(3, 2, 2), (9, 3, 2), (5, 4, 3)])
def test_transpose_matches_reference_enumeration(order, size):
    data = np.arange(int(np.prod(size)), dtype=np.float64)
    want = np.array(getattr(oracle, "transpose_" + order)(list(data), list(size)))
    got = host(rt.ri_transpose(dev(data), size, order))
    torch.cuda.synchronize()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("order", sorted(PERMS))
@pytest.mark.parametrize("size", [(257, 129, 33), (600, 600, 24), (1, 700, 300), (70, 1, 90)])
def test_transpose_large_and_ragged(order, size):
    rng = np.random.default_rng(11)
    a = rng.standard_normal(int(np.prod(size)))
    want = np.transpose(a.reshape(size, order="F"), PERMS[order]).reshape(-1, order="F")
    got = host(rt.ri_transpose(dev(a), size, order))
    assert np.array_equal(got, want)


def test_transpose_rejects_bad_orders():
    a = dev(np.zeros(24))
    for bad in ["iik", "ij", "abc"]:
        with pytest.raises(rt.RTError):
            rt.ri_transpose(a, (2, 3, 4), bad)


# ----------------------------------------------------------------- packing --
@pytest.mark.parametrize("nao,naux", [(1, 1), (7, 3), (33, 5)])
def test_pack_symm_matches_reference_enumeration(nao, naux):
    data = np.arange(nao * nao * naux, dtype=np.float64)
    want = np.array(oracle.rifull_to_matfull_symm(list(data), nao, naux))
    got = host(rt.ri_pack_symm(dev(data), nao, naux))
    assert np.array_equal(got, want)


def test_pack_symm_at_full_basis_size():
    nao, naux = 600, 40
    B = torch.from_numpy(oracle.synth_ri3ao(4, nao, naux).reshape(-1, order="F")).cuda()
    got = host(rt.ri_pack_symm(B, nao, naux)).reshape((-1, naux), order="F")
    R = host(B).reshape((nao, nao, naux), order="F")
    r, c = np.triu_indices(nao)
    o = np.lexsort((r, c))
    assert np.array_equal(got, R[r[o], c[o], :])
