"""GPU parity of the native RI path against the CPU oracle, through the C ABI.

Tolerances (written here, judged against the oracle's float64 results):
  * float64 form: 1e-12 relative to max|reference| (the reference path is
    IEEE float64 with a different summation order);
  * split form (6 BF16 digits): ov and ri3mo within 1e-10 absolute (values are
    O(0.1-1)), K within 1e-11 relative to max|K|, E_x within 1e-9 relative.
"""
import json
import os

import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_doctests.json")))


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))).cuda()


def host(t, shape):
    return t.cpu().numpy().reshape(shape, order="F")


def inputs(nb, naux, seed=0):
    return oracle.synth_coef(seed, nb), oracle.synth_ri3ao(seed, nb, naux)


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b))))


# ------------------------------------------------------------- GEMM seam --
@pytest.mark.parametrize("name", ["general_dgemm_f", "_dgemm_0", "_dgemm_1", "_dgemm_2"])
def test_gemm_seam_doctests_on_gpu(name):
    c = next(x for x in GOLD["cases"] if x["name"] == name)
    a = np.arange(1, 10, dtype=np.float64)
    b = a + 5.0
    out = np.full(9, c["c_init"])
    rt.general_dgemm_f(a, [3, 3], range(*c["rows_a"]), range(*c["cols_a"]), c["opa"],
                       b, [3, 3], range(*c["rows_b"]), range(*c["cols_b"]), c["opb"],
                       out, [3, 3], range(*c["rows_c"]), range(*c["cols_c"]), c["alpha"], c["beta"])
    m = out.reshape(3, 3, order="F")
    r0, r1 = c["check_rows"]
    c0, c1 = c["check_cols"]
    assert m[r0:r1, c0:c1].flatten(order="F").tolist() == c["expected"]


# Shapes cover every float64 tile form: 64x64, 128x32 (n <= 32), 32x128 (m <= 32),
# 256x16 (n <= 16) and 16x256 (m <= 16), under all four op pairs.
@pytest.mark.parametrize("opa,opb,m,n,k", [("N", "N", 70, 33, 129), ("T", "N", 64, 64, 17), ("N", "T", 1, 200, 5),
                                           ("T", "T", 129, 65, 300), ("N", "N", 40, 30, 5000),
                                           ("T", "N", 20, 100, 50), ("N", "T", 300, 7, 90), ("T", "T", 9, 333, 77),
                                           ("N", "N", 257, 16, 33), ("T", "N", 100, 31, 64), ("N", "T", 31, 97, 19)])
def test_rt_dgemm_matches_oracle(opa, opb, m, n, k):
    rng = np.random.default_rng(m * 7 + n)
    A = np.asfortranarray(rng.standard_normal((m, k) if opa == "N" else (k, m)))
    B = np.asfortranarray(rng.standard_normal((k, n) if opb == "N" else (n, k)))
    C = np.asfortranarray(rng.standard_normal((m, n)))
    ref = oracle.dgemm(opa, opb, A, B, alpha=0.75, beta=-0.5, c=C.copy(order="F"))
    dC = dev(C)
    rt.dgemm(opa, opb, m, n, k, 0.75, dev(A), A.shape[0], dev(B), B.shape[0], -0.5, dC, m)
    assert relerr(host(dC, (m, n)), ref) < 1e-12


# ---------------------------------------------------------------- ao2mo --
def test_ri_ao2mo_f_bench_known_answer():
    c = next(x for x in GOLD["cases"] if x["name"] == "bench_ao2mo")
    nb, _, naux = c["ri3fn_size"]
    ri = rt.RIFull.new([nb, nb, naux], c["ri3fn_fill"])
    ev = rt.MatrixFull.new(c["eigenvector_size"], c["eigenvector_fill"])
    out = ri.ao2mo(ev)
    assert out.size == [naux, 10, 10]
    assert np.all(out.data == c["expected_every_element"])


@pytest.mark.parametrize("nb,ns,naux", [(24, 24, 9), (33, 33, 7), (65, 65, 3), (100, 100, 40), (1, 1, 2)])
def test_ri_ao2mo_f_dropin_matches_oracle(nb, ns, naux):
    C, B = inputs(nb, naux, seed=nb)
    ref = oracle.ri_ao2mo(C, B)
    ri = rt.RIFull.from_vec([nb, nb, naux], B.reshape(-1, order="F"))
    out = ri.ao2mo(rt.MatrixFull.from_vec([nb, ns], C[:, :ns].reshape(-1, order="F")))
    assert relerr(out.to_numpy(), ref) < 1e-12


def test_ri_ao2mo_fewer_states_is_the_intended_math():
    nb, ns, naux = 40, 17, 5
    C, B = inputs(nb, naux, seed=2)
    Cs = np.asfortranarray(C[:, :ns])
    ref = np.einsum("mp,mnP,nq->Ppq", Cs, B, Cs)
    out = rt.ri_ao2mo(dev(Cs), dev(B), nb, ns, naux, form="fp64")
    assert relerr(host(out, (naux, ns, ns)), ref) < 1e-12


@pytest.mark.parametrize("nb,naux", [(24, 9), (65, 13), (100, 40)])
def test_ri_ao2mo_split_matches_oracle(nb, naux):
    C, B = inputs(nb, naux, seed=nb + 1)
    ref = oracle.ri_ao2mo(C, B)
    out = rt.ri_ao2mo(dev(C), dev(B), nb, nb, naux, form="split")
    rt.sync_status()
    assert np.max(np.abs(host(out, (naux, nb, nb)) - ref)) < 1e-10


# ------------------------------------------------------------ ov + RI-K --
CASES = [(20, 12, 4), (33, 7, 5), (100, 400, 20), (64, 16, 64), (130, 9, 1)]


@pytest.mark.parametrize("nb,naux,nocc", CASES)
def test_ri_ov_k_fp64_matches_oracle(nb, naux, nocc):
    C, B = inputs(nb, naux, seed=nocc)
    nvir = nb - nocc
    ov_ref, K_ref = oracle.ri_ov_k(C, B, nocc)
    ov, K = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nvir, form="fp64")
    if nvir:
        assert relerr(host(ov, (nocc, nvir, naux)), ov_ref) < 1e-12
    assert relerr(host(K, (nb, nb)), K_ref) < 1e-12


@pytest.mark.parametrize("nb,naux,nocc", CASES)
def test_ri_ov_k_split_matches_oracle(nb, naux, nocc):
    C, B = inputs(nb, naux, seed=nocc)
    nvir = nb - nocc
    ov_ref, K_ref = oracle.ri_ov_k(C, B, nocc)
    ov, K = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nvir, form="split", nslices=6)
    rt.sync_status()
    if nvir:
        assert np.max(np.abs(host(ov, (nocc, nvir, naux)) - ov_ref)) < 1e-10
    Kh = host(K, (nb, nb))
    assert relerr(Kh, K_ref) < 1e-11
    assert np.array_equal(Kh, Kh.T)


@pytest.mark.parametrize("S,nb", [(6, 850), (7, 700)])
def test_split_multichunk_contraction(S, nb):
    # nb above the exact-chunk length (800 terms at S = 6, 672 at S = 7) forces two
    # exact chunks along the contraction in the first half-transform.
    naux, nocc = 3, 6
    C, B = inputs(nb, naux, seed=11)
    ov_ref, K_ref = oracle.ri_ov_k(C, B, nocc)
    ov, K = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nb - nocc, form="split", nslices=S)
    assert np.max(np.abs(host(ov, (nocc, nb - nocc, naux)) - ov_ref)) < 1e-10
    assert relerr(host(K, (nb, nb)), K_ref) < 1e-11


@pytest.mark.parametrize("S", [3, 4, 5, 7, 8])
def test_split_slice_counts_converge(S):
    nb, naux, nocc = 48, 6, 8
    C, B = inputs(nb, naux, seed=S)
    ov_ref, _ = oracle.ri_ov_k(C, B, nocc)
    ov, _ = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nb - nocc, form="split", nslices=S)
    err = np.max(np.abs(host(ov, (nocc, nb - nocc, naux)) - ov_ref))
    # each extra BF16 digit carries 7 more bits
    assert err < 2.0 ** (-(7 * S - 10))


def test_split_is_bitwise_deterministic():
    nb, naux, nocc = 64, 20, 8
    C, B = inputs(nb, naux, seed=5)
    a = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nb - nocc, form="split")
    b = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nb - nocc, form="split")
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


def test_empty_and_degenerate_shapes():
    nb, naux = 10, 4
    C, B = inputs(nb, naux, seed=3)
    for form in ("fp64", "split"):
        ov, K = rt.ri_ov_k(dev(C), dev(B), nb, naux, 0, nb, form=form)
        assert torch.count_nonzero(K).item() == 0
        ov, K = rt.ri_ov_k(dev(C), dev(B), nb, 0, 3, 7, form=form)
        assert torch.count_nonzero(K).item() == 0


# ------------------------------------------------------------ J and E_x --
# Even and odd slab lengths (16-byte and scalar J kernels), naux above the 1024 slabs of one w stage.
@pytest.mark.parametrize("nb,naux", [(20, 12), (33, 7), (100, 400), (40, 1100), (600, 96), (750, 33), (1200, 20)])
def test_ri_j_matches_oracle(nb, naux):
    C, B = inputs(nb, naux, seed=1)
    D = np.asfortranarray(C[:, :5] @ C[:, :5].T)
    w_ref, J_ref = oracle.ri_j(B, D)
    w, J = rt.ri_j(dev(B), dev(D), nb, naux)
    assert relerr(w.cpu().numpy(), w_ref) < 1e-12
    assert relerr(host(J, (nb, nb)), J_ref) < 1e-12
    w2, J2 = rt.ri_j(dev(B), dev(D), nb, naux)  # fixed reduction orders: bitwise repeatable
    assert torch.equal(w, w2) and torch.equal(J, J2)


# The synthetic ri3ao is symmetric per slab; odd and even nb, one column pair
# per warp and many, naux above one 1024-slab w stage and split over blocks.
@pytest.mark.parametrize("nb,naux", [(1, 3), (2, 5), (20, 12), (33, 7), (100, 400), (40, 1100), (600, 96), (751, 33)])
def test_ri_j_symmetric_matches_oracle(nb, naux):
    C, B = inputs(nb, naux, seed=1)
    D = np.asfortranarray(C[:, :5] @ C[:, :5].T)
    D = np.asfortranarray(0.5 * (D + D.T))
    w_ref, J_ref = oracle.ri_j(B, D)
    w, J = rt.ri_j(dev(B), dev(D), nb, naux, symmetric=True)
    assert relerr(w.cpu().numpy(), w_ref) < 1e-12
    Jh = host(J, (nb, nb))
    assert relerr(Jh, J_ref) < 1e-12
    assert np.array_equal(Jh, Jh.T)
    w2, J2 = rt.ri_j(dev(B), dev(D), nb, naux, symmetric=True)
    assert torch.equal(w, w2) and torch.equal(J, J2)


def test_ri_j_symmetric_reads_only_the_upper_triangles():
    nb, naux = 90, 70
    C, B = inputs(nb, naux, seed=2)
    D = np.asfortranarray(C[:, :7] @ C[:, :7].T)
    D = np.asfortranarray(0.5 * (D + D.T))
    w_ref, J_ref = rt.ri_j(dev(B), dev(D), nb, naux, symmetric=True)
    low = np.tril(np.ones((nb, nb), dtype=bool), -1)
    Bg, Dg = B.copy(order="F"), D.copy(order="F")
    Bg[low, :] = 1e300  # anything below the diagonal must be ignored
    Dg[low] = -1e300
    w, J = rt.ri_j(dev(Bg), dev(Dg), nb, naux, symmetric=True)
    assert torch.equal(w, w_ref) and torch.equal(J, J_ref)


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_exchange_energy(form):
    nb, naux, nocc = 100, 400, 20
    C, B = inputs(nb, naux, seed=0)
    _, K_ref = oracle.ri_ov_k(C, B, nocc)
    D = np.asfortranarray(C[:, :nocc] @ C[:, :nocc].T)
    ex_ref = oracle.exchange_energy(D, K_ref)
    _, K = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nb - nocc, form=form)
    ex = rt.exchange_energy(dev(D), K, nb).item()
    tol = 1e-12 if form == "fp64" else 1e-9
    assert abs(ex - ex_ref) < tol * abs(ex_ref)


# ------------------------------------------------------- host entry point --
def test_host_entry_matches_device_entry_and_flags_nonfinite():
    nb, naux, nocc = 40, 10, 6
    C, B = inputs(nb, naux, seed=9)
    nvir = nb - nocc
    ov_h = np.zeros(nocc * nvir * naux)
    K_h = np.zeros(nb * nb)
    Cf, Bf = C.reshape(-1, order="F").copy(), B.reshape(-1, order="F").copy()
    rt.ri_ov_k_host(Cf, Bf, nb, naux, nocc, nvir, ov_h, K_h, form="split")
    ov, K = rt.ri_ov_k(dev(C), dev(B), nb, naux, nocc, nvir, form="split")
    assert np.array_equal(ov_h, ov.cpu().numpy()) and np.array_equal(K_h, K.cpu().numpy())
    Bf[17] = np.nan
    with pytest.raises(rt.RTError) as e:
        rt.ri_ov_k_host(Cf, Bf, nb, naux, nocc, nvir, ov_h, K_h, form="split")
    assert e.value.status == 5


def test_device_synth_matches_host_formula():
    nb, naux = 16, 3
    ref = oracle.synth_ri3ao(7, nb, naux)
    got = host(rt.synth_ri3ao(7, nb, naux), (nb, nb, naux))
    assert np.max(np.abs(got - ref)) < 1e-14


# ------------------------------------------------ split GEMM exactness --
@pytest.mark.parametrize("opa,opb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("S", [5, 7, 8])
@pytest.mark.parametrize("k", [1000, 1500])  # one-pass (8-row) and two-pass slicing of strided rows
def test_split_gemm_is_exact_on_short_integers(opa, opb, S, k):
    """Integers of at most 20 significant bits need only digits 0..2; every
    dropped digit pair is then zero, the float64 products are exact, and the
    split form must reproduce them bit for bit (the exact-accumulation claim)."""
    rng = np.random.default_rng(S)
    m, n = 200, 130  # k spans two or three exact chunks at S = 7
    A = rng.integers(-(2 ** 19), 2 ** 19, size=(m, k) if opa == "N" else (k, m)).astype(np.float64)
    B = rng.integers(-(2 ** 19), 2 ** 19, size=(k, n) if opb == "N" else (n, k)).astype(np.float64)
    # Give every row of op(A) and column of op(B) the same maximum exponent, so 20 bits fit in 3 digits.
    A.flat[0::7] = 2.0 ** 19 - 1
    B.flat[0::5] = -(2.0 ** 19 - 1)
    A, B = np.asfortranarray(A), np.asfortranarray(B)
    ref = (A if opa == "N" else A.T) @ (B if opb == "N" else B.T)
    assert np.all(np.abs(ref) < 2.0 ** 52)  # exact in float64
    dC = torch.zeros(m * n, dtype=torch.float64, device="cuda")
    rt.dgemm_split(opa, opb, m, n, k, dev(A), A.shape[0], dev(B), B.shape[0], dC, m, nslices=S)
    got = host(dC, (m, n))
    assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))


def test_split_rounding_has_no_bias_on_ties():
    """Values on a 2^-48 grid with row maximum 1.5 put every odd multiple
    exactly on a rounding tie of the last (7th) digit.  Ties must not all go
    one way: the diagonal of X X^T must match the exact sum of squares with
    no mean bias (ties rounded away from zero gave about +1e-14)."""
    rng = np.random.default_rng(3)
    nb, k = 64, 5000
    J = np.clip(np.rint(rng.standard_normal((nb, k)) * 0.3 * 2.0 ** 48), -1.4 * 2 ** 48, 1.4 * 2 ** 48).astype(np.int64)
    J[:, 0] = int(1.5 * 2 ** 48)
    X = np.asfortranarray(J.astype(np.float64) * 2.0 ** -48)
    dX = dev(X)
    K = torch.zeros(nb * nb, dtype=torch.float64, device="cuda")
    rt.dgemm_split("N", "T", nb, nb, k, dX, nb, dX, nb, K, nb, nslices=7)
    d = torch.diagonal(K.view(nb, nb)).cpu().numpy()
    exact = [sum(int(j) * int(j) for j in J[i].tolist()) for i in range(nb)]
    rel = np.array([(d[i] * 2.0 ** 96 - exact[i]) / exact[i] for i in range(nb)])
    assert abs(rel.mean()) < 2e-15 and np.max(np.abs(rel)) < 1e-13


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_pipelined_host_entry_is_bitwise_equal_to_device_entry(form):
    # 864 MB of ri3ao: the host entry streams it in two slab blocks, overlapping
    # copies with compute; every element's arithmetic is unchanged by blocking.
    nb, naux, nocc = 600, 300, 60
    nvir = nb - nocc
    B = rt.synth_ri3ao(11, nb, naux)
    C = rt.synth_coef(11, nb)
    ov, K = rt.ri_ov_k(C, B, nb, naux, nocc, nvir, form=form, nslices=7)
    hB = torch.empty(B.numel(), dtype=torch.float64).pin_memory()
    hB.copy_(B)
    hC = C.cpu()
    hO = np.zeros(nocc * nvir * naux)
    hK = np.zeros(nb * nb)
    rt.ri_ov_k_host(hC.data_ptr(), hB.data_ptr(), nb, naux, nocc, nvir, hO, hK, form=form, nslices=7)
    assert np.array_equal(hO, ov.cpu().numpy())
    assert np.array_equal(hK, K.cpu().numpy())


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_symmetric_host_entry_is_bitwise_equal_to_device_entry(form):
    # The synthetic ri3ao is exactly symmetric per slab, so reading only the
    # upper triangles across the host link changes nothing.
    nb, naux, nocc = 600, 300, 60
    nvir = nb - nocc
    B = rt.synth_ri3ao(11, nb, naux)
    C = rt.synth_coef(11, nb)
    ov, K = rt.ri_ov_k(C, B, nb, naux, nocc, nvir, form=form, nslices=7)
    hB = torch.empty(B.numel(), dtype=torch.float64).pin_memory()
    hB.copy_(B)
    hC = C.cpu()  # held for the call: the entry reads it through a raw address
    hO = np.zeros(nocc * nvir * naux)
    hK = np.zeros(nb * nb)
    rt.ri_ov_k_host(hC.data_ptr(), hB.data_ptr(), nb, naux, nocc, nvir, hO, hK, form=form, nslices=7,
                    symmetric=True)
    assert np.array_equal(hO, ov.cpu().numpy())
    assert np.array_equal(hK, K.cpu().numpy())


@pytest.mark.parametrize("nb", [1, 31, 33, 100])
def test_symmetric_host_entry_mirrors_the_upper_triangle(nb):
    # Non-symmetric input: the result is that of the slabs symmetrised from their
    # upper triangles (mu <= nu), for sizes around the 32-wide column blocks.
    naux, nocc = 7, max(1, nb // 5)
    nvir = nb - nocc
    rng = np.random.default_rng(nb)
    Bh = rng.standard_normal((nb, nb, naux))
    up = np.triu(np.ones((nb, nb), dtype=bool))
    Bsym = np.where(up[:, :, None], Bh, np.transpose(Bh, (1, 0, 2)))
    C = oracle.synth_coef(nb, nb)
    ov_ref, K_ref = oracle.ri_ov_k(C, Bsym, nocc)
    hO = np.zeros(max(1, nocc * nvir * naux))
    hK = np.zeros(nb * nb)
    rt.ri_ov_k_host(np.asfortranarray(C), np.asfortranarray(Bh), nb, naux, nocc, nvir, hO, hK, form="fp64",
                    symmetric=True)
    if nvir:
        assert relerr(hO[:nocc * nvir * naux].reshape(nocc, nvir, naux, order="F"), ov_ref) < 1e-12
    assert relerr(hK.reshape(nb, nb, order="F"), K_ref) < 1e-12


def test_split_ov_k_replays_from_a_cuda_graph():
    """The single-molecule split path captured in a CUDA graph (scratch as graph
    allocation nodes) replays to the uncaptured result, bit for bit."""
    nb, naux, nocc = 64, 48, 8
    C, B = inputs(nb, naux, seed=3)
    dC, dB = dev(C), dev(B)
    ov0, K0 = rt.ri_ov_k(dC, dB, nb, naux, nocc, nb - nocc, form="split")  # uncaptured first call
    torch.cuda.synchronize()
    ov = torch.zeros_like(ov0)
    K = torch.zeros_like(K0)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rt.ri_ov_k(dC, dB, nb, naux, nocc, nb - nocc, ov=ov, K=K, form="split", stream=s)
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(ov, ov0) and torch.equal(K, K0)
    _, K_ref = oracle.ri_ov_k(C, B, nocc)
    assert relerr(host(K, (nb, nb)), K_ref) < 1e-11
