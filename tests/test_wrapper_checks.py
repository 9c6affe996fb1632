"""Size checks of the device-tensor wrappers, on the CPU.

Each wrapper passes the extent the native call will touch to ``_dptr``, which
refuses a tensor with fewer elements (ValueError) before any native call.
Here the native library is a stub and ``_dptr`` a recorder applying the same
rule to stand-in tensors, so the extents each wrapper asks for are checked
without a GPU.
"""
import pytest

import rest_tensors_gb300 as rt


class Fake:
    """Stand-in for a device tensor with n elements."""

    def __init__(self, n):
        self.n = n
        self.device = "fake"

    def numel(self):
        return self.n


@pytest.fixture
def stub(monkeypatch):
    calls = []

    class Lib:
        def __getattr__(self, name):
            def f(*a):
                calls.append(name)
                return 0
            return f

    def dptr(t, need=0, name="tensor"):
        if t is None or isinstance(t, int):
            return t
        if t.numel() < need:
            raise ValueError(f"{name}: {t.numel()} elements, the call needs {need}")
        return 1

    monkeypatch.setattr(rt, "lib", lambda: Lib())
    monkeypatch.setattr(rt, "_dptr", dptr)
    monkeypatch.setattr(rt, "_stream", lambda s: 0)
    return calls


def test_mat_extent_and_gemm_extents():
    assert rt._mat_extent(10, 7, 3) == 27
    assert rt._mat_extent(10, 0, 3) == 0
    # C = A^T B^T, m=4, n=5, k=6: A is 6 x 4 (lda 8), B is 5 x 6 (ldb 5), C 4 x 5 (ldc 4)
    assert rt._gemm_extents("T", "T", 4, 5, 6, 8, 5, 4) == (3 * 8 + 6, 5 * 5 + 5, 4 * 4 + 4)
    assert rt._gemm_extents("N", "N", 4, 5, 6, 4, 6, 4) == (5 * 4 + 4, 4 * 6 + 6, 4 * 4 + 4)


def test_ri_ov_k_refuses_short_tensors(stub):
    nb, naux, nocc, nvir = 10, 4, 3, 7
    good = dict(C=Fake(nb * nb), B=Fake(nb * nb * naux), ov=Fake(nocc * nvir * naux), K=Fake(nb * nb))
    rt.ri_ov_k(good["C"], good["B"], nb, naux, nocc, nvir, ov=good["ov"], K=good["K"])
    assert stub == ["rt_ri_ov_k"]
    for key in good:
        bad = dict(good)
        bad[key] = Fake(good[key].n - 1)
        with pytest.raises(ValueError, match=key):
            rt.ri_ov_k(bad["C"], bad["B"], nb, naux, nocc, nvir, ov=bad["ov"], K=bad["K"])
    assert stub == ["rt_ri_ov_k"]  # no native call after a refusal


def test_other_wrappers_refuse_short_tensors(stub):
    nb, naux = 6, 5
    with pytest.raises(ValueError, match="B"):
        rt.ri_j(Fake(nb * nb * naux - 1), Fake(nb * nb), nb, naux, w=Fake(naux), J=Fake(nb * nb))
    with pytest.raises(ValueError, match="J"):
        rt.ri_j(Fake(nb * nb * naux), Fake(nb * nb), nb, naux, w=Fake(naux), J=Fake(nb * nb - 1))
    with pytest.raises(ValueError, match="out"):
        rt.ri_ao2mo(Fake(nb * nb), Fake(nb * nb * naux), nb, nb, naux, out=Fake(naux * nb * nb - 1))
    with pytest.raises(ValueError, match="C"):
        rt.dgemm("N", "N", 4, 5, 6, 1.0, Fake(24), 4, Fake(30), 6, 0.0, Fake(19), 4)
    with pytest.raises(ValueError, match="A"):
        rt.dgemm_split("T", "N", 4, 5, 6, Fake(23), 6, Fake(30), 6, Fake(20), 4)
    with pytest.raises(ValueError, match="K"):
        rt.exchange_energy(Fake(nb * nb), Fake(nb * nb - 1), nb, out=Fake(1))
    with pytest.raises(ValueError, match="out"):
        rt.ri_transpose(Fake(60), (3, 4, 5), "jik", out=Fake(59))
    with pytest.raises(ValueError, match="out"):
        rt.ri_pack_symm(Fake(nb * nb * naux), nb, naux, out=Fake(nb * (nb + 1) // 2 * naux - 1))
    with pytest.raises(ValueError, match="M"):
        rt.ri_iajb(Fake(40), 8, 5, M=Fake(63))
    with pytest.raises(ValueError, match="AX"):
        rt.ri_response_matvec(Fake(40), Fake(8), 8, 5, Fake(16), 2, AX=Fake(15))
    with pytest.raises(ValueError, match="ten3_a"):
        rt.special_dgemm_01(Fake(3 * 4 * 5 - 1), (3, 4, 5), range(3), range(5), Fake(25), (5, 5), range(5),
                            range(5))
    with pytest.raises(ValueError, match="t_ri"):
        rt.copy_rr((1, 1, 1), Fake(8), (2, 2, 2), (0, 0, 0), Fake(7), (2, 2, 2), (0, 0, 0))
    with pytest.raises(ValueError, match="problem 1 B"):
        rt.ri_ov_k_batched([dict(C=Fake(16), B=Fake(32), ov=None, K=Fake(16), nb=4, naux=2, nocc=1, nvir=3),
                            dict(C=Fake(16), B=Fake(31), ov=None, K=Fake(16), nb=4, naux=2, nocc=1, nvir=3)])
    assert stub == []
