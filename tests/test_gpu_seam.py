"""The Fortran seam's host-buffer paths on the GPU.

* rt_ri_ao2mo_host (the body of the drop-in ri_ao2mo_f_) pipelines ri3ao in
  and ri3mo out over the host link in blocks; its results must be bitwise those
  of the device entry rt_ri_ao2mo on the same inputs, in both forms, from
  pageable and from page-locked host memory.  nbas=300, naux=1200 gives two
  slab blocks and two ri3mo column blocks.
* Under RT_FORM=split the three drop-ins (ri_ao2mo_f_, general_dgemm_f_,
  special_dgemm_f_01_) run the split form; the form is read once per process,
  so that check runs in a fresh interpreter.  Tolerances: ri3mo 1e-10
  absolute, the GEMMs 1e-11 relative to max|oracle|.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
import rest_tensors_gb300 as rt

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("form", ["fp64", "split"])
def test_ao2mo_host_entry_is_bitwise_the_device_entry(form):
    nb, naux = 300, 1200
    B = rt.synth_ri3ao(5, nb, naux)
    C = rt.synth_coef(5, nb)
    R = rt.ri_ao2mo(C, B, nb, nb, naux, form=form)
    rt.sync_status()
    want = R.cpu().numpy()
    Ch, Bh = C.cpu().numpy(), B.cpu().numpy()
    got = np.full(naux * nb * nb, np.nan)
    rt.ri_ao2mo_host(Ch, Bh, got, nb, nb, naux, form=form)  # pageable, like a Rust Vec
    assert np.array_equal(got, want)
    pB = torch.empty(nb * nb * naux, dtype=torch.float64, pin_memory=True)
    pB.copy_(torch.from_numpy(Bh))
    pR = torch.full((naux * nb * nb,), float("nan"), dtype=torch.float64, pin_memory=True)
    rt.ri_ao2mo_host(Ch, pB.data_ptr(), pR.data_ptr(), nb, nb, naux, form=form)
    assert np.array_equal(pR.numpy(), want)
    if form == "fp64":
        Bf = Bh.reshape(naux, nb, nb).transpose(2, 1, 0)
        ref = oracle.ri_ao2mo(Ch.reshape(nb, nb, order="F"), Bf)
        assert np.max(np.abs(got.reshape(naux, nb, nb, order="F") - ref)) / np.max(np.abs(ref)) < 1e-12


SPLIT_SEAM = r"""
import numpy as np
import oracle
import rest_tensors_gb300 as rt

def split_launches():
    return rt.profile_get(rt.PROF_OZ_GEMM)[1]


rt.profile_enable(True)
nb, naux = 100, 40
C, B = oracle.synth_coef(3, nb), oracle.synth_ri3ao(3, nb, naux)
ri = rt.RIFull.from_vec([nb, nb, naux], B.reshape(-1, order="F"))
out = ri.ao2mo(rt.MatrixFull.from_vec([nb, nb], C.reshape(-1, order="F")))
err = np.max(np.abs(out.to_numpy() - oracle.ri_ao2mo(C, B)))
assert err < 1e-10, err
n0 = split_launches()
assert n0 > 0, "ri_ao2mo_f_ did not run the split GEMM"

rng = np.random.default_rng(1)
a, b = rng.standard_normal((70, 90)), rng.standard_normal((50, 90))
c = np.asfortranarray(rng.standard_normal((80, 60)))
want = c.copy(order="F")
oracle.general_dgemm_f(a, (3, 63), (10, 90), "N", b, (0, 50), (5, 85), "T", want, (4, 64), (7, 57), 0.75, -0.5)
got = c.reshape(-1, order="F").copy()
rt.general_dgemm_f(np.asfortranarray(a).reshape(-1, order="F"), [70, 90], range(3, 63), range(10, 90), "N",
                   np.asfortranarray(b).reshape(-1, order="F"), [50, 90], range(0, 50), range(5, 85), "T",
                   got, [80, 60], range(4, 64), range(7, 57), 0.75, -0.5)
gerr = np.max(np.abs(got.reshape(80, 60, order="F") - want)) / np.max(np.abs(want))
assert gerr < 1e-11, gerr
n1 = split_launches()
assert n1 > n0, "general_dgemm_f_ did not run the split GEMM"

size_a, size_b = (30, 7, 40), (45, 50)
t = rng.standard_normal(30 * 7 * 40)
m = rng.standard_normal(45 * 50)
want = oracle.special_dgemm_f_01(t, size_a, (2, 27), (5, 35), m, size_b, (10, 40), (12, 42), 1.5, 0.25)
got = t.copy()
rt.special_dgemm_f_01(got, size_a, range(2, 27), 0, range(5, 35), m, size_b, range(10, 40), range(12, 42), 1.5, 0.25)
serr = np.max(np.abs(got - want)) / np.max(np.abs(want))
assert serr < 1e-11, serr
assert split_launches() > n1, "special_dgemm_f_01_ did not run the split GEMM"
print("split seam ok", err, gerr, serr)
"""


def test_seam_runs_the_split_form_when_asked():
    env = {**os.environ, "RT_FORM": "split", "RT_NSLICES": "7"}
    r = subprocess.run([sys.executable, "-c", SPLIT_SEAM], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "split seam ok" in r.stdout, r.stdout + r.stderr


SYMMETRY_CHECK = r"""
import numpy as np, torch
import oracle, rest_tensors_gb300 as rt
nb, naux, nocc = 40, 6, 5
C, B = oracle.synth_coef(3, nb), oracle.synth_ri3ao(3, nb, naux)
D = np.asfortranarray(C[:, :nocc] @ C[:, :nocc].T); D = np.asfortranarray(0.5 * (D + D.T))
Bn = B.copy(order="F"); Bn[7, 30, :] += 1.0  # one mirror pair broken in every slab (slab 0 is checked whole)
dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).cuda()
rt.ri_j(dev(B), dev(D), nb, naux, symmetric=True); rt.sync_status()
rt.ri_j(dev(Bn), dev(D), nb, naux, symmetric=True)
try:
    rt.sync_status(); print("ri_j not refused")
except rt.RTError as e:
    assert e.status == 1, e; print("ri_j refused")
ov = np.zeros((nocc, nb - nocc, naux), order="F"); K = np.zeros((nb, nb), order="F")
rt.ri_ov_k_host(C, B, nb, naux, nocc, nb - nocc, ov, K, form="fp64", symmetric=True)
try:
    rt.ri_ov_k_host(C, Bn, nb, naux, nocc, nb - nocc, ov, K, form="fp64", symmetric=True); print("host not refused")
except rt.RTError as e:
    assert e.status == 1, e; print("host refused")
"""


def test_symmetric_entries_check_their_input_when_asked():
    env = dict(os.environ, RT_CHECK_SYMMETRY="1")
    r = subprocess.run([sys.executable, "-c", SYMMETRY_CHECK], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "ri_j refused" in r.stdout and "host refused" in r.stdout, r.stdout + r.stderr
