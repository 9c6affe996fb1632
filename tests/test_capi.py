"""C ABI checks that need no GPU: the library builds, loads, exports every
function declared in include/*.h, and rejects bad arguments before touching
the device."""
import ctypes
import glob
import os
import re

import pytest

import rest_tensors_gb300 as rt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    """Names of the function prototypes (declarations ending in ';', not
    inline definitions) in include/*.h."""
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
        text = text.replace('extern "C" {', "")
        text = re.sub(r"^\s*\}\s*$", "", text, flags=re.M)
        text = re.sub(r"\{[^{}]*\}", ";", text)  # drop bodies (one nesting level at a time)
        text = re.sub(r"\{[^{}]*\}", ";", text)
        for stmt in text.split(";"):
            stmt = " ".join(stmt.split())
            if stmt.startswith("typedef"):
                continue
            m = re.match(r"^(?:extern \"C\" )?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(.*\)$", stmt)
            if m and not re.search(r"\b(static|inline|RT_SYNTH_FN)\b", stmt):
                names.add(m.group(1))
    return sorted(n for n in names if n.startswith(("rt_", "ri_", "general_", "special_")))


def test_header_declares_the_seam():
    names = declared_functions()
    for n in ["ri_ao2mo_f_", "general_dgemm_f_", "special_dgemm_f_01_", "rt_ri_ov_k", "rt_ri_ao2mo", "rt_ri_j",
              "rt_dgemm", "rt_special_dgemm_01", "rt_copy_rr", "rt_ri_transpose", "rt_ri_pack_symm",
              "rt_newton_schulz_inv_sqrt", "rt_ri_ao2mo_host"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    L = rt.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert missing == []


def test_version_and_status_text():
    L = rt.lib()
    assert L.rt_version() >> 16 == 1
    assert L.rt_status_string(0) == b"ok"
    assert L.rt_status_string(5) == b"non-finite input"


@pytest.mark.parametrize("args", [
    (b"N", b"N", -1, 2, 2, 1.0, None, 1, None, 2, 0.0, None, 1, None),
    (b"X", b"N", 2, 2, 2, 1.0, None, 2, None, 2, 0.0, None, 2, None),
    (b"N", b"N", 4, 2, 2, 1.0, None, 2, None, 2, 0.0, None, 4, None),  # lda < m
])
def test_dgemm_rejects_bad_arguments(args):
    L = rt.lib()
    assert L.rt_dgemm(*args) == 1
    assert b"rt_dgemm" in L.rt_last_error()


def test_split_form_rejects_bad_slice_count():
    L = rt.lib()
    st = L.rt_ri_ov_k(None, None, 4, 4, 2, 2, None, None, 1, 9, None)
    assert st == 1 and b"nslices" in L.rt_last_error()
    st = L.rt_ri_ao2mo(None, None, None, 4, 4, 4, 7, 6, None)
    assert st == 1


def test_general_dgemm_f_rejects_inconsistent_blocks():
    import numpy as np
    a = np.zeros((3, 3), order="F")
    with pytest.raises(rt.RTError):
        # op(A) is 2x2 but C block is 1x2
        rt.general_dgemm_f(a.reshape(-1, order="F"), [3, 3], range(1, 3), range(1, 3), "N",
                           a.reshape(-1, order="F"), [3, 3], range(0, 2), range(0, 2), "N",
                           np.zeros(9), [3, 3], range(1, 2), range(0, 2), 1.0, 1.0)


def test_dgemm_shape_check_mirrors_reference():
    A = rt.MatrixFull.new([3, 3], 1.0)
    with pytest.raises(ValueError):
        rt._dgemm(A, (range(0, 2), range(0, 3)), "N", A, (range(0, 2), range(0, 2)), "N",
                  A, (range(0, 2), range(0, 2)), 1.0, 0.0)


# ----------------------------------------------- next rows: argument checks --
def test_special_dgemm_rejects_blocks_before_touching_the_device():
    L = rt.lib()
    L.rt_special_dgemm_01.restype = ctypes.c_int
    # matr_b block 7 x 6 with len_z_a 7
    st = L.rt_special_dgemm_01(None, 7, 5, 12, 2, 4, 3, 7, None, 11, 13, 1, 7, 4, 6, ctypes.c_double(1.0),
                               ctypes.c_double(0.0), 0, 7, None)
    assert st == 1 and b"len_z_a" in L.rt_last_error()
    # block of ten3_a outside the tensor
    st = L.rt_special_dgemm_01(None, 7, 5, 12, 2, 6, 3, 7, None, 11, 13, 1, 7, 4, 7, ctypes.c_double(1.0),
                               ctypes.c_double(0.0), 0, 7, None)
    assert st == 1 and b"outside" in L.rt_last_error()
    # split form with a bad slice count
    st = L.rt_special_dgemm_01(None, 7, 5, 12, 2, 4, 3, 7, None, 11, 13, 1, 7, 4, 7, ctypes.c_double(1.0),
                               ctypes.c_double(0.0), 1, 2, None)
    assert st == 1


def test_layout_calls_reject_bad_modes_orders_and_ranges():
    L = rt.lib()
    assert L.rt_copy_mr(2, 2, None, 6, 5, 0, 0, None, 4, 5, 6, 0, 0, 0, 3, None) == 1  # mode 3
    assert b"mode" in L.rt_last_error()
    assert L.rt_copy_rm(4, 2, None, 4, 5, 6, 1, 0, 0, 0, None, 6, 5, 0, 0, None) == 1  # rows 1..5 of 4
    assert L.rt_copy_mm(3, 3, None, 2, 5, 0, 0, None, 4, 4, 0, 0, None) == 1  # source rows 0..3 of 2
    assert L.rt_copy_rr(2, 2, 2, None, 2, 2, 2, 1, 0, 0, None, 4, 4, 4, 0, 0, 0, None) == 1
    for bad in (b"iik", b"ij", b"xyz"):
        assert L.rt_ri_transpose(None, 2, 3, 4, bad, None, None) == 1
    assert L.rt_ri_pack_symm(None, -1, 3, None, None) == 1
    # empty blocks are accepted and do nothing
    assert L.rt_copy_mr(0, 2, None, 6, 5, 0, 0, None, 4, 5, 6, 0, 0, 0, 0, None) == 0
    assert L.rt_ri_transpose(None, 0, 3, 4, b"kji", None, None) == 0


def test_newton_schulz_rejects_bad_arguments():
    L = rt.lib()
    shifts = (ctypes.c_double * 1)(0.0)
    call = lambda n, nshift, form, nsl: L.rt_newton_schulz_inv_sqrt(  # noqa: E731
        None, n, ctypes.c_double(1e-8), ctypes.c_double(1.0), 10, shifts, nshift, form, nsl, None, None, None, None)
    assert call(4, 0, 0, 7) == 1  # no level shift
    assert call(0, 1, 0, 7) == 1  # empty matrix
    assert call(4, 1, 1, 9) == 1  # split form, bad slice count
    assert call(4, 1, 0, 7) == 1  # null pointers


@pytest.mark.parametrize("env", [{"RT_FORM": "single"}, {"RT_NSLICES": "9"}, {"RT_FORM": "split", "RT_NSLICES": "x"}])
def test_seam_refuses_an_unknown_form_before_any_device_work(env):
    # The seam's form is read once per process, so each setting runs in a fresh interpreter.
    import subprocess
    import sys

    code = ("import numpy as np, rest_tensors_gb300 as rt\n"
            "out = np.ones(2 * 2 * 3)\n"
            "try:\n"
            "    rt.ri_ao2mo_f(np.ones(4), np.ones(12), out, 2, 2, 3)\n"
            "except rt.RTError as e:\n"
            "    assert e.status == 1 and b'RT_' in rt.lib().rt_last_error(), e\n"
            "    assert not out.any()\n"
            "    print('refused')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env={**os.environ, **env}, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0 and "refused" in r.stdout, r.stderr


def test_symmetric_host_entry_refuses_asymmetric_input_when_asked():
    # RT_CHECK_SYMMETRY is read once per process; the host-memory check runs before any device work.
    import subprocess
    import sys

    code = ("import numpy as np, rest_tensors_gb300 as rt\n"
            "nb, naux, nocc = 12, 3, 2\n"
            "B = np.asfortranarray(np.random.default_rng(0).standard_normal((nb, nb, naux)))\n"
            "C = np.asfortranarray(np.eye(nb)); ov = np.zeros((nocc, nb - nocc, naux), order='F')\n"
            "K = np.zeros((nb, nb), order='F')\n"
            "st = rt.lib().rt_ri_ov_k_host_symmetric(C.ctypes.data, B.ctypes.data, nb, naux, nocc, nb - nocc,\n"
            "                                         ov.ctypes.data, K.ctypes.data, 0, 7, None)\n"
            "assert st == 1 and b'not symmetric' in rt.lib().rt_last_error(), (st, rt.lib().rt_last_error())\n"
            "print('refused')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env={**os.environ, "RT_CHECK_SYMMETRY": "1"},
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "refused" in r.stdout, r.stdout + r.stderr
