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
    return sorted(n for n in names if n.startswith(("rt_", "ri_", "general_")))


def test_header_declares_the_seam():
    names = declared_functions()
    for n in ["ri_ao2mo_f_", "general_dgemm_f_", "rt_ri_ov_k", "rt_ri_ao2mo", "rt_ri_j", "rt_dgemm"]:
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
