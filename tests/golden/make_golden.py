"""Regenerate tests/golden/reference_doctests.json from the reference sources.

The reference (a Rust crate) cannot be built or run here, so its known-answer
tests are read as text: the doctest blocks that assert numeric results on the
GEMM seam and the symmetric eigen-solver, plus the criterion bench input whose
ao2mo result follows in closed form.  Each vector records the file:line it
came from.  Run from the repository root with the reference checked out:

    python tests/golden/make_golden.py /path/to/rest_tensors
"""
from __future__ import annotations

import json
import os
import re
import sys


def _floats(s: str):
    return [float(x) for x in re.findall(r"-?\d+\.\d+(?:[eE]-?\d+)?", s)]


def _line_of(lines, pattern, start=0):
    for i in range(start, len(lines)):
        if re.search(pattern, lines[i]):
            return i
    raise ValueError(f"pattern not found: {pattern}")


def _range(s: str):
    a, b = s.split("..")
    return [int(a), int(b)]


def extract(ref: str) -> dict:
    out = {"source": "rest_tensors doctests and benches, read as text", "cases": []}

    # general_dgemm_f doctest, src/external_libs/mod.rs
    p = os.path.join(ref, "src/external_libs/mod.rs")
    L = open(p).read().splitlines()
    i = _line_of(L, r"general_dgemm_f\(\s*$")
    call = " ".join(L[i:i + 6])
    rngs = re.findall(r"(\d+\.\.\d+)", call)
    ops = re.findall(r"'([NT])'", call)
    j = _line_of(L, r"assert_eq!\(matr_c\.get_submatrix", i)
    m = re.search(r"get_submatrix\((\d+\.\.\d+),\s*(\d+\.\.\d+)\)", L[j])
    out["cases"].append({
        "name": "general_dgemm_f", "where": f"src/external_libs/mod.rs:{i + 1}-{j + 1}",
        "a": "1..10 as 3x3 column-major", "b": "6..15 as 3x3 column-major", "c_init": 2.0,
        "rows_a": _range(rngs[0]), "cols_a": _range(rngs[1]), "opa": ops[0],
        "rows_b": _range(rngs[2]), "cols_b": _range(rngs[3]), "opb": ops[1],
        "rows_c": _range(rngs[4]), "cols_c": _range(rngs[5]), "alpha": 1.0, "beta": 1.0,
        "check_rows": _range(m.group(1)), "check_cols": _range(m.group(2)),
        "expected": _floats(L[j].split("vec!")[1]),
    })

    # _dgemm doctest (three calls), src/matrix/matrix_blas_lapack.rs
    p = os.path.join(ref, "src/matrix/matrix_blas_lapack.rs")
    L = open(p).read().splitlines()
    start = 0
    for n in range(3):
        i = _line_of(L, r"_dgemm\(&matr_a,", start)
        call = " ".join(L[i:i + 4])
        rngs = re.findall(r"(\d+\.\.\d+)", call)
        ops = re.findall(r"'([NT])'", call)
        j = _line_of(L, r"assert_eq!\(matr_c\.get_submatrix", i)
        m = re.search(r"get_submatrix\((\d+\.\.\d+),\s*(\d+\.\.\d+)\)", L[j])
        out["cases"].append({
            "name": f"_dgemm_{n}", "where": f"src/matrix/matrix_blas_lapack.rs:{i + 1}-{j + 1}",
            "a": "1..10 as 3x3 column-major", "b": "6..15 as 3x3 column-major", "c_init": 2.0,
            "rows_a": _range(rngs[0]), "cols_a": _range(rngs[1]), "opa": ops[0],
            "rows_b": _range(rngs[2]), "cols_b": _range(rngs[3]), "opb": ops[1],
            "rows_c": _range(rngs[4]), "cols_c": _range(rngs[5]), "alpha": 1.0, "beta": 1.0,
            "check_rows": _range(m.group(1)), "check_cols": _range(m.group(2)),
            "expected": _floats(L[j].split("vec!")[1]),
        })
        start = j + 1

    # _dsyev doctest: packed upper 1..7 -> eigenpairs
    i = _line_of(L, r"let eigvec_benchmark = vec!\[")
    vec_txt = " ".join(L[i:i + 4])
    k = _line_of(L, r"let eigval_benchmark = vec!\[", i)
    out["cases"].append({
        "name": "_dsyev", "where": f"src/matrix/matrix_blas_lapack.rs:{i - 9}-{k + 3}",
        "packed_upper": [float(x) for x in range(1, 7)], "uplo_used": "L", "tol_sq": 10e-7,
        "eigvec": _floats(vec_txt.split("vec!")[1]), "eigval": _floats(L[k].split("vec!")[1]),
    })

    # lapack_power test inputs (the tests print their results without asserting): the
    # 3x3 SPD matrix of test_sqrt_inverse and the 8x8 matrix of matfull_inverse_and_power.
    num = r"(-?\d+(?:\.\d+)?(?:[eE]-?\d+)?)"
    i = _line_of(L, r"fn test_sqrt_inverse")
    j = _line_of(L, r"lapack_power\(", i)
    vec_txt = " ".join(L[i:j])
    pm = re.search(r"lapack_power\(" + num + r",\s*" + num + r"\)", L[j])
    out["cases"].append({
        "name": "lapack_power_3x3", "where": f"src/matrix/matrix_blas_lapack.rs:{i + 1}-{j + 1}",
        "n": 3, "matrix": _floats(vec_txt.split("vec!")[1]), "p": float(pm.group(1)),
        "threshold": float(pm.group(2)),
    })
    p = os.path.join(ref, "src/lib.rs")
    L = open(p).read().splitlines()
    i = _line_of(L, r"fn matfull_inverse_and_power")
    k = _line_of(L, r"let orig_a = vec!\[", i)
    j = _line_of(L, r"lapack_power\(", k)
    pm = re.search(r"lapack_power\(" + num + r",\s*" + num + r"\)", L[j])
    mat = _floats(L[k].split("vec!")[1])
    out["cases"].append({
        "name": "lapack_power_8x8", "where": f"src/lib.rs:{k + 1}-{j + 1}",
        "n": int(round(len(mat) ** 0.5)), "matrix": mat, "p": float(pm.group(1)), "threshold": float(pm.group(2)),
    })

    # criterion bench input: RIFull [10,10,20] filled with 2.0, eigenvector ones(10,10)
    p = os.path.join(ref, "benches/bench_tensors.rs")
    L = open(p).read().splitlines()
    i = _line_of(L, r"RIFull::new\(\[")
    j = _line_of(L, r"MatrixFull::new\(\[")
    size = [int(x) for x in re.search(r"\[(\d+),(\d+),(\d+)\]", L[i]).groups()]
    fill = float(re.search(r"\],\s*([\d.]+)\)", L[i]).group(1))
    cshape = [int(x) for x in re.search(r"\[(\d+),(\d+)\]", L[j]).groups()]
    cfill = float(re.search(r"\],\s*([\d.]+)\)", L[j]).group(1))
    out["cases"].append({
        "name": "bench_ao2mo", "where": f"benches/bench_tensors.rs:{i + 1}-{j + 3}",
        "ri3fn_size": size, "ri3fn_fill": fill, "eigenvector_size": cshape, "eigenvector_fill": cfill,
        "expected_every_element": fill * cfill * cfill * size[0] * size[1],
        "note": "ri3mo[P,p,q] = sum_{mu,nu} C[mu,p] B[mu,nu,P] C[nu,q] in closed form",
    })
    return out


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the reference checkout>")
    data = extract(sys.argv[1])
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_doctests.json")
    with open(dst, "w") as f:
        json.dump(data, f, indent=1)
    print(dst, len(data["cases"]), "cases")
