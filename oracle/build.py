"""Build recipe for the CPU oracle (test infrastructure, never product code).

Compiles oracle.c into oracle/liboracle.so with gcc.  The reference itself
(Rust crate + one Fortran file) cannot be compiled here: the image has no
rustc/cargo and no Fortran compiler, so there is no oracle/_ref build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.c")
OUT = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "..", "include", "rt_synth.h"))
    ):
        return OUT
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11", SRC, "-o", OUT + ".tmp", "-ldl", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
