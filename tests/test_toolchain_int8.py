"""The 7-slice INT8 split form is not built because GB300's tensor cores offer
this toolkit no INT8 MMA: ptxas rejects ``tcgen05.mma ... kind::i8`` for
sm_103a, while the same instruction assembles for sm_100a, and the BF16 form
the library uses (``kind::f16``) assembles for both.

The probe is a hand-written PTX kernel holding that one instruction.  Only
ptxas's exit status and message are read; the assembled output is discarded.
Nothing runs on a GPU.
"""
import os
import shutil
import subprocess

import pytest

PTX = """.version 9.0
.target {arch}
.address_size 64

.visible .entry mma_probe(.param .u32 d, .param .u64 a, .param .u64 b, .param .u32 idesc)
{{
    .reg .b32 %r<4>;
    .reg .b64 %rd<3>;
    .reg .pred p;
    ld.param.u32 %r1, [d];
    ld.param.u64 %rd1, [a];
    ld.param.u64 %rd2, [b];
    ld.param.u32 %r2, [idesc];
    setp.ne.b32 p, %r2, 0;
    tcgen05.mma.cta_group::1.kind::{kind} [%r1], %rd1, %rd2, %r2, p;
    ret;
}}
"""


def _ptxas():
    p = shutil.which("ptxas") or "/usr/local/cuda/bin/ptxas"
    if not os.path.exists(p):
        pytest.skip("ptxas not found")
    return p


def _assemble(tmp_path, kind, arch):
    src = tmp_path / f"probe_{kind}_{arch}.ptx"
    src.write_text(PTX.format(kind=kind, arch=arch))
    return subprocess.run([_ptxas(), f"-arch={arch}", str(src), "-o", os.devnull], capture_output=True, text=True,
                          timeout=120)


def test_no_int8_tensor_mma_on_sm_103a(tmp_path):
    r = _assemble(tmp_path, "i8", "sm_103a")
    assert r.returncode != 0
    assert "kind::i8" in r.stderr and "sm_103a" in r.stderr, r.stderr


@pytest.mark.parametrize("kind,arch", [("i8", "sm_100a"), ("f16", "sm_103a"), ("f16", "sm_100a")])
def test_the_probe_itself_assembles_elsewhere(tmp_path, kind, arch):
    r = _assemble(tmp_path, kind, arch)
    assert r.returncode == 0, r.stderr
