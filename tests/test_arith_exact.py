"""The FP64 shortcuts of the exact schemes return the FP64 instruction's result:
tests/arith/div_check.cu compares the seeded Markstein division, the division
by a two-term reciprocal and the 1e-30 + x shortcut with the division and
addition instructions (and the host's division) over about four million operand
pairs (GPU); it compiles for sm_103a here (CPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "arith", "div_check.cu")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _compile(out, *extra):
    subprocess.run([NVCC, "-std=c++17", "-O2", "--fmad=false", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "mom5_gb300", "csrc"), *extra, SRC, "-o", out], check=True)


@pytest.mark.skipif(not os.path.exists(NVCC), reason="nvcc not found")
def test_division_check_compiles(tmp_path):
    _compile(str(tmp_path / "div_check.o"), "-c")


@pytest.mark.gpu
def test_division_and_tiny_add_are_exact(tmp_path):
    exe = str(tmp_path / "div_check")
    _compile(exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
