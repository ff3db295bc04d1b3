"""The C ABI from a C host: include/mom5gpu.h compiles as C11 (CPU) and a small
C program creates a domain, steps it and checks the status-code contract (GPU)."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "c_abi", "host_example.c")


def test_header_and_host_compile_as_c(tmp_path):
    obj = str(tmp_path / "host.o")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-c", SRC, "-o", obj,
                    "-I", os.path.join(ROOT, "include")], check=True)


@pytest.mark.gpu
def test_c_host_runs(gpu_lib, tmp_path):
    from mom5_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "host")
    subprocess.run(["gcc", "-std=c11", "-O1", SRC, "-o", exe, "-I", os.path.join(ROOT, "include"),
                    "-L", os.path.dirname(lib), "-lmom5gpu", "-Wl,-rpath," + os.path.dirname(lib), "-lm"],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
