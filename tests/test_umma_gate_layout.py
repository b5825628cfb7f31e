"""The gate block of a complex128 tensor-memory pass, as libhqs.so writes it
(plan_launches + write_umma_pool), decoded on the CPU at the rows and
swizzled 16-byte chunks the kernel's MMAs read (umma_pass.cu: plane-major
rows for passes with diagonal runs, rows by output half for passes that hold
only the dense gate): every gate real of the real form is rebuilt from its
six fp16 digits to half a unit of its column's 54-bit grid, and every column
exponent is the column's largest (`umma_gate_block.cpp`)."""
import os
import shutil
import subprocess

import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    return None


def test_umma_gate_block_layouts(hqs, tmp_path):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("g++ or the CUDA runtime headers are missing")
    pkg = os.path.join(ROOT, "hiqsimulator_gb300")
    exe = str(tmp_path / "umma_gate_block")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(pkg, "csrc"), "-I", os.path.join(ROOT, "include"),
                    "-I", inc, os.path.join(TESTS, "umma_gate_block.cpp"), "-o", exe, "-L", pkg, "-lhqs",
                    "-Wl,-rpath," + pkg], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    lines = r.stdout.strip().splitlines()
    assert r.returncode == 0, r.stdout + r.stderr
    assert lines == [l for l in lines if l.endswith(" ok")] and len(lines) == 2, lines
    assert lines[0].startswith("dense halves=1") and lines[1].startswith("dense+diagonal halves=0"), lines
