"""The traversal divides by a per-ray reciprocal (Markstein's method) where
the operand magnitudes allow it; this compiles tests/gpu_div_check.cu
against the library's trace.cuh and checks that division against IEEE a / b
bit for bit on 2^32 random operand pairs of that domain."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_reciprocal_division_is_correctly_rounded(tmp_path):
    exe = tmp_path / "div_check"
    csrc = os.path.join(ROOT, "qubatron_gb300", "csrc")
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false",
                    "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-I", csrc, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "gpu_div_check.cu"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(1 << 32)], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0 " in out.stdout
