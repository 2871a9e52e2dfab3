"""The integer multiplication of csrc/emul64.cuh is also a host function:
compiled for the host with nvcc and compared bit for bit with the host's
IEEE double multiplication (random bit patterns, moderate and wide exponent
ranges, few-bit significands whose products are exact or ties, signed zeros,
and products next to the overflow and underflow thresholds)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "emul_host_check.cpp")


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not on PATH")
def test_host_mul_rn_is_ieee(tmp_path):
    exe = tmp_path / "emul_host_check"
    inc = os.path.join(os.path.dirname(HERE), "euler2d_cudafortran_gb300", "csrc")
    subprocess.run(["nvcc", "-O2", "-std=c++17", "-x", "cu", "-I", inc, "-o", str(exe), SRC], check=True)
    out = subprocess.run([str(exe), "3000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 mismatches" in out.stdout
