"""The fixed-point conversions of the kernels (pysic_gb300/csrc/fixed.cuh),
compiled for the host with g++ and checked against correctly rounded
references on random values: float and double to 2^-32 fixed point (round to
nearest), fixed point back to double (round to nearest even), exact 128-bit
totals, the two-word atomic add with carry, and NaN propagation."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fixed_point_conversions(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "fixed_point_check")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", cuda_inc, "-o", exe,
                    os.path.join(HERE, "native", "fixed_point_check.cpp")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    assert "bad=0" in out, out
    assert "nan: nan nan nan" in out, out
