"""The integer-pipe FP64 -> FP32 conversion used by the mixed solves' FP32
copy of A (ddla_gb300/csrc/convert.cuh), compiled for the host and checked bit
for bit against the compiler's round-to-nearest-even conversion: specials,
ties at every exponent, FP32 subnormal results, overflow, random bits."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_d2f_bits_matches_hardware_rounding(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "d2f_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "ddla_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "d2f_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "mismatches 0" in out.stdout
