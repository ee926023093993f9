"""The FP32 reproduction of the reference's double-precision norm sum
(mestrado_gb300/csrc/exact_round.cuh) against (float)(D + (double)f), on
random, integer-valued, near-midpoint and edge inputs (host build, CPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_add_norms_rn_matches_double_rounding(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "xr_check")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", "-I",
                    os.path.join(ROOT, "mestrado_gb300", "csrc"), "-o", exe,
                    os.path.join(ROOT, "tests", "native", "xr_check.cpp")], check=True)
    r = subprocess.run([exe, "1500000"], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0" in r.stdout
