"""Exact fixed-point products of the hybrid CGS kernels
(hlanc_gb300/csrc/fixed_point.cuh), checked on the host against 128-bit
integer arithmetic: the split of a double into two 29-bit limbs rounds to
nearest, limb accumulation is exact under the documented carry and
magnitude rules, the conversion back is the nearest double, and dot
products stay within the input quantisation bound."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_fixed_point_helpers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "fixed_point_test")
    src = os.path.join(ROOT, "tests", "cpp", "fixed_point_test.cpp")
    subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-Werror", "-o", exe, src], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
