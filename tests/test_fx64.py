"""Exactness of the fixed-point binary64 emulation (npbench_gb300/csrc/fx64.cuh) on the host.

The same header the CUDA kernels include is compiled for the CPU and checked
bit for bit against IEEE binary64 arithmetic (tests/fx64_check.cpp).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fx64_matches_ieee_binary64(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "fx64_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "fx64_check.cpp")], check=True)
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
