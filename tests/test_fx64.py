"""Exactness of the binary64 emulations (npbench_gb300/csrc/fx64.cuh, f64emu.cuh) on the host.

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


def test_f64emu_addition_matches_ieee_binary64(tmp_path):
    """npbench_gb300/csrc/f64emu.cuh: exact binary64 addition on integers (tests/f64emu_check.cpp)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "f64emu_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "f64emu_check.cpp")], check=True)
    r = subprocess.run([exe, "2000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
