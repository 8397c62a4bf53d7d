"""The library's software binary128 (sweeping_fd_weno_gb300/csrc/swfd_quad.cuh,
host and device code) against GCC's _Float128 on the CPU: add, sub, mul, div,
a smoothness-indicator chain and the rounding to binary64 (subnormal results
included) on random and edge-case operands, compiled with the host compiler."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "sweeping_fd_weno_gb300" / "csrc"


def test_binary128_matches_float128(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = tmp_path / "quad_check"
    r = subprocess.run([cxx, "-O2", "-std=gnu++17", "-ffp-contract=off", "-I", str(CSRC), str(HERE / "quad" / "quad_check.cpp"),
                        "-o", str(exe), "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "300000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    counts = dict(line.split() for line in r.stdout.strip().splitlines())
    assert all(v == "0" for v in counts.values()), counts
