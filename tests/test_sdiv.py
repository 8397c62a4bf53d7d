"""The software binary64 division and power-of-two scaling of
csrc/swfd_sdiv.cuh (host and device code) against the host's IEEE
arithmetic, on the CPU: 2M random and edge-case
operand pairs (subnormals, infinities, NaN, exponent limits, long runs of
ones and zeros, exact quotients) must give the same bits."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
CSRC = HERE.parent / "sweeping_fd_weno_gb300" / "csrc"


def test_sdiv_matches_ieee_division(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "sdiv_check"
    r = subprocess.run([cxx, "-O2", "-std=gnu++17", "-ffp-contract=off", "-I", str(CSRC),
                        str(HERE / "sdiv" / "sdiv_check.cpp"), "-o", str(exe), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "1000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("div 0 scale 0 "), r.stdout
