"""The C host request loop (sweeping_fd_weno_gb300/host/swfd_serve.c) over
the batch C-ABI: a small Poisson stream served by continuous batching, every
request finished, and requests solved again alone equal to the last bit."""
import json
import subprocess

import pytest

from sweeping_fd_weno_gb300 import abi

pytestmark = pytest.mark.gpu

SERVE = abi.LIB_PATH.parent / "swfd_serve"


def test_c_host_serving_loop(swfd):
    assert SERVE.exists(), "build() builds the C serving loop next to libswfd.so"
    r = subprocess.run([str(SERVE), "--small", "--requests", "12", "--rate", "200", "--seed", "7",
                        "--slots", "8", "--chunk", "4", "--check", "2"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["finished"] == out["requests"] == 12
    assert out["failed"] == 0 and out["errors"] == 0
    assert out["fp32_bulk_requests"] > 0 and out["fp64_requests"] > 0
    assert out["p99_s"] >= out["p50_s"] > 0
    assert out["check"]["compared"] >= 2
    assert out["check"]["equal"] == out["check"]["compared"]
