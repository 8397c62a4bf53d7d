"""The serving loop: a seeded Poisson stream of mixed solves through the
batched engine with continuous batching (an FP32-bulk batch beside an FP64
batch for the problems that stay FP64), against the same stream solved one
request at a time by single-instance handles."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Batch, abi, problems
from sweeping_fd_weno_gb300.serving import (fp32_accepted, poisson_arrivals, serve_batched,
                                            serve_one_at_a_time)

pytestmark = pytest.mark.gpu


def draw_small(precision):
    def draw(rng):
        kind = int(rng.integers(0, 4))
        if kind == 0:
            n = int(rng.choice([24, 45]))
            c = problems.make_config(abi.VORTEX_2D, nx=n, ny=n, time_terminal=0.004)
        elif kind == 1:
            n = int(rng.integers(24, 65))
            c = problems.make_config(abi.SEDOV_2D, nx=n, ny=n, time_terminal=0.01)
        elif kind == 2:
            c = problems.make_config(abi.JET_2D, nx=64, ny=16, time_terminal=2e-5)
        else:
            c = problems.make_config(abi.SHOCK_DIFFRACTION, total=12, time_terminal=0.03)
        c.precision = precision if fp32_accepted(c) else abi.PRECISION_FP64
        return c
    return draw


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32_BULK])
def test_stream_results_equal_one_at_a_time(swfd, precision):
    arr = poisson_arrivals(200.0, 12, seed=7, draw=draw_small(precision))
    got, ref = {}, {}
    batches = [Batch(max_slots=4, max_nx=160, max_ny=160, precision=abi.PRECISION_FP64,
                     ubar_mode=abi.UBAR_SEQUENTIAL)]
    if precision == abi.PRECISION_FP32_BULK:
        batches.insert(0, Batch(max_slots=4, max_nx=64, max_ny=64, precision=precision,
                                ubar_mode=abi.UBAR_SEQUENTIAL))
    try:
        r = serve_batched(arr, batches, step_chunk=3, keep=got)
    finally:
        for b in batches:
            b.close()
    r1 = serve_one_at_a_time(arr, keep=ref)
    assert sorted(got) == list(range(12)) and sorted(ref) == list(range(12))
    assert all(s == 0 for s in r.status.values())
    assert any(c.problem == abi.SHOCK_DIFFRACTION for _, c in arr)
    for k in range(12):
        (u, t), (u1, t1) = got[k], ref[k]
        assert t == t1, k
        assert not (~(u == u1)).any(), k
    s = r.summary()
    assert s["requests"] == 12 and s["p99_s"] >= s["p50_s"] > 0
    assert s["cell_updates"] == r1.summary()["cell_updates"]
