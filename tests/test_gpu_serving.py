"""The serving loop: a seeded Poisson stream of mixed solves through the
batched engine with continuous batching, against the same stream solved one
request at a time by single-instance handles."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Batch, abi, problems
from sweeping_fd_weno_gb300.serving import poisson_arrivals, serve_batched, serve_one_at_a_time

pytestmark = pytest.mark.gpu


def draw_small(precision):
    def draw(rng):
        kind = int(rng.integers(0, 3))
        if kind == 0:
            n = int(rng.choice([24, 45]))
            return problems.make_config(abi.VORTEX_2D, nx=n, ny=n, time_terminal=0.004,
                                        precision=precision)
        if kind == 1:
            n = int(rng.integers(24, 65))
            return problems.make_config(abi.SEDOV_2D, nx=n, ny=n, time_terminal=0.01,
                                        precision=precision)
        return problems.make_config(abi.JET_2D, nx=64, ny=16, time_terminal=2e-5,
                                    precision=precision)
    return draw


def rel_l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32_BULK])
def test_stream_results_equal_one_at_a_time(swfd, precision):
    arr = poisson_arrivals(200.0, 10, seed=7, draw=draw_small(precision))
    got, ref = {}, {}
    with Batch(max_slots=4, max_nx=64, max_ny=64, precision=precision,
               ubar_mode=abi.UBAR_SEQUENTIAL) as b:
        r = serve_batched(arr, b, step_chunk=3, keep=got)
    r1 = serve_one_at_a_time(arr, keep=ref)
    assert sorted(got) == list(range(10)) and sorted(ref) == list(range(10))
    assert all(s == 0 for s in r.status.values())
    for k in range(10):
        (u, t), (u1, t1) = got[k], ref[k]
        assert t == t1, k
        assert not (~(u == u1)).any(), k
    s = r.summary()
    assert s["requests"] == 10 and s["p99_s"] >= s["p50_s"] > 0
    assert s["cell_updates"] == r1.summary()["cell_updates"]
