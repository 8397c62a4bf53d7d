"""The batched engine (swfd_batch_*): many instances advanced together.

With the FP64 precision and the sequential u_bar, every batched kernel runs
the single-instance arithmetic, so each instance must equal its own
single-instance run value for value -- alone, and in a mix whose members are
admitted at different times (continuous batching).
"""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Batch, Solver, abi, problems

pytestmark = pytest.mark.gpu

MIX = [
    dict(problem=abi.VORTEX_2D, nx=45, ny=45),
    dict(problem=abi.SEDOV_2D, nx=40, ny=40),
    dict(problem=abi.JET_2D, nx=96, ny=24),
    dict(problem=abi.VORTEX_2D, nx=64, ny=48),
    dict(problem=abi.SEDOV_2D, nx=33, ny=57),
]


def cfg_of(case, **extra):
    kw = dict(case)
    p = kw.pop("problem")
    kw.update(extra)
    return problems.make_config(p, **kw)


def single_run(case, steps, precision):
    s = Solver(cfg_of(case, precision=precision))
    s.init_problem()
    for _ in range(steps):
        if s.time > s.cfg.time_terminal - 1e-10:
            break
        s.step()
    return s.state(), s.time, s.stats()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32_BULK])
def test_batch_equals_single_instance_runs(swfd, precision):
    steps = 6
    with Batch(max_slots=8, max_nx=128, max_ny=128, precision=precision,
               ubar_mode=abi.UBAR_SEQUENTIAL) as b:
        for k, case in enumerate(MIX):
            assert b.admit(cfg_of(case), k)
        assert b.run(steps) >= 1
        for k, case in enumerate(MIX):
            u, t = b.download(k)
            ref, tref, sref = single_run(case, steps, precision)
            assert t == tref, (k, t, tref)
            bad = ~(u == ref)
            assert not bad.any(), f"instance {k}: {int(bad.sum())} values differ"
            assert b.stats(k) == sref, k


def test_continuous_batching_alone_equals_in_mix(swfd):
    """Requests admitted while others run give the same result as alone."""
    prec = abi.PRECISION_FP32_BULK
    with Batch(max_slots=4, max_nx=128, max_ny=128, precision=prec,
               ubar_mode=abi.UBAR_SEQUENTIAL) as b:
        assert b.admit(cfg_of(MIX[0]), 10)
        b.run(3)
        assert b.admit(cfg_of(MIX[1]), 11)   # joins while 10 is mid-run
        b.run(2)
        assert b.admit(cfg_of(MIX[2]), 12)
        b.run(4)
        got = {k: b.download(k) for k in (10, 11, 12)}
    ref10 = single_run(MIX[0], 9, prec)
    ref11 = single_run(MIX[1], 6, prec)
    ref12 = single_run(MIX[2], 4, prec)
    for k, ref in ((10, ref10), (11, ref11), (12, ref12)):
        u, t = got[k]
        assert t == ref[1], k
        assert not (~(u == ref[0])).any(), k


def test_instances_stop_at_their_own_time_and_are_polled(swfd):
    short = dict(problem=abi.VORTEX_2D, nx=45, ny=45, time_terminal=0.005)
    with Batch(max_slots=4, max_nx=64, max_ny=64, precision=abi.PRECISION_FP64,
               ubar_mode=abi.UBAR_SEQUENTIAL) as b:
        assert b.admit(cfg_of(short), 1)
        assert b.admit(cfg_of(MIX[0]), 2)  # T = 0.01
        done = []
        for _ in range(50):
            b.run(1)
            done += b.poll()
            if len(done) == 2:
                break
        assert sorted(done) == [(1, 0), (2, 0)]
        u1, t1 = b.download(1)
        ref = Solver(cfg_of(short))
        ref.init_problem()
        ref.run()
        assert t1 == ref.time
        assert not (~(u1 == ref.state())).any()
        b.release(1)
        assert b.info()["free_slots"] == 3


def test_admission_respects_the_hbm_budget(swfd):
    with Batch(max_slots=8, max_nx=256, max_ny=256, precision=abi.PRECISION_FP32_BULK,
               pool_bytes=30 << 20) as b:
        big = dict(problem=abi.SEDOV_2D, nx=256, ny=256)
        assert b.admit(cfg_of(big), 1)       # ~20 MB of state and FP32 planes
        assert not b.admit(cfg_of(big), 2)   # over the 30 MB budget: waits
        b.release(1)
        assert b.admit(cfg_of(big), 2)
