"""The persistent kernels' grid barrier and the 1D solve's grid reduction
(csrc/swfd_gridsync.cuh) end their waits by themselves: with one block of a
cooperative launch absent, the other block's wait runs out after its limit
and reports the timeout bit, without a fault, and the context stays usable.
No GPU fault is made: the failure is a block that never arrives."""
import ctypes as C
import time

import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

TIMEOUT_BIT = 64


def _probe(absent, wait_ms):
    err, passed = C.c_int32(-1), C.c_int32(-1)
    t0 = time.perf_counter()
    st = abi.load_probe().swfd_probe_barrier_timeout(0, absent, wait_ms, C.byref(err),
                                                     C.byref(passed))
    return st, err.value, passed.value, time.perf_counter() - t0


def test_grid_barrier_passes_with_every_block(swfd):
    st, err, passed, _ = _probe(0, 200.0)
    assert st == abi.OK and err == 0 and passed == 2


def test_grid_barrier_wait_runs_out_without_a_fault(swfd):
    st, err, passed, dt = _probe(1, 200.0)
    assert st == abi.OK, "the probe launch must end without a CUDA error"
    assert err == TIMEOUT_BIT and passed == 0
    assert 0.15 < dt < 5.0, dt
    # the context is still usable: a solve runs and matches a fresh one
    cfg = problems.make_config(abi.SEDOV_1D, nx=160)
    with Solver(cfg) as s:
        s.init_problem()
        assert s.run(5) == 5
        assert np.isfinite(s.state()).all()


def _reduce(absent, wait_ms):
    err, passed = C.c_int32(-1), C.c_int32(-1)
    am, bad = (C.c_double * 2)(-1.0, -1.0), (C.c_int32 * 2)(-1, -1)
    t0 = time.perf_counter()
    st = abi.load_probe().swfd_probe_reduce_timeout(0, absent, wait_ms, C.byref(err),
                                                    C.byref(passed), am, bad)
    return st, err.value, passed.value, list(am), list(bad), time.perf_counter() - t0


def test_grid_reduction_folds_every_block(swfd):
    # block b posts b + 1, block 0 the flag: both receive the maximum 2 and the flag
    st, err, passed, am, bad, _ = _reduce(0, 200.0)
    assert st == abi.OK and err == 0 and passed == 2
    assert am == [2.0, 2.0] and bad == [1, 1]


def test_grid_reduction_wait_runs_out_without_a_fault(swfd):
    st, err, passed, _, _, dt = _reduce(1, 200.0)
    assert st == abi.OK, "the probe launch must end without a CUDA error"
    assert err == TIMEOUT_BIT and passed == 0
    assert 0.15 < dt < 5.0, dt
    cfg = problems.make_config(abi.SEDOV_1D, nx=160)
    with Solver(cfg) as s:
        s.init_problem()
        assert s.run(5) == 5
        assert np.isfinite(s.state()).all()
