"""swfd_step_async / swfd_finish: enqueued steps give the synchronous steps'
results value for value, and every other call finishes them first."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

CASES = {
    "vortex64": dict(problem=abi.VORTEX_2D, nx=64, ny=64),
    "sedov2d_48": dict(problem=abi.SEDOV_2D, nx=48, ny=48),   # sweeps in the first steps
    "sedov1d_restart": dict(problem=abi.SEDOV_1D, nx=200, cfl=3.0, rk_choice=2),
}


def make(case):
    kw = dict(CASES[case])
    s = Solver(problems.make_config(kw.pop("problem"), **kw))
    s.init_problem()
    return s


@pytest.mark.parametrize("case", list(CASES))
def test_async_steps_equal_sync_steps(swfd, case):
    a, b = make(case), make(case)
    for s in (a, b):
        s.set_profiling(True)
    for _ in range(6):
        a.step()
        b.step_async()
    b.finish()
    assert a.time == b.time
    assert np.array_equal(a.state(), b.state())
    assert a.stats() == b.stats()
    assert a.profile()["kernel_launches"] == b.profile()["kernel_launches"]
    a.close()
    b.close()


def test_other_calls_finish_pending_steps(swfd):
    a, b = make("sedov2d_48"), make("sedov2d_48")
    for _ in range(3):
        a.step()
        b.step_async()
    assert b.time == a.time                 # get_time finishes the enqueued steps
    assert np.array_equal(b.state(), a.state())
    b.step_async()
    a.step()
    assert b.stats() == a.stats()
    b.finish()
    b.finish()                              # nothing pending: a no-op
    a.close()
    b.close()
