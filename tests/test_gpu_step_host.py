"""swfd_step_host (upload, step, download with one synchronisation) against
swfd_upload_state + swfd_step + swfd_download_state: the same state bits,
time, dt and statistics, with sweeps (the jet), in FP32-bulk, and through
the detonation engine's path."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

CASES = [
    ("vortex64", dict(problem=abi.VORTEX_2D, nx=64, ny=64), {}),
    ("jet_96x24", dict(problem=abi.JET_2D, nx=96, ny=24), {}),
    ("vortex64_fp32", dict(problem=abi.VORTEX_2D, nx=64, ny=64),
     dict(precision=abi.PRECISION_FP32_BULK)),
    ("detonation_40", dict(problem=abi.DETONATION, total=8, cut_x=2, cut_y=2), {}),
]


@pytest.mark.parametrize("name,case,extra", CASES, ids=[c[0] for c in CASES])
def test_step_host_equals_the_three_calls(swfd, name, case, extra):
    kw = dict(case)
    p = kw.pop("problem")
    a = Solver(problems.make_config(p, **kw, **extra))
    b = Solver(problems.make_config(p, **kw, **extra))
    for s in (a, b):
        s.init_problem()
    ua = a.state()
    ub = ub_out = b.state()
    dts = []
    for _ in range(12):
        a.set_state(ua)
        da = a.step()
        a.state(out=ua)
        db = b.step_host(ub, ub_out)
        dts.append((da, db))
    assert all(x == y for x, y in dts)
    assert a.time == b.time
    assert np.array_equal(ua.view(np.uint64), ub_out.view(np.uint64))
    assert a.stats() == b.stats()
    a.close()
    b.close()
