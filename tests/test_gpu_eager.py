"""SWFD_LAUNCH=eager runs the graph sections as plain stream launches (for
profilers); the results must be those of the graphs, value for value."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

CASES = [
    ("sedov2d", dict(problem=abi.SEDOV_2D, nx=64, ny=64), 6),
    ("sedov1d", dict(problem=abi.SEDOV_1D, nx=800, cfl=0.6, swp_num=2, e_background=1e-12), 8),
    ("jet", dict(problem=abi.JET_2D, nx=96, ny=24), 4),
    ("vortex_fp32_fused", dict(problem=abi.VORTEX_2D, nx=64, ny=48,
                               precision=abi.PRECISION_FP32_BULK), 6),
    ("detonation", dict(problem=abi.DETONATION, total=8, cut_x=2, cut_y=2), 6),
]


def run(monkeypatch, mode, case, steps, solve=False):
    if mode == "eager":
        monkeypatch.setenv("SWFD_LAUNCH", "eager")
    else:
        monkeypatch.delenv("SWFD_LAUNCH", raising=False)
    kw = dict(case)
    s = Solver(problems.make_config(kw.pop("problem"), **kw))
    s.init_problem()
    if solve:
        n = s.run()
    else:
        n = steps
        for _ in range(steps):
            s.step()
    out = (s.state(), s.time, s.stats(), n)
    s.close()
    return out


@pytest.mark.parametrize("name,case,steps", CASES, ids=[c[0] for c in CASES])
def test_eager_equals_graphs(swfd, monkeypatch, name, case, steps):
    g = run(monkeypatch, "graph", case, steps)
    e = run(monkeypatch, "eager", case, steps)
    assert g[1] == e[1] and g[2] == e[2] and g[3] == e[3]
    assert not (~(g[0] == e[0])).any()


def test_eager_solve_equals_graphs(swfd, monkeypatch):
    case = dict(problem=abi.VORTEX_2D, nx=45, ny=45)
    g = run(monkeypatch, "graph", case, 0, solve=True)
    e = run(monkeypatch, "eager", case, 0, solve=True)
    assert g[1] == e[1] and g[2] == e[2] and g[3] == e[3]
    assert not (~(g[0] == e[0])).any()
