"""The FP32-bulk precision form against the FP64 oracle.

WENO fluxes, flux differences and the Lax-Friedrichs splitting run in FP32;
pressure recovery, the RK accumulation into the state, the positivity test,
the CFL reduction and the sweeps stay FP64.  Accepted where the relative L1
density error against the FP64 oracle stays below 1e-6 (the vortex and the
point-energy problems); the jet (kinetic-dominated) is only checked to stay
finite and positive.
"""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu


def rel_l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


def interior(u, ndim):
    return u[0, 3:-3] if ndim == 1 else u[3:-3, 3:-3]


@pytest.mark.parametrize("n", [45, 90, 180])
def test_vortex_fp32_bulk_within_1e6_of_fp64_oracle(swfd, oracle_mod, n):
    g = Solver(problems.workload(f"vortex{n}", precision=abi.PRECISION_FP32_BULK))
    o = oracle_mod.Oracle(problems.workload(f"vortex{n}"))
    g.init_problem()
    o.init_problem()
    ng, no = g.run(), o.run()
    assert ng == no
    ug, uo = interior(g.state(), 2), interior(o.state(), 2)
    err = rel_l1(ug[..., 0], uo[..., 0])
    assert err < 1e-6, err
    p = 0.4 * (ug[..., 3] - 0.5 * (ug[..., 1] ** 2 + ug[..., 2] ** 2) / ug[..., 0])
    assert (ug[..., 0] > 0).all() and (p > 0).all()


@pytest.mark.parametrize("case", [
    dict(problem=abi.SEDOV_2D, nx=64, ny=64, steps=20),
    dict(problem=abi.SEDOV_1D, nx=800, cfl=0.6, swp_num=2, e_background=1e-12, steps=40),
])
def test_point_energy_fp32_bulk_close_to_fp64(swfd, oracle_mod, case):
    kw = dict(case)
    steps = kw.pop("steps")
    p = kw.pop("problem")
    g = Solver(problems.make_config(p, precision=abi.PRECISION_FP32_BULK, **kw))
    o = oracle_mod.Oracle(problems.make_config(p, **kw))
    g.init_problem()
    o.init_problem()
    for _ in range(steps):
        g.step()
        o.step()
    ndim = 1 if p in (abi.SEDOV_1D, abi.MATLAB_1D) else 2
    ug, uo = interior(g.state(), ndim), interior(o.state(), ndim)
    err = rel_l1(ug[..., 0], uo[..., 0])
    assert err < 1e-6, err
    assert np.isfinite(ug).all()


def test_jet_fp32_bulk_stays_physical(swfd):
    g = Solver(problems.make_config(abi.JET_2D, nx=96, ny=24, precision=abi.PRECISION_FP32_BULK))
    g.init_problem()
    for _ in range(10):
        g.step()
    u = interior(g.state(), 2)
    assert np.isfinite(u).all() and (u[..., 0] > 0).all()
