"""The dt-halving restart RK of ex2 (rk_choice 2, ex2_sedov_1d/main.f90:
330-374) on the GPU against the oracle, value for value: state, time, dt and
the number of restarts, step by step, through the solve graph and in the
eager launch mode."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

CASES = {
    # cfl 1.2 (ex2's own): a few restarts; cfl 3.0: restarts in most steps,
    # many from a stale stage-2/3 flux
    "cfl1.2": (dict(nx=200, cfl=1.2), 40),
    "cfl3.0": (dict(nx=200, cfl=3.0), 20),
    "cfl3.0_n801": (dict(nx=801, cfl=3.0, e_background=1e-12), 12),
}


def pair(oracle_mod, kw, **extra):
    cfg = dict(kw, rk_choice=2, **extra)
    g = Solver(problems.make_config(abi.SEDOV_1D, **cfg))
    o = oracle_mod.Oracle(problems.make_config(abi.SEDOV_1D, **cfg))
    g.init_problem()
    o.init_problem()
    return g, o


@pytest.mark.parametrize("case", list(CASES))
def test_restart_rk_steps_match(swfd, oracle_mod, case):
    kw, steps = CASES[case]
    g, o = pair(oracle_mod, kw)
    for k in range(steps):
        dg = g.step()
        o.step()
        assert dg == o.dt, (k, dg, o.dt)
        assert g.time == o.time
        assert np.array_equal(g.state(), o.state()), f"state after step {k + 1}"
        assert g.restarts() == o.restarts
    assert o.restarts > 0
    g.close()


@pytest.mark.parametrize("case", ["cfl1.2", "cfl3.0"])
def test_restart_rk_solve_graph_matches(swfd, oracle_mod, case):
    kw, steps = CASES[case]
    g, o = pair(oracle_mod, kw)
    assert g.run(steps) == o.run(steps) == steps
    assert g.time == o.time
    assert np.array_equal(g.state(), o.state())
    assert g.restarts() == o.restarts > 0
    g.close()


def test_restart_rk_eager_matches_graphs(swfd, oracle_mod, monkeypatch):
    kw, steps = CASES["cfl3.0"]
    monkeypatch.setenv("SWFD_LAUNCH", "eager")
    g, o = pair(oracle_mod, kw)
    for _ in range(steps):
        g.step()
        o.step()
    assert np.array_equal(g.state(), o.state())
    assert g.restarts() == o.restarts > 0
    g.close()


def test_restart_rk_fp32_bulk_tracks_fp64(swfd):
    """FP32-bulk fluxes with the FP64 restart logic: the same restart pattern
    on ex2's own CFL and a close state."""
    kw, steps = CASES["cfl1.2"]
    a = Solver(problems.make_config(abi.SEDOV_1D, rk_choice=2, **kw))
    b = Solver(problems.make_config(abi.SEDOV_1D, rk_choice=2,
                                    precision=abi.PRECISION_FP32_BULK, **kw))
    for s in (a, b):
        s.init_problem()
        for _ in range(steps):
            s.step()
    ua, ub = a.state()[0, 3:-3, 0], b.state()[0, 3:-3, 0]
    assert np.abs(ua - ub).sum() / np.abs(ua).sum() < 1e-4
    a.close()
    b.close()


def test_restart_limit_matches_oracle(swfd, oracle_mod):
    """A uniform state below the positivity threshold fails every stage 1:
    both stop the step after SWFD_RESTART_LIMIT halvings with the same status,
    and the GPU leaves u at u0."""
    kw, _ = CASES["cfl1.2"]
    g, o = pair(oracle_mod, kw)
    u = o.state()
    u[...] = 0.0
    u[..., 0] = 1.0
    u[..., 2] = 1e-14      # uniform: RHS = 0, and E - m^2/(2 rho) <= eps = 1e-13
    g.set_state(u)
    o.set_state(u)
    with pytest.raises(RuntimeError, match=str(abi.ERR_RESTART_LIMIT)):
        o.step()
    with pytest.raises(abi.SwfdError) as e:
        g.step()
    assert e.value.status == abi.ERR_RESTART_LIMIT
    assert np.array_equal(g.state(), u)
    g.close()
