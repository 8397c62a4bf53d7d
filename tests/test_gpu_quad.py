"""literals = QUAD: the reference's own build (-fdefault-real-8, which makes
its double-kind literals binary128, so that the WENO smoothness indicators
and alphas, the RK stage combinations, the Roe regularisers of ex4/ex6 and
the literal thresholds are evaluated in binary128 and rounded once).  The GPU
evaluates those subexpressions with software binary128 and must equal the
oracle's _Float128 restatement value for value -- including the cases where
the binary64-literal form drifts away from it (the shock diffraction by 1e-9
after ten steps, ex2 at its own CFL 1.2 by 1e-3)."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

Q = abi.LITERALS_QUAD

CASES = {
    "vortex64x48": (dict(problem=abi.VORTEX_2D, nx=64, ny=48), 6),
    "sedov2d_40": (dict(problem=abi.SEDOV_2D, nx=40, ny=40), 12),
    "jet_96x24": (dict(problem=abi.JET_2D, nx=96, ny=24), 8),
    "sedov1d_ref": (dict(problem=abi.SEDOV_1D, nx=160), 60),
    "sedov1d_200": (dict(problem=abi.SEDOV_1D, nx=200, cfl=0.6, swp_num=2, e_background=1e-12), 30),
    "shock12": (dict(problem=abi.SHOCK_DIFFRACTION, total=12), 6),
    "vortex48_limiter": (dict(problem=abi.VORTEX_2D, nx=48, ny=48, use_limiter=1), 5),
    "sedov1d_restart": (dict(problem=abi.SEDOV_1D, nx=200, cfl=3.0, rk_choice=2), 10),
}


def pair(oracle_mod, kw):
    kw = dict(kw)
    p = kw.pop("problem")
    g = Solver(problems.make_config(p, literals=Q, **kw))
    o = oracle_mod.Oracle(problems.make_config(p, literals=Q, **kw))
    g.init_problem()
    o.init_problem()
    return g, o


def test_weno5_batch_quad_matches_oracle(swfd, oracle_mod):
    rng = np.random.default_rng(9)
    st = np.concatenate([rng.standard_normal((3000, 5)), rng.standard_normal((1000, 5)) * 1e-7,
                         np.cumsum(rng.standard_normal((1000, 5)), axis=1), np.zeros((4, 5))])
    for eps in (1e-6, 1e-12):
        ul_o, ur_o = oracle_mod.weno5(st, eps, 1)
        ul, ur = np.empty(len(st)), np.empty(len(st))
        abi.check(abi.load().swfd_weno5_batch(abi.dptr(np.ascontiguousarray(st)), len(st), eps, Q,
                                              0, abi.dptr(ul), abi.dptr(ur)))
        np.testing.assert_array_equal(ul, ul_o)
        np.testing.assert_array_equal(ur, ur_o)


@pytest.mark.parametrize("case", list(CASES))
def test_quad_steps_match_oracle(swfd, oracle_mod, case):
    kw, steps = CASES[case]
    g, o = pair(oracle_mod, kw)
    for k in range(steps):
        dg = g.step()
        o.step()
        assert dg == o.dt, (k, dg, o.dt)
        assert g.time == o.time
        np.testing.assert_array_equal(g.state(), o.state(), err_msg=f"step {k + 1}")
    assert g.stats() == o.stats()
    g.close()


def test_quad_vortex45_full_run(swfd, oracle_mod):
    g, o = pair(oracle_mod, dict(problem=abi.VORTEX_2D, nx=45, ny=45, time_terminal=0.2))
    n = g.run()
    assert n == o.run() and n > 5
    np.testing.assert_array_equal(g.state(), o.state())
    assert g.stats() == o.stats()
    g.close()


def test_quad_solve_graph_and_eager_match(swfd, oracle_mod, monkeypatch):
    """the solve graph (time loop on the device, binary128 time test) and the
    eager launch mode of the binary128-literal form"""
    kw = dict(problem=abi.SEDOV_2D, nx=40, ny=40, time_terminal=0.02)
    g, o = pair(oracle_mod, kw)
    n = g.run()
    assert n == o.run() and n > 3
    np.testing.assert_array_equal(g.state(), o.state())
    assert g.stats() == o.stats()
    g.close()
    monkeypatch.setenv("SWFD_LAUNCH", "eager")
    e, o2 = pair(oracle_mod, kw)
    for _ in range(4):
        e.step()
        o2.step()
    np.testing.assert_array_equal(e.state(), o2.state())
    e.close()
