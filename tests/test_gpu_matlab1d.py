"""The MATLAB script of the reference's first example
(ex1_double_rarefaction_1d/FD_WENO_Application.m) on the GPU against the
oracle's restatement, value for value: state, time, dt and sweep counts."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu


def pair(oracle_mod, variant, **kw):
    cfg = dict(problems.matlab_problem(variant), **kw)
    g = Solver(problems.make_config(abi.MATLAB_1D, **cfg))
    o = oracle_mod.Oracle(problems.make_config(abi.MATLAB_1D, **cfg))
    g.init_problem()
    o.init_problem()
    return g, o


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6, 7])
def test_initial_state_matches(swfd, oracle_mod, variant):
    g, o = pair(oracle_mod, variant)
    assert np.array_equal(g.state(), o.state())
    g.close()


@pytest.mark.parametrize("variant,steps", [(5, 12), (3, 10), (4, 10), (1, 10), (2, 8), (6, 3)])
def test_steps_match(swfd, oracle_mod, variant, steps):
    g, o = pair(oracle_mod, variant)
    for k in range(steps):
        dg = g.step()
        o.step()
        assert dg == o.dt, (k, dg, o.dt)
        assert g.time == o.time
        np.testing.assert_array_equal(g.state(), o.state(), err_msg=f"step {k + 1}")
    assert g.stats() == o.stats()
    g.close()


def test_double_rarefaction_full_run_matches(swfd, oracle_mod):
    """The script as shipped (problem 5, 200 cells, T = 0.3): the whole time
    loop in one call, with the sweeps it triggers."""
    g, o = pair(oracle_mod, 5)
    n = g.run()
    assert n == o.run() and n > 50
    assert g.time == o.time == 0.3
    np.testing.assert_array_equal(g.state(), o.state())
    s = g.stats()
    assert s == o.stats() and s["sweep_count"] >= 1
    for a, b in zip(g.tracks(), o.tracks()):
        assert np.array_equal(a, b)
    g.close()


def test_without_sweeping_matches(swfd, oracle_mod):
    g, o = pair(oracle_mod, 5, use_limiter=0)
    assert g.run() == o.run()
    np.testing.assert_array_equal(g.state(), o.state())
    g.close()
