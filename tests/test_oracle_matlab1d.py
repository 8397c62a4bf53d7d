"""The oracle's restatement of the MATLAB script (ex1_double_rarefaction_1d):
properties of the script's own algorithm.  MATLAB is not available, so the
restatement's evaluation order is not pinned against MATLAB's output."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import abi, problems


def run(oracle_mod, variant, steps=None, **kw):
    o = oracle_mod.Oracle(problems.make_config(abi.MATLAB_1D, **dict(problems.matlab_problem(variant), **kw)))
    o.init_problem()
    if steps is None:
        o.run()
    else:
        for _ in range(steps):
            o.step()
    return o


def test_uniform_state_stays_uniform(oracle_mod):
    o = run(oracle_mod, 7)
    u = o.state()[0, 3:-3]
    assert np.all(u == u[0])
    assert o.time == 1e-5


def test_double_rarefaction_is_symmetric_conserving_and_positive(oracle_mod):
    """Problem 5 (the script as shipped): the 1-2-3 problem is mirror
    symmetric, the sweeps keep density and pressure positive, and the
    constant-extension boundaries let little mass leave by T = 0.3."""
    o = run(oracle_mod, 5)
    u = o.state()[0, 3:-3]
    assert o.time == 0.3
    np.testing.assert_allclose(u[:, 0], u[::-1, 0], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(u[:, 1], -u[::-1, 1], rtol=1e-9, atol=1e-12)
    p = 0.4 * (u[:, 2] - 0.5 * u[:, 1] ** 2 / u[:, 0])
    assert u[:, 0].min() > 0 and p.min() > 0
    assert u[:, 0].min() < 0.1                       # the near-vacuum centre
    assert o.stats()["sweep_count"] >= 1


def test_sod_keeps_its_plateaus(oracle_mod):
    o = run(oracle_mod, 3)
    rho = o.state()[0, 3:-3, 0]
    assert abs(rho[0] - 1.0) < 1e-6 and abs(rho[-1] - 0.125) < 1e-6
    assert rho.max() <= 1.0 + 1e-3 and rho.min() >= 0.125 - 1e-3


def test_linear_advection_converges(oracle_mod):
    """Problem 1 (rho = 1 + 0.2 sin(x) carried at speed 1 on [0, 2 pi]): the
    error against the exact solution falls with the grid."""
    errs = []
    for n in (20, 40, 80):
        o = run(oracle_mod, 1, nx=n, time_terminal=0.5)
        h = 2 * np.pi / n
        x = -0.0 + (np.arange(1, n + 1) - 0.5) * h
        rho = o.state()[0, 3:-3, 0]
        errs.append(np.abs(rho - (1 + 0.2 * np.sin(x - o.time))).mean())
    assert errs[1] < errs[0] / 4 and errs[2] < errs[1] / 4
