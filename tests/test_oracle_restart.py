"""The dt-halving restart RK of ex2 (RK_choice /= 1, ex2_sedov_1d/main.f90:
330-374) in the CPU oracle: properties that hold for the reference's
algorithm itself."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import abi, problems


def make(oracle_mod, **kw):
    o = oracle_mod.Oracle(problems.make_config(abi.SEDOV_1D, nx=200, **kw))
    o.init_problem()
    return o


def test_without_restarts_equals_rk3_without_sweeps(oracle_mod):
    """While no stage fails checkpositivity, `rk` runs exactly the operations
    of `rk3` with the sweeps switched off."""
    a = make(oracle_mod, rk_choice=2, cfl=0.3)
    b = make(oracle_mod, rk_choice=1, cfl=0.3, use_limiter=0)
    for _ in range(15):
        a.step()
        b.step()
        assert a.dt == b.dt
        assert np.array_equal(a.state(), b.state())
    assert a.restarts == 0


@pytest.mark.parametrize("cfl,steps,min_restarts", [(1.2, 40, 1), (3.0, 20, 20)])
def test_restarts_halve_dt_and_keep_positivity(oracle_mod, cfl, steps, min_restarts):
    """Every accepted step passes checkpositivity (rho, P > eps in the
    interior), and each restart halves the step's dt: the accepted dt is
    dx*cfl/alphamax / 2^r for the step's r restarts."""
    o = make(oracle_mod, rk_choice=2, cfl=cfl)
    for _ in range(steps):
        before = o.restarts
        u0 = o.state()
        alpha = o.find_alpha()
        o.set_state(u0)
        o.step()
        r = o.restarts - before
        assert o.dt == (o.dx * cfl / alpha) / 2.0 ** r
        u = o.state()[0, 3:-3]
        assert (u[:, 0] > 1e-13).all()
        assert (u[:, 2] - u[:, 1] ** 2 / u[:, 0] / 2.0 > 1e-13).all()
    assert o.restarts >= min_restarts


def test_a_state_that_never_turns_positive_ends_at_the_restart_limit(oracle_mod):
    """A uniform state whose pressure term is below eps has RHS = 0, so every
    stage 1 returns u0 and fails checkpositivity however small dt gets: the
    oracle stops after SWFD_RESTART_LIMIT halvings (the reference would loop
    on)."""
    o = make(oracle_mod, rk_choice=2)
    u = o.state()
    u[...] = 0.0
    u[..., 0] = 1.0
    u[..., 2] = 1e-14      # uniform: RHS = 0, and E - m^2/(2 rho) <= eps = 1e-13
    o.set_state(u)
    with pytest.raises(RuntimeError, match=str(abi.ERR_RESTART_LIMIT)):
        o.step()
    assert o.restarts == 0 or o.restarts <= abi.RESTART_LIMIT
