"""Known-answer checks of the oracle's shock-diffraction restatement
(ex6_shock_diffraction/main.f90), on the CPU."""
import numpy as np

from sweeping_fd_weno_gb300 import abi, problems


def test_post_shock_state_satisfies_rankine_hugoniot(oracle_mod):
    """The inflow state of initdata (:1113-1129) is the post-shock state of a
    Mach 5.09 shock into rho = gamma, p = 1, u = 0: mass, momentum and
    energy fluxes agree across the shock in its frame (speed ss = 5.09)."""
    o = oracle_mod.Oracle(problems.workload("shock8"))
    o.init_problem()
    u = o.state()
    g, ss = 1.4, 5.09
    r2, m2, e2 = u[60, 3, 0], u[60, 3, 1], u[60, 3, 3]  # a post-shock cell
    u2 = m2 / r2
    p2 = (g - 1) * (e2 - 0.5 * r2 * u2 * u2)
    r1, u1, p1 = g, 0.0, 1.0
    e1 = p1 / (g - 1)
    # fluxes in the shock frame: w = u - ss
    w1, w2 = u1 - ss, u2 - ss
    mass = (r1 * w1, r2 * w2)
    mom = (r1 * w1 * w1 + p1, r2 * w2 * w2 + p2)
    ene = ((e1 + 0.5 * r1 * (w1 * w1 - u1 * u1) + p1) * w1 + 0.0,
           (e2 - 0.5 * r2 * u2 * u2 + 0.5 * r2 * w2 * w2 + p2) * w2)
    assert abs(mass[0] - mass[1]) < 1e-12 * abs(mass[0])
    assert abs(mom[0] - mom[1]) < 1e-12 * abs(mom[0])
    assert abs(ene[0] - ene[1]) < 1e-12 * abs(ene[0])
    # the shock Mach number: ss = 5.09 relative to the pre-shock sound speed
    assert abs(ss / np.sqrt(g * p1 / r1) - 5.09) < 1e-12


def test_uniform_state_has_no_flux_divergence_away_from_walls(oracle_mod):
    """A uniform pre-shock state: every interior cell away from the walls,
    the inflow and the boundaries has RHS == 0 exactly, including cells at
    the rank boundaries (each rank's alpha differs, but the split fluxes of a
    uniform state cancel)."""
    o = oracle_mod.Oracle(problems.workload("shock8"))
    o.init_problem()
    u = o.state()
    u[...] = np.array([1.4, 0.0, 0.0, 1.0 / 0.4])
    o.set_state(u)
    rhs = o.flux_divergence()
    # rows above the step top and away from the left inflow / walls
    inner = rhs[3 + 52:3 + 80, 3 + 12:3 + 100]
    assert np.all(inner == 0.0)


def test_rank_layout_matters_and_is_reproducible(oracle_mod):
    """The rank grid is part of the arithmetic: a 2 x 2 layout of the same
    grid gives a different (finite) result from 4 x 8 after a few steps,
    and the same layout reproduces itself exactly."""
    def run(cx, cy):
        cfg = problems.make_config(abi.SHOCK_DIFFRACTION, **problems.shock_grid(8, cx, cy))
        o = oracle_mod.Oracle(cfg)
        o.init_problem()
        for _ in range(6):
            o.step()
        return o.state()
    a, b, c = run(4, 8), run(4, 8), run(2, 2)
    assert np.array_equal(a, b)
    assert np.isfinite(c).all() and not np.array_equal(a, c)
