"""Size-independent properties at full sizes, where the oracle would take
minutes to hours per solve:

- the GPU path is deterministic: two solves from the same initial state agree
  value for value, with the same step count, time and sweep statistics (the
  max-reductions are order-independent and the sweeps run in the reference's
  sequential order);
- the reference's own positivity test (checkpositivity,
  ex3_vortex_accuracy_2d/main.f90:634-651) passes on the state a step leaves;
- on the periodic vortex the interior totals of all four conserved
  variables stay constant to rounding: the flux differences telescope and the
  sweeps (density sweep, pressure passes with nodal adjustment) move
  conserved quantities between cells without changing the totals.

The point-energy problem is not a conservation case: at its reflective
walls (ex4_sedov_2d/main.f90:922-948) the wall-face fluxes, zero in exact
arithmetic by mirror symmetry, are not zero in rounded arithmetic, where the
characteristic projection of the near-vacuum background (sound speed ~1e-6)
is ill-conditioned.  The reference's scheme itself changes the interior
totals there (at 128^2 the oracle's t=0 mass flux divergence sums to -7e-4
and the first step gains 1.5e-4 of the energy), so only determinism and
positivity are checked for it.
"""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, problems

pytestmark = pytest.mark.gpu


def _interior(s, u):
    # state arrays are [j+2, i+2, c] for i, j in -2..n+3: cells 1..n at 3..n+2
    return u[3:s.ny + 3, 3:s.nx + 3, :]


def _solve_twice(name, steps=None, checkpoints=()):
    out = []
    for rep in range(2):
        with Solver(problems.workload(name)) as s:
            s.init_problem()
            first = _interior(s, s.state()).copy()
            if steps is None:
                n = s.run()
            else:
                n = steps
                for k in range(steps):
                    s.step()
                    if rep == 0 and (k + 1) in checkpoints:
                        assert s.check_positivity() == 0, f"{name}: step {k + 1}"
            u = s.state()
            out.append(dict(n=n, u=u, first=first, inner=_interior(s, u).copy(),
                            stats=s.stats(), t=s.time, pos=s.check_positivity()))
    a, b = out
    assert a["n"] == b["n"] and a["t"] == b["t"] and a["stats"] == b["stats"], name
    bad = ~(a["u"] == b["u"])
    assert not bad.any(), f"{name}: {int(bad.sum())} values differ between two identical solves"
    assert np.isfinite(a["inner"]).all()
    assert a["pos"] == 0
    assert (a["inner"][..., 0] > 0).all()
    return a


def test_jet_800x200_full_run_is_deterministic_and_positive(swfd):
    """The jet (800x200 half domain, gamma 5/3, T=0.001) run to the end twice."""
    T = problems.workload("jet").time_terminal
    a = _solve_twice("jet")
    assert a["n"] > 100
    assert T - 1e-10 < a["t"] <= T + 1e-12


def test_point_energy_640_is_deterministic_and_positive(swfd):
    """The 640x640 point-energy instance ([0,1.3]^2, corner blast, E=1e-12
    background) for 200 steps, twice; the positivity test checked every 50."""
    a = _solve_twice("sedov2d640", steps=200, checkpoints=(50, 100, 150, 200))
    assert a["t"] > 0.0


def test_vortex_1024_conserves_and_is_deterministic(swfd):
    """The near-vacuum vortex at 1024^2 (periodic, T=0.01) run to the end
    twice: all four interior totals conserved to 1e-12 relative."""
    a = _solve_twice("vortex1024")
    t0, t1 = a["first"].sum(axis=(0, 1)), a["inner"].sum(axis=(0, 1))
    rel = np.abs(t1 - t0) / np.abs(t0)
    assert (rel <= 1e-12).all(), rel
