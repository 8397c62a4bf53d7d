"""Parity at the sizes of the named configurations: the GPU path against the
oracle on the same inputs, every value equal and the sweep statistics
identical (full runs where the oracle finishes in seconds, leading steps
otherwise)."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu


def pair(oracle_mod, cfg_fn):
    g, o = Solver(cfg_fn()), oracle_mod.Oracle(cfg_fn())
    g.init_problem()
    o.init_problem()
    return g, o


def same(g, o, what):
    a, b = g.state(), o.state()
    bad = ~(a == b)
    assert not bad.any(), f"{what}: {int(bad.sum())} values differ"
    assert g.time == o.time, what
    assert g.stats() == o.stats(), what


@pytest.mark.parametrize("name", ["sedov1d_fp64", "vortex45", "vortex90", "vortex180", "vortex360"])
def test_full_run(swfd, oracle_mod, name):
    """C1 (800 points, CFL 0.6, swp_num 2, E=1e-12, T=0.001) and C2 (the
    vortex at 45^2..360^2 to T=0.01), run to the end."""
    g, o = pair(oracle_mod, lambda: problems.workload(name))
    ng, no = g.run(), o.run()
    assert ng == no
    same(g, o, name)


def test_sedov1d_shipped_parameters_full_run(swfd, oracle_mod):
    """C1 with the shipped PARAMETERs (CFL 1.2, swp_num 50, E=1d-9/gamma1)."""
    g, o = pair(oracle_mod, lambda: problems.make_config(abi.SEDOV_1D))
    ng, no = g.run(), o.run()
    assert ng == no
    same(g, o, "sedov1d shipped")


@pytest.mark.parametrize("name,steps", [("jet", 5), ("sedov2d128", 40), ("sedov2d640", 3)])
def test_leading_steps(swfd, oracle_mod, name, steps):
    """C4 (jet 800x200 half domain) and C3 instances (point energy 128^2, 640^2)."""
    g, o = pair(oracle_mod, lambda: problems.workload(name))
    for k in range(steps):
        g.step()
        o.step()
    same(g, o, f"{name} after {steps} steps")
