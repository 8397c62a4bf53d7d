"""Detonation (ex7_detonation): the GPU engine, which keeps the reference's
cut_x x cut_y ranks as slices of one buffer, against the oracle, which runs
them as separate local grids -- value for value: five components, the q*Y
equation of state, the chemistry source (exp evaluated in binary128 by both),
the 5x5 eigenvectors, the wall mirrors, the ex7 boundaries and the sweep with
the reference's ordering-II indexing."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

# (total, cut_x, cut_y): 40 x 40 on 2 x 2 ranks, 160 x 160 on the reference's 4 x 8
CASES = [(8, 2, 2), (32, 4, 8)]


def pair(oracle_mod, total, cx, cy, **kw):
    cfg = problems.make_config(abi.DETONATION, total=total, cut_x=cx, cut_y=cy, **kw)
    g = Solver(cfg)
    o = oracle_mod.Oracle(problems.make_config(abi.DETONATION, total=total, cut_x=cx, cut_y=cy,
                                               **kw))
    g.init_problem()
    o.init_problem()
    return g, o


def assert_same(a, b, what):
    bad = ~(a == b)
    if bad.any():
        idx = np.argwhere(bad)[:5]
        rel = np.max(np.abs(a - b)[bad] / np.maximum(np.abs(b[bad]), 1e-300))
        raise AssertionError(f"{what}: {int(bad.sum())} values differ, max rel {rel:.3e}, "
                             f"first {idx.tolist()}")


@pytest.mark.parametrize("case", CASES)
def test_initial_state(swfd, oracle_mod, case):
    g, o = pair(oracle_mod, *case)
    assert g.state().shape[2] == 5
    assert_same(g.state(), o.state(), f"init {case}")
    g.close()


@pytest.mark.parametrize("case", CASES)
def test_find_alpha(swfd, oracle_mod, case):
    g, o = pair(oracle_mod, *case)
    for _ in range(2):
        g.step()
        o.step()
    assert g.find_alpha() == o.find_alpha()
    g.close()


@pytest.mark.parametrize("case,steps", [((8, 2, 2), 60), ((32, 4, 8), 30)])
def test_steps_match_the_oracle(swfd, oracle_mod, case, steps):
    g, o = pair(oracle_mod, *case)
    for k in range(steps):
        dg = g.step()
        do = o.step()
        assert dg == do, (k, dg, do)
        if k % 10 == 9:
            assert_same(g.state(), o.state(), f"{case} step {k + 1}")
    assert g.time == o.time
    assert_same(g.state(), o.state(), f"{case} after {steps} steps")
    assert g.stats() == o.stats()
    g.close()


def test_full_run_with_sweeps(swfd, oracle_mod):
    """40 x 40 to T = 0.6: several sweeps, with both nod_lim branches."""
    g, o = pair(oracle_mod, 8, 2, 2)
    n = g.run()
    m = o.run()
    assert n == m
    assert g.time == o.time
    assert_same(g.state(), o.state(), "T = 0.6")
    st = g.stats()
    assert st == o.stats()
    assert st["sweep_count"] > 0 and st["total_pos"] > 0
    g.close()


def test_state_round_trip_and_unsupported_entry_points(swfd, oracle_mod):
    g, o = pair(oracle_mod, 8, 2, 2)
    for _ in range(3):
        o.step()
    u = o.state()
    g.set_state(u)
    assert_same(g.state(), u, "upload/download")
    g.time = o.time
    assert g.step() == o.step()
    assert_same(g.state(), o.state(), "step after upload")
    with pytest.raises(RuntimeError):
        g.flux_divergence()
    g.close()


@pytest.mark.parametrize("case,steps", [((8, 2, 2), 0), ((32, 4, 8), 6)])
def test_binary128_literals_match_the_oracle(swfd, oracle_mod, case, steps):
    """literals QUAD (the reference's -fdefault-real-8 build): the WENO
    indicators and alphas, the RK combinations, the 1d-15 Roe regularisers,
    rho < 1d-8 and the time loop with binary128 literals; steps 0 runs to
    T = 0.6 (with sweeps)."""
    g, o = pair(oracle_mod, *case, literals=abi.LITERALS_QUAD)
    if steps == 0:
        assert g.run() == o.run()
    else:
        for k in range(steps):
            assert g.step() == o.step(), k
    assert g.time == o.time
    assert_same(g.state(), o.state(), f"quad {case}")
    assert g.stats() == o.stats()
    g.close()


@pytest.mark.parametrize("literals", [abi.LITERALS_DOUBLE, abi.LITERALS_QUAD])
def test_flux_limiter_run(swfd, oracle_mod, literals):
    """use_limiter = 1: the five-component positivity limiter (q*Y in both
    pressures) on a whole 40 x 40 run; the density and pressure limitings
    are counted in den_count and pre_count."""
    g, o = pair(oracle_mod, 8, 2, 2, use_limiter=1, literals=literals)
    assert g.run() == o.run()
    assert g.time == o.time
    assert_same(g.state(), o.state(), f"limiter, literals {literals}")
    st = g.stats()
    assert st == o.stats()
    assert st["den_count"] > 0 and st["pre_count"] > 0
    g.close()
