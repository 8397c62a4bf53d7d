"""Parity of the CUDA library (through the C ABI) with the CPU oracle.

Both run the same problem from the same configuration on the same machine.
The FP64 path is compared for exact equality of every value (x == y, so only
the sign of an exact zero may differ), the sweep statistics for identity.
Against the oracle's quad-literal mode (the reference's own -fdefault-real-8
build) the bar is 1e-12 relative with identical statistics.
"""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

CASES = {
    "vortex45": dict(problem=abi.VORTEX_2D, nx=45, ny=45),
    "vortex64x48": dict(problem=abi.VORTEX_2D, nx=64, ny=48),
    "sedov2d_40": dict(problem=abi.SEDOV_2D, nx=40, ny=40),
    "jet_96x24": dict(problem=abi.JET_2D, nx=96, ny=24),
    # the jet's full domain [0,1]x[-0.25,0.25] (variant 1)
    "jet_full_96x48": dict(problem=abi.JET_2D, nx=96, ny=48, variant=1),
    "sedov1d_200": dict(problem=abi.SEDOV_1D, nx=200, cfl=0.6, swp_num=2, e_background=1e-12),
    "sedov1d_ref": dict(problem=abi.SEDOV_1D, nx=160),
}


def make_pair(oracle_mod, case, **extra):
    kw = dict(CASES[case])
    p = kw.pop("problem")
    kw.update(extra)
    cfg = problems.make_config(p, **kw)
    g = Solver(cfg)
    o = oracle_mod.Oracle(problems.make_config(p, **kw))
    g.init_problem()
    o.init_problem()
    return g, o


def assert_same(a, b, what=""):
    assert a.shape == b.shape
    bad = ~(a == b)
    if bad.any():
        idx = np.argwhere(bad)[:5]
        rel = np.max(np.abs(a - b)[bad] / np.maximum(np.abs(b[bad]), 1e-300))
        raise AssertionError(f"{what}: {bad.sum()} values differ, max rel {rel:.3e}, first {idx.tolist()}")


def test_weno5_batch_matches_oracle(swfd, oracle_mod):
    rng = np.random.default_rng(7)
    st = np.concatenate([
        rng.standard_normal((4000, 5)),
        rng.standard_normal((2000, 5)) * 1e-9,
        np.cumsum(rng.standard_normal((2000, 5)), axis=1),
        np.zeros((8, 5)),
    ])
    ul_o, ur_o = oracle_mod.weno5(st, 1e-6, 0)
    ul = np.empty(len(st))
    ur = np.empty(len(st))
    abi.check(abi.load().swfd_weno5_batch(abi.dptr(np.ascontiguousarray(st)), len(st), 1e-6,
                                          abi.LITERALS_DOUBLE, 0, abi.dptr(ul), abi.dptr(ur)))
    assert_same(ul, ul_o, "weno_left")
    assert_same(ur, ur_o, "weno_right")


@pytest.mark.parametrize("case", list(CASES))
def test_initial_state_matches(swfd, oracle_mod, case):
    g, o = make_pair(oracle_mod, case)
    assert_same(g.state(), o.state(), "initdata + bc")


@pytest.mark.parametrize("case", list(CASES))
def test_flux_divergence_matches(swfd, oracle_mod, case):
    g, o = make_pair(oracle_mod, case)
    assert g.find_alpha() == o.find_alpha()
    assert_same(g.flux_divergence(), o.flux_divergence(), "wenofd + scheme")


@pytest.mark.parametrize("sweep_mode", [abi.SWEEP_PARALLEL, abi.SWEEP_SEQUENTIAL])
@pytest.mark.parametrize("case", list(CASES))
def test_three_steps_match(swfd, oracle_mod, case, sweep_mode):
    g, o = make_pair(oracle_mod, case, sweep_mode=sweep_mode)
    for k in range(3):
        dt_g = g.step()
        dt_o = o.step()
        assert dt_g == dt_o, (k, dt_g, dt_o)
        assert g.time == o.time
        assert_same(g.state(), o.state(), f"state after step {k + 1}")
    assert g.stats() == o.stats()
    for a, b in zip(g.tracks(), o.tracks()):
        assert np.array_equal(a, b)


def test_vortex45_full_run_matches_and_is_within_1e12_of_quad_reference(swfd, oracle_mod):
    g, o = make_pair(oracle_mod, "vortex45")
    n_g = g.run()
    n_o = o.run()
    assert n_g == n_o
    assert_same(g.state(), o.state(), "vortex45 at T")
    assert g.stats() == o.stats()
    q = oracle_mod.Oracle(problems.make_config(abi.VORTEX_2D, nx=45, ny=45,
                                               literals=abi.LITERALS_QUAD))
    q.init_problem()
    assert q.run() == n_g
    u, uq = g.state(), q.state()
    rel = np.abs(u - uq) / np.maximum(np.abs(uq), 1e-300)
    assert rel.max() <= 1e-12, rel.max()
    assert g.stats() == q.stats()


def _poison(u, ndim, cells, rng):
    """Make some cells non-positive in pressure or density (a state a stage can leave)."""
    u = u.copy()
    for (j, i) in cells:
        v = u[j, i]
        if ndim == 2:
            kin = 0.5 * (v[1] ** 2 + v[2] ** 2) / v[0]
            v[3] = kin * (1.0 - rng.uniform(0, 1e-3))
        else:
            kin = 0.5 * v[1] ** 2 / v[0]
            v[2] = kin * (1.0 - rng.uniform(0, 1e-3))
        if rng.uniform() < 0.3:
            v[0] = rng.uniform(1e-16, 5e-14)
    return u


@pytest.mark.parametrize("case", ["vortex45", "vortex64x48", "jet_96x24", "sedov1d_200"])
def test_sweep_on_poisoned_state_matches(swfd, oracle_mod, case):
    g, o = make_pair(oracle_mod, case)
    rng = np.random.default_rng(11)
    u = o.state()
    ndim = 1 if u.shape[0] == 1 else 2
    if ndim == 2:
        ny, nx = u.shape[0] - 6, u.shape[1] - 6
        cells = [(3 + rng.integers(0, ny), 3 + rng.integers(0, nx)) for _ in range(12)]
        j0, i0 = 3 + ny // 2, 3 + nx // 3
        cells += [(j0, i0 + d) for d in range(5)] + [(j0 + d, i0) for d in range(4)]
    else:
        n = u.shape[1] - 6
        cells = [(0, 3 + rng.integers(0, n)) for _ in range(8)] + [(0, 3 + n // 2 + d) for d in range(6)]
    u = _poison(u, ndim, cells, rng)
    g.set_state(u)
    o.set_state(u)
    assert g.check_positivity() == o.check_positivity() == 1
    g.sweep()
    assert o.sweep() == 0
    assert_same(g.state(), o.state(), "after sweep_lim")
    assert g.stats() == o.stats()
    s = g.stats()
    assert s["sweep_count"] == 1 and s["pre_count"] >= 1


def _dense_poison(u, rng, frac=0.5, block=(12, 12), ndim=2):
    u = u.copy()
    if ndim == 2:
        ny, nx = u.shape[0] - 6, u.shape[1] - 6
        j0 = 3 + rng.integers(0, ny - block[0])
        i0 = 3 + rng.integers(0, nx - block[1])
        cells = [(j, i) for j in range(j0, j0 + block[0]) for i in range(i0, i0 + block[1])
                 if rng.uniform() < frac]
    else:
        n = u.shape[1] - 6
        i0 = 3 + rng.integers(0, n - 40)
        cells = [(0, i) for i in range(i0, i0 + 40) if rng.uniform() < frac]
    return _poison(u, ndim, cells, rng)


@pytest.mark.parametrize("case", ["vortex64x48", "jet_96x24", "sedov1d_200", "sedov2d_40"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_parallel_sweep_equals_sequential_and_oracle_on_dense_damage(swfd, oracle_mod, case, seed):
    # swp_num 40: a sweep that does not converge must fail identically
    # (SWEEP FAIL stops ex4; ex2, ex3, ex5 go on)
    g, o = make_pair(oracle_mod, case, swp_num=40)
    gs, _ = make_pair(oracle_mod, case, swp_num=40, sweep_mode=abi.SWEEP_SEQUENTIAL)
    rng = np.random.default_rng(seed)
    u = o.state()
    ndim = 1 if u.shape[0] == 1 else 2
    u = _dense_poison(u, rng, frac=0.6, ndim=ndim)
    for s in (g, gs):
        s.set_state(u)
    o.set_state(u)
    st_o = o.sweep()

    def status(solver):
        try:
            solver.sweep()
            return 0
        except abi.SwfdError as e:
            return e.status

    assert status(g) == st_o
    assert status(gs) == st_o
    assert_same(gs.state(), o.state(), "sequential GPU sweep")
    assert_same(g.state(), o.state(), "parallel GPU sweep")
    assert g.stats() == gs.stats() == o.stats()


def test_parallel_sweep_many_chains_256(swfd, oracle_mod):
    """A ring of damaged cells on a 256^2 grid: hundreds of independent chains."""
    cfg = dict(problem=abi.VORTEX_2D, nx=256, ny=256)
    g = Solver(problems.make_config(**cfg))
    gs = Solver(problems.make_config(**cfg, sweep_mode=abi.SWEEP_SEQUENTIAL))
    o = oracle_mod.Oracle(problems.make_config(**cfg))
    for s in (g, gs, o):
        s.init_problem()
    u = o.state()
    rng = np.random.default_rng(9)
    jj, ii = np.meshgrid(np.arange(256), np.arange(256), indexing="ij")
    r = np.hypot(jj - 128, ii - 128)
    cells = [(3 + j, 3 + i) for j, i in zip(*np.nonzero((np.abs(r - 60) < 1.5)))
             if rng.uniform() < 0.7]
    u = _poison(u, 2, cells, rng)
    for s in (g, gs, o):
        s.set_state(u)
    o.sweep()
    g.sweep()
    gs.sweep()
    assert_same(g.state(), o.state(), "parallel sweep 256^2")
    assert_same(gs.state(), o.state(), "sequential sweep 256^2")
    assert g.stats() == o.stats() == gs.stats()
