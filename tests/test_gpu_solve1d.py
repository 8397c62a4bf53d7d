"""The persistent 1D solve (one cooperative launch runs the time loop of
ex2_sedov_1d/main.f90:38-53 over rk3 :287-328) against the graph kernels
(SWFD_SOLVE1D=graph) and the oracle, value for value: the point-energy run of
the benchmark, the reference's own configuration (CFL 1.2, whose run sweeps:
the launch pauses, sweep_lim runs, the next launch resumes at the following
stage), step bounds that split the run over several launches, and a
sweep-heavy run (CFL 1.8)."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu


def _run(cfg, graph, monkeypatch, state=None, chunks=(0,)):
    if graph:
        monkeypatch.setenv("SWFD_SOLVE1D", "graph")
    else:
        monkeypatch.delenv("SWFD_SOLVE1D", raising=False)
    with Solver(cfg) as s:
        s.init_problem()
        if state is not None:
            s.set_state(state)
        n = 0
        for c in chunks:
            try:
                n += s.run(c)
            except abi.SwfdError as e:
                if e.status != abi.ERR_MAX_STEPS:
                    raise
                n += c
        return n, s.time, s.state(), s.stats(), s.tracks(), s.profile()


def _same(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("kw", [dict(nx=800, cfl=0.6, swp_num=2, e_background=1e-12),
                                dict(nx=160), dict(nx=400), dict(nx=800)],
                         ids=["point_energy_800", "ref_160", "ref_400", "ref_800"])
def test_persistent_solve_equals_graph_and_oracle(swfd, oracle_mod, monkeypatch, kw):
    cfg = problems.make_config(abi.SEDOV_1D, **kw)
    n_p, t_p, u_p, st_p, tr_p, pr_p = _run(cfg, False, monkeypatch)
    n_g, t_g, u_g, st_g, tr_g, _ = _run(cfg, True, monkeypatch)
    o = oracle_mod.Oracle(problems.make_config(abi.SEDOV_1D, **kw))
    o.init_problem()
    n_o = o.run()
    assert n_p == n_g == n_o and t_p == t_g == o.time
    assert _same(u_p, u_g), "persistent and graph solves differ"
    assert np.array_equal(u_p, o.state()), "persistent solve differs from the oracle"
    assert st_p == st_g == o.stats()
    for a, b in zip(tr_p, tr_g):
        assert np.array_equal(a, b)
    assert pr_p["stages"] == 3 * n_p
    # one launch per run, one more per sweep, plus the sweeps' own kernels
    assert pr_p["kernel_launches"] >= 1 + st_p["sweep_count"]
    if kw.get("cfl") is None:  # the reference's CFL 1.2 sweeps
        assert st_p["sweep_count"] >= 1


def test_persistent_solve_over_step_bounds(swfd, monkeypatch):
    # run(k) chunks: the launch stops at the bound and the next continues
    cfg = problems.make_config(abi.SEDOV_1D, nx=160)
    n1, t1, u1, st1, _, _ = _run(cfg, False, monkeypatch, chunks=(7, 50, 1, 0))
    n2, t2, u2, st2, _, _ = _run(cfg, True, monkeypatch, chunks=(0,))
    assert n1 == n2 and t1 == t2 and st1 == st2
    assert _same(u1, u2)


def test_persistent_solve_sweep_heavy_run(swfd, oracle_mod, monkeypatch):
    # CFL 1.8: 26 sweeps in the first 20 steps (both nod_lim branches), so
    # launches pause and resume at every stage kind
    kw = dict(nx=200, cfl=1.8)
    cfg = problems.make_config(abi.SEDOV_1D, **kw)
    res = [_run(cfg, g, monkeypatch, chunks=(20,)) for g in (False, True)]
    o = oracle_mod.Oracle(problems.make_config(abi.SEDOV_1D, **kw))
    o.init_problem()
    o.run(20)
    (n_p, t_p, u_p, st_p, tr_p, _), (n_g, t_g, u_g, st_g, tr_g, _) = res
    assert n_p == n_g == 20 and t_p == t_g == o.time
    assert st_p == st_g == o.stats()
    assert st_p["sweep_count"] > 20 and st_p["total_neg"] > 0 and st_p["total_pos"] > 0
    assert _same(u_p, u_g)
    assert np.array_equal(u_p, o.state())
    for a, b in zip(tr_p, tr_g):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("nx", [160, 800])
def test_limiter_1d_persistent_graph_and_oracle(swfd, oracle_mod, monkeypatch, nx):
    # use_limiter 1 (ex2_sedov_1d/main.f90:159-245): the positivity limiter of
    # the split fluxes instead of sweeps; the reference's configuration limits
    # two pressures on the way to T
    kw = dict(nx=nx, use_limiter=1)
    cfg = problems.make_config(abi.SEDOV_1D, **kw)
    n_p, t_p, u_p, st_p, _, _ = _run(cfg, False, monkeypatch)
    n_g, t_g, u_g, st_g, _, _ = _run(cfg, True, monkeypatch)
    o = oracle_mod.Oracle(problems.make_config(abi.SEDOV_1D, **kw))
    o.init_problem()
    n_o = o.run()
    assert n_p == n_g == n_o and t_p == t_g == o.time
    assert st_p == st_g == o.stats()
    assert st_p["pre_count"] == 2 and st_p["sweep_count"] == 0
    assert _same(u_p, u_g)
    assert np.array_equal(u_p, o.state())
