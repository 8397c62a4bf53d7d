"""The high-speed jet of ex5_mach2000_jet run to its final time, against the
oracle: the sweep and adjustment counts of the run the reference prints
(ex5_mach2000_jet/main.f90:853-875; total sweeps, negative pairs, positive
neighbours, pre_count), its per-sweep tracks and the final state.

- At the configured size (800x200 half domain, T = 0.001: 3272 steps that
  sweep in most stages) the oracle takes about 40 minutes on one core, so its
  run is a committed fixture (tests/golden/jet_800x200_to_T.npz, made by
  `python -m tests.golden.make_golden --jet-full`): step count, time, last
  dt, the statistics block, the three tracks, the SHA-256 of the final state's
  bytes and its per-row sums.
- A 200x50 jet to T (775 steps, 2111 sweeps, up to 252 negative cells per
  sweep) runs in the same process on the GPU and in the oracle and is
  compared value for value.  Its sweeps come from the flow itself, not from a
  planted state.
"""
from pathlib import Path

import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "jet_800x200_to_T.npz"


def _sha(u):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(u, np.float64).astype("<f8").tobytes()).hexdigest()


def _assert_stats_and_tracks(st, tracks, ref_stats, ref_tracks):
    assert st == ref_stats, (st, ref_stats)
    for name, a, b in zip(("sweep_track", "neg_track", "pos_track"), tracks, ref_tracks):
        assert a.shape == b.shape, (name, a.shape, b.shape)
        bad = np.flatnonzero(a != b)
        assert bad.size == 0, f"{name}: {bad.size} sweeps differ, first at sweep {bad[0] + 1}"


def test_jet_800x200_to_T_matches_the_oracle_run(swfd):
    ref = np.load(GOLDEN)
    with Solver(problems.workload("jet")) as s:
        s.init_problem()
        n = s.run()
        u = s.state()
        st, tr, t = s.stats(), s.tracks(), s.time
    assert n == int(ref["steps"][0])
    assert t == float(ref["time"][0])
    ref_stats = dict(zip(sorted(st), (int(v) for v in ref["stats"])))
    _assert_stats_and_tracks(st, tr, ref_stats,
                             (ref["sweep_track"], ref["neg_track"], ref["pos_track"]))
    rows = u.sum(axis=1)
    bad_rows = np.flatnonzero(~(rows == ref["row_sums"]).all(axis=1))
    assert bad_rows.size == 0, f"row sums differ in rows {bad_rows[:8].tolist()}"
    assert _sha(u) == str(ref["state_sha256"])
    # the statistics the reference prints for this run sweep in most stages
    assert st["sweep_count"] > 9000 and st["max_neg"] > 100


def test_jet_200x50_to_T_matches_the_oracle_live(swfd, oracle_mod):
    cfg = dict(nx=200, ny=50)
    with Solver(problems.make_config(abi.JET_2D, **cfg)) as s:
        s.init_problem()
        n = s.run()
        u, st, tr, t = s.state(), s.stats(), s.tracks(), s.time
    o = oracle_mod.Oracle(problems.make_config(abi.JET_2D, **cfg))
    o.init_problem()
    no = o.run()
    assert n == no and t == o.time
    _assert_stats_and_tracks(st, tr, o.stats(), o.tracks())
    bad = ~(u == o.state())
    assert not bad.any(), f"{int(bad.sum())} state values differ from the oracle"
    # the flow sweeps by itself: both nod_lim branches and many sweeps
    assert st["sweep_count"] > 1000 and st["total_neg"] > 0 and st["total_pos"] > 0
