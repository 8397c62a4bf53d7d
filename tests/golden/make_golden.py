"""Generate the golden fixtures of the CPU oracle.

    python -m tests.golden.make_golden            # the small runs (seconds)
    python -m tests.golden.make_golden --jet-full # the 800x200 jet to T (~40 min, one core)

Each fixture stores the final state, the sweep statistics and tracks, the
time and the last dt of one small run of the oracle.  The reference ships no
outputs of its own, so these fixtures pin the oracle against regressions;
they are regenerated only when the oracle's restatement is deliberately
changed.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from sweeping_fd_weno_gb300 import abi, problems  # noqa: E402

CASES = {
    # name: (problem, config overrides, steps (0 = run to T))
    "vortex45_run": (abi.VORTEX_2D, dict(nx=45, ny=45), 0),
    "vortex45_run_quad": (abi.VORTEX_2D, dict(nx=45, ny=45, literals=abi.LITERALS_QUAD), 0),
    "vortex90_2steps": (abi.VORTEX_2D, dict(nx=90, ny=90), 2),
    "sedov1d_fp64_n200_40steps": (abi.SEDOV_1D, dict(nx=200, cfl=0.6, swp_num=2,
                                                     e_background=1e-12), 40),
    "sedov2d_32_6steps": (abi.SEDOV_2D, dict(nx=32, ny=32), 6),
    "jet_80x20_6steps": (abi.JET_2D, dict(nx=80, ny=20), 6),
    "shock8_20steps": (abi.SHOCK_DIFFRACTION, dict(total=8), 20),
}


def run_case(oracle_mod, name):
    problem, kw, steps = CASES[name]
    o = oracle_mod.Oracle(problems.make_config(problem, **kw))
    o.init_problem()
    if steps == 0:
        o.run()
    else:
        for _ in range(steps):
            o.step()
    st = o.stats()
    tr = o.tracks()
    return {
        "state": o.state(),
        "stats": np.array([st[k] for k in sorted(st)], np.int64),
        "sweep_track": tr[0], "neg_track": tr[1], "pos_track": tr[2],
        "time": np.array([o.time]), "dt": np.array([o.dt]),
    }


def state_digest(u):
    """SHA-256 of the state's bytes (C order, float64, little endian) and the
    per-row sums of each component, so that a mismatch can be located."""
    import hashlib
    u = np.ascontiguousarray(u, np.float64)
    return hashlib.sha256(u.astype("<f8").tobytes()).hexdigest(), u.sum(axis=1)


def jet_full(oracle_mod):
    """The jet of ex5_mach2000_jet at its configured size (800x200 half domain,
    T=0.001) run to T by the oracle: step count, time, last dt, the
    statistics block, the three tracks and a digest of the final state."""
    import time as _time
    o = oracle_mod.Oracle(problems.workload("jet"))
    o.init_problem()
    t0 = _time.time()
    steps = o.run()
    wall = _time.time() - t0
    st = o.stats()
    tr = o.tracks()
    sha, rows = state_digest(o.state())
    return {
        "steps": np.array([steps], np.int64),
        "stats": np.array([st[k] for k in sorted(st)], np.int64),
        "sweep_track": tr[0], "neg_track": tr[1], "pos_track": tr[2],
        "time": np.array([o.time]), "dt": np.array([o.dt]),
        "state_sha256": np.array(sha), "row_sums": rows,
        "oracle_wall_s": np.array([wall]),
    }


def main():
    import oracle
    oracle.build()
    out = Path(__file__).resolve().parent
    if "--jet-full" in sys.argv:
        d = jet_full(oracle)
        np.savez_compressed(out / "jet_800x200_to_T.npz", **d)
        print("jet_800x200_to_T steps", d["steps"][0], "time", d["time"][0],
              "wall", d["oracle_wall_s"][0], "sha", str(d["state_sha256"]))
        return
    for name in CASES:
        d = run_case(oracle, name)
        np.savez_compressed(out / f"{name}.npz", **d)
        print(name, {k: v.shape for k, v in d.items()}, "time", d["time"][0])


if __name__ == "__main__":
    main()
