#!/usr/bin/env python
"""Benchmark of the sweeping FD-WENO Euler step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one SSP-RK3 time step (three RK stages, each with its CFL reduction,
characteristic WENO5 fluxes, RK update, positivity test, sweep when flagged and
boundary conditions) of the 360x360 near-vacuum isentropic vortex in plain
FP64, on state resident in HBM.  The metric is cell-updates/s per RK stage:
interior cells x stages / time.  One JSON line is printed by rank 0.

Under torchrun (N > 1) every rank advances its own replica (the path does not
shard within one grid); the value is the sum of all ranks' work over the
slowest rank's time.

--impl reference times the reference's algorithm on the host CPU instead: the
CPU restatement of the reference (the oracle) on the same 360x360 vortex with
the same binary64 literals as the GPU line, one solve per host core; beside it
the binary128-literal pair (the arithmetic of the reference's -fdefault-real-8
build) on the same grid.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s per RK stage, FP32-batched vs plain FP64; p50/p99 solve latency"
UNIT = "cell-updates/s"
# compulsory HBM traffic of one fused 2D FP64 RK stage, bytes per cell
# (read u_k and u0, write u_k+1: 85.3 B averaged over the three stages)
STAGE_BYTES_PER_CELL = (64 + 96 + 96) / 3.0
# FP64 work of one interface flux (Roe eigenvectors, 40 projections, 8 WENO5
# reconstructions, back projection): 800 adds/multiplies + 50 divisions + 1
# square root in the source.  With the hardware division this executes 1197
# FP64 pipe instructions (379 DADD, 465 DMUL, 353 DFMA -- the DFMAs are the
# divisions and the square root); with the divisions and the products by
# 2, 4, 0.25 and 0.5 on the integer pipes (the same bits), 739 (355 DADD,
# 379 DMUL, 5 DFMA).  Both counted by ncu on the one-lane k_flux_xy<double>;
# the default kernel, k_flux_xy_share<5> (two lanes per interface, the
# eigenvectors formed once per interface and shared), executes 737 (ncu on
# the 1024x1024 vortex), and 739 stays the work the roofline counts.
FLUX_FLOPS_PER_INTERFACE = 800 + 50 + 1
FLUX_FP64_INST_PER_INTERFACE = 739
FLUX_FP64_INST_PER_INTERFACE_EXECUTED = 737
FLUX_FP64_INST_PER_INTERFACE_HW_DIV = 1197
# DRAM bytes of one k_flux_xy_share<5> launch per interior cell, from an ncu
# capture of the 1024x1024 vortex (313.9 MB per launch, inputs above L2)
FLUX_DRAM_BYTES_PER_CELL = 313.9e6 / (1024 * 1024)
# the same for k_flux_xy<float> of the FP32-bulk form's separate kernels
# (134.4 MB per launch) and for its fused stage kernel k_stage32<256, 4>
# (107.9 MB per launch)
FLUX_F32_DRAM_BYTES_PER_CELL = 134.4e6 / (1024 * 1024)
STAGE32_DRAM_BYTES_PER_CELL = 107.9e6 / (1024 * 1024)
# algorithmic bytes of one fused FP32-bulk stage per interior cell: the nine
# splitting terms and four Roe planes (FP32) read once, u and u0 read and u
# written (FP64)
STAGE32_BYTES_PER_CELL = 9 * 4 + 4 * 4 + 3 * 32


def precision_errors(u32, u64, gamma=1.4):
    """The FP32-bulk state against the FP64 path's (value-for-value the
    oracle's) on the interior cells: relative L1 and Linf errors of density and
    pressure, and the relative drift of total mass and total energy."""
    import numpy as np
    a, b = u32[3:-3, 3:-3], u64[3:-3, 3:-3]

    def pres(u):
        return (gamma - 1.0) * (u[..., 3] - 0.5 * (u[..., 1] ** 2 + u[..., 2] ** 2) / u[..., 0])

    out = {}
    for name, x, y in (("density", a[..., 0], b[..., 0]), ("pressure", pres(a), pres(b))):
        d = np.abs(x - y)
        out[f"rel_l1_{name}"] = float(d.sum() / np.abs(y).sum())
        out[f"rel_linf_{name}"] = float(d.max() / np.abs(y).max())
    out["mass_drift"] = float((a[..., 0].sum() - b[..., 0].sum()) / b[..., 0].sum())
    out["energy_drift"] = float((a[..., 3].sum() - b[..., 3].sum()) / b[..., 3].sum())
    return out


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[4:8]) if v == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(nx: int, budget_s: float = 10.0) -> dict:
    """The CPU oracle on the host, one thread, on a bounded sample of the workload."""
    import oracle
    from sweeping_fd_weno_gb300 import problems
    oracle.build()
    o = oracle.Oracle(problems.workload(f"vortex{nx}"))
    o.init_problem()
    t0 = time.perf_counter()
    steps = 0
    while True:
        o.step()
        steps += 1
        if time.perf_counter() - t0 >= budget_s or steps >= 200:
            break
    el = time.perf_counter() - t0
    v = nx * nx * 3 * steps / el
    # the reference's own build promotes its double literals to REAL(16):
    # one RK3 step of a 120x120 vortex in that arithmetic
    q = oracle.Oracle(problems.workload("vortex120", literals=1))
    q.init_problem()
    t1 = time.perf_counter()
    q.step()
    qel = time.perf_counter() - t1
    return {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} SSP-RK3 steps of the {nx}x{nx} vortex, double literals "
                      f"(the arithmetic of the GPU path), single thread, {el:.1f} s",
            "quad_literal_value": 120 * 120 * 3 / qel,
            "quad_literal_sample": f"1 SSP-RK3 step of a 120x120 vortex with REAL(16) literals "
                                   f"(the reference's -fdefault-real-8 build), {qel:.1f} s"}


# --- batched point-energy instances and the serving stream -------------------

BATCH_SEED = 20261203
SERVE_SEED = 20261204


def point_energy_sizes(n_inst: int, seed: int = BATCH_SEED):
    """Side lengths of the batched point-energy instances: uniform on 128..640."""
    import numpy as np
    return [int(n) for n in np.random.default_rng(seed).integers(128, 641, size=n_inst)]


def _oracle_steps(args):
    """One CPU oracle instance (a worker of the host-core baseline)."""
    n, steps = args
    import oracle
    from sweeping_fd_weno_gb300 import abi, problems
    o = oracle.Oracle(problems.make_config(abi.SEDOV_2D, nx=n, ny=n))
    o.init_problem()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    return n * n * 3 * steps, time.perf_counter() - t0


def cpu_batched_baseline(sizes, steps: int = 1) -> dict:
    """The CPU oracle, one instance per host core, on the first instances of
    the batched workload (a process pool started with spawn)."""
    import multiprocessing as mp
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    sample = sizes[:cores]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        out = pool.map(_oracle_steps, [(n, steps) for n in sample])
    wall = time.perf_counter() - t0
    upd = sum(u for u, _ in out)
    busy = max(t for _, t in out)
    return {"value": upd / busy, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{len(sample)} of the point-energy instances ({min(sample)}^2..."
                      f"{max(sample)}^2), {steps} SSP-RK3 step(s) each, one instance per core, "
                      f"FP64 double literals; value = updates / slowest instance's time "
                      f"({busy:.1f} s; pool wall {wall:.1f} s)"}


def bench_batched(args, local, flush):
    """256 point-energy instances (seeded sizes 128^2..640^2 on [0,1.3]^2) in the
    batched engine with the FP32-bulk precision, against the plain FP64 path one
    instance at a time on a seeded sample of the same instances."""
    import numpy as np
    import torch
    from sweeping_fd_weno_gb300 import Batch, Solver, abi, problems
    sizes = point_energy_sizes(args.batch_instances)
    dev = torch.device("cuda", local)
    cfg_of = lambda n, **kw: problems.make_config(abi.SEDOV_2D, nx=n, ny=n, device=local, **kw)
    b = Batch(max_slots=len(sizes), max_nx=640, max_ny=640,
              precision=abi.PRECISION_FP32_BULK, ubar_mode=abi.UBAR_TREE, device=local)
    t_adm = time.perf_counter()
    for k, n in enumerate(sizes):
        if not b.admit(cfg_of(n), k):
            raise RuntimeError(f"instance {k} ({n}^2) not admitted")
    t_adm = time.perf_counter() - t_adm
    tile_cells = b.autotune()   # cell-tile size of the per-cell kernels for this mix
    ext = torch.cuda.ExternalStream(b.stream_ptr(), device=dev)
    b.run(args.warmup)
    before = [b.progress(k)[1] for k in range(len(sizes))]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    b.run(args.batch_steps)
    e1.record(ext)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    done = [b.progress(k)[1] - before[k] for k in range(len(sizes))]
    upd = sum(n * n * 3 * d for n, d in zip(sizes, done))
    from sweeping_fd_weno_gb300.replicas import aggregate
    value = aggregate(upd, ms * 1e-3)[2]  # every replica's instances over the slowest
    # accuracy: the smallest instances against the FP64 path after the same steps
    check = sorted(range(len(sizes)), key=lambda k: sizes[k])[:3]
    errs, full = [], {}
    for k in check:
        u32, _ = b.download(k)
        s = Solver(cfg_of(sizes[k]))
        s.init_problem()
        for _ in range(args.warmup + args.batch_steps):
            s.step()
        u64 = s.state()
        s.close()
        r32, r64 = u32[3:-3, 3:-3, 0], u64[3:-3, 3:-3, 0]
        errs.append(float(np.abs(r32 - r64).sum() / np.abs(r64).sum()))
        full[f"{sizes[k]}^2"] = precision_errors(u32, u64)
    b.close()
    # the same instances and steps in an FP64 batch (the form for problems where
    # FP32-bulk does not hold 1e-6 to the end of the run)
    b64 = Batch(max_slots=len(sizes), max_nx=640, max_ny=640, precision=abi.PRECISION_FP64,
                ubar_mode=abi.UBAR_SEQUENTIAL, device=local)
    for k, n in enumerate(sizes):
        if not b64.admit(cfg_of(n), k):
            raise RuntimeError(f"instance {k} ({n}^2) not admitted to the FP64 batch")
    tile64 = b64.autotune()
    ext64 = torch.cuda.ExternalStream(b64.stream_ptr(), device=dev)
    b64.run(args.warmup)
    before64 = [b64.progress(k)[1] for k in range(len(sizes))]
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(ext64)
    b64.run(args.batch_steps)
    f1.record(ext64)
    torch.cuda.synchronize()
    ms64 = f0.elapsed_time(f1)
    done64 = [b64.progress(k)[1] - before64[k] for k in range(len(sizes))]
    value64 = aggregate(sum(n * n * 3 * d for n, d in zip(sizes, done64)), ms64 * 1e-3)[2]
    b64.close()
    # the plain FP64 path (and the FP32 path unbatched), one instance at a time
    rng = np.random.default_rng(BATCH_SEED + 1)
    sample = [sizes[k] for k in rng.choice(len(sizes), size=args.plain_sample, replace=False)]
    plain = {}
    for name, prec in (("fp64", abi.PRECISION_FP64), ("fp32_bulk_single", abi.PRECISION_FP32_BULK)):
        tot_ms, tot_upd = 0.0, 0
        for n in sample:
            s = Solver(cfg_of(n, precision=prec))
            s.init_problem()
            s.autotune()
            se = torch.cuda.ExternalStream(s.stream_ptr(), device=dev)
            for _ in range(args.warmup):   # the same steps as the batch's timed ones
                s.step()
            torch.cuda.synchronize()
            for _ in range(args.plain_steps):
                with torch.cuda.stream(se):
                    flush.zero_()
                    a = torch.cuda.Event(enable_timing=True)
                    z = torch.cuda.Event(enable_timing=True)
                    a.record(se)
                s.step_async()
                z.record(se)
                torch.cuda.synchronize()
                s.finish()
                tot_ms += a.elapsed_time(z)
            tot_upd += n * n * 3 * args.plain_steps
            s.close()
        plain[name] = {"value": tot_upd / (tot_ms * 1e-3), "instances": len(sample),
                       "steps_each": args.plain_steps}
    return {
        "workload": f"{len(sizes)} point-energy instances, sides uniform 128..640 "
                    f"(numpy default_rng({BATCH_SEED})), [0,1.3]^2, corner E=0.244816/(dx*dy), "
                    "E=1e-12 background, CFL 0.5",
        "precision": "FP32-bulk (FP32 fluxes; FP64 pressure, RK accumulation, positivity, sweeps)",
        "cells": int(sum(n * n for n in sizes)),
        "value": value, "unit": UNIT, "ms": ms, "steps": args.batch_steps,
        "graph_launches": 1, "admission_s": t_adm, "tile_cells": tile_cells,
        "l2": "not flushed: the batch's resident state (GBs) is far above L2",
        "fp64_batch": {"value": value64, "ms": ms64, "steps": args.batch_steps,
                       "tile_cells": tile64},
        "plain_fp64_one_at_a_time": plain["fp64"],
        "fp32_bulk_one_at_a_time": plain["fp32_bulk_single"],
        "speedup_vs_plain_fp64": value / plain["fp64"]["value"],
        "fp64_batch_speedup_vs_plain_fp64": value64 / plain["fp64"]["value"],
        "rel_l1_density_err_vs_fp64": {f"{sizes[k]}^2": e for k, e in zip(check, errs)},
        "errors_vs_fp64": full,
    }


def bench_batched_full(args, local):
    """The point-energy configuration run to completion: every instance to
    T = 1 in the batched engine (graph launches of --batch-chunk steps, each
    instance retiring at its own time); wall time, whole-run cell-updates/s and
    the instances' completion times."""
    import numpy as np
    from sweeping_fd_weno_gb300 import Batch, abi, problems
    sizes = point_energy_sizes(args.batch_instances)
    b = Batch(max_slots=len(sizes), max_nx=640, max_ny=640,
              precision=abi.PRECISION_FP32_BULK, ubar_mode=abi.UBAR_TREE, device=local)
    for k, n in enumerate(sizes):
        if not b.admit(problems.make_config(abi.SEDOV_2D, nx=n, ny=n, device=local), k):
            raise RuntimeError(f"instance {k} not admitted")
    t0 = time.perf_counter()
    done, steps_of, status = {}, {}, {}
    launches = 0
    while len(done) < len(sizes):
        b.run(args.batch_chunk)
        launches += 1
        for rid, st in b.poll():
            done[rid] = time.perf_counter() - t0
            steps_of[rid] = b.progress(rid)[1]
            status[rid] = st
        if time.perf_counter() - t0 > args.batch_full_timeout:
            break
    wall = time.perf_counter() - t0
    upd = sum(sizes[k] ** 2 * 3 * steps_of[k] for k in done)
    b.close()
    t = np.array(sorted(done.values()))
    return {"workload": f"{len(sizes)} point-energy instances 128^2..640^2 to T=1, FP32-bulk",
            "finished": len(done), "failed": sum(1 for v in status.values() if v != 0),
            "wall_s": wall, "cell_updates": upd, "value": upd / wall, "unit": UNIT,
            "graph_launches": launches, "steps_per_launch": args.batch_chunk,
            "steps_min_max": [min(steps_of.values()), max(steps_of.values())] if steps_of else None,
            "completion_p50_s": float(np.percentile(t, 50)) if len(t) else None,
            "completion_p99_s": float(np.percentile(t, 99)) if len(t) else None}


def bench_accuracy(args, local):
    """The vortex accuracy table: the near-vacuum vortex at 45^2..360^2 to
    T = 0.01 in plain FP64 and in FP32-bulk on the GPU, with the L1 and Linf
    density errors against the exact translated solution and the observed
    orders between successive grids (the methodology of
    ex3_vortex_accuracy_2d/main.f90:725-777), and the FP32-bulk state's errors
    against the FP64 state at T."""
    import math
    import torch
    from sweeping_fd_weno_gb300 import Solver, abi, output, problems
    rows, prev = [], {}
    for n in args.accuracy_sizes:
        row, states = {"n": n}, {}
        for name, prec in (("fp64", abi.PRECISION_FP64), ("fp32_bulk", abi.PRECISION_FP32_BULK)):
            s = Solver(problems.workload(f"vortex{n}", device=local, precision=prec))
            s.init_problem()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            steps = s.run()
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            u, t = s.state(), s.time
            s.close()
            l1, linf = output.vortex_errors(u, t)
            r = {"steps": steps, "t": t, "l1": l1, "linf": linf, "gpu_s": wall}
            if name in prev:
                pn, pl1, plinf = prev[name]
                r["order_l1"] = math.log(pl1 / l1) / math.log(n / pn)
                r["order_linf"] = math.log(plinf / linf) / math.log(n / pn)
            prev[name] = (n, l1, linf)
            states[name] = u
            row[name] = r
        row["fp32_bulk_vs_fp64"] = precision_errors(states["fp32_bulk"], states["fp64"])
        rows.append(row)
    return {"workload": "near-vacuum vortex (eps 10.0828, min density ~7.8e-15), periodic "
                        "[0,10]^2, mean flow (1,1), T=0.01, dt = dx^(5/3)*0.5/alpha",
            "errors": "density against the exact translated vortex at the final time: L1 the "
                      "mean absolute error, Linf the maximum; orders log(e_coarse/e_fine) / "
                      "log(n_fine/n_coarse)",
            "table": rows}


def bench_sedov_precision(args, local):
    """The FP32-bulk batch's error at a late time: a seeded sample of the
    point-energy instances (the 640^2 one included) is run to T = 1 in the
    FP32-bulk batch to learn each instance's step count; then every instance
    runs to the common time T_s by which all of them have taken at least a
    quarter of those steps, in the FP32-bulk batch and in plain FP64 one at a
    time (the oracle's arithmetic), and the FP32-bulk states are compared with
    the FP64 ones (L1/Linf density and pressure, mass and energy drift)."""
    import numpy as np
    import torch
    from sweeping_fd_weno_gb300 import Batch, Solver, abi, problems
    sizes = point_energy_sizes(args.batch_instances)
    rng = np.random.default_rng(BATCH_SEED + 2)
    pick = [int(n) for n in rng.choice(sorted(set(sizes) - {640}), size=args.late_sample - 1,
                                       replace=False)] + [640]
    cfg_of = lambda n, **kw: problems.make_config(abi.SEDOV_2D, nx=n, ny=n, device=local, **kw)
    # 1. step counts to T = 1 in the FP32-bulk batch, with (time, steps) samples
    t0 = time.perf_counter()
    hist = {k: [(0.0, 0)] for k in range(len(pick))}
    with Batch(max_slots=len(pick), max_nx=640, max_ny=640, precision=abi.PRECISION_FP32_BULK,
               ubar_mode=abi.UBAR_TREE, device=local) as b:
        for k, n in enumerate(pick):
            assert b.admit(cfg_of(n), k)
        done = set()
        while len(done) < len(pick):
            b.run(args.batch_chunk)
            for k in range(len(pick)):
                if k not in done:
                    hist[k].append(b.progress(k))
            for rid, st in b.poll():
                if st != 0:
                    raise RuntimeError(f"instance {pick[rid]}^2 failed with status {st}")
                done.add(rid)
    steps_t1 = [hist[k][-1][1] for k in range(len(pick))]
    t_quarter = [next(t for t, st in hist[k] if st >= 0.25 * steps_t1[k])
                 for k in range(len(pick))]
    ts = float(f"{max(t_quarter):.2g}")
    if any(next(st for t, st in hist[k] if t >= ts) < 0.25 * steps_t1[k] for k in range(len(pick))):
        ts = float(f"{max(t_quarter):.3g}")
    find_s = time.perf_counter() - t0
    # 2. every instance to T_s: FP32-bulk batch and plain FP64 one at a time
    t1 = time.perf_counter()
    u32 = {}
    with Batch(max_slots=len(pick), max_nx=640, max_ny=640, precision=abi.PRECISION_FP32_BULK,
               ubar_mode=abi.UBAR_TREE, device=local) as b:
        for k, n in enumerate(pick):
            assert b.admit(cfg_of(n, time_terminal=ts), k)
        left = set(range(len(pick)))
        while left:
            b.run(args.batch_chunk)
            for rid, st in b.poll():
                if st != 0:
                    raise RuntimeError(f"instance {pick[rid]}^2 failed with status {st}")
                u32[rid] = (b.download(rid)[0], b.progress(rid)[1], b.stats(rid))
                left.discard(rid)
    fp32_s = time.perf_counter() - t1
    # 3. the FP32-bulk and FP64 single-instance solves side by side through the
    # checkpoints 0.02, 0.05 and T_s (each segment ends on its checkpoint with
    # a clamped step, the same in both forms): the error as the run goes on
    checks = [t for t in (0.02, 0.05) if t < ts] + [ts]
    out = {}
    t2 = time.perf_counter()
    for k, n in enumerate(pick):
        st = {p_: None for p_ in ("fp32", "fp64")}
        t_prev, errs = 0.0, {}
        for tc in checks:
            states = {}
            for name, prec in (("fp32", abi.PRECISION_FP32_BULK), ("fp64", abi.PRECISION_FP64)):
                with Solver(cfg_of(n, time_terminal=tc, precision=prec)) as s:
                    if st[name] is None:
                        s.init_problem()
                    else:
                        s.set_state(st[name])
                        s.time = t_prev
                    s.run()
                    st[name] = s.state()
                    states[name] = st[name]
            errs[f"T={tc:g}"] = precision_errors(states["fp32"], states["fp64"])["rel_l1_density"]
            t_prev = tc
        ua, steps32, st32 = u32[k]
        e = precision_errors(ua, st["fp64"])
        e.update({"steps_to_T1_fp32": steps_t1[k], "steps_to_Ts_fp32_batch": steps32,
                  "quarter_reached_at": t_quarter[k], "sweeps_fp32_batch": st32["sweep_count"],
                  "rel_l1_density_single_fp32_at": errs})
        out[f"{n}^2"] = e
    fp64_s = time.perf_counter() - t2
    worst = max(v["rel_l1_density"] for v in out.values())
    worst_at = {f"T={tc:g}": max(v["rel_l1_density_single_fp32_at"][f"T={tc:g}"]
                                 for v in out.values()) for tc in checks}
    return {"workload": f"{len(pick)} of the point-energy instances (seeded sample, 640^2 "
                        "included) to a common late time",
            "T_s": ts, "instances": out, "worst_rel_l1_density": worst,
            "worst_rel_l1_density_at": worst_at,
            "accepted_at_1e-6": bool(worst < 1e-6),
            "fp32": "FP32-bulk batch (tree u_bar) for the T_s comparison; FP32-bulk single "
                    "instances (sequential u_bar) for the checkpoints",
            "fp64": "plain FP64, one at a time (sequential u_bar: the oracle's arithmetic)",
            "seconds": {"steps_to_T1": find_s, "fp32_batch_to_Ts": fp32_s,
                        "single_checkpoints": fp64_s}}


def profile_jet(args, local):
    """Launch-list mode for the sweep-heavy jet: the 800x200 jet advances
    --profile-after steps as graphs, its state moves to a solver that runs its
    sections as plain stream launches (SWFD_LAUNCH=eager: the same kernels and
    arguments, conditions read on the host; profilers see every kernel), and
    --profile-steps steps run between cudaProfilerStart and cudaProfilerStop.
    Under `ncu --profile-from-start off` only those steps' launches are
    captured.  Prints one JSON line describing the window."""
    import torch
    from sweeping_fd_weno_gb300 import Solver, problems
    torch.cuda.set_device(local)
    with Solver(problems.workload("jet", device=local)) as g:
        g.init_problem()
        g.run(args.profile_after)
        u, t, n0 = g.state(), g.time, g.stats()
    prev = os.environ.get("SWFD_LAUNCH")
    os.environ["SWFD_LAUNCH"] = "eager"
    try:
        e = Solver(problems.workload("jet", device=local))
    finally:
        if prev is None:
            del os.environ["SWFD_LAUNCH"]
        else:
            os.environ["SWFD_LAUNCH"] = prev
    with e:
        e.set_state(u)
        e.time = t
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        t0 = time.perf_counter()
        for _ in range(args.profile_steps):
            e.step()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        torch.cuda.profiler.stop()
        st = e.stats()
    print(json.dumps({"mode": "profile_jet", "after_steps": args.profile_after,
                      "steps": args.profile_steps, "wall_ms_per_step_eager":
                      wall * 1e3 / args.profile_steps, "sweeps": st["sweep_count"],
                      "sweep_pairs": st["pre_count"], "max_neg": st["max_neg"],
                      "time_at_start": t, "stats_before": n0}))
    return 0


def serving_draw(device, plain_fp64=False):
    """Requests of the serving mix, drawn uniformly from three problems: the
    vortex (45^2..360^2, T=0.01), a point-energy instance (128^2..640^2,
    shortened to T=0.02) and the Mach 5.09 shock diffraction (total 20..80:
    260x216..1040x880, shortened to T=0.05).  The first two run in FP32-bulk
    (accepted: relative L1 density error < 1e-6), the shock in FP64; with
    plain_fp64 every request is FP64."""
    from sweeping_fd_weno_gb300 import abi, problems
    from sweeping_fd_weno_gb300.serving import fp32_accepted

    def draw(rng):
        kind = int(rng.integers(0, 3))
        if kind == 0:
            n = int(rng.choice([45, 90, 180, 360]))
            c = problems.make_config(abi.VORTEX_2D, nx=n, ny=n, device=device)
        elif kind == 1:
            n = int(rng.integers(128, 641))
            c = problems.make_config(abi.SEDOV_2D, nx=n, ny=n, time_terminal=0.02, device=device)
        else:
            total = int(rng.choice([20, 40, 60, 80]))
            c = problems.make_config(abi.SHOCK_DIFFRACTION, total=total, time_terminal=0.05,
                                     device=device)
        c.precision = (abi.PRECISION_FP32_BULK if fp32_accepted(c) and not plain_fp64
                       else abi.PRECISION_FP64)
        return c
    return draw


def bench_point_energy_1d(args, local):
    """The reference's CPU-runnable case (1D point energy, 800 cells on [-2,2],
    E=1e-12 background, CFL 0.6, swp_num 2, T = 0.001): the whole run on the
    GPU (the time loop on the device, one solve graph) next to the oracle on
    one host core -- a CPU baseline leg -- and the MATLAB script of ex1 (its
    double rarefaction as shipped) on the GPU."""
    import numpy as np
    import oracle
    import torch
    from sweeping_fd_weno_gb300 import Solver, abi, problems
    out = {}
    for name, cfg in (("point_energy_1d", problems.workload("sedov1d_fp64", device=local)),
                      ("matlab_double_rarefaction",
                       problems.make_config(abi.MATLAB_1D, device=local,
                                            **problems.matlab_problem(5)))):
        s = Solver(cfg)
        s.init_problem()
        s.run(3)                      # captures the solve graph
        s.init_problem()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n = s.run()
        torch.cuda.synchronize()
        gpu_s = time.perf_counter() - t0
        u = s.state()
        s.close()
        o = oracle.Oracle(cfg)
        o.init_problem()
        t0 = time.perf_counter()
        n_o = o.run()
        cpu_s = time.perf_counter() - t0
        out[name] = {"cells": int(cfg.nx), "steps": int(n), "t_end": float(cfg.time_terminal),
                     "gpu_s": gpu_s, "gpu_us_per_step": gpu_s / n * 1e6,
                     "cpu_oracle_s": cpu_s, "cpu_cores": 1,
                     "same_result": bool(n == n_o and np.array_equal(u, o.state())),
                     "speedup_vs_cpu": cpu_s / gpu_s}
    return out


def bench_jet(args, local):
    """The high-speed jet of ex5 (gamma 5/3, 800x200 half domain with the y=0
    symmetry plane, u=800 inflow, T=0.001), plain FP64 only: the whole solve
    to T as one graph (device-side loop over steps, sweeps as conditional
    nodes), wall clock with a device synchronize on both sides, with the
    sweep and adjustment counts it printed; the oracle on one host core for a
    bounded sample of the leading steps, with a value-for-value check."""
    import numpy as np
    import oracle
    import torch
    from sweeping_fd_weno_gb300 import Solver, problems
    cfg = problems.workload("jet", device=local)
    cells = cfg.nx * cfg.ny
    w = Solver(cfg)                       # warm-up: the same graph shape, a few steps
    w.init_problem()
    w.run(max(1, args.warmup))
    w.close()
    s = Solver(cfg)
    s.init_problem()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps = s.run()
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    st, t_end = s.stats(), s.time
    s.close()
    # where a sweeping step's time goes: 20 steps after the first 1000 (the
    # sweep runs in almost every stage by then), the flux launches bracketed
    # by the handle's CUDA events; step() adds one host round trip per step
    q = Solver(cfg)
    q.init_problem()
    q.run(1000)
    q.set_profiling(True)
    q.step()  # untimed: captures the step graph with the flux events
    q.reset_profile()
    sweeps0 = q.stats()["sweep_count"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(20):
        q.step()
    torch.cuda.synchronize()
    prof_s = time.perf_counter() - t0
    pr = q.profile()
    split = {"after_steps": 1001, "steps": 20, "wall_ms_per_step": prof_s / 20 * 1e3,
             "flux_ms_per_step": pr["flux_ms"] / 20,
             "sweeps": int(q.stats()["sweep_count"] - sweeps0)}
    q.close()
    sample = max(1, args.jet_sample)
    g = Solver(cfg)
    g.init_problem()
    o = oracle.Oracle(cfg)
    o.init_problem()
    t0 = time.perf_counter()
    for _ in range(sample):
        o.step()
    cpu_s = time.perf_counter() - t0
    for _ in range(sample):
        g.step()
    same = bool(np.array_equal(g.state(), o.state()) and g.time == o.time
                and g.stats() == o.stats())
    g.close()
    gpu_rate = cells * 3 * steps / gpu_s
    cpu_rate = cells * 3 * sample / cpu_s
    return {"workload": "jet: ex5 high-speed jet, gamma 5/3, 800x200 half domain, u=800 "
                        "inflow, T=0.001, plain FP64 with the sweeping limiter",
            "cells": int(cells), "steps": int(steps), "t_end": t_end, "gpu_s": gpu_s,
            "gpu_ms_per_step": gpu_s / max(steps, 1) * 1e3,
            "value": gpu_rate, "unit": "cell-updates/s",
            "sweeps": {k: int(v) for k, v in st.items()},
            "cpu_oracle": {"value": cpu_rate, "cores": 1, "steps": int(sample),
                           "s": cpu_s, "kind": "port"},
            "speedup_vs_cpu": gpu_rate / cpu_rate, "same_result_after_sample": same,
            "step_split": split,
            "cpu_sample_note": "the oracle's sample is the leading steps, which run no "
                               "sweep; the solve sweeps in most later stages, so the "
                               "ratio understates the speed-up over a full CPU solve",
            "timing": "wall clock around the whole-solve graph launch with a device "
                      "synchronize on both sides"}


def bench_detonation(args, local):
    """The reactive Euler detonation of ex7 at the reference's size (400x400 on
    its 4 x 8 ranks): each GPU step one graph launch (the sweep decisions and
    its pass loop are conditional nodes) and one read-back of the scalars,
    and the oracle on one host core for a bounded sample of the same steps,
    with a value-for-value check of the state after them."""
    import numpy as np
    import oracle
    import torch
    from sweeping_fd_weno_gb300 import Solver, problems
    cfg = problems.workload("detonation80", device=local)
    cells = cfg.nx * cfg.ny
    s = Solver(cfg)
    s.init_problem()
    for _ in range(args.warmup):
        s.step()
    s.init_problem()
    steps = max(args.steps, 10)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        s.step()
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    st = s.stats()
    # the oracle: a bounded sample of the first steps, same result checked
    sample = max(1, min(steps, args.detonation_sample))
    g = Solver(cfg)
    g.init_problem()
    o = oracle.Oracle(cfg)
    o.init_problem()
    t0 = time.perf_counter()
    for _ in range(sample):
        o.step()
    cpu_s = time.perf_counter() - t0
    for _ in range(sample):
        g.step()
    same = bool(np.array_equal(g.state(), o.state()) and g.time == o.time)
    g.close()
    s.close()
    gpu_rate = cells * 3 * steps / gpu_s
    cpu_rate = cells * 3 * sample / cpu_s
    return {"workload": "detonation80: ex7 reactive Euler, 400x400 on 4 x 8 ranks, five "
                        "components, sweeping limiter",
            "cells": int(cells), "steps": int(steps), "gpu_ms_per_step": gpu_s / steps * 1e3,
            "value": gpu_rate, "unit": "cell-updates/s",
            "sweeps": {k: int(v) for k, v in st.items()},
            "cpu_oracle": {"value": cpu_rate, "cores": 1, "steps": int(sample),
                           "s": cpu_s, "kind": "port"},
            "speedup_vs_cpu": gpu_rate / cpu_rate, "same_result_after_sample": same,
            "timing": "wall clock around the steps with a device synchronize on both sides "
                      "(each step one graph launch with device-side sweep control and one "
                      "read-back of the scalars)"}


def bench_serving(args, local):
    """Poisson arrivals (mean 50 req/s) served by continuous batching (an
    FP32-bulk batch and an FP64 batch side by side) and, for comparison, one
    at a time by the plain FP64 path."""
    from sweeping_fd_weno_gb300 import Batch, abi
    from sweeping_fd_weno_gb300.serving import (poisson_arrivals, serve_batched,
                                                serve_one_at_a_time)
    arr = poisson_arrivals(args.serve_rate, args.serve_requests, SERVE_SEED,
                           serving_draw(local))
    with Batch(max_slots=args.serve_slots, max_nx=640, max_ny=640,
               precision=abi.PRECISION_FP32_BULK, ubar_mode=abi.UBAR_TREE, device=local) as b32, \
            Batch(max_slots=max(4, args.serve_slots // 4), max_nx=1040, max_ny=880,
                  precision=abi.PRECISION_FP64, ubar_mode=abi.UBAR_SEQUENTIAL,
                  device=local) as b64:
        rb = serve_batched(arr, [b32, b64], step_chunk=args.serve_chunk)
    # the same stream (same seed: same arrivals and requests) in plain FP64
    plain = poisson_arrivals(args.serve_rate, args.serve_requests, SERVE_SEED,
                             serving_draw(local, plain_fp64=True))
    rp = serve_one_at_a_time(plain)
    sb, sp = rb.summary(), rp.summary()
    # the same kind of stream through the C host request loop over the batch
    # C-ABI (host/swfd_serve.c, its own seeded draw of the same mix)
    c_host = None
    serve = ROOT / "sweeping_fd_weno_gb300" / "_lib" / "swfd_serve"
    if serve.exists():
        r = subprocess.run([str(serve), "--requests", str(args.serve_requests), "--rate",
                            str(args.serve_rate), "--seed", str(SERVE_SEED), "--slots",
                            str(args.serve_slots), "--chunk", str(args.serve_chunk),
                            "--check", "4", "--device", str(local)],
                           capture_output=True, text=True, timeout=900)
        if r.returncode == 0:
            c_host = json.loads(r.stdout.strip().splitlines()[-1])
        else:
            c_host = {"error": r.stderr.strip()[-300:]}
    kinds = {}
    for _, c in arr:
        kinds[int(c.problem)] = kinds.get(int(c.problem), 0) + 1
    return {
        "workload": f"{len(arr)} requests, Poisson arrivals mean {args.serve_rate:g}/s "
                    f"(numpy default_rng({SERVE_SEED})), uniformly: vortex 45^2..360^2 to "
                    "T=0.01, point energy 128^2..640^2 to T=0.02, shock diffraction total "
                    "20..80 to T=0.05",
        "requests_by_problem": {"vortex": kinds.get(3, 0), "point_energy": kinds.get(4, 0),
                                "shock_diffraction": kinds.get(6, 0)},
        "precision": "FP32-bulk batch (vortex; point energy to T <= 0.05) beside an FP64 "
                     "batch (shock diffraction: FP32 error 1e-3 fails the 1e-6 bar)",
        "batched": sb, "plain_fp64_one_at_a_time": sp,
        "throughput_ratio": (sb["value"] / sp["value"]) if sp["value"] else None,
        "slots": args.serve_slots, "step_chunk": args.serve_chunk,
        "c_host_loop": c_host,
    }


def _reference_worker(args):
    """One serial solve of the reference's algorithm (a worker of the reference
    arm): warm-up steps, then the timed steps."""
    n, warmup, steps, literals = args
    import oracle
    from sweeping_fd_weno_gb300 import problems
    o = oracle.Oracle(problems.workload(f"vortex{n}", literals=literals))
    o.init_problem()
    for _ in range(warmup):
        o.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    return n * n * 3 * steps, time.perf_counter() - t0


# the workload description both arms print (the driver pairs the lines on it)
L2_NOTE = ("GPU arm: L2 flushed between timed steps (256 MiB write); CPU arm: each core's "
           "solve resident in its own caches and DRAM")


def bench_config(workload, precision, nx, ny, n_gpus):
    return {"workload": f"{workload}_{precision}", "nx": nx, "ny": ny, "stages_per_step": 3,
            "precision": "plain FP64 (double literals)" if precision == "fp64"
            else "FP32-bulk (FP32 fluxes; FP64 pressure, RK accumulation, sweeps)",
            "l2": L2_NOTE,
            "parallelism": f"GPU arm: replicas x{n_gpus} (one grid per GPU); CPU arm: one solve "
                           "per host core"}


def reference_pool(n, warmup, steps, literals, cores):
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(cores) as pool:
        out = pool.map(_reference_worker, [(n, warmup, steps, literals)] * cores)
    return sum(u for u, _ in out), max(t for _, t in out)


def run_reference(args, rank):
    """The reference's algorithm on the host CPU: its CPU restatement (the
    oracle) on the GPU line's workload -- the 360x360 vortex with binary64
    literals, the GPU line's arithmetic -- with every host core running its
    own solve (the reference's vortex program is serial); the value is all
    cores' updates over the slowest core's timed steps.  Beside it, the
    binary128-literal pair: the same grid in the arithmetic of the reference's
    -fdefault-real-8 build, against which the GPU line's quad_literals leg
    compares."""
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    n = args.reference_nx or int(args.workload[len("vortex"):] or 180)
    cores = os.cpu_count() or 1
    upd, el = reference_pool(n, args.warmup, args.steps, 0, cores)
    v = upd / el
    qsteps = max(1, args.reference_quad_steps)
    qupd, qel = reference_pool(n, 0, qsteps, 1, cores)
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: ex3 initdata of the near-vacuum isentropic vortex (no dataset)",
        "config": bench_config(args.workload, "fp64", n, n, args.gpus),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} SSP-RK3 steps (after {args.warmup} untimed) of "
                                   f"the {n}x{n} vortex per core, {cores} independent solves, "
                                   "binary64 literals (the GPU line's arithmetic); the reference "
                                   "itself is serial Fortran and no Fortran compiler exists "
                                   "here or on the GPU box"},
        "quad_literals": {"value": qupd / qel, "unit": UNIT, "cores": cores, "kind": "port",
                          "ms_per_step": qel * 1e3 / qsteps,
                          "sample": f"{qsteps} SSP-RK3 step(s) of the {n}x{n} vortex per core, "
                                    "binary128 literals (the reference's -fdefault-real-8 "
                                    "build); pairs with the GPU line's quad_literals leg"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="vortex360")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32_bulk"],
                    help="arithmetic of the main measurement (the headline is fp64)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--reference-nx", type=int, default=0,
                    help="grid of the reference arm (default: the workload's own)")
    ap.add_argument("--reference-quad-steps", type=int, default=1,
                    help="binary128-literal steps per core of the reference arm (~4 s each)")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-quad", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-detonation", action="store_true")
    ap.add_argument("--detonation-sample", type=int, default=2,
                    help="oracle steps of the detonation leg (about 1.5 s each)")
    ap.add_argument("--no-jet", action="store_true")
    ap.add_argument("--jet-sample", type=int, default=3,
                    help="oracle steps of the jet leg (about 0.3 s each)")
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--plain-sample", type=int, default=8)
    ap.add_argument("--plain-steps", type=int, default=10)
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-slots", type=int, default=64)
    ap.add_argument("--serve-chunk", type=int, default=4)
    ap.add_argument("--profile-jet", action="store_true",
                    help="launch-list mode: jet steps as plain launches inside a profiler range")
    ap.add_argument("--profile-after", type=int, default=1000)
    ap.add_argument("--profile-steps", type=int, default=20)
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--accuracy-sizes", type=int, nargs="+", default=[45, 90, 180, 360])
    ap.add_argument("--no-late-precision", action="store_true")
    ap.add_argument("--late-sample", type=int, default=8,
                    help="point-energy instances of the late-time FP32-bulk error sample")
    ap.add_argument("--batch-full", action="store_true",
                    help="also run the point-energy batch to T=1 (minutes)")
    ap.add_argument("--batch-chunk", type=int, default=64)
    ap.add_argument("--batch-full-timeout", type=float, default=1800.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.profile_jet:
        return profile_jet(args, local)

    import numpy as np
    import torch
    from sweeping_fd_weno_gb300 import Solver, abi, problems

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    main_prec = abi.PRECISION_FP64 if args.precision == "fp64" else abi.PRECISION_FP32_BULK
    cfg = problems.workload(args.workload, device=local, precision=main_prec)
    solver = Solver(cfg)
    solver.init_problem()
    flux_min_blocks = solver.autotune()  # launch shape of the flux kernel on this state
    cells = solver.nx * solver.ny
    ext = torch.cuda.ExternalStream(solver.stream_ptr(), device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    # profiling on from the warm-up: the step graph with the flux events is
    # captured before the timed steps
    solver.set_profiling(True)
    for _ in range(args.warmup):
        solver.step()

    solver.reset_profile()
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = []
    # steps are enqueued without a host round trip (step_async), so each
    # event pair brackets one step graph on the device; finish() then waits
    # and reports their status
    for _ in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()  # evict L2 (129 MB) between timed steps
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
        solver.step_async()
        e1.record(ext)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    solver.finish()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in evs)
    prof = solver.profile()
    solver.set_profiling(False)
    # whole job: every replica's updates over the slowest replica's time
    from sweeping_fd_weno_gb300.replicas import aggregate
    updates, max_s, value = aggregate(cells * 3 * args.steps, total_ms * 1e-3)
    total_ms = max_s * 1e3

    # end to end through the public API with host buffers: upload the step's
    # input from pinned memory, step, read the result back
    host = torch.empty(int(np.prod(solver.shape)), dtype=torch.float64).pin_memory()
    hu = host.numpy().reshape(solver.shape)
    solver.state(out=hu)
    solver.step_host(hu)  # untimed: captures the step graph of this (unprofiled) setting
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        solver.step_host(hu)  # upload, step, download: one synchronisation
    e2e_s = time.perf_counter() - t0
    _, e2e_s, e2e_value = aggregate(cells * 3 * args.e2e_steps, e2e_s)
    state_bytes = int(np.prod(solver.shape)) * 8
    e2e = {"value": e2e_value, "unit": UNIT,
           "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes,
           "steps": args.e2e_steps, "call": "swfd_step_host (pinned host state in and out)"}

    # dominant kernel: the WENO flux kernel (one launch per stage, both directions)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    import ctypes as C
    fp64 = C.c_double(0.0)
    abi.load_probe().swfd_probe_fp64_peak(local, C.byref(fp64))
    flux_ms_per_launch = prof["flux_ms"] / max(prof["flux_launches"], 1)
    # per launch (both directions of one stage): read the split fluxes (8
    # doubles) and Roe averages (4 doubles) of every cell once per direction,
    # write 8 doubles per interface
    f32 = args.precision != "fp64"
    fused32 = f32 and os.environ.get("SWFD_FP32_STAGE") != "split"
    launch_bytes = (cells * STAGE32_BYTES_PER_CELL if fused32
                    else 2 * cells * (12 + 8) * (4.0 if f32 else 8.0))
    achieved = launch_bytes / (flux_ms_per_launch * 1e-3) / 1e9
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": achieved / hbm_peak,
        "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
        "launch_ms": flux_ms_per_launch,
        "stage_hbm": {"achieved": STAGE_BYTES_PER_CELL * value / 1e9, "peak": hbm_peak,
                      "frac": STAGE_BYTES_PER_CELL * value / 1e9 / hbm_peak,
                      "bytes_per_cell_stage": STAGE_BYTES_PER_CELL},
    }
    if not f32:
        launch_inst = 2 * cells * FLUX_FP64_INST_PER_INTERFACE
        fp64_inst_rate = launch_inst / (flux_ms_per_launch * 1e-3) / 1e9
        fp64_peak_inst = fp64.value / 2.0  # the probe counts a DFMA as 2 flops
        roofline.update({
            "traffic": FLUX_DRAM_BYTES_PER_CELL * cells,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                              "k_flux_xy_share<5> on the 1024x1024 vortex (313.9 MB), scaled "
                              "per cell to this grid",
            "kernel": "k_flux_xy_share<5> (characteristic WENO5 interface fluxes, both "
                      "directions in one code path, two lanes per interface, the fields "
                      "in a loop, each interface's eigenvectors formed once; the default "
                      "FP64 shape)",
            "compute_bound": "fp64 (the FP64 pipe; divisions and power-of-two products run "
                             "on the integer pipes)",
            "fp64": {"achieved_ginst_per_s": fp64_inst_rate, "peak_ginst_per_s": fp64_peak_inst,
                     "frac": fp64_inst_rate / fp64_peak_inst if fp64_peak_inst else None,
                     "peak_source": "measured by swfd_probe_fp64_peak (DFMA chains; 2 flops "
                                    "each)",
                     "inst_per_interface": FLUX_FP64_INST_PER_INTERFACE,
                     "inst_per_interface_executed": FLUX_FP64_INST_PER_INTERFACE_EXECUTED,
                     # the all-hardware instruction stream of the same arithmetic
                     # (hardware divisions) over the measured time: above 1.0 means
                     # faster than that stream could run at the FP64 peak
                     "hw_division_equivalent_frac":
                         2 * cells * FLUX_FP64_INST_PER_INTERFACE_HW_DIV
                         / (flux_ms_per_launch * 1e-3) / 1e9 / fp64_peak_inst
                         if fp64_peak_inst else None,
                     "hw_division_inst_per_interface": FLUX_FP64_INST_PER_INTERFACE_HW_DIV,
                     "achieved_gflops_source_count": 2 * cells * FLUX_FLOPS_PER_INTERFACE
                     / (flux_ms_per_launch * 1e-3) / 1e9,
                     "flops_per_interface": FLUX_FLOPS_PER_INTERFACE}})
    elif fused32:
        roofline.update({
            "traffic": STAGE32_DRAM_BYTES_PER_CELL * cells,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                              "k_stage32<256, 4> on the 1024x1024 vortex (107.9 MB), scaled "
                              "per cell to this grid",
            "kernel": "k_stage32<256, 4> (the fused FP32-bulk stage: split fluxes in shared "
                      "memory, interface fluxes, RHS, RK combination, positivity)",
            "compute_bound": "issue (ncu on the 1024x1024 vortex: 68 % issue active, FMA "
                             "pipe 36 %, FP64 pipe 33 %, DRAM 10 %)"})
    else:
        roofline.update({
            "traffic": FLUX_F32_DRAM_BYTES_PER_CELL * cells,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                              "k_flux_xy<float> on the 1024x1024 vortex (134.4 MB), scaled "
                              "per cell to this grid",
            "kernel": "k_flux_xy<float> (characteristic WENO5 interface fluxes, both directions)",
            "compute_bound": "none: latency-bound (ncu on the 1024x1024 vortex: FMA pipe "
                             "35 %, DRAM 9 %, issue 55 % active, long-scoreboard stalls)"})
    # the FP32-bulk precision form on the same workload, from the same state:
    # timed the same way, with its relative L1 density error against FP64
    fp32 = None
    if not args.no_fp32:
        u_start = np.empty(solver.shape)
        s64 = Solver(problems.workload(args.workload, device=local))
        s32 = Solver(problems.workload(args.workload, device=local,
                                       precision=abi.PRECISION_FP32_BULK))
        s64.init_problem()
        s32.init_problem()
        ext32 = torch.cuda.ExternalStream(s32.stream_ptr(), device=torch.device("cuda", local))
        for _ in range(args.warmup):
            s32.step()
        s32.set_state(s64.state(out=u_start))
        s32.time = s64.time
        minb32 = s32.autotune()
        torch.cuda.synchronize()
        ev32 = []
        for _ in range(args.steps):
            with torch.cuda.stream(ext32):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(ext32)
            s32.step_async()
            b.record(ext32)
            ev32.append((a, b))
        torch.cuda.synchronize()
        s32.finish()
        ms32 = sum(a.elapsed_time(b) for a, b in ev32)
        for _ in range(args.steps):
            s64.step()
        u64f, u32f = s64.state(), s32.state()
        r64, r32 = u64f[3:-3, 3:-3, 0], u32f[3:-3, 3:-3, 0]
        fp32 = {"value": aggregate(cells * 3 * args.steps, ms32 * 1e-3)[2],
                "ms_per_step": ms32 / args.steps,
                "speedup_vs_fp64": total_ms / ms32 if ms32 else None,
                "flux_min_blocks": minb32,
                "stage_kernels": ("split: findalpha, splitting, fluxes, RK + positivity, bc"
                                  if os.environ.get("SWFD_FP32_STAGE") == "split" else
                                  "fused: [bc +] findalpha + splitting terms, then one tile "
                                  "kernel for split fluxes, interface fluxes, RHS, RK and "
                                  "positivity"),
                "rel_l1_density_err_vs_fp64": float(np.abs(r32 - r64).sum() / np.abs(r64).sum()),
                "errors_vs_fp64": precision_errors(u32f, u64f),
                "arithmetic": "FP32 LF splitting, WENO5 fluxes and flux differences; FP64 pressure "
                              "recovery, RK accumulation, positivity, CFL reduction and sweeps"}
        s32.close()
        s64.close()
    # the reference build's own arithmetic (literals = QUAD: its binary128
    # subexpressions in software on the GPU), same workload, timed the same way
    quad = None
    if args.precision == "fp64" and not args.no_quad:
        sq_ = Solver(problems.workload(args.workload, device=local, literals=abi.LITERALS_QUAD))
        sd_ = Solver(problems.workload(args.workload, device=local))
        for s_ in (sq_, sd_):
            s_.init_problem()
        extq = torch.cuda.ExternalStream(sq_.stream_ptr(), device=torch.device("cuda", local))
        sq_.step()                            # captures the step graph
        sq_.init_problem()
        nq = max(1, min(args.steps, 3))
        torch.cuda.synchronize()
        evq = []
        for _ in range(nq):
            with torch.cuda.stream(extq):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(extq)
            sq_.step_async()
            b.record(extq)
            evq.append((a, b))
        torch.cuda.synchronize()
        sq_.finish()
        msq = sum(a.elapsed_time(b) for a, b in evq)
        for _ in range(nq):
            sd_.step()
        uq, ud = sq_.state(), sd_.state()
        quad = {"value": aggregate(cells * 3 * nq, msq * 1e-3)[2], "ms_per_step": msq / nq,
                "steps": nq, "slowdown_vs_fp64": (msq / nq) / (total_ms / args.steps),
                "max_rel_diff_vs_double_literals": float(np.max(np.abs(uq - ud)) /
                                                         np.max(np.abs(ud))),
                "arithmetic": "the reference's -fdefault-real-8 build: its double-kind "
                              "literals' subexpressions in binary128 (software, integer pipes), "
                              "the rest FP64"}
        sq_.close()
        sd_.close()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic: ex3 initdata of the near-vacuum isentropic vortex (no dataset)",
        "config": bench_config(args.workload, args.precision, solver.nx, solver.ny, world),
        "tuning": {"flux_min_blocks": flux_min_blocks},
        "clocks": clk,
        "e2e": e2e,
        "gpu_launches": prof["kernel_launches"],
        "roofline": roofline,
        "sweep": {"invocations": prof["sweep_invocations"], "ms": prof["sweep_ms"]},
        "fp32_bulk": fp32,
        "quad_literals": quad,
    }
    if not args.no_batched:
        line["batched"] = bench_batched(args, local, flush)
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            line["batched"]["cpu_baseline"] = cpu_batched_baseline(
                point_energy_sizes(args.batch_instances))
    if not args.no_serving:
        line["serving"] = bench_serving(args, local)
    if not args.no_accuracy:
        line["accuracy"] = bench_accuracy(args, local)
    if not args.no_late_precision:
        line["late_precision"] = bench_sedov_precision(args, local)
    if args.batch_full:
        line["batched_to_completion"] = bench_batched_full(args, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["one_d"] = bench_point_energy_1d(args, local)
        if not args.no_detonation:
            line["detonation"] = bench_detonation(args, local)
        if not args.no_jet:
            line["jet"] = bench_jet(args, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(solver.nx, args.cpu_budget)
    if rank == 0:
        print(json.dumps(line))
    solver.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
