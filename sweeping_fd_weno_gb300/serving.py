"""Serving loops: a stream of independent Euler solves arriving over time.

`serve_batched` is continuous batching over the batched engine: a request is
admitted as soon as it has arrived and the batch has a free slot and enough
of its HBM budget; while any request runs, the loop advances every running
request together by `step_chunk` SSP-RK3 steps (one graph launch); finished
requests are polled, their final state read back to the host, their
time-to-solution (arrival to result on the host) recorded and their slots
released for the requests still waiting.

`serve_one_at_a_time` is the plain form the batched one is compared with:
the same stream, first come first served, each request solved alone by a
single-instance handle.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .batch import Batch
from .solver import Solver


@dataclass
class ServeResult:
    latencies: dict = field(default_factory=dict)   # request id -> seconds
    status: dict = field(default_factory=dict)      # request id -> swfd status
    updates: dict = field(default_factory=dict)     # request id -> interior cells x stages
    wall: float = 0.0
    launches: int = 0                                # graph launches (batched) / solves

    def percentile(self, q):
        v = np.array(list(self.latencies.values()))
        return float(np.percentile(v, q)) if len(v) else float("nan")

    def summary(self) -> dict:
        upd = float(sum(self.updates.values()))
        return {"requests": len(self.latencies),
                "p50_s": self.percentile(50), "p99_s": self.percentile(99),
                "max_s": max(self.latencies.values()) if self.latencies else None,
                "wall_s": self.wall, "cell_updates": upd,
                "value": upd / self.wall if self.wall else None,
                "failed": sum(1 for s in self.status.values() if s != 0),
                "launches": self.launches}


def serve_batched(arrivals, batch: Batch, step_chunk: int = 4, timeout: float = 600.0,
                  keep=None) -> ServeResult:
    """arrivals: list of (arrival time in s after the start, swfd_config).
    `keep` (optional dict) receives each request's final (state, time)."""
    pending = deque(sorted(((t, k, c) for k, (t, c) in enumerate(arrivals)), key=lambda x: x[0]))
    waiting = deque()
    arrived_at, cells_of = {}, {}
    res = ServeResult()
    n_total, done = len(pending), 0
    t0 = time.perf_counter()
    while done < n_total:
        now = time.perf_counter() - t0
        if now > timeout:
            raise TimeoutError(f"serving stream not finished after {timeout} s")
        while pending and pending[0][0] <= now:
            waiting.append(pending.popleft())
        while waiting:
            t, k, c = waiting[0]
            if not batch.admit(c, k):
                break
            waiting.popleft()
            arrived_at[k] = t
            cells_of[k] = c.nx * c.ny
        if batch.info()["running"] == 0:
            if pending:
                time.sleep(max(0.0, min(pending[0][0] - (time.perf_counter() - t0), 0.005)))
            continue
        batch.run(step_chunk)
        res.launches += 1
        for rid, st in batch.poll():
            u, tt = batch.download(rid)
            _, steps = batch.progress(rid)
            res.latencies[rid] = time.perf_counter() - t0 - arrived_at[rid]
            res.status[rid] = st
            res.updates[rid] = cells_of[rid] * 3 * steps
            if keep is not None:
                keep[rid] = (u, tt)
            batch.release(rid)
            done += 1
    res.wall = time.perf_counter() - t0
    return res


def serve_one_at_a_time(arrivals, timeout: float = 600.0, keep=None) -> ServeResult:
    """The same stream, first come first served, one single-instance solve at a time."""
    order = sorted(((t, k, c) for k, (t, c) in enumerate(arrivals)), key=lambda x: x[0])
    res = ServeResult()
    t0 = time.perf_counter()
    for t, k, c in order:
        now = time.perf_counter() - t0
        if now > timeout:
            raise TimeoutError(f"serving stream not finished after {timeout} s")
        if t > now:
            time.sleep(t - now)
        s = Solver(c)
        s.init_problem()
        steps = s.run()
        u = s.state()
        res.latencies[k] = time.perf_counter() - t0 - t
        res.status[k] = 0
        res.updates[k] = c.nx * c.ny * 3 * steps
        if keep is not None:
            keep[k] = (u, s.time)
        s.close()
        res.launches += 1
    res.wall = time.perf_counter() - t0
    return res


def poisson_arrivals(rate_hz: float, n: int, seed: int, draw):
    """n requests with exponential inter-arrival times of mean 1/rate_hz; request
    k's configuration is draw(rng) from the same seeded generator."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=n))
    return [(float(t[k]), draw(rng)) for k in range(n)]
