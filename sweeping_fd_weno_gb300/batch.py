"""Host side of the batched engine (swfd_batch_* of the C ABI).

Many independent 2D problem instances resident on one GPU advance together;
instances are admitted and retired between runs (continuous batching).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class Batch:
    def __init__(self, max_slots=64, max_nx=640, max_ny=640, precision=abi.PRECISION_FP32_BULK,
                 ubar_mode=abi.UBAR_TREE, device=0, pool_bytes=0):
        self.lib = abi.load()
        cfg = abi.SwfdBatchConfig()
        abi.check(self.lib.swfd_batch_config_default(C.byref(cfg)))
        cfg.max_slots, cfg.max_nx, cfg.max_ny = max_slots, max_nx, max_ny
        cfg.precision, cfg.ubar_mode, cfg.device, cfg.pool_bytes = precision, ubar_mode, device, pool_bytes
        self.cfg = cfg
        h = C.c_void_p()
        abi.check(self.lib.swfd_batch_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.shapes = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.swfd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def admit(self, cfg: abi.SwfdConfig, request_id: int) -> bool:
        """False when the batch is full (no slot or HBM budget): the request waits."""
        st = self.lib.swfd_batch_admit(self.h, C.byref(cfg), int(request_id))
        if st == abi.ERR_OOM:
            return False
        abi.check(st)
        self.shapes[int(request_id)] = (cfg.ny + 6, cfg.nx + 6, 4)
        return True

    def run(self, max_steps: int) -> int:
        n = C.c_int64()
        abi.check(self.lib.swfd_batch_run(self.h, int(max_steps), C.byref(n)))
        return n.value

    def poll(self, cap: int = 1024):
        ids = (C.c_int64 * cap)()
        sts = (C.c_int32 * cap)()
        n = C.c_int32()
        abi.check(self.lib.swfd_batch_poll(self.h, ids, sts, cap, C.byref(n)))
        return [(ids[k], sts[k]) for k in range(n.value)]

    def download(self, request_id: int):
        u = np.empty(self.shapes[int(request_id)], np.float64)
        t = C.c_double()
        abi.check(self.lib.swfd_batch_download(self.h, int(request_id), abi.dptr(u), C.byref(t)))
        return u, t.value

    def stats(self, request_id: int) -> dict:
        s = abi.SwfdSweepStats()
        abi.check(self.lib.swfd_batch_stats(self.h, int(request_id), C.byref(s)))
        return s.as_dict()

    def release(self, request_id: int):
        abi.check(self.lib.swfd_batch_release(self.h, int(request_id)))
        self.shapes.pop(int(request_id), None)

    def progress(self, request_id: int):
        """(simulated time, steps taken) of a request as of the last run."""
        t, n = C.c_double(), C.c_int64()
        abi.check(self.lib.swfd_batch_progress(self.h, int(request_id), C.byref(t), C.byref(n)))
        return t.value, n.value

    def autotune(self) -> int:
        """Time the cell-tile sizes of the per-cell kernels on the running
        instances and keep the fastest; returns the tile size in cells."""
        v = C.c_int32(0)
        abi.check(self.lib.swfd_batch_autotune(self.h, C.byref(v)))
        return v.value

    def stream_ptr(self) -> int:
        v = C.c_void_p()
        abi.check(self.lib.swfd_batch_get_stream(self.h, C.byref(v)))
        return v.value or 0

    def info(self):
        r, f, b = C.c_int32(), C.c_int32(), C.c_int64()
        abi.check(self.lib.swfd_batch_info(self.h, C.byref(r), C.byref(f), C.byref(b)))
        return {"running": r.value, "free_slots": f.value, "free_bytes": b.value}
