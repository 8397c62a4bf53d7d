"""Host-side mirror of the reference PROGRAMs over the C ABI.

``Solver`` owns one ``swfd_handle``: it replaces the module-level state of an
example's main.f90 and exposes the same procedures (initdata, rk, the time
loop, findalpha, checkpositivity, sweep_lim) plus the output stage (the .dat
files and the sweep statistics block printed by ``output``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi
from .problems import make_config


class Solver:
    """One problem instance resident on one GPU."""

    def __init__(self, cfg: abi.SwfdConfig | int, **overrides):
        if isinstance(cfg, int):
            cfg = make_config(cfg, **overrides)
        elif overrides:
            raise TypeError("overrides only apply when a problem id is given")
        self.cfg = cfg
        self.lib = abi.load()
        h = C.c_void_p()
        abi.check(self.lib.swfd_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.ndim = 1 if cfg.problem in (abi.SEDOV_1D, abi.MATLAB_1D) else 2
        self.nc = 3 if self.ndim == 1 else (5 if cfg.problem == abi.DETONATION else 4)
        self.nx = cfg.nx
        self.ny = 1 if self.ndim == 1 else cfg.ny
        self.shape = (1, self.nx + 6, 3) if self.ndim == 1 else (self.ny + 6, self.nx + 6, self.nc)

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.swfd_destroy(self.h)
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

    def _chk(self, st):
        return abi.check(st, self.h)

    # -- state --------------------------------------------------------------
    def init_problem(self):
        self._chk(self.lib.swfd_init_problem(self.h))

    def state(self, out: np.ndarray | None = None) -> np.ndarray:
        """u(nc,-2:nx+3,-2:ny+3) as a C array [j+2, i+2, c] (into ``out`` if given)."""
        if out is None:
            out = np.empty(self.shape, dtype=np.float64)
        assert out.shape == self.shape and out.dtype == np.float64 and out.flags["C_CONTIGUOUS"]
        self._chk(self.lib.swfd_download_state(self.h, abi.dptr(out)))
        return out

    def set_state(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(self.shape)
        self._chk(self.lib.swfd_upload_state(self.h, abi.dptr(u)))

    @property
    def time(self) -> float:
        t = C.c_double()
        self._chk(self.lib.swfd_get_time(self.h, C.byref(t)))
        return t.value

    @time.setter
    def time(self, t: float):
        self._chk(self.lib.swfd_set_time(self.h, float(t)))

    # -- procedures ---------------------------------------------------------
    def step(self) -> float:
        dt = C.c_double()
        self._chk(self.lib.swfd_step(self.h, C.byref(dt)))
        return dt.value

    def step_host(self, u_in: np.ndarray, u_out: np.ndarray | None = None) -> float:
        """One step from a host state to a host state (upload, step, download,
        one synchronisation); u_out may be u_in.  Returns dt."""
        assert u_in.shape == self.shape and u_in.dtype == np.float64 and u_in.flags["C_CONTIGUOUS"]
        if u_out is None:
            u_out = u_in
        assert u_out.shape == self.shape and u_out.dtype == np.float64 and \
            u_out.flags["C_CONTIGUOUS"]
        dt = C.c_double()
        self._chk(self.lib.swfd_step_host(self.h, abi.dptr(u_in), abi.dptr(u_out), C.byref(dt)))
        return dt.value

    def step_async(self):
        """Enqueue one step on the solver's stream without waiting; finish()
        (or any other call) waits for it and reports its status."""
        self._chk(self.lib.swfd_step_async(self.h))

    def autotune(self) -> int:
        """Time the flux kernel's launch shapes on the current state and keep
        the fastest; returns its resident blocks per SM (0: not tuned)."""
        v = C.c_int32(0)
        self._chk(self.lib.swfd_autotune(self.h, C.byref(v)))
        return v.value

    def finish(self):
        self._chk(self.lib.swfd_finish(self.h))

    def run(self, max_steps: int = 0) -> int:
        n = C.c_int64()
        st = self.lib.swfd_run(self.h, int(max_steps), C.byref(n))
        if st not in (abi.OK, abi.ERR_MAX_STEPS):
            self._chk(st)
        return n.value

    def flux_divergence(self) -> np.ndarray:
        out = np.empty(self.shape, dtype=np.float64)
        self._chk(self.lib.swfd_flux_divergence(self.h, abi.dptr(out)))
        return out

    def sweep(self):
        self._chk(self.lib.swfd_sweep(self.h))

    def check_positivity(self) -> int:
        v = C.c_int32()
        self._chk(self.lib.swfd_check_positivity(self.h, C.byref(v)))
        return v.value

    def find_alpha(self) -> float:
        v = C.c_double()
        self._chk(self.lib.swfd_find_alpha(self.h, C.byref(v)))
        return v.value

    def restarts(self) -> int:
        """dt halvings of the restart RK (rk_choice 2) over all steps"""
        n = C.c_int64(0)
        self._chk(self.lib.swfd_get_restarts(self.h, C.byref(n)))
        return n.value

    def stats(self) -> dict:
        s = abi.SwfdSweepStats()
        self._chk(self.lib.swfd_get_sweep_stats(self.h, C.byref(s)))
        return s.as_dict()

    def tracks(self):
        n = C.c_int64()
        self._chk(self.lib.swfd_get_sweep_tracks(self.h, None, None, None, 0, C.byref(n)))
        k = n.value
        a = np.zeros(k, np.int32), np.zeros(k, np.int32), np.zeros(k, np.int32)
        ip = C.POINTER(C.c_int32)
        self._chk(self.lib.swfd_get_sweep_tracks(
            self.h, a[0].ctypes.data_as(ip), a[1].ctypes.data_as(ip), a[2].ctypes.data_as(ip), k,
            C.byref(n)))
        return a

    # -- instrumentation ----------------------------------------------------
    def stream_ptr(self) -> int:
        v = C.c_void_p()
        self._chk(self.lib.swfd_get_stream(self.h, C.byref(v)))
        return v.value or 0

    def set_profiling(self, on: bool = True):
        self._chk(self.lib.swfd_set_profiling(self.h, 1 if on else 0))

    def profile(self) -> dict:
        pr = abi.SwfdProfile()
        self._chk(self.lib.swfd_get_profile(self.h, C.byref(pr)))
        return pr.as_dict()

    def reset_profile(self):
        self._chk(self.lib.swfd_reset_profile(self.h))

    # -- output (ex3_vortex_accuracy_2d/main.f90:720-841) ----------------------
    def stats_text(self) -> str:
        """The statistics block printed by ``output`` (list-directed records)."""
        from .output import stats_block
        return stats_block(self.stats())

    def write_output(self, out_dir=".", new_table=False, ierror=None) -> str:
        """The example's ``output``: its .dat files in out_dir; returns the
        printed text (errors and orders where computed, then the statistics)."""
        from .output import write_output
        return write_output(self, out_dir, new_table=new_table, ierror=ierror)

    def write_dat(self, out_dir=".") -> str:
        return self.write_output(out_dir)

    def _dx(self):
        p = self.cfg.problem
        if p == abi.VORTEX_2D:
            return 10.0 / self.nx
        if p == abi.SEDOV_2D:
            return 1.3 / self.nx
        if p == abi.SHOCK_DIFFRACTION:  # (13/cut_x - 0)/nxl, the same for every rank
            return (13.0 / self.cfg.cut_x) / (self.nx // self.cfg.cut_x)
        if p == abi.DETONATION:  # (5/cut_x - 0)/nxl
            return (5.0 / self.cfg.cut_x) / (self.nx // self.cfg.cut_x)
        return 1.0 / self.nx

    def _dy(self):
        p = self.cfg.problem
        if p == abi.VORTEX_2D:
            return 10.0 / self.ny
        if p == abi.SEDOV_2D:
            return 1.3 / self.ny
        if p == abi.SHOCK_DIFFRACTION:
            return (11.0 / self.cfg.cut_y) / (self.ny // self.cfg.cut_y)
        if p == abi.DETONATION:
            return (5.0 / self.cfg.cut_y) / (self.ny // self.cfg.cut_y)
        return 0.25 / self.ny


