"""TEST INFRASTRUCTURE ONLY: ctypes wrapper over the CPU oracle.

The oracle (swfd_oracle.c) restates the reference's algorithm on the CPU.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libswfd_oracle.so"
_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    lib = C.CDLL(str(LIB))
    P, DP, I64P, I32P = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int32)
    sig = {
        "oracle_create": (P, [C.c_void_p]),
        "oracle_destroy": (None, [P]),
        "oracle_init": (None, [P]),
        "oracle_state_len": (C.c_int64, [P]),
        "oracle_get_state": (None, [P, DP]),
        "oracle_set_state": (None, [P, DP]),
        "oracle_get_time": (C.c_double, [P]),
        "oracle_set_time": (None, [P, C.c_double]),
        "oracle_get_dt": (C.c_double, [P]),
        "oracle_get_restarts": (C.c_int64, [P]),
        "oracle_get_alphamax": (C.c_double, [P]),
        "oracle_get_dx": (C.c_double, [P]),
        "oracle_get_dy": (C.c_double, [P]),
        "oracle_get_status": (C.c_int, [P]),
        "oracle_step": (C.c_int, [P]),
        "oracle_run": (C.c_int64, [P, C.c_int64]),
        "oracle_time_loop_continue": (C.c_int, [P]),
        "oracle_find_alpha": (C.c_double, [P]),
        "oracle_flux_divergence": (None, [P, DP]),
        "oracle_check_positivity": (C.c_int, [P]),
        "oracle_sweep": (C.c_int, [P]),
        "oracle_bc": (None, [P]),
        "oracle_get_stats": (None, [P, I64P]),
        "oracle_get_tracks": (C.c_int64, [P, I32P, I32P, I32P, C.c_int64]),
        "oracle_weno5": (None, [DP, C.c_int64, C.c_double, C.c_int, DP, DP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


STATS_FIELDS = ["sweep_count", "total_sweep", "max_sweep", "total_neg", "max_neg", "total_pos",
                "max_pos", "den_count", "pre_count", "sweep_fail_count"]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """One CPU problem instance; same config struct and state layout as the library."""

    def __init__(self, cfg):
        self.lib = load()
        self.cfg = cfg
        self.o = self.lib.oracle_create(C.byref(cfg))
        ndim = 1 if cfg.problem in (1, 2) else 2  # the MATLAB script and ex2 are 1D
        nc = 5 if cfg.problem == 7 else 4  # ex7: rho, m_x, m_y, E, rho*Y
        self.shape = (1, cfg.nx + 6, 3) if ndim == 1 else (cfg.ny + 6, cfg.nx + 6, nc)

    def close(self):
        if self.o:
            self.lib.oracle_destroy(self.o)
            self.o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_problem(self):
        self.lib.oracle_init(self.o)

    def state(self):
        out = np.empty(self.shape, np.float64)
        self.lib.oracle_get_state(self.o, _dp(out))
        return out

    def set_state(self, u):
        u = np.ascontiguousarray(u, np.float64).reshape(self.shape)
        self.lib.oracle_set_state(self.o, _dp(u))

    @property
    def time(self):
        return self.lib.oracle_get_time(self.o)

    @time.setter
    def time(self, t):
        self.lib.oracle_set_time(self.o, float(t))

    @property
    def dt(self):
        return self.lib.oracle_get_dt(self.o)

    @property
    def restarts(self):
        """dt halvings of the restart RK (rk_choice 2) over all steps"""
        return self.lib.oracle_get_restarts(self.o)

    @property
    def dx(self):
        return self.lib.oracle_get_dx(self.o)

    @property
    def dy(self):
        return self.lib.oracle_get_dy(self.o)

    def step(self):
        st = self.lib.oracle_step(self.o)
        if st != 0:
            raise RuntimeError(f"oracle step status {st}")
        return self.dt

    def run(self, max_steps=0):
        return self.lib.oracle_run(self.o, int(max_steps))

    def loop_continues(self):
        return bool(self.lib.oracle_time_loop_continue(self.o))

    def find_alpha(self):
        return self.lib.oracle_find_alpha(self.o)

    def flux_divergence(self):
        out = np.empty(self.shape, np.float64)
        self.lib.oracle_flux_divergence(self.o, _dp(out))
        return out

    def check_positivity(self):
        return self.lib.oracle_check_positivity(self.o)

    def sweep(self):
        return self.lib.oracle_sweep(self.o)

    def bc(self):
        self.lib.oracle_bc(self.o)

    def stats(self):
        a = np.zeros(10, np.int64)
        self.lib.oracle_get_stats(self.o, a.ctypes.data_as(C.POINTER(C.c_int64)))
        return {k: int(v) for k, v in zip(STATS_FIELDS, a)}

    def tracks(self):
        n = self.lib.oracle_get_tracks(self.o, None, None, None, 0)
        a = [np.zeros(n, np.int32) for _ in range(3)]
        ip = C.POINTER(C.c_int32)
        self.lib.oracle_get_tracks(self.o, *(x.ctypes.data_as(ip) for x in a), n)
        return tuple(a)


def weno5(stencils, weno_eps=1e-6, literals=0):
    lib = load()
    st = np.ascontiguousarray(stencils, np.float64).reshape(-1, 5)
    n = st.shape[0]
    ul = np.empty(n)
    ur = np.empty(n)
    lib.oracle_weno5(_dp(st), n, weno_eps, literals, _dp(ul), _dp(ur))
    return ul, ur
