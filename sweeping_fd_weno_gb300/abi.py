"""ctypes view of the C ABI declared in include/swfd.h.

The shared library is loaded from the package's own ``_lib`` directory.  There
is no fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libswfd.so"
ABI_VERSION = 2

# status codes
OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_SWEEP_NOCONV = -3
ERR_PUBAR_NONPOS = -4
ERR_NONFINITE = -5
ERR_OOM = -6
ERR_TIMEOUT = -7
ERR_UNSUPPORTED = -8
ERR_MAX_STEPS = -9
ERR_SWEEP_CHECK = -10
ERR_RESTART_LIMIT = -11
RESTART_LIMIT = 1100

# problems (one per reference example)
MATLAB_1D = 1  # ex1_double_rarefaction_1d (MATLAB)
SEDOV_1D = 2   # ex2_sedov_1d
VORTEX_2D = 3  # ex3_vortex_accuracy_2d
SEDOV_2D = 4   # ex4_sedov_2d
JET_2D = 5     # ex5_mach2000_jet
SHOCK_DIFFRACTION = 6  # ex6_shock_diffraction
DETONATION = 7  # ex7_detonation: five components (rho, m_x, m_y, E, rho*Y)

LITERALS_DOUBLE = 0
LITERALS_QUAD = 1
PRECISION_FP64 = 0
PRECISION_FP32_BULK = 1
UBAR_SEQUENTIAL = 0
UBAR_TREE = 1
SWEEP_PARALLEL = 0
SWEEP_SEQUENTIAL = 1


class SwfdConfig(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32),
        ("problem", C.c_int32),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("use_limiter", C.c_int32),
        ("swp_num", C.c_int32),
        ("literals", C.c_int32),
        ("precision", C.c_int32),
        ("ubar_mode", C.c_int32),
        ("device", C.c_int32),
        ("cfl", C.c_double),
        ("time_terminal", C.c_double),
        ("gamma", C.c_double),
        ("e_background", C.c_double),
        ("e_blast", C.c_double),
        ("sweep_mode", C.c_int32),
        ("total", C.c_int32),
        ("cut_x", C.c_int32),
        ("cut_y", C.c_int32),
        ("rk_choice", C.c_int32),
        ("variant", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class SwfdSweepStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "sweep_count", "total_sweep", "max_sweep", "total_neg", "max_neg", "total_pos",
        "max_pos", "den_count", "pre_count", "sweep_fail_count")]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


STATS_FIELDS = [f for f, _ in SwfdSweepStats._fields_]


class SwfdProfile(C.Structure):
    _fields_ = [("kernel_launches", C.c_int64), ("stages", C.c_int64),
                ("flux_launches", C.c_int64), ("flux_ms", C.c_double),
                ("sweep_invocations", C.c_int64), ("sweep_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}

class SwfdBatchConfig(C.Structure):
    _fields_ = [("max_slots", C.c_int32), ("max_nx", C.c_int32), ("max_ny", C.c_int32),
                ("precision", C.c_int32), ("ubar_mode", C.c_int32), ("device", C.c_int32),
                ("pool_bytes", C.c_int64), ("reserved", C.c_int32 * 8)]


# name -> (restype, argtypes) for every entry point of include/swfd.h
_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_SIGS = {
    "swfd_config_default": (C.c_int32, [C.POINTER(SwfdConfig), C.c_int32]),
    "swfd_create": (C.c_int32, [C.POINTER(SwfdConfig), C.POINTER(_P)]),
    "swfd_destroy": (C.c_int32, [_P]),
    "swfd_init_problem": (C.c_int32, [_P]),
    "swfd_upload_state": (C.c_int32, [_P, _DP]),
    "swfd_download_state": (C.c_int32, [_P, _DP]),
    "swfd_flux_divergence": (C.c_int32, [_P, _DP]),
    "swfd_step": (C.c_int32, [_P, _DP]),
    "swfd_step_host": (C.c_int32, [_P, _DP, _DP, _DP]),
    "swfd_run": (C.c_int32, [_P, C.c_int64, C.POINTER(C.c_int64)]),
    "swfd_sweep": (C.c_int32, [_P]),
    "swfd_check_positivity": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "swfd_find_alpha": (C.c_int32, [_P, _DP]),
    "swfd_get_time": (C.c_int32, [_P, _DP]),
    "swfd_set_time": (C.c_int32, [_P, C.c_double]),
    "swfd_get_sweep_stats": (C.c_int32, [_P, C.POINTER(SwfdSweepStats)]),
    "swfd_get_restarts": (C.c_int32, [_P, C.POINTER(C.c_int64)]),
    "swfd_step_async": (C.c_int32, [_P]),
    "swfd_autotune": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "swfd_batch_autotune": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "swfd_finish": (C.c_int32, [_P]),
    "swfd_get_sweep_tracks": (C.c_int32, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32), C.c_int64,
                                          C.POINTER(C.c_int64)]),
    "swfd_weno5_batch": (C.c_int32, [_DP, C.c_int64, C.c_double, C.c_int32, C.c_int32, _DP, _DP]),
    "swfd_get_stream": (C.c_int32, [_P, C.POINTER(_P)]),
    "swfd_set_profiling": (C.c_int32, [_P, C.c_int32]),
    "swfd_get_profile": (C.c_int32, [_P, C.POINTER(SwfdProfile)]),
    "swfd_reset_profile": (C.c_int32, [_P]),
    "swfd_flux_divergence_static": (C.c_int32, [C.POINTER(SwfdConfig), _P, _P, _P]),
    "swfd_batch_config_default": (C.c_int32, [C.POINTER(SwfdBatchConfig)]),
    "swfd_batch_create": (C.c_int32, [C.POINTER(SwfdBatchConfig), C.POINTER(_P)]),
    "swfd_batch_destroy": (C.c_int32, [_P]),
    "swfd_batch_admit": (C.c_int32, [_P, C.POINTER(SwfdConfig), C.c_int64]),
    "swfd_batch_run": (C.c_int32, [_P, C.c_int64, C.POINTER(C.c_int64)]),
    "swfd_batch_poll": (C.c_int32, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int32,
                                    C.POINTER(C.c_int32)]),
    "swfd_batch_download": (C.c_int32, [_P, C.c_int64, _DP, _DP]),
    "swfd_batch_stats": (C.c_int32, [_P, C.c_int64, C.POINTER(SwfdSweepStats)]),
    "swfd_batch_release": (C.c_int32, [_P, C.c_int64]),
    "swfd_batch_info": (C.c_int32, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int64)]),
    "swfd_batch_get_stream": (C.c_int32, [_P, C.POINTER(_P)]),
    "swfd_sequential_sum": (C.c_int32, [_DP, C.c_int64, C.c_double, C.c_int32,
                                        C.POINTER(C.c_double)]),
    "swfd_batch_progress": (C.c_int32, [_P, C.c_int64, C.POINTER(C.c_double),
                                        C.POINTER(C.c_int64)]),
    "swfd_last_error": (C.c_int32, [_P, C.c_char_p, C.c_size_t]),
    "swfd_status_string": (C.c_char_p, [C.c_int32]),
}

# libswfd_probe.so (include/swfd_probe.h): measurement and test probes
PROBE_PATH = LIB_PATH.parent / "libswfd_probe.so"
_PROBE_SIGS = {
    "swfd_probe_fp64_peak": (C.c_int32, [C.c_int32, _DP]),
    "swfd_probe_rcp_bulk": (C.c_int32, [C.c_int32, _DP, C.c_int64, _DP]),
    "swfd_probe_convert": (C.c_int32, [C.c_int32, _DP, C.c_int64, C.POINTER(C.c_float), _DP]),
    "swfd_probe_barrier_timeout": (C.c_int32, [C.c_int32, C.c_int32, C.c_double,
                                              C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "swfd_probe_solve1d_layout": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32,
                                             C.POINTER(C.c_int32)]),
    "swfd_probe_reduce_timeout": (C.c_int32, [C.c_int32, C.c_int32, C.c_double,
                                             C.POINTER(C.c_int32), C.POINTER(C.c_int32), _DP,
                                             C.POINTER(C.c_int32)]),
}

_lib = None
_probe = None


def load_probe() -> C.CDLL:
    """Load libswfd_probe.so (once).  Raises if absent."""
    global _probe
    if _probe is not None:
        return _probe
    if not PROBE_PATH.exists():
        raise FileNotFoundError(f"{PROBE_PATH} is missing: build it with __graft_entry__.build()")
    lib = C.CDLL(str(PROBE_PATH))
    for name, (res, args) in _PROBE_SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _probe = lib
    return lib


def probe_names() -> list[str]:
    return list(_PROBE_SIGS)


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libswfd.so (once) and attach the prototypes.  Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def exported_names() -> list[str]:
    return list(_SIGS)


class SwfdError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"swfd status {status}: {msg}")
        self.status = status


def last_error(handle=None) -> str:
    lib = load()
    buf = C.create_string_buffer(1024)
    lib.swfd_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, handle=None) -> int:
    if status != OK:
        raise SwfdError(status, last_error(handle) or load().swfd_status_string(status).decode())
    return status


def config_default(problem: int) -> SwfdConfig:
    cfg = SwfdConfig()
    check(load().swfd_config_default(C.byref(cfg), problem))
    return cfg


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_DP)
