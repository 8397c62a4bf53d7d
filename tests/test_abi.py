"""CPU checks of the C ABI: the library loads, exports every entry point that
include/swfd.h declares, and validates configurations before touching CUDA."""
import ctypes as C
import re

import pytest

from sweeping_fd_weno_gb300 import abi, problems

HEADER = abi.LIB_PATH.parents[2] / "include" / "swfd.h"
PROBE_HEADER = abi.LIB_PATH.parents[2] / "include" / "swfd_probe.h"


def declared_functions(header=HEADER):
    text = header.read_text()
    return sorted(set(re.findall(r"^\s*(?:swfd_status|const char\*)\s+(swfd_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(swfd):
    lib = abi.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(abi.exported_names()) == names


def test_probe_library_is_apart_from_the_product(swfd):
    names = declared_functions(PROBE_HEADER)
    assert names == sorted(abi.probe_names())
    probe = abi.load_probe()
    for n in names:
        assert hasattr(probe, n), n
    # the product library exports none of them
    import subprocess
    syms = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], capture_output=True,
                          text=True).stdout
    for n in names:
        assert f" {n}\n" not in syms, n


@pytest.mark.parametrize("problem", [abi.MATLAB_1D, abi.SEDOV_1D, abi.VORTEX_2D, abi.SEDOV_2D,
                                     abi.JET_2D, abi.SHOCK_DIFFRACTION, abi.DETONATION])
def test_config_default_matches_reference_parameters(swfd, problem):
    c = abi.config_default(problem).as_dict()
    ref = problems.reference_defaults(problem)
    for k, v in ref.items():
        assert c[k] == v, (k, c[k], v)


def test_create_rejects_bad_configs_without_cuda(swfd):
    lib = abi.load()
    h = C.c_void_p()
    cfg = problems.make_config(abi.VORTEX_2D, abi_version=99)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.make_config(abi.VORTEX_2D, nx=4)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.make_config(abi.VORTEX_2D, use_limiter=3)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.make_config(abi.VORTEX_2D, rk_choice=2)    # the restart RK is ex2's only
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.make_config(abi.SEDOV_1D, rk_choice=3)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.make_config(abi.MATLAB_1D, variant=9)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.make_config(abi.MATLAB_1D, precision=abi.PRECISION_FP32_BULK)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_UNSUPPORTED
    cfg = problems.make_config(abi.VORTEX_2D, swp_num=0)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    assert "swp_num" in abi.last_error()
    assert lib.swfd_config_default(C.byref(cfg), 42) == abi.ERR_INVALID


def test_status_strings(swfd):
    lib = abi.load()
    for st in range(0, -12, -1):
        assert lib.swfd_status_string(st)
    assert lib.swfd_status_string(abi.ERR_SWEEP_NOCONV) == b"sweep did not converge within swp_num"


def test_null_handle_is_rejected(swfd):
    lib = abi.load()
    assert lib.swfd_step(None, None) == abi.ERR_INVALID
    assert lib.swfd_destroy(None) == abi.OK


def test_shock_diffraction_config_checks(swfd):
    """The wall rows must sit inside one rank, away from its ghost rows."""
    import ctypes as C
    from sweeping_fd_weno_gb300 import problems
    lib = abi.load()
    h = C.c_void_p()
    cfg = problems.workload("shock8")       # step top at local row 4 of its rank
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_UNSUPPORTED
    cfg = problems.workload("shock12")
    cfg.nx += 4                              # not cut_x*(13*total/cut_x)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.workload("shock12", cut_x=3)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_UNSUPPORTED


def test_detonation_config_checks(swfd):
    """ex7: grid from total and the rank grid, the wall row inside a rank's
    local rows, FP64 and the SSP-RK3 of its rk."""
    import ctypes as C
    from sweeping_fd_weno_gb300 import problems
    lib = abi.load()
    h = C.c_void_p()
    # total 8 on 4 x 8 ranks: the wall row is local row 6 = nyl + 1 of rank row 2
    cfg = problems.make_config(abi.DETONATION, total=8)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_UNSUPPORTED
    cfg = problems.make_config(abi.DETONATION, total=32)
    cfg.ny += 8                              # not cut_y*(5*total/cut_y)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
    cfg = problems.make_config(abi.DETONATION, total=32, precision=abi.PRECISION_FP32_BULK)
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_UNSUPPORTED
    cfg = problems.make_config(abi.DETONATION, total=32, rk_choice=2)  # ex2's restart RK only
    assert lib.swfd_create(C.byref(cfg), C.byref(h)) == abi.ERR_INVALID
