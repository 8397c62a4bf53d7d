"""Problem configurations: the reference examples' compile-time PARAMETERs and
the benchmark workloads built on them.

``reference_defaults`` restates the PARAMETER blocks of each example's
main.f90; ``workload`` returns the named benchmark configurations (grid sizes,
CFL, swp_num, final time) on synthetic initial data generated by the same
initdata formulas.
"""
from __future__ import annotations

from . import abi


def reference_defaults(problem: int) -> dict:
    """PARAMETERs of the reference example behind ``problem``."""
    base = dict(abi_version=abi.ABI_VERSION, problem=problem, use_limiter=2, swp_num=20000,
                literals=abi.LITERALS_DOUBLE, precision=abi.PRECISION_FP64,
                ubar_mode=abi.UBAR_SEQUENTIAL, sweep_mode=abi.SWEEP_PARALLEL, device=0, gamma=1.4,
                e_background=0.0,
                e_blast=0.0, ny=1, total=0, cut_x=0, cut_y=0, rk_choice=1, variant=0)
    if problem == abi.MATLAB_1D:     # FD_WENO_Application.m:10,17,95-110,207 (problem = 5)
        base.update(matlab_problem(5), swp_num=200000)
    elif problem == abi.SEDOV_1D:      # ex2_sedov_1d/main.f90:4-7,423-425 (RK_choice = 1)
        base.update(nx=800, ny=1, swp_num=50, cfl=1.2, time_terminal=0.001,
                    e_background=1e-9 / (1.4 - 1.0), e_blast=3200000.0)
    elif problem == abi.VORTEX_2D:   # ex3_vortex_accuracy_2d/main.f90:5-7,570
        base.update(nx=180, ny=180, cfl=0.5, time_terminal=0.01)
    elif problem == abi.SEDOV_2D:    # ex4_sedov_2d/main.f90:18-20,687,1172,1182
        base.update(nx=640, ny=640, cfl=0.5, time_terminal=1.0, e_background=1e-12,
                    e_blast=0.244816)
    elif problem == abi.JET_2D:      # ex5_mach2000_jet/main.f90:4-6,597
        base.update(nx=800, ny=200, cfl=1.0 / 4.0, time_terminal=0.001, gamma=5.0 / 3.0)
    elif problem == abi.SHOCK_DIFFRACTION:  # ex6_shock_diffraction/main.f90:16-20,695
        base.update(shock_grid(80), cfl=0.9, time_terminal=2.3)
    elif problem == abi.DETONATION:  # ex7_detonation/main.f90:11-19,43,812
        base.update(detonation_grid(80), cfl=0.88, time_terminal=0.6, gamma=1.2,
                    swp_num=20000)
    else:
        raise ValueError(f"unknown problem {problem}")
    return base


# The MATLAB script's problems (ex1_double_rarefaction_1d/FD_WENO_Application.m
# :27-150 and its nArray :158-165): gamma, final time and grid size.  The
# script defines cfl = 0.85 for problem 5 only; the others take the same.
MATLAB_PROBLEMS = {
    1: dict(gamma=1.4, time_terminal=2.0, nx=80),      # linear advection (nArray 20..320)
    2: dict(gamma=3.0, time_terminal=0.3, nx=80),      # nonlinear (nArray 20..320)
    3: dict(gamma=1.4, time_terminal=0.4, nx=200),     # Sod shock tube
    4: dict(gamma=1.4, time_terminal=1.3, nx=200),     # Lax
    5: dict(gamma=1.4, time_terminal=0.3, nx=200),     # double rarefaction (as shipped)
    6: dict(gamma=1.4, time_terminal=0.0004, nx=801),  # point energy
    7: dict(gamma=1.4, time_terminal=0.00001, nx=200), # jet ambient state (no nArray)
}


def matlab_problem(variant: int) -> dict:
    d = dict(MATLAB_PROBLEMS[variant])
    return dict(d, variant=variant, ny=1, cfl=0.85, use_limiter=2)


def shock_grid(total: int, cut_x: int = 4, cut_y: int = 8) -> dict:
    """Grid of the shock-diffraction example for its `total` and rank grid:
    nx = cut_x*(13*total/cut_x), ny = cut_y*(11*total/cut_y) in integer
    arithmetic (ex6_shock_diffraction/main.f90:16-18)."""
    return dict(total=total, cut_x=cut_x, cut_y=cut_y, nx=cut_x * (13 * total // cut_x),
                ny=cut_y * (11 * total // cut_y))


def detonation_grid(total: int, cut_x: int = 4, cut_y: int = 8) -> dict:
    """Grid of the detonation example: nx = cut_x*(5*total/cut_x),
    ny = cut_y*(5*total/cut_y) in integer arithmetic
    (ex7_detonation/main.f90:11-13)."""
    return dict(total=total, cut_x=cut_x, cut_y=cut_y, nx=cut_x * (5 * total // cut_x),
                ny=cut_y * (5 * total // cut_y))


def make_config(problem: int, **overrides) -> abi.SwfdConfig:
    d = reference_defaults(problem)
    if problem == abi.SHOCK_DIFFRACTION and "total" in overrides:
        d.update(shock_grid(overrides["total"], overrides.get("cut_x", 4),
                            overrides.get("cut_y", 8)))
    if problem == abi.DETONATION and "total" in overrides:
        d.update(detonation_grid(overrides["total"], overrides.get("cut_x", 4),
                                 overrides.get("cut_y", 8)))
    unknown = set(overrides) - set(d) - {"reserved"}
    if unknown:
        raise KeyError(f"unknown config fields {sorted(unknown)}")
    d.update(overrides)
    cfg = abi.SwfdConfig()
    for k, v in d.items():
        setattr(cfg, k, v)
    return cfg


# Benchmark workloads (sizes and parameters of the named configurations).
def workload(name: str, **overrides) -> abi.SwfdConfig:
    if name == "sedov1d_fp64":
        # 1D point energy: n=800 on [-2,2], E=1e-12 background, E=3.2e6/dx centre,
        # CFL 0.6, swp_num=2, T=0.001
        return make_config(abi.SEDOV_1D, cfl=0.6, swp_num=2, e_background=1e-12,
                           **overrides)
    if name.startswith("vortex"):
        # near-vacuum isentropic vortex on [0,10]^2, T=0.01; name 'vortex<n>'
        n = int(name[len("vortex"):] or 180)
        return make_config(abi.VORTEX_2D, nx=n, ny=n, **overrides)
    if name == "jet":
        # Mach-2000-type jet, 800x200 half domain with the y=0 symmetry plane, T=0.001
        return make_config(abi.JET_2D, **overrides)
    if name == "jet_full":
        # the same jet on the full domain [0,1]x[-0.25,0.25] at 800x400 (inflow for
        # |y| <= 0.05, outflow at the bottom instead of the symmetry plane)
        return make_config(abi.JET_2D, **dict(dict(ny=400, variant=1), **overrides))
    if name.startswith("shock"):
        # Mach 5.09 shock diffraction around a step; name 'shock<total>'
        # (total 20..80: 260x216 .. 1040x880 cells)
        return make_config(abi.SHOCK_DIFFRACTION, total=int(name[len("shock"):] or 80),
                           **overrides)
    if name.startswith("detonation"):
        # reactive Euler detonation past a step; name 'detonation<total>'
        # (total 80: 400x400 cells on 4 x 8 ranks)
        return make_config(abi.DETONATION, total=int(name[len("detonation"):] or 80),
                           **overrides)
    if name.startswith("sedov2d"):
        n = int(name[len("sedov2d"):] or 640)
        return make_config(abi.SEDOV_2D, nx=n, ny=n, **overrides)
    raise KeyError(name)
