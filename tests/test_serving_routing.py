"""Which requests the serving loop gives the FP32-bulk form (no GPU needed):
those whose FP32-bulk error against FP64 was measured below 1e-6 relative L1
density -- the vortex, and the point energy up to T = 0.05."""
from sweeping_fd_weno_gb300 import abi, problems
from sweeping_fd_weno_gb300.serving import POINT_ENERGY_FP32_T_MAX, fp32_accepted


def test_vortex_is_fp32():
    assert fp32_accepted(problems.workload("vortex360"))


def test_point_energy_is_fp32_only_for_short_runs():
    assert fp32_accepted(problems.make_config(abi.SEDOV_2D, nx=128, ny=128, time_terminal=0.02))
    assert fp32_accepted(problems.make_config(abi.SEDOV_2D, nx=640, ny=640,
                                              time_terminal=POINT_ENERGY_FP32_T_MAX))
    # the batched configuration runs to T = 1: FP64
    assert not fp32_accepted(problems.make_config(abi.SEDOV_2D, nx=640, ny=640))


def test_jet_and_shock_stay_fp64():
    assert not fp32_accepted(problems.workload("jet"))
    assert not fp32_accepted(problems.workload("shock20"))
