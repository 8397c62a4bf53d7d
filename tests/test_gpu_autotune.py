"""The autotuners change launch shapes only: results stay value for value
those of the default shapes."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Batch, Solver, abi, problems

pytestmark = pytest.mark.gpu


# FP32-bulk: the separate splitting, flux and RK kernels (SWFD_FP32_STAGE=
# split, the batch engine's kernels); the fused stage has one launch shape
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32_BULK])
def test_flux_launch_shape_tuning_keeps_results(swfd, monkeypatch, precision):
    monkeypatch.setenv("SWFD_FP32_STAGE", "split")
    cfg = problems.make_config(abi.VORTEX_2D, nx=64, ny=64, precision=precision)
    a, b = Solver(cfg), Solver(cfg)
    for s in (a, b):
        s.init_problem()
    minb = b.autotune()
    assert minb in ((3, 2, 4, 13, 14, 15, 16, 24, 25, 44, 45)
                    if precision == abi.PRECISION_FP64 else (4, 5, 6))
    for _ in range(4):
        assert a.step() == b.step()
    assert np.array_equal(a.state(), b.state())
    a.close()
    b.close()


# FP64 13..16: the lane-pair flux kernel (two lanes per interface) with 3..6
# resident blocks per SM; 24, 25: its short form (one code path for both
# directions, the fields in a loop) with 4, 5; 44, 45: the short form with
# each interface's eigenvectors formed once and shared
@pytest.mark.parametrize("precision,minb", [(abi.PRECISION_FP64, 2), (abi.PRECISION_FP64, 3),
                                            (abi.PRECISION_FP64, 4),
                                            (abi.PRECISION_FP64, 13), (abi.PRECISION_FP64, 14),
                                            (abi.PRECISION_FP64, 15), (abi.PRECISION_FP64, 16),
                                            (abi.PRECISION_FP64, 24), (abi.PRECISION_FP64, 25),
                                            (abi.PRECISION_FP64, 44), (abi.PRECISION_FP64, 45),
                                            (abi.PRECISION_FP32_BULK, 5),
                                            (abi.PRECISION_FP32_BULK, 6)])
def test_each_flux_launch_shape_keeps_results(swfd, monkeypatch, precision, minb):
    # SWFD_FLUX_MIN_BLOCKS pins a candidate: every shape runs, not only the fastest
    monkeypatch.setenv("SWFD_FLUX_MIN_BLOCKS", str(minb))
    monkeypatch.setenv("SWFD_FP32_STAGE", "split")
    cfg = problems.make_config(abi.VORTEX_2D, nx=72, ny=56, precision=precision)
    a, b = Solver(cfg), Solver(cfg)
    for s in (a, b):
        s.init_problem()
    assert b.autotune() == minb
    for _ in range(3):
        assert a.step() == b.step()
    assert np.array_equal(a.state(), b.state())
    a.close()
    b.close()


def test_flux_tuning_skips_segmented_and_limited_problems(swfd):
    s = Solver(problems.make_config(abi.VORTEX_2D, nx=48, ny=48, use_limiter=1))
    s.init_problem()
    assert s.autotune() == 0
    s.close()


def test_flux_tuning_skips_the_fused_fp32_stage(swfd, monkeypatch):
    monkeypatch.delenv("SWFD_FP32_STAGE", raising=False)
    s = Solver(problems.make_config(abi.VORTEX_2D, nx=48, ny=48,
                                    precision=abi.PRECISION_FP32_BULK))
    s.init_problem()
    assert s.autotune() == 0
    s.close()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32_BULK])
def test_batch_tile_tuning_keeps_results(swfd, precision):
    mix = [dict(nx=45, ny=45), dict(nx=64, ny=48), dict(nx=96, ny=80)]
    out = []
    for tune in (False, True):
        with Batch(max_slots=4, max_nx=128, max_ny=128, precision=precision) as b:
            for k, m in enumerate(mix):
                assert b.admit(problems.make_config(abi.VORTEX_2D, precision=precision, **m), k)
            if tune:
                assert b.autotune() in (512, 1024, 2048, 4096, 8192)
            b.run(5)
            out.append([b.download(k) for k in range(len(mix))])
    for (ua, ta), (ub, tb) in zip(*out):
        assert ta == tb
        assert np.array_equal(ua, ub)


@pytest.mark.parametrize("minb", [3, 14, 16, 24, 25, 44, 45])
@pytest.mark.parametrize("case", [dict(problem=abi.SEDOV_2D, nx=48, ny=40),
                                  dict(problem=abi.JET_2D, nx=96, ny=24)],
                         ids=["point_energy", "jet"])
def test_lane_pair_flux_kernel_matches_the_oracle(swfd, oracle_mod, monkeypatch, minb, case):
    """The FP64 flux kernels (3: one lane per interface; 14, 16: the lane-pair
    kernel; 24, 25: its short form; 44, 45: the short form with shared
    eigenvectors, the default 45) on the ex4 form (alpha
    pre-multiplied, y-pass regulariser planes) and the ex5 form, against the
    oracle's steps."""
    monkeypatch.setenv("SWFD_FLUX_MIN_BLOCKS", str(minb))
    kw = dict(case)
    prob = kw.pop("problem")
    g = Solver(problems.make_config(prob, **kw))
    o = oracle_mod.Oracle(problems.make_config(prob, **kw))
    g.init_problem()
    o.init_problem()
    assert g.autotune() == minb
    for _ in range(3):
        assert g.step() == o.step()
    assert np.array_equal(g.state(), o.state())
    assert g.stats() == o.stats()
    g.close()


@pytest.mark.parametrize("block", [32, 256, 1024])
def test_heavy_kernel_block_size_keeps_results(swfd, monkeypatch, block):
    """SWFD_HEAVY_BLOCK sets the largest block of the splitting and RK kernels
    (default 128): launch shape only, the same bits (ex4 form, 6 steps)."""
    cfg = problems.make_config(abi.SEDOV_2D, nx=70, ny=50)
    monkeypatch.delenv("SWFD_HEAVY_BLOCK", raising=False)
    a = Solver(cfg)
    monkeypatch.setenv("SWFD_HEAVY_BLOCK", str(block))
    b = Solver(cfg)
    for s in (a, b):
        s.init_problem()
    for _ in range(6):
        assert a.step() == b.step()
    assert np.array_equal(a.state(), b.state())
    assert a.stats() == b.stats()
    a.close()
    b.close()
