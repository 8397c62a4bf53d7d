"""The fused FP32-bulk stage (k_alpha_terms32: [bc,] findalpha and the
splitting terms; k_stage32: split fluxes, interface fluxes, RHS, RK
combination and checkpositivity per 32 x 8 tile) against the separate
splitting, flux and RK kernels (SWFD_FP32_STAGE=split): the same bits for
every state value, the time and every statistic, on grids whose sides are
not multiples of the tile (partial tiles), with the ex4 switches (fluxes
scaled by alpha, regularised y-pass Roe planes, strict positivity) and with
sweeps (the jet)."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

F32 = abi.PRECISION_FP32_BULK
CASES = [
    ("vortex45_to_T", dict(problem=abi.VORTEX_2D, nx=45, ny=45), 0),
    ("vortex64", dict(problem=abi.VORTEX_2D, nx=64, ny=64), 20),
    ("sedov2d_70x50", dict(problem=abi.SEDOV_2D, nx=70, ny=50), 25),
    ("jet_96x24", dict(problem=abi.JET_2D, nx=96, ny=24), 60),
    ("jet_full_96x48", dict(problem=abi.JET_2D, nx=96, ny=48, variant=1), 30),
]


def run(monkeypatch, mode, case, steps):
    monkeypatch.setenv("SWFD_FP32_STAGE", mode)
    kw = dict(case)
    s = Solver(problems.make_config(kw.pop("problem"), precision=F32, **kw))
    s.init_problem()
    s.set_profiling(True)
    if steps == 0:
        n = s.run()
    else:
        n = steps
        for _ in range(steps):
            s.step()
    out = dict(u=s.state(), t=s.time, stats=s.stats(), n=n,
               launches=s.profile()["kernel_launches"], tracks=s.tracks())
    s.close()
    return out


@pytest.mark.parametrize("name,case,steps", CASES, ids=[c[0] for c in CASES])
def test_fused_stage_equals_separate_kernels(swfd, monkeypatch, name, case, steps):
    a = run(monkeypatch, "split", case, steps)
    b = run(monkeypatch, "fused", case, steps)
    assert a["n"] == b["n"] and a["t"] == b["t"], (a["n"], b["n"], a["t"], b["t"])
    assert a["stats"] == b["stats"]
    for x, y in zip(a["tracks"], b["tracks"]):
        assert np.array_equal(x, y)
    # bit patterns: the sign of a zero and a NaN's payload count too
    bad = a["u"].view(np.uint64) != b["u"].view(np.uint64)
    assert not bad.any(), f"{int(bad.sum())} state values differ, first at {np.argwhere(bad)[:4]}"
    # two kernels per stage instead of four (sweeps aside)
    assert b["launches"] < a["launches"], (a["launches"], b["launches"])
    if name == "jet_96x24":
        assert b["stats"]["sweep_count"] > 0  # the sweeps ran in both


def test_fused_stage_kernel_count_per_step(swfd, monkeypatch):
    """vortex 64x64: findalpha+terms, then per stage the stage kernel and
    bc+findalpha+terms (the bc alone after stage 3), and the time advance --
    8 kernels per step against 14 with the separate kernels (the sweeps'
    kernels are the same in both)."""
    case = dict(problem=abi.VORTEX_2D, nx=64, ny=64)
    a = run(monkeypatch, "split", case, 4)
    b = run(monkeypatch, "fused", case, 4)
    assert a["stats"] == b["stats"]
    assert a["launches"] - b["launches"] == (14 - 8) * 4, (a["launches"], b["launches"])


@pytest.mark.parametrize("shape", [1, 2, 3, 4, 5])
def test_every_stage_kernel_shape_gives_the_same_bits(swfd, monkeypatch, shape):
    """SWFD_STAGE32_SHAPE pins the stage kernel's launch shape (threads per
    tile x tiles per SM: 256x2, 320x2, 256x3, 256x4, 320x3); each gives the
    separate kernels' bits (ex4 switches, partial tiles, 12 steps)."""
    case = dict(problem=abi.SEDOV_2D, nx=70, ny=50)
    a = run(monkeypatch, "split", case, 12)
    monkeypatch.setenv("SWFD_STAGE32_SHAPE", str(shape))
    b = run(monkeypatch, "fused", case, 12)
    monkeypatch.delenv("SWFD_STAGE32_SHAPE")
    assert a["t"] == b["t"] and a["stats"] == b["stats"]
    assert np.array_equal(a["u"].view(np.uint64), b["u"].view(np.uint64))


def test_batched_fused_stage_equals_separate_kernels(swfd, monkeypatch):
    """The batch engine takes the fused FP32 stage when every running slot is
    2D without rank segments or limiter (kb_alpha_terms32, kb_stage32 over
    all slots' tiles); against its separate kernels each instance keeps its
    bits, time and statistics."""
    from sweeping_fd_weno_gb300 import Batch
    mix = [dict(problem=abi.VORTEX_2D, nx=45, ny=45), dict(problem=abi.SEDOV_2D, nx=70, ny=50),
           dict(problem=abi.JET_2D, nx=96, ny=24), dict(problem=abi.VORTEX_2D, nx=64, ny=48)]
    out = {}
    for mode in ("split", "fused"):
        monkeypatch.setenv("SWFD_FP32_STAGE", mode)
        with Batch(max_slots=4, max_nx=128, max_ny=128, precision=F32) as b:
            for k, m in enumerate(mix):
                kw = dict(m)
                assert b.admit(problems.make_config(kw.pop("problem"), precision=F32, **kw), k)
            assert b.run(8) >= 1
            out[mode] = [(b.download(k), b.stats(k)) for k in range(len(mix))]
    for k, (((ua, ta), sa), ((ub, tb), sb)) in enumerate(zip(out["split"], out["fused"])):
        assert ta == tb and sa == sb, k
        assert np.array_equal(ua.view(np.uint64), ub.view(np.uint64)), k
