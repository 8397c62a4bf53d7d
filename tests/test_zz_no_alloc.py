"""swfd_flux_divergence_static, the entry point that allocates nothing.

Some callers cannot call cudaMalloc (a framework allocator owns the device
memory, or allocation is not allowed in their loop); they hand the library
device pointers for the input state and the output, and the library keeps its
intermediates in one static device array.  This test calls that entry point
through the C ABI on device buffers and checks its RHS against the handle
based swfd_flux_divergence, value for value, on two calls in a row (the second
call sees the first call's leftovers in the shared array), and for the FP64
forms also against the CPU oracle's wenofd + scheme.  The FP32-bulk form has
no oracle counterpart (it is not bit-exact by design); there the handle path
is the reference.  The file sorts last so that a run stopping at the first
failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Solver, abi, problems

pytestmark = pytest.mark.gpu

CASES = [
    dict(problem=abi.VORTEX_2D, nx=45, ny=45),
    dict(problem=abi.JET_2D, nx=96, ny=24),
    dict(problem=abi.SEDOV_2D, nx=64, ny=40),
    dict(problem=abi.SEDOV_1D, nx=800, cfl=0.6, swp_num=2, e_background=1e-12),
    # the FP32-bulk planes and flux kernel
    dict(problem=abi.VORTEX_2D, nx=45, ny=45, precision=abi.PRECISION_FP32_BULK),
    # the positivity flux limiter epilogue (use_limiter = 1)
    dict(problem=abi.SEDOV_2D, nx=48, ny=48, use_limiter=1),
]


def _case_id(c):
    tag = f"p{c['problem']}_{c['nx']}"
    if c.get("precision") == abi.PRECISION_FP32_BULK:
        tag += "_fp32bulk"
    if c.get("use_limiter") == 1:
        tag += "_limiter"
    return tag


def _perturbed(u, rng):
    v = u.copy()
    v[..., 0] *= 1.0 + 1e-3 * rng.standard_normal(v.shape[:-1])
    v[..., -1] *= 1.0 + 1e-3 * rng.standard_normal(v.shape[:-1])
    return v


@pytest.mark.parametrize("case", CASES, ids=_case_id)
def test_static_entry_matches_handle_entry_on_two_calls(case, oracle_mod):
    torch = pytest.importorskip("torch")
    kw = dict(case)
    p = kw.pop("problem")
    cfg = problems.make_config(p, **kw)
    lib = abi.load()
    rng = np.random.default_rng(17)
    with Solver(problems.make_config(p, **kw)) as s:
        s.init_problem()
        inputs = [s.state()]
        inputs.append(_perturbed(inputs[0], rng))
        refs = []
        for u in inputs:
            s.set_state(u)
            refs.append(s.flux_divergence())
    if kw.get("precision", abi.PRECISION_FP64) == abi.PRECISION_FP64:
        o = oracle_mod.Oracle(problems.make_config(p, **kw))
        o.init_problem()
        for u, ref in zip(inputs, refs):
            o.set_state(u)
            assert not (~(o.flux_divergence() == ref)).any(), "handle path differs from the oracle"
    stream = torch.cuda.current_stream(0)
    for u, ref in zip(inputs, refs):
        du = torch.from_numpy(u).to("cuda:0")
        dr = torch.full_like(du, float("nan"))
        st = lib.swfd_flux_divergence_static(C.byref(cfg), C.c_void_p(du.data_ptr()),
                                             C.c_void_p(dr.data_ptr()),
                                             C.c_void_p(stream.cuda_stream))
        assert st == abi.OK, abi.last_error()
        stream.synchronize()
        out = dr.cpu().numpy()
        bad = ~(out == ref)
        assert not bad.any(), f"{int(bad.sum())} RHS values differ from swfd_flux_divergence"


def test_static_entry_rejects_grids_beyond_its_scratch():
    cfg = problems.make_config(abi.VORTEX_2D, nx=200, ny=200)
    lib = abi.load()
    st = lib.swfd_flux_divergence_static(C.byref(cfg), C.c_void_p(1), C.c_void_p(1), None)
    assert st == abi.ERR_INVALID
    assert "static limit" in abi.last_error()
