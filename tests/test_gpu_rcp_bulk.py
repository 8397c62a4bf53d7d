"""The FP32-bulk form's integer-pipe helpers against the hardware: the
reciprocal (sd::div(1, x)) equals IEEE division bit for bit, and the
binary64 <-> binary32 conversions equal the round-to-nearest conversions."""
import ctypes as C

import numpy as np
import pytest

from sweeping_fd_weno_gb300 import abi

pytestmark = pytest.mark.gpu


def test_rcp_bulk_is_the_ieee_reciprocal(swfd):
    rng = np.random.default_rng(5)
    x = np.concatenate([
        10.0 ** rng.uniform(-30, 30, 200000) * rng.choice([-1.0, 1.0], 200000),
        np.array([1.0, 3.0, 7.0, 0.1, 1e-14, 7.8e-15, 1 - 2.0 ** -53, 1 + 2.0 ** -52, 2.0 ** 100,
                  2.0 ** -100, 1e-300, 1e300, 5e-324, -1e-310, 0.0, -0.0, np.inf, 1.7e308]),
    ])
    out = np.empty_like(x)
    dp = C.POINTER(C.c_double)
    st = abi.load_probe().swfd_probe_rcp_bulk(0, x.ctypes.data_as(dp), x.size, out.ctypes.data_as(dp))
    assert st == abi.OK
    with np.errstate(divide="ignore", over="ignore"):
        ref = 1.0 / x
    assert np.array_equal(out.view(np.uint64), ref.view(np.uint64))


def test_conversions_match_hardware(swfd):
    """d2f / f2d (integer pipes) equal numpy's round-to-nearest-even
    conversions bit for bit, on every class of binary64 value."""
    rng = np.random.default_rng(11)
    bits = rng.integers(0, 2**63, size=1 << 18, dtype=np.uint64) | \
        (rng.integers(0, 2, size=1 << 18, dtype=np.uint64) << np.uint64(63))
    x = bits.view(np.float64)
    near = rng.uniform(-1, 1, 1 << 18) * np.exp2(rng.integers(-160, 140, 1 << 18).astype(np.float64))
    ties = (rng.integers(1, 2**23, 1 << 14).astype(np.float64) + 0.5) * np.exp2(
        rng.integers(-150, 100, 1 << 14).astype(np.float64))  # binary32 midpoints
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 3.4028235677973366e38,
                        3.4028234663852886e38, 1.1754943508222875e-38, 1.401298464324817e-45,
                        7.006492321624085e-46, 1e-50, -1e-50, 1e300, -1e300])
    x = np.ascontiguousarray(np.concatenate([x, near, ties, special]))
    f = np.empty(x.size, np.float32)
    d = np.empty(x.size, np.float64)
    dp = C.POINTER(C.c_double)
    st = abi.load_probe().swfd_probe_convert(0, x.ctypes.data_as(dp), x.size,
                                       f.ctypes.data_as(C.POINTER(C.c_float)), d.ctypes.data_as(dp))
    assert st == 0
    with np.errstate(over="ignore", invalid="ignore"):
        ref = x.astype(np.float32)
    same_f = (f.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(f) & np.isnan(ref))
    assert same_f.all(), x[~same_f][:5]
    ref_d = ref.astype(np.float64)
    same_d = (d.view(np.uint64) == ref_d.view(np.uint64)) | (np.isnan(d) & np.isnan(ref_d))
    assert same_d.all(), ref[~same_d][:5]
