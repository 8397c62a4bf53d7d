"""The FP32-bulk form's reciprocal (FP32 seed, two Newton steps in FP64)
against IEEE division: within two ulp over the magnitudes the form meets,
and the IEEE division itself outside the seed's range."""
import ctypes as C

import numpy as np
import pytest

from sweeping_fd_weno_gb300 import abi

pytestmark = pytest.mark.gpu


def test_rcp_bulk_within_two_ulp(swfd):
    rng = np.random.default_rng(5)
    x = np.concatenate([
        10.0 ** rng.uniform(-30, 30, 200000) * rng.choice([-1.0, 1.0], 200000),
        np.array([1.0, 3.0, 7.0, 0.1, 1e-14, 7.8e-15, 1 - 2.0 ** -53, 1 + 2.0 ** -52, 2.0 ** 100,
                  2.0 ** -100, 1e-300, 1e300, 5e-324, -1e-310]),
    ])
    out = np.empty_like(x)
    dp = C.POINTER(C.c_double)
    st = abi.load().swfd_probe_rcp_bulk(0, x.ctypes.data_as(dp), x.size, out.ctypes.data_as(dp))
    assert st == abi.OK
    with np.errstate(divide="ignore", over="ignore"):
        ref = 1.0 / x
    fin = np.isfinite(ref)
    assert np.array_equal(out[~fin], ref[~fin])
    err = np.abs(out[fin] - ref[fin]) / np.spacing(np.abs(ref[fin]))
    assert err.max() <= 2.0, (x[fin][err.argmax()], err.max())
    lg = np.log2(np.abs(x))
    far = (lg < -121) | (lg > 122)
    assert np.array_equal(out[far], ref[far])   # the IEEE division there
