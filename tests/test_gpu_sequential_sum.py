"""The u_bar summation of sweep_lim, s = s + w*x(m) rounded in order, as the
GPU evaluates it (integer runs inside a binade plus single hardware steps)
against the plain sequential loop in IEEE double, on inputs built to hit
every branch: rounding ties, binade crossings both ways, sign changes, zero,
subnormal and non-finite values."""
import ctypes as C
import math

import numpy as np
import pytest

from sweeping_fd_weno_gb300 import abi

pytestmark = pytest.mark.gpu


def seq(x, w):
    s = 0.0
    for v in x.tolist():
        s = s + w * v
    return s


def gpu(x, w):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = C.c_double()
    abi.check(abi.load().swfd_sequential_sum(abi.dptr(x), x.size, w, 0, C.byref(out)))
    return out.value


def same(a, b):
    return (math.isnan(a) and math.isnan(b)) or a == b and math.copysign(1, a) == math.copysign(1, b)


def cases():
    rng = np.random.default_rng(11)
    n384 = 384 * 384
    yield "empty", np.zeros(0), 1.0
    yield "one", np.array([3.0]), 0.1
    yield "uniform density", np.ones(n384), 1.0 / n384
    yield "random mixed signs", rng.normal(size=100_000), 1.0 / 100_000
    yield "positive lognormal", rng.lognormal(0, 6, size=50_000), 1.0 / 50_000
    # ties: 2^53 + 1 rounds to even, then half-ulp steps at several binades
    t = [2.0 ** 53] + [1.0, 1.0, 3.0, 1.0, -1.0, 5.0] * 500
    yield "ties at 2^53", np.array(t), 1.0
    k = rng.integers(-40, 40, size=20_000)
    yield "ties at many binades", np.ldexp(rng.integers(1, 4, size=20_000) * 1.0, k), 1.0
    yield "half-integers", rng.integers(-8, 9, size=30_000) * 0.5 + 2.0 ** 52, 1.0
    # the running sum crossing zero and binade edges both ways
    a = np.tile([1.0, -1.0, 0.75, -0.75, 2.0 ** -30, -2.0 ** -30], 4000)
    yield "sign changes", a + rng.normal(scale=1e-9, size=a.size), 0.5
    yield "exact binade edges", np.array([1.0, 1.0, 2.0, 4.0, -4.0, -3.0, 1.5, 0.25] * 3000), 1.0
    yield "negative sums", -rng.lognormal(0, 3, size=40_000), 1.0 / 40_000
    big = rng.normal(size=10_000)
    big[::7] *= 1e300
    big[::11] *= 1e-300
    yield "huge range", big, 1.0
    yield "subnormals", np.concatenate([np.full(5000, 5e-324), rng.normal(size=5000) * 1e-310,
                                        np.full(5000, 2.2e-308)]), 1.0
    yield "near vacuum background", np.concatenate([[0.244816 / 1e-6], np.full(n384, 1e-12)]), 1.0 / n384
    yield "zeros and signed zeros", np.array([0.0, -0.0, 0.0, -0.0] * 1000), 1.0
    inf = np.ones(6000)
    inf[3000] = np.inf
    yield "infinity", inf, 1.0
    nan = np.ones(6000)
    nan[10] = np.inf
    nan[20] = -np.inf
    yield "inf - inf", nan, 1.0
    yield "overflow", np.full(5000, 1.7e308), 1.0
    # lengths at the 2048-term chunks of the summation, a tie on a chunk edge,
    # and a random walk (a sum that keeps changing binade: many single steps)
    for n in (2047, 2048, 2049, 6145):
        yield f"chunk edge {n}", rng.lognormal(0, 2, size=n), 1.0 / n
    t = np.ones(3 * 2048)
    t[0] = 2.0 ** 53
    yield "ties across chunk edges", t, 1.0
    yield "random walk", rng.normal(size=60_000), 1.0 / 60_000


@pytest.mark.parametrize("name,x,w", list(cases()), ids=[c[0] for c in cases()])
def test_sequential_sum_bit_exact(swfd, name, x, w):
    a, b = gpu(x, w), seq(x, w)
    assert same(a, b), (name, a.hex() if math.isfinite(a) else a, b.hex() if math.isfinite(b) else b)
