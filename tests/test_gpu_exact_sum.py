"""The exact sums behind the resident CG's reductions (exactsum.cuh) against
math.fsum, the correctly rounded sum: bit-equal whenever the terms span
fewer than 2^64 below the largest term's last bit; otherwise within 2^-100
of the largest term."""
import math

import numpy as np
import pytest

from help_gb300 import native

pytestmark = pytest.mark.gpu


def exact_sums(x):
    x = np.ascontiguousarray(x, np.float64)
    out = np.zeros(3)
    assert native.gpu_lib().help_exact_sum(native.ptr(x), len(x), native.ptr(out)) == native.HELP_OK
    return out


def bits(v):
    return np.float64(v).view(np.int64)


@pytest.mark.parametrize("seed", range(12))
def test_bit_equal_to_fsum(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 257))
    spread = [0, 10, 40, 55][seed % 4]
    x = rng.standard_normal(n) * np.exp2(rng.integers(-spread, 1, n).astype(float))
    if seed % 3 == 1:  # heavy cancellation
        x[: n // 2] = -x[n - n // 2 - (n // 2):][: n // 2] if n > 1 else x[: n // 2]
    out = exact_sums(x)
    assert bits(out[0]) == bits(math.fsum(x))
    assert bits(out[1]) == bits(math.fsum(x[:16]))
    assert bits(out[2]) == bits(math.fsum(x[:96]))


def test_special_values():
    z = exact_sums(np.zeros(40))
    assert np.all(z == 0.0)
    sub = np.array([5e-324, 5e-324, -1e-320, 3e-310])
    assert bits(exact_sums(sub)[0]) == bits(math.fsum(sub))
    big = np.array([1e308, 1e308, -1e308])
    assert exact_sums(big)[0] == 1e308  # the exact sum fits though a running sum would overflow
    nan = np.ones(20)
    nan[7] = np.nan
    assert np.all(np.isnan(exact_sums(nan)))
    inf = np.ones(20)
    inf[3] = np.inf
    assert np.all(exact_sums(inf) == np.inf)


def test_wide_spread_error_bound():
    rng = np.random.default_rng(7)
    x = rng.standard_normal(256) * np.exp2(rng.integers(-300, 1, 256).astype(float))
    got = exact_sums(x)[0]
    assert abs(got - math.fsum(x)) <= 2.0 ** -100 * np.abs(x).max()
