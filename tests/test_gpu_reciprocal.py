"""The pivot reciprocal of the banded solves, LU5decompStep's 1.0d0/A(i,0)
(rbparmat_blocking.f90:41), formed by Newton-Raphson iteration on the FP64
pipe: against the correctly rounded quotient over the normal range, and the
IEEE quotient for zeros, subnormals, the largest magnitudes, Inf and NaN."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pivot_reciprocal_is_the_rounded_quotient(gpu_lib):
    from channel_gb300.lib import pivot_reciprocal

    rng = np.random.default_rng(0)
    n = 1 << 20
    m = rng.uniform(1.0, 2.0, n)
    m[:64] = 1.0  # significands at the ends of the FP32 start's range
    m[64:128] = np.nextafter(2.0, 0.0)
    m[128:192] = 1.0 + rng.integers(0, 1 << 23, 64) * 2.0**-23  # exact FP32 significands
    e = rng.integers(-1022, 1022, n)  # every normal binary exponent the iteration takes
    e[:8] = -1022
    e[8:16] = 1021
    x = np.ldexp(m, e) * rng.choice([-1.0, 1.0], n)
    y = pivot_reciprocal(x)
    ref = 1.0 / x
    ulps = np.abs(y.view(np.int64) - ref.view(np.int64))
    assert int(ulps.max()) <= 1, x[np.argmax(ulps)]
    # the iteration's value lies within 2^-88 relative of 1/x, so only a
    # quotient that close to a rounding midpoint can round the other way: the
    # significands next to 2 are such (1/(2 - 2^-52) = 0.5 + 2^-54 + 2^-106),
    # random ones practically never
    assert np.count_nonzero(ulps[192:]) <= 2, np.count_nonzero(ulps[192:])


def test_pivot_reciprocal_outside_the_iteration_range(gpu_lib):
    from channel_gb300.lib import pivot_reciprocal

    x = np.array([0.0, -0.0, 5e-324, -2.2e-308, 2.0**1022, -1.5 * 2.0**1022, 1.7e308, np.inf, -np.inf, np.nan])
    with np.errstate(divide="ignore", over="ignore"):
        ref = 1.0 / x
    y = pivot_reciprocal(x)
    assert np.array_equal(np.isnan(y), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.array_equal(y[ok], ref[ok]) and np.array_equal(np.signbit(y[ok]), np.signbit(ref[ok]))
