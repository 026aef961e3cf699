"""The float-float square root and division of the sphere intersections (ff_sqrt, ff_div in
zl_common.cuh), emulated in numpy float32 on the CPU.

Both take one Newton correction from an FP32 estimate and form the residual (a - s^2, a - b q)
with three additions, relying on the leading difference being exact: the estimate is within a
few ulps, so s^2 (or b q) lies within a factor 2 of a.hi (Sterbenz).  The emulation perturbs
the reciprocal-square-root and reciprocal estimates by up to two ulps, as the approximate
instructions may be off, checks that the leading difference is exact, and bounds the relative
error: 2^-42 for both (float-float operands carry 2^-48).
"""

import numpy as np

f = np.float32


def fma(a, b, c):
    # float32 a * b is exact in float64; one rounding of the sum to float64, then to float32 (a
    # double rounding only where the float64 sum is inexact, far below the bounds checked here)
    return f(np.float64(a) * np.float64(b) + np.float64(c))


def quick(a, b):
    s = f(a + b)
    return s, f(b - f(s - a))


def split(x):
    hi = f(x)
    return hi, f(x - np.float64(hi))


def nudge(x, rng):
    for _ in range(int(rng.integers(0, 3))):
        x = np.nextafter(x, f(np.inf) if rng.random() < 0.5 else f(-np.inf))
    return x


def test_sqrt_residual_is_exact_and_accurate():
    rng = np.random.default_rng(1)
    worst = 0.0
    for _ in range(20000):
        a = np.float64(10 ** rng.uniform(-6, 2))
        ah, al = split(a)
        r = nudge(f(1 / np.sqrt(np.float64(ah))), rng)
        s = f(ah * r)
        p = f(s * s)
        pe = fma(s, s, -p)
        assert np.float64(ah) - np.float64(p) == np.float64(f(ah - p))  # Sterbenz
        d = f(f(f(ah - p) - pe) + al)
        hi, lo = quick(s, f(f(d * f(0.5)) * r))
        ref = np.sqrt(np.float64(ah) + np.float64(al))
        worst = max(worst, abs(np.float64(hi) + np.float64(lo) - ref) / ref)
    assert worst < 2.0**-42, worst


def test_division_residual_is_exact_and_accurate():
    rng = np.random.default_rng(2)
    worst = 0.0
    for _ in range(20000):
        b = np.float64(rng.uniform(-20, 20))
        c = np.float64(rng.uniform(-20, 20))
        if abs(b) < 1e-3:
            continue
        bh, bl = split(b)
        ch, cl = split(c)
        rb = nudge(f(1 / np.float64(bh)), rng)
        q = f(ch * rb)
        p = f(bh * q)
        pe = fma(bh, q, -p)
        assert np.float64(ch) - np.float64(p) == np.float64(f(ch - p))  # Sterbenz
        res = fma(-bl, q, f(f(f(ch - p) - pe) + cl))
        hi, lo = quick(q, f(res * rb))
        ref = (np.float64(ch) + np.float64(cl)) / (np.float64(bh) + np.float64(bl))
        worst = max(worst, abs(np.float64(hi) + np.float64(lo) - ref) / abs(ref))
    assert worst < 2.0**-42, worst


def test_zero_divisor_gives_an_infinite_or_nan_quotient():
    """rcp(+-0) = +-inf: q = c * rcp is +-inf (c != 0) or NaN (c = 0), as c / 0 is; the
    intersection then takes its NaN branch."""
    with np.errstate(divide="ignore", invalid="ignore"):
        for c in (f(1.5), f(-2.0), f(0.0)):
            for z in (f(0.0), f(-0.0)):
                rb = f(1.0) / z
                q = f(c * rb)
                ieee = f(c / z)
                assert (np.isnan(q) and np.isnan(ieee)) or q == ieee
