"""Fit of the polynomial in atan2_poly (zodipy_gb300/csrc/zl_common.cuh).

atan t = t + t^3 Q(t^2) on t in [0, 1]; Q of degree 7 minimises the maximum relative
error of atan by iteratively reweighted least squares (Lawson's method) on
Chebyshev-distributed points.  Prints the coefficients (low order first) as float32
literals and the float32-evaluated error of atan on [0, 1] and of the octant-reduced
atan2 on random points (FMA emulated in float64, the reciprocal correctly rounded).

    python tests/atan2_fit.py

tests/test_atan2_fit.py re-derives the coefficients with this fit and checks them
against the ones compiled into the kernels.
"""

import numpy as np

DEG = 7


def fit(deg: int, iters: int = 80) -> np.ndarray:
    n = 6000
    t = 0.5 * (1 - np.cos(np.pi * (np.arange(n) + 0.5) / n))
    t = t[t > 1e-4]
    s = t * t
    g = (np.arctan(t) - t) / t**3
    a = np.vstack([s**k for k in range(deg + 1)]).T
    wt = t**3 / np.arctan(t)  # error of Q -> relative error of atan
    w = np.ones_like(s)
    for _ in range(iters):
        sw = np.sqrt(w) * wt
        c, *_ = np.linalg.lstsq(a * sw[:, None], g * sw, rcond=None)
        e = np.abs(a @ c - g) * wt
        w = w * (e / e.max()) ** 0.5 + 1e-30
        w /= w.sum()
    return c


def f32(x):
    return np.asarray(x, dtype=np.float64).astype(np.float32).astype(np.float64)


def fma(a, b, c):
    return f32(a * b + c)


def atan_poly(c, t):
    s = f32(t * t)
    q = np.full_like(t, f32(c[-1]))
    for k in range(len(c) - 2, -1, -1):
        q = fma(q, s, f32(c[k]))
    return fma(f32(t * s), q, t)


def atan2_model(c, y, x):
    ax, ay = np.abs(x), np.abs(y)
    t = f32(np.minimum(ax, ay) * f32(1.0 / np.maximum(np.maximum(ax, ay), 1e-37)))
    r = atan_poly(c, t)
    r = np.where(ay > ax, f32(f32(np.pi / 2) - r), r)
    r = np.where(x < 0, f32(f32(np.pi) - r), r)
    return np.copysign(r, y)


def main() -> None:
    c = fit(DEG)
    print("coefficients:", ", ".join(str(np.float32(v)) + "f" for v in c))
    t = f32(np.linspace(0, 1, 400001))
    ref = np.arctan(t)
    ulp = np.spacing(np.maximum(ref, 1e-30).astype(np.float32)).astype(np.float64)
    print("atan on [0, 1]: max", np.max(np.abs(atan_poly(c, t) - ref) / ulp), "ulp")
    rng = np.random.default_rng(1)
    y, x = f32(rng.standard_normal(1 << 21)), f32(rng.standard_normal(1 << 21))
    ref2 = np.arctan2(y, x)
    err = np.abs(atan2_model(c, y, x) - ref2) / np.spacing(np.abs(ref2).astype(np.float32)).astype(np.float64)
    print("atan2: max", err.max(), "ulp")


if __name__ == "__main__":
    main()
