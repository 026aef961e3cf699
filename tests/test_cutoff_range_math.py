"""The geometry behind the kernels' inner-cutoff ranges, on the CPU.

A band's inner-cutoff factor 1 - e^-y, y = (R/delta_r)^20 (number_density.py:109), is exactly
1.0f in float32 once e^-y is below half an ulp of 1 (y > 17.3), and the adjoint's log-derivative
y e^-y / (1 - e^-y) exactly +0 once ex2.approx.ftz of -y log2(e) flushes to zero (y > 88).  The
paired DIRBE kernels evaluate both only at the nodes of a warp-uniform range: the nodes whose
abscissa lies in the interval where R < 1.26 delta_r (cutoff_interval in zl_f32.cuh), united
over the warp.  This mirrors the interval in float32 and checks, in float64 geometry over random
observers, directions, band widths and quadrature degrees, that every node outside it has
y > 88 -- so the constants the kernels take there are the values they would compute.
"""

import numpy as np

Y_FLUSH = 127.0 / np.log2(np.e)  # y beyond which ex2.approx.ftz(-y log2 e) is flushed to zero


def cutoff_interval(h, w, b2, inv_dr2):
    """numpy float32 mirror of cutoff_interval: (x1, x2), x1 > x2 when empty."""
    f = np.float32
    h, w, b2, inv_dr2 = f(h), f(w), f(b2), f(inv_dr2)
    D = f(1.5876) / inv_dr2 - b2
    if not D > 0:
        return np.inf, -np.inf
    sq = np.sqrt(D)
    if not h > 0:
        return (-np.inf, np.inf) if abs(w) < sq else (np.inf, -np.inf)
    ih = f(1) / h
    return float((-w - sq) * ih), float((sq - w) * ih)


def node_range(nodes, x1, x2):
    """Node indices [lo, hi) with x1 <= x <= x2 (warp_node_range for one lane)."""
    if not x1 <= x2:
        return 0, 0
    lo = int(np.searchsorted(nodes, x1, side="left"))
    hi = int(np.searchsorted(nodes, x2, side="right"))
    return lo, hi


def test_nodes_outside_the_range_have_exact_constants():
    rng = np.random.default_rng(11)
    checked = inside = 0
    for degree in (50, 100):
        nodes = np.polynomial.legendre.leggauss(degree)[0].astype(np.float32).astype(np.float64)
        for _ in range(3000):
            delta_r = rng.uniform(0.5, 2.0)  # the bands' inner-cutoff radii (0.94 and 1.5 AU for DIRBE)
            r_obs = rng.uniform(0.3, 5.0)
            phi = rng.uniform(0, 2 * np.pi)
            obs = np.array([r_obs * np.cos(phi), r_obs * np.sin(phi), rng.normal(0, 0.05)])
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            beta = u @ obs
            disc = beta * beta - (obs @ obs - 5.2**2)
            if disc <= 0:
                continue
            start = 0.0 if r_obs < 5.2 else max(-beta - np.sqrt(disc), 0.0)
            stop = -beta + np.sqrt(disc)
            hs, mid = 0.5 * (stop - start), 0.5 * (stop + start)
            b2 = max(obs @ obs - beta * beta, 0.0)
            x1, x2 = cutoff_interval(hs, mid + beta, b2, 1.0 / delta_r**2)
            lo, hi = node_range(nodes, x1, x2)
            inside += hi - lo
            outside = np.r_[nodes[:lo], nodes[hi:]]
            if outside.size == 0:
                continue
            X = obs[:, None] + (hs * outside + mid)[None, :] * u[:, None]
            y = (np.linalg.norm(X, axis=0) / delta_r) ** 20
            assert np.all(y > Y_FLUSH), (float(np.min(y)), delta_r, r_obs)
            checked += outside.size
    assert checked > 100_000 and inside > 10_000


def test_constants_are_what_float32_computes_beyond_the_flush():
    """At y > 88: 1 - e^-y is 1.0f and y e^-y / (1 - e^-y) is +0 when e^-y is flushed, and
    1 - e^-y already rounds to 1.0f from y = 18 on (the forward's margin)."""
    f = np.float32
    for y in (f(18.0), f(88.1), f(101.0), f(1e4)):
        e = np.exp2(-y * f(np.log2(np.e)), dtype=np.float32)
        if y > Y_FLUSH:
            e = f(0)  # ex2.approx.ftz: the subnormal result is flushed
        t4 = f(1) - e
        assert t4 == f(1)
        if y > Y_FLUSH:
            assert (y * e) * (f(1) / t4) == f(0)


def test_empty_and_whole_ranges():
    # a line of sight that never comes within 1.26 delta_r of the Sun: no node needs the factor
    assert cutoff_interval(2.0, 3.0, 9.0, 1.0) == (np.inf, -np.inf)
    # a point-like range (h = 0) inside the radius: every node
    assert cutoff_interval(0.0, 0.1, 0.2, 1.0) == (-np.inf, np.inf)
    nodes = np.linspace(-0.99, 0.99, 50)
    assert node_range(nodes, np.inf, -np.inf) == (0, 0)
    assert node_range(nodes, -np.inf, np.inf) == (0, 50)
