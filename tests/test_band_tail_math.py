"""The geometry behind the kernels' band tails, on the CPU.

The float32 kernels stop evaluating a band at the nodes beyond the larger root of
    (a1 x + a0)^2 - c^2 ((h x + m)^2 + b^2) > 0,   c = 2.2 delta_zeta,
where a line of sight at node abscissa x has height Z = a1 x + a0 above the band's plane and
heliocentric distance R^2 = (h x + m)^2 + b^2.  Past that root the band factor
e^-(zeta/delta_zeta)^6 must be zero in float32 (zeta > 2.11 delta_zeta).  This mirrors the
estimate in float32 (zl_f32.cuh: band_zero_tail) and checks the claim in float64 geometry over
random observers and directions, including lines of sight that cross the plane.
"""

import numpy as np

FLUSH = (127.0 / np.log2(np.e)) ** (1.0 / 6.0)  # zeta / delta_zeta beyond which ex2 flushes to 0


def tail_root(a1, a0, h, m, b2, dzeta):
    """numpy float32 mirror of band_zero_tail (without the warp vote): +inf = no tail."""
    f = np.float32
    a1, a0, h, m, b2 = f(a1), f(a0), f(h), f(m), f(b2)
    c = f(2.2) * f(dzeta)
    c2 = c * c
    A = a1 * a1 - c2 * (h * h)
    if not A > 0:
        return np.inf
    B = f(2) * (a1 * a0 - c2 * (h * m))
    C = a0 * a0 - c2 * (m * m + b2)
    disc = B * B - f(4) * A * C
    if disc < 0:
        return -np.inf
    q = f(-0.5) * (B + np.copysign(np.sqrt(disc), B))
    with np.errstate(divide="ignore", invalid="ignore"):
        r = max(q / A, C / q)
    return np.inf if np.isnan(r) else float(r)


def test_nodes_past_the_root_are_flushed():
    rng = np.random.default_rng(7)
    checked = tails = 0
    for _ in range(4000):
        # band plane: inclination up to 2 deg; width 2-15 deg (DIRBE bands: 2, 8.8, 15)
        inc, node = np.radians(rng.uniform(0, 2)), rng.uniform(0, 2 * np.pi)
        n = np.array([np.sin(node) * np.sin(inc), -np.cos(node) * np.sin(inc), np.cos(inc)])
        dzeta = np.radians(rng.uniform(2, 15))
        r_obs = rng.uniform(0.5, 3.0)
        phi = rng.uniform(0, 2 * np.pi)
        obs = np.array([r_obs * np.cos(phi), r_obs * np.sin(phi), rng.normal(0, 0.05)])
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        # line of sight from the observer to the 5.2 AU sphere, nodes x in [-1, 1]
        beta = u @ obs
        stop = -beta + np.sqrt(beta * beta - (obs @ obs - 5.2**2))
        hs, mid = 0.5 * stop, 0.5 * stop
        a1, a0 = (u @ n) * hs, (u @ n) * mid + obs @ n
        m = mid + beta
        b2 = obs @ obs - beta * beta
        root = tail_root(a1, a0, hs, m, b2, dzeta)
        if root == np.inf:
            continue
        tails += 1
        xs = np.linspace(-1, 1, 2001)
        xs = xs[xs > root]
        if xs.size == 0:
            continue
        X = obs[:, None] + (hs * xs + mid)[None, :] * u[:, None]
        zeta = np.abs(n @ X) / np.linalg.norm(X, axis=0)
        assert np.all(zeta / dzeta > FLUSH), (root, float(np.min(zeta / dzeta)))
        checked += xs.size
    assert tails > 200 and checked > 100000


def test_no_tail_where_the_direction_stays_in_the_band():
    # a direction within 2.2 delta_zeta of the plane never leaves it: A <= 0, no tail
    dzeta = np.radians(8.0)
    u_n = 0.5 * 2.2 * dzeta
    assert tail_root(u_n * 2.0, 0.01, 2.0, 2.5, 0.3, dzeta) == np.inf
