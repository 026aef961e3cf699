"""HEALPix RING-scheme pixel centres (Gorski et al. 2005, ApJ 622, 759, sec. 4).

Only what the benchmarks and tests need: the unit vector of every pixel centre
of a full-sky map, vectorised over int64 pixel indices.  The polar-cap
co-latitude is carried as 1 - z = i^2 / (3 nside^2) so that sin(theta) keeps
full precision near the poles.
"""

from __future__ import annotations

import numpy as np


def npix(nside: int) -> int:
    return 12 * nside * nside


def pix2vec_ring(nside: int, pix=None) -> np.ndarray:
    """(3, n) float64 unit vectors of RING pixel centres (all pixels if ``pix`` is None)."""
    nside = int(nside)
    if nside < 1:
        raise ValueError("nside must be >= 1")
    n_pix = npix(nside)
    p = np.arange(n_pix, dtype=np.int64) if pix is None else np.asarray(pix, dtype=np.int64)
    if np.any((p < 0) | (p >= n_pix)):
        raise ValueError("pixel index out of range")
    ncap = 2 * nside * (nside - 1)
    z = np.empty(p.shape, dtype=np.float64)
    one_minus_z = np.empty(p.shape, dtype=np.float64)
    phi = np.empty(p.shape, dtype=np.float64)
    fact = 1.0 / (3.0 * nside * nside)

    north = p < ncap
    if np.any(north):
        pn = p[north]
        i = (1 + np.floor(np.sqrt(1.0 + 2.0 * pn)).astype(np.int64)) // 2  # ring index 1..nside-1
        # guard the float sqrt at ring boundaries
        i = np.where(2 * i * (i - 1) > pn, i - 1, i)
        i = np.where(2 * (i + 1) * i <= pn, i + 1, i)
        j = pn + 1 - 2 * i * (i - 1)
        omz = i.astype(np.float64) ** 2 * fact
        one_minus_z[north] = omz
        z[north] = 1.0 - omz
        phi[north] = (j - 0.5) * np.pi / (2.0 * i)

    south = p >= n_pix - ncap
    if np.any(south):
        ps = n_pix - p[south]  # 1..ncap
        i = (1 + np.floor(np.sqrt(2.0 * ps - 1.0)).astype(np.int64)) // 2
        i = np.where(2 * i * (i - 1) >= ps, i - 1, i)
        i = np.where(2 * (i + 1) * i < ps, i + 1, i)
        j = 4 * i + 1 - (ps - 2 * i * (i - 1))
        omz = i.astype(np.float64) ** 2 * fact  # 1 + z
        z[south] = omz - 1.0
        one_minus_z[south] = 2.0 - omz
        phi[south] = (j - 0.5) * np.pi / (2.0 * i)

    belt = ~(north | south)
    if np.any(belt):
        pb = p[belt] - ncap
        i = pb // (4 * nside) + nside  # ring index nside..3 nside
        j = pb % (4 * nside) + 1
        s = (i - nside + 1) % 2
        zb = (2.0 * nside - i) * 2.0 / (3.0 * nside)
        z[belt] = zb
        one_minus_z[belt] = 1.0 - zb
        phi[belt] = (j - s / 2.0) * np.pi / (2.0 * nside)

    sin_theta = np.sqrt(one_minus_z * (1.0 + z))
    return np.stack([sin_theta * np.cos(phi), sin_theta * np.sin(phi), z])


def random_sphere(n: int, seed: int) -> np.ndarray:
    """(3, n) unit vectors uniform on the sphere (normalised Gaussians), seeded."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((3, int(n)))
    return v / np.linalg.norm(v, axis=0)


def pix2vec_ring_torch(nside: int, device="cuda"):
    """(3, 12 nside^2) float64 RING pixel centres computed on the device (same formulas as pix2vec_ring)."""
    import torch

    nside = int(nside)
    n_pix = npix(nside)
    p = torch.arange(n_pix, dtype=torch.int64, device=device)
    ncap = 2 * nside * (nside - 1)
    fact = 1.0 / (3.0 * nside * nside)
    z = torch.empty(n_pix, dtype=torch.float64, device=device)
    omz = torch.empty_like(z)
    phi = torch.empty_like(z)

    north = p < ncap
    pn = p[north]
    i = (1 + torch.floor(torch.sqrt(1.0 + 2.0 * pn.double())).long()) // 2
    i = torch.where(2 * i * (i - 1) > pn, i - 1, i)
    i = torch.where(2 * (i + 1) * i <= pn, i + 1, i)
    j = pn + 1 - 2 * i * (i - 1)
    o = i.double() ** 2 * fact
    omz[north], z[north] = o, 1.0 - o
    phi[north] = (j.double() - 0.5) * torch.pi / (2.0 * i.double())

    south = p >= n_pix - ncap
    ps = n_pix - p[south]
    i = (1 + torch.floor(torch.sqrt(2.0 * ps.double() - 1.0)).long()) // 2
    i = torch.where(2 * i * (i - 1) >= ps, i - 1, i)
    i = torch.where(2 * (i + 1) * i < ps, i + 1, i)
    j = 4 * i + 1 - (ps - 2 * i * (i - 1))
    o = i.double() ** 2 * fact
    z[south], omz[south] = o - 1.0, 2.0 - o
    phi[south] = (j.double() - 0.5) * torch.pi / (2.0 * i.double())

    belt = ~(north | south)
    pb = p[belt] - ncap
    i = pb // (4 * nside) + nside
    j = pb % (4 * nside) + 1
    s = (i - nside + 1) % 2
    zb = (2.0 * nside - i.double()) * 2.0 / (3.0 * nside)
    z[belt], omz[belt] = zb, 1.0 - zb
    phi[belt] = (j.double() - s.double() / 2.0) * torch.pi / (2.0 * nside)

    st = torch.sqrt(omz * (1.0 + z))
    return torch.stack([st * torch.cos(phi), st * torch.sin(phi), z])
