"""Approximate heliocentric positions of Earth and Mars (host-side set-up only).

The reference asks astropy/erfa for Earth's heliocentric ecliptic position
(``zodipy/bodies.py:53-62``).  astropy is optional here, so without it the
positions come from the published low-precision method of E. M. Standish,
"Keplerian Elements for Approximate Positions of the Major Planets" (JPL,
Table 1, valid 1800-2050): mean J2000 ecliptic elements with linear rates,
Kepler's equation solved by Newton iteration.  It is good to ~1e-4 AU for
the Earth-Moon barycentre, which is what is returned for "earth".  The
position only enters the Earth-trailing feature's longitude and the default
observer; callers that need ephemeris-grade positions pass them explicitly.
When astropy is importable the front end uses it instead.
"""

from __future__ import annotations

import numpy as np

# (a [AU], e, I [deg], L [deg], long. perihelion [deg], long. asc. node [deg]) and rates per century
_ELEMENTS = {
    "earth": (
        (1.00000261, 0.01671123, -0.00001531, 100.46457166, 102.93768193, 0.0),
        (0.00000562, -0.00004392, -0.01294668, 35999.37244981, 0.32327364, 0.0),
    ),
    "mars": (
        (1.52371034, 0.09339410, 1.84969142, -4.55343205, -23.94362959, 49.55953891),
        (0.00001847, 0.00007882, -0.00813131, 19140.30268499, 0.44441088, -0.29257343),
    ),
}

MEAN_DIST_TO_L2 = 0.009896235034000056  # AU, zodipy/bodies.py:13


def _position(body: str, jd: np.ndarray) -> np.ndarray:
    el0, rate = _ELEMENTS[body]
    T = (np.asarray(jd, dtype=np.float64) - 2451545.0) / 36525.0
    a, e, inc, L, varpi, node = (el0[k] + rate[k] * T for k in range(6))
    omega = np.radians(varpi - node)
    M = np.radians(np.mod(L - varpi + 180.0, 360.0) - 180.0)
    E = M + e * np.sin(M)
    for _ in range(8):
        E = E - (E - e * np.sin(E) - M) / (1.0 - e * np.cos(E))
    xp = a * (np.cos(E) - e)
    yp = a * np.sqrt(1.0 - e * e) * np.sin(E)
    co, so = np.cos(omega), np.sin(omega)
    cn, sn = np.cos(np.radians(node)), np.sin(np.radians(node))
    ci, si = np.cos(np.radians(inc)), np.sin(np.radians(inc))
    x = (co * cn - so * sn * ci) * xp + (-so * cn - co * sn * ci) * yp
    y = (co * sn + so * cn * ci) * xp + (-so * sn + co * cn * ci) * yp
    z = (so * si) * xp + (co * si) * yp
    return np.stack([x, y, z])


def mjd_to_jd(mjd) -> np.ndarray:
    return np.asarray(mjd, dtype=np.float64) + 2400000.5


def body_position(body: str, mjd) -> np.ndarray:
    """Heliocentric ecliptic (J2000) position [AU], shape (3,) or (3, n)."""
    body = body.lower()
    if body in _ELEMENTS:
        return _position(body, mjd_to_jd(mjd))
    if body == "sun":
        shape = np.shape(mjd)
        return np.zeros((3, *shape))
    if body == "semb-l2":
        return semb_l2(_position("earth", mjd_to_jd(mjd)))
    raise ValueError(
        f"Invalid observer string: '{body}'. Valid observers without astropy are: earth, mars, sun, semb-l2"
    )


def semb_l2(earth_xyz: np.ndarray) -> np.ndarray:
    """SEMB-L2: Earth's direction from the Sun, pushed out by the mean L2 distance (``bodies.py:38-50``)."""
    d = np.linalg.norm(earth_xyz, axis=0)
    return earth_xyz / d * (d + MEAN_DIST_TO_L2)


def iso_to_mjd(iso: str) -> float:
    """ISO-8601 'YYYY-MM-DD[ THH:MM[:SS]]' (UTC taken as TT) to MJD."""
    iso = iso.strip().replace("T", " ")
    date, _, clock = iso.partition(" ")
    y, mo, d = (int(v) for v in date.split("-"))
    hh = mm = 0
    ss = 0.0
    if clock:
        parts = clock.split(":")
        hh = int(parts[0])
        mm = int(parts[1]) if len(parts) > 1 else 0
        ss = float(parts[2]) if len(parts) > 2 else 0.0
    # Fliegel & Van Flandern (1968) Julian day number
    a = (14 - mo) // 12
    yy = y + 4800 - a
    m2 = mo + 12 * a - 3
    jdn = d + (153 * m2 + 2) // 5 + 365 * yy + yy // 4 - yy // 100 + yy // 400 - 32045
    jd = jdn - 0.5 + (hh + mm / 60.0 + ss / 3600.0) / 24.0
    return jd - 2400000.5


def earth_position(mjd) -> np.ndarray:
    return body_position("earth", mjd)


__all__ = ["body_position", "earth_position", "iso_to_mjd", "semb_l2"]
