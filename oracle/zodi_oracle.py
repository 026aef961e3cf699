"""CPU oracle for ZodiPy's line-of-sight integral — TEST INFRASTRUCTURE ONLY.

This is a numpy restatement of the reference's hot path (zodipy v1.1.3).  It is
the checker for the CUDA kernels: only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline / reference arm may import it.  The product
package never calls it, and nothing here is used as a fallback.

Pinning: every function below is validated against outputs of the reference's
own modules (executed in place under an astropy stand-in by
``tests/golden/make_golden.py``) through the committed fixtures in
``tests/golden/``.  The blackbody table restates astropy's ``BlackBody`` and is
pinned only through the DIRBE IDL known-answer test at 1 % (see
``planck_table``).

Arithmetic follows the reference operation by operation (same expression
order, float64 throughout) so that the oracle agrees with the reference to a
few ulp, not merely to a tolerance.
"""

from __future__ import annotations

import numpy as np

# line_of_sight.py:14 — the "zero" radius used for the inner cutoff of the
# cloud and bands, and the value returned when the observer lies outside a
# cutoff sphere (line_of_sight.py:73).
EPS = np.finfo(np.float64).eps

# line_of_sight.py:19-26 — (inner, outer) cutoff radii per component type.
KELSALL_CUTOFFS = {
    "cloud": (EPS, 5.2),
    "band1": (EPS, 5.2),
    "band2": (EPS, 5.2),
    "band3": (EPS, 5.2),
    "ring": (1 - 0.2, 1 + 0.2),
    "feature": (1 - 0.3, 1 + 0.3),
}

# Physical constants (exact SI 2019 values, as in astropy 6 / CODATA 2018).
_H = 6.62607015e-34
_KB = 1.380649e-23
_C = 299792458.0


def planck_table(x, weights=None, unit="micron", n_temps=100, t_min=40.0, t_max=550.0):
    """Blackbody table ``[T_K, B_MJy/sr]`` of shape (2, n_temps).

    Restates ``zodipy/blackbody.py:9-13,33-49``: temperatures
    ``linspace(40, 550, 100)`` K, B_nu from astropy's ``BlackBody``
    (``2 h nu^3 / c^2 / expm1(h nu / k T)`` per steradian) converted to MJy/sr
    (x 1e20 from SI), and for a bandpass the trapezoid integral of
    ``weights * B`` over ``x`` with ``weights`` already normalised
    (``model.py:94``).  astropy is absent here, so this formula is parity
    unpinned beyond the 1 % DIRBE IDL known-answer test.
    """
    temps = np.linspace(t_min, t_max, n_temps)
    x = np.asarray(x, dtype=np.float64)
    if unit in ("micron", "um"):
        freq = _C / (x * 1e-6)
    elif unit == "GHz":
        freq = x * 1e9
    else:
        raise ValueError(unit)

    def bnu(f):
        f = np.asarray(f, dtype=np.float64)[..., np.newaxis]
        log_boltz = _H * f / (_KB * temps)
        return 2.0 * _H * f**3 / (_C**2 * np.expm1(log_boltz)) * 1e20

    if weights is None:
        vals = bnu(freq)
    else:
        vals = np.trapezoid(np.asarray(weights) * bnu(freq).T, x)
    return np.asarray([temps, np.asarray(vals, dtype=np.float64).reshape(n_temps)])


def component_geometry(comp: dict) -> dict:
    """Derived geometry of a component (``component.py:39-44,87-89,133-136``)."""
    g = {
        "X_0": np.expand_dims([comp["x_0"], comp["y_0"], comp["z_0"]], axis=-1),
        "sin_i_rad": np.sin(np.radians(comp["i"])),
        "cos_i_rad": np.cos(np.radians(comp["i"])),
        "sin_Omega_rad": np.sin(np.radians(comp["Omega"])),
        "cos_Omega_rad": np.cos(np.radians(comp["Omega"])),
    }
    if "delta_zeta" in comp:
        g["delta_zeta_rad"] = np.radians(comp["delta_zeta"])
    if "theta" in comp:
        g["theta_rad"] = np.radians(comp["theta"])
        g["sigma_theta_rad"] = np.radians(comp["sigma_theta"])
    return g


def sphere_intersection(obs_pos, unit_vectors, cutoff, fix_b0=False):
    """Distance from the observer to the heliocentric sphere of radius ``cutoff``.

    Follows ``line_of_sight.py:64-85`` including its three quirks: if ANY
    observer lies outside the sphere every line of sight gets ``EPS``
    (``:72-73``); ``b`` omits ``z_obs * u_z`` (``:80``); and ``b == 0`` gives
    nan (``:83``).  ``fix_b0=True`` evaluates the same root as
    ``-0.5 (b + copysign(sqrt(D), b))`` where ``b == 0`` — the documented
    behaviour of the CUDA kernels — and is otherwise identical.
    """
    x_0, y_0, z_0 = obs_pos
    r_obs = np.sqrt(x_0**2 + y_0**2 + z_0**2)
    if (r_obs > cutoff).any():
        return np.full(obs_pos.shape[-1], EPS)
    u_x, u_y, u_z = unit_vectors
    lon = np.arctan2(u_y, u_x)
    lat = np.arcsin(u_z)
    cos_lat = np.cos(lat)
    b = 2 * (x_0 * cos_lat * np.cos(lon) + y_0 * cos_lat * np.sin(lon))
    c = r_obs**2 - cutoff**2
    with np.errstate(divide="ignore", invalid="ignore"):
        q = -0.5 * b * (1 + np.sqrt(b**2 - 4 * c) / np.abs(b))
        if fix_b0:
            b_arr = np.broadcast_to(b, q.shape)
            zero = b_arr == 0
            if np.any(zero):
                q = np.array(q, copy=True)
                sq = np.sqrt(np.broadcast_to(b**2 - 4 * c, q.shape))
                q[zero] = -0.5 * (b_arr[zero] + np.copysign(sq[zero], b_arr[zero]))
        return np.maximum(q, c / q)


def los_range(comp_labels, cutoffs, unit_vectors, obs_pos, fix_b0=False):
    """Per-component (start, stop) arrays (``line_of_sight.py:88-105``)."""
    start = {c: sphere_intersection(obs_pos, unit_vectors, cutoffs[c][0], fix_b0) for c in comp_labels}
    stop = {c: sphere_intersection(obs_pos, unit_vectors, cutoffs[c][1], fix_b0) for c in comp_labels}
    return start, stop


def _dist_and_z(X_helio, geom):
    X = X_helio - geom["X_0"]
    R = np.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
    Z = (
        X[0] * geom["sin_Omega_rad"] * geom["sin_i_rad"]
        - X[1] * geom["cos_Omega_rad"] * geom["sin_i_rad"]
        + X[2] * geom["cos_i_rad"]
    )
    return X, R, Z


def cloud_density(X_helio, comp, geom):
    """Smooth cloud (``number_density.py:47-73``)."""
    _, R, Z = _dist_and_z(X_helio, geom)
    zeta = np.abs(Z / R)
    mu = comp["mu"]
    g = np.where(zeta < mu, zeta**2 / (2 * mu), zeta - (mu / 2))
    return comp["n_0"] * R ** -comp["alpha"] * np.exp(-comp["beta"] * g ** comp["gamma"])


def band_density(X_helio, comp, geom):
    """Asteroidal dust band (``number_density.py:76-110``)."""
    _, R, Z = _dist_and_z(X_helio, geom)
    zeta = np.abs(Z / R)
    zz = zeta / geom["delta_zeta_rad"]
    term1 = 3 * comp["n_0"] / R
    term2 = np.exp(-(zz**6))
    term3 = 1 + (zz ** comp["p"]) / comp["v"]
    term4 = 1 - np.exp(-((R / comp["delta_r"]) ** 20))
    return term1 * term2 * term3 * term4


def ring_density(X_helio, comp, geom):
    """Circumsolar ring (``number_density.py:113-139``)."""
    _, R, Z = _dist_and_z(X_helio, geom)
    term1 = -((R - comp["R"]) ** 2) / comp["sigma_r"] ** 2
    term2 = np.abs(Z) / comp["sigma_z"]
    return comp["n_0"] * np.exp(term1 - term2)


def feature_density(X_helio, comp, geom, X_earth):
    """Earth-trailing feature (``number_density.py:142-181``), floor-mod angle wrap."""
    X, R, Z = _dist_and_z(X_helio, geom)
    Xe = X_earth - geom["X_0"]
    theta_comp = np.arctan2(X[1], X[0]) - np.arctan2(Xe[1], Xe[0])
    dtheta = theta_comp - geom["theta_rad"]
    dtheta = (dtheta + np.pi) % (2 * np.pi) - np.pi
    e = (R - comp["R"]) ** 2 / comp["sigma_r"] ** 2
    e += np.abs(Z) / comp["sigma_z"]
    e += dtheta**2 / geom["sigma_theta_rad"] ** 2
    return comp["n_0"] * np.exp(-e)


def _masked(R, lo, hi):
    """Radial mask of the RRM densities; outside it the reference leaves zeros (np.zeros_like + filtered fill)."""
    return np.logical_and(R >= lo, R <= hi)


def fan_density(X_helio, comp, geom):
    """RRM fan (``number_density.py:184-218``)."""
    _, R, Z = _dist_and_z(X_helio, geom)
    keep = R <= comp["R_outer"]
    beta = np.arcsin(Z / R)
    Z_abs = np.abs(Z)
    eps = np.where(Z_abs < comp["Z_0"], 2 - (Z_abs / comp["Z_0"]), 1)
    f = np.cos(beta) ** comp["Q"] * np.exp(-comp["P"] * np.sin(np.abs(beta) ** eps))
    return np.where(keep, (R ** (-comp["gamma"])) * f, 0.0)


def comet_density(X_helio, comp, geom):
    """RRM comet (``number_density.py:221-256``)."""
    _, R, Z = _dist_and_z(X_helio, geom)
    keep = _masked(R, comp["R_inner"], comp["R_outer"])
    beta = np.arcsin(Z / R)
    Z_abs = np.abs(Z)
    eps = np.where(Z_abs < comp["Z_0"], 2 - (Z_abs / comp["Z_0"]), 1)
    f = np.exp(-comp["P"] * np.sin(np.abs(beta) ** eps))
    return np.where(keep, comp["amp"] * (R ** (-comp["gamma"])) * f, 0.0)


def interstellar_density(X_helio, comp, geom):
    """RRM interstellar dust (``number_density.py:259-264``): a constant."""
    return np.full(np.shape(X_helio)[1:], comp["amp"])


def narrow_band_density(X_helio, comp, geom):
    """RRM narrow band (``number_density.py:267-304``)."""
    _, R, Z = _dist_and_z(X_helio, geom)
    keep = _masked(R, comp["R_inner"], comp["R_outer"])
    beta_abs = np.abs(np.rad2deg(np.arcsin(Z / R)))
    f = np.where(beta_abs < comp["beta_nb"], np.exp(comp["G"] * (beta_abs - comp["beta_nb"])), 0)
    return np.where(keep, comp["A"] * ((R / comp["R_outer"]) ** (-comp["gamma"])) * f, 0.0)


def broad_band_density(X_helio, comp, geom):
    """RRM broad band (``number_density.py:307-342``)."""
    _, R, Z = _dist_and_z(X_helio, geom)
    keep = _masked(R, comp["R_inner"], comp["R_outer"])
    beta = np.rad2deg(np.arcsin(Z / R))
    f = np.exp(-0.5 * ((beta - comp["beta_bb"]) / comp["sigma_bb"]) ** 2) + np.exp(
        -0.5 * ((beta + comp["beta_bb"]) / comp["sigma_bb"]) ** 2
    )
    return np.where(keep, comp["A"] * ((R / comp["R_outer"]) ** (-comp["gamma"])) * f, 0.0)


def ring_rrm_density(X_helio, comp, geom):
    """RRM ring: A times the Kelsall ring (``number_density.py:345-370``)."""
    return comp["A"] * ring_density(X_helio, comp, geom)


def feature_rrm_density(X_helio, comp, geom, X_earth):
    """RRM feature: A times the Kelsall feature (``number_density.py:373-403``)."""
    return comp["A"] * feature_density(X_helio, comp, geom, X_earth)


def rrm_brightness_at_step(r, start, stop, X_obs, u_los, bb_table, density, T_0, delta, calibration):
    """RRM integrand at one quadrature node (``brightness.py:59-83``)."""
    R_los = 0.5 * (stop - start) * r + 0.5 * (stop + start)
    X_los = R_los * u_los
    X_helio = X_los + X_obs
    R_helio = np.sqrt(X_helio[0] ** 2 + X_helio[1] ** 2 + X_helio[2] ** 2)
    temperature = T_0 * R_helio**-delta  # blackbody.py:16-30
    bb = np.interp(temperature, *bb_table)
    return bb * density(X_helio) * calibration * 0.5 * (stop - start)


def phase_normalization(C1, C2, C3):
    """Analytic phase-function normalisation (``scattering.py:53-59``)."""
    t1 = 2 * np.pi
    t2 = 2 * C1
    t3 = np.pi * C2
    t4 = (np.exp(C3 * np.pi) + 1) / (C3**2 + 1)
    return 1 / (t1 * (t2 + t3 + t4))


def scattering_angle(R_los, R_helio, X_los, X_helio):
    """``scattering.py:11-31``."""
    cos_theta = (X_los * X_helio).sum(axis=0) / (R_los * R_helio)
    cos_theta = np.clip(cos_theta, -1, 1)
    return np.arccos(-cos_theta)


def phase_function(Theta, C1, C2, C3):
    """``scattering.py:34-50``."""
    return phase_normalization(C1, C2, C3) * (C1 + C2 * Theta + np.exp(C3 * Theta))


def brightness_at_step(r, start, stop, X_obs, u_los, bb_table, density, T_0, delta, emissivity, albedo, C1, C2, C3, S):
    """Kelsall integrand at one quadrature node (``brightness.py:21-56``)."""
    R_los = 0.5 * (stop - start) * r + 0.5 * (stop + start)
    X_los = R_los * u_los
    X_helio = X_los + X_obs
    R_helio = np.sqrt(X_helio[0] ** 2 + X_helio[1] ** 2 + X_helio[2] ** 2)
    temperature = T_0 * R_helio**-delta  # blackbody.py:16-30
    bb = np.interp(temperature, *bb_table)
    emission = (1 - albedo) * (emissivity * bb)
    if albedo != 0:
        solar_flux = S / R_helio**2
        theta = scattering_angle(R_los, R_helio, X_los, X_helio)
        emission += albedo * solar_flux * phase_function(theta, C1, C2, C3)
    return emission * density(X_helio) * 0.5 * (stop - start)


def integrate_leggauss(func, points, weights):
    """Sequential quadrature sum in node order (``line_of_sight.py:55-61``)."""
    return np.squeeze(sum(func(x) * w for x, w in zip(points, weights)))


_DENSITY = {
    "cloud": cloud_density,
    "band": band_density,
    "ring": ring_density,
    "feature": feature_density,
    "fan": fan_density,
    "comet": comet_density,
    "interstellar": interstellar_density,
    "narrow_band": narrow_band_density,
    "broad_band": broad_band_density,
    "ring_rrm": ring_rrm_density,
    "feature_rrm": feature_rrm_density,
}
_NEEDS_EARTH = ("feature", "feature_rrm")


def comp_type(label: str) -> str:
    if label.startswith("band"):
        return "band"
    if label.endswith("narrow_band"):
        return "narrow_band"
    return label


def evaluate(desc: dict, unit_vectors, obs_xyz, earth_xyz, fix_b0=False) -> np.ndarray:
    """Per-component emission (C, N) for one call, as ``model.py:253-277``.

    ``desc`` holds, in component order: ``labels``, ``comps`` (init parameters
    as in ``to_dict()``), ``cutoffs`` {label: (inner, outer)}, ``T_0``,
    ``delta``, ``emissivity`` / ``albedo`` lists, ``C1``..``C3``,
    ``solar_irradiance``, ``bb_table`` (2, n_T) and ``gauss_quad_degree``.
    An RRM model (``family`` = "rrm") has ``T_0`` / ``delta`` as
    {label: value} and a ``calibration`` [Jy/cm] instead of the Kelsall
    spectral scalars.  ``obs_xyz`` / ``earth_xyz`` are (3,) or (3, N).
    """
    u = np.asarray(unit_vectors, dtype=np.float64)
    obs = np.asarray(obs_xyz, dtype=np.float64)
    if obs.ndim == 1:
        obs = obs[:, np.newaxis]
    earth = np.asarray(earth_xyz, dtype=np.float64)
    if earth.ndim == 1:
        earth = earth[:, np.newaxis]
    labels = list(desc["labels"])
    start, stop = los_range(labels, desc["cutoffs"], u, obs, fix_b0)
    pts, wts = np.polynomial.legendre.leggauss(desc["gauss_quad_degree"])
    out = np.zeros((len(labels), u.shape[-1]))
    for idx, label in enumerate(labels):
        comp = desc["comps"][label]
        geom = component_geometry(comp)
        kind = comp_type(label)
        if kind in _NEEDS_EARTH:
            density = lambda X, c=comp, g=geom, f=_DENSITY[kind]: f(X, c, g, earth)  # noqa: E731
        else:
            density = lambda X, c=comp, g=geom, f=_DENSITY[kind]: f(X, c, g)  # noqa: E731
        if desc.get("family") == "rrm":
            with np.errstate(all="ignore"):
                out[idx] = integrate_leggauss(
                    lambda r: rrm_brightness_at_step(
                        r,
                        start[label],
                        stop[label],
                        obs,
                        u,
                        desc["bb_table"],
                        density,
                        desc["T_0"][label],
                        desc["delta"][label],
                        desc["calibration"],
                    ),
                    pts,
                    wts,
                )
            continue
        with np.errstate(all="ignore"):
            out[idx] = integrate_leggauss(
                lambda r: brightness_at_step(
                    r,
                    start[label],
                    stop[label],
                    obs,
                    u,
                    desc["bb_table"],
                    density,
                    desc["T_0"],
                    desc["delta"],
                    desc["emissivity"][idx],
                    desc["albedo"][idx],
                    desc["C1"],
                    desc["C2"],
                    desc["C3"],
                    desc["solar_irradiance"],
                ),
                pts,
                wts,
            )
    return out


def grid_number_density(desc: dict, x, y, z, earth_xyz) -> np.ndarray:
    """Component densities on ``numpy.meshgrid(x, y, z)`` (``number_density.py:482-536``).

    Returns (C, ny, nx, nz) float64, the reference's layout; ``earth_xyz`` is
    Earth's heliocentric position (the feature's longitude origin).
    """
    grid = np.asarray(np.meshgrid(np.asarray(x, float), np.asarray(y, float), np.asarray(z, float)))
    earth = np.asarray(earth_xyz, dtype=np.float64).reshape(3, 1, 1, 1)
    labels = list(desc["labels"])
    out = np.zeros((len(labels), *grid.shape[1:]))
    for idx, label in enumerate(labels):
        comp = desc["comps"][label]
        geom = component_geometry(comp)
        geom["X_0"] = geom["X_0"].reshape(3, 1, 1, 1)
        kind = comp_type(label)
        with np.errstate(all="ignore"):
            if kind in _NEEDS_EARTH:
                out[idx] = _DENSITY[kind](grid, comp, geom, earth)
            else:
                out[idx] = _DENSITY[kind](grid, comp, geom)
    return out


def evaluate_chunked(desc, unit_vectors, obs_xyz, earth_xyz, nprocesses=1, fix_b0=False, start_method="fork"):
    """``evaluate`` split over coordinate chunks like ``model.py:182-200``.

    By default the pool is created with the fork start method exactly like the
    reference; a process that has initialised CUDA must pass
    ``start_method="spawn"`` (a pool forked after CUDA initialisation can hang).
    """
    u = np.asarray(unit_vectors, dtype=np.float64)
    n = u.shape[-1]
    if not (n > nprocesses > 1):
        return evaluate(desc, u, obs_xyz, earth_xyz, fix_b0)
    import multiprocessing

    obs = np.asarray(obs_xyz, dtype=np.float64)
    per_pixel_obs = obs.ndim > 1 and obs.shape[-1] == n and n > 1
    u_splits = np.array_split(u, nprocesses, axis=-1)
    o_splits = np.array_split(obs, nprocesses, axis=-1) if per_pixel_obs else [obs] * nprocesses
    with multiprocessing.get_context(start_method).Pool(nprocesses) as pool:
        parts = [
            pool.apply_async(evaluate, (desc, us, os_, earth_xyz, fix_b0)) for us, os_ in zip(u_splits, o_splits)
        ]
        return np.concatenate([p.get() for p in parts], axis=-1)
