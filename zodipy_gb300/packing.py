"""Pack a model (Kelsall or RRM) and its spectral set-up into the C ABI's ``ZlModel``.

Components keep their order (the reference's output order,
``zodipy/model.py:267-277``).  Components with identical (inner, outer)
cutoffs -- and, for RRM, identical grain temperature law -- share one
line-of-sight range, so their node positions, temperature and blackbody value
are computed once per node in the kernels.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .components import (
    COMPONENT_TYPE_CODE,
    Band,
    BroadBand,
    Cloud,
    Comet,
    Fan,
    Feature,
    FeatureRRM,
    Interstellar,
    NarrowBand,
    Ring,
    RingRRM,
)
from .zodiacal_light_model import COMPONENT_CUTOFFS, RRM


def component_params(comp) -> list[float]:
    """``ZlComponent.p`` of one component (order as in ``include/zodigb.h``)."""
    if isinstance(comp, RingRRM):
        return [comp.R, comp.sigma_r, comp.sigma_z, comp.A]
    if isinstance(comp, FeatureRRM):
        return [comp.R, comp.sigma_r, comp.sigma_z, comp.theta_rad, comp.sigma_theta_rad, comp.A]
    if isinstance(comp, Fan):
        return [comp.gamma, comp.Z_0, comp.Q, comp.P, comp.R_outer]
    if isinstance(comp, Comet):
        return [comp.gamma, comp.Z_0, comp.P, comp.amp, comp.R_inner, comp.R_outer]
    if isinstance(comp, Interstellar):
        return [comp.amp]
    if isinstance(comp, NarrowBand):
        return [comp.gamma, comp.A, comp.G, comp.R_inner, comp.R_outer, comp.beta_nb]
    if isinstance(comp, BroadBand):
        return [comp.gamma, comp.A, comp.R_inner, comp.R_outer, comp.beta_bb, comp.sigma_bb]
    if isinstance(comp, Cloud):
        return [comp.alpha, comp.beta, comp.gamma, comp.mu]
    if isinstance(comp, Band):
        return [comp.delta_zeta_rad, comp.v, comp.p, comp.delta_r]
    if isinstance(comp, Feature):
        return [comp.R, comp.sigma_r, comp.sigma_z, comp.theta_rad, comp.sigma_theta_rad]
    if isinstance(comp, Ring):
        return [comp.R, comp.sigma_r, comp.sigma_z]
    raise TypeError(f"component type {type(comp).__name__} is not supported by the kernels")


def pack_model(ipd_model, spectra: list[dict], bb_tables: list[np.ndarray], gl_x, gl_w) -> _lib.ZlModel:
    """Build the ``ZlModel`` for ``len(spectra)`` fused spectral sets.

    ``spectra[s]`` holds ``emissivity``/``albedo`` (one per component, model
    order) and the scalars ``C1``, ``C2``, ``C3``, ``solar_irradiance`` (and
    ``calibration`` for an RRM model); ``bb_tables[s]`` is the (2, n_T)
    blackbody table.
    """
    comps = list(ipd_model.comps.items())
    if not 1 <= len(comps) <= _lib.ZL_MAX_COMPS:
        raise ValueError(f"models with {len(comps)} components are not supported (max {_lib.ZL_MAX_COMPS})")
    if not 1 <= len(spectra) <= _lib.ZL_MAX_SPEC:
        raise ValueError(f"1..{_lib.ZL_MAX_SPEC} spectral sets can be fused, got {len(spectra)}")
    gl_x = np.asarray(gl_x, dtype=np.float64)
    gl_w = np.asarray(gl_w, dtype=np.float64)
    if not 1 <= gl_x.size <= _lib.ZL_MAX_NODES:
        raise ValueError(f"gauss_quad_degree must be in [1, {_lib.ZL_MAX_NODES}] for the GPU kernels")
    temps = np.asarray(bb_tables[0][0], dtype=np.float64)
    if temps.size > _lib.ZL_MAX_TEMPS:
        raise ValueError("blackbody table too long")

    m = _lib.ZlModel()
    m.abi_version = _lib.ZL_ABI_VERSION
    m.n_comps = len(comps)
    m.n_spec = len(spectra)
    m.n_nodes = gl_x.size
    m.n_temps = temps.size
    rrm = isinstance(ipd_model, RRM)
    m.family = _lib.ZL_RRM if rrm else _lib.ZL_KELSALL
    if rrm:
        for c, (label, _) in enumerate(comps):
            m.comp_T_0[c] = float(ipd_model.T_0[label])
            m.comp_delta[c] = float(ipd_model.delta[label])
    else:
        m.T_0 = float(ipd_model.T_0)
        m.delta = float(ipd_model.delta)
    ranges: list[tuple] = []
    cutoffs: list[tuple[float, float]] = []
    for c, (label, comp) in enumerate(comps):
        cut = tuple(float(v) for v in COMPONENT_CUTOFFS[label])
        key = (cut, m.comp_T_0[c], m.comp_delta[c]) if rrm else cut
        if key not in ranges:
            ranges.append(key)
            cutoffs.append(cut)
        k = m.comp[c]
        k.type = COMPONENT_TYPE_CODE[type(comp)]
        k.range = ranges.index(key)
        k.offset[:] = [float(v) for v in comp.X_0]
        k.sin_i, k.cos_i = comp.sin_i_rad, comp.cos_i_rad
        k.sin_Omega, k.cos_Omega = comp.sin_Omega_rad, comp.cos_Omega_rad
        k.n_0 = float(getattr(comp, "n_0", 1.0))
        p = component_params(comp)
        for j, v in enumerate(p):
            k.p[j] = float(v)
    if len(ranges) > _lib.ZL_MAX_RANGES:
        raise ValueError(f"models with {len(ranges)} distinct line-of-sight ranges are not supported")
    m.n_ranges = len(ranges)
    for r, (lo, hi) in enumerate(cutoffs):
        m.cutoff[r][0] = lo
        m.cutoff[r][1] = hi
    m.temps[: temps.size] = temps.tolist()
    m.gl_x[: gl_x.size] = gl_x.tolist()
    m.gl_w[: gl_w.size] = gl_w.tolist()
    for s, (sp, tab) in enumerate(zip(spectra, bb_tables)):
        if not np.array_equal(np.asarray(tab[0]), temps):
            raise ValueError("all fused spectral sets must share the table temperatures")
        ks = m.spec[s]
        for c in range(len(comps)):
            ks.emissivity[c] = float(sp["emissivity"][c])
            ks.albedo[c] = float(sp["albedo"][c])
        ks.C1 = float(sp["C1"])
        ks.C2 = float(sp["C2"])
        ks.C3 = float(sp["C3"])
        ks.solar_irradiance = float(sp["solar_irradiance"])
        ks.calibration = float(sp.get("calibration", 0.0))
        ks.bb[: temps.size] = np.asarray(tab[1], dtype=np.float64).tolist()
    lib = _lib.load()
    _lib.check(lib.zl_model_check(ctypes.byref(m)), "zl_model_check")
    return m


def pack_densities(ipd_model) -> _lib.ZlModel:
    """``ZlModel`` carrying only the components' geometry, for ``zl_density_grid``.

    The spectral block is a placeholder (one zero spectrum, a two-point table,
    one node) that satisfies ``zl_model_check``; densities never read it.
    """
    zero = {"emissivity": [0.0] * len(ipd_model.comps), "albedo": [0.0] * len(ipd_model.comps)}
    zero.update(C1=0.0, C2=0.0, C3=0.0, solar_irradiance=0.0)
    table = np.array([[1.0, 2.0], [0.0, 0.0]])
    return pack_model(ipd_model, [zero], [table], [0.0], [2.0])


def observer_table(model: _lib.ZlModel, obs_xyz: np.ndarray, earth_xyz: np.ndarray, pix_begin, any_mode: bool):
    """ctypes array of ``ZlObserver`` with the cutoff flags filled in."""
    obs_xyz = np.asarray(obs_xyz, dtype=np.float64).reshape(3, -1)
    earth_xyz = np.asarray(earth_xyz, dtype=np.float64).reshape(3, -1)
    n = obs_xyz.shape[1]
    if earth_xyz.shape[1] not in (1, n):
        raise ValueError("earth positions must be (3,) or (3, n_obs)")
    pix_begin = np.asarray(pix_begin, dtype=np.int64).reshape(-1)
    if pix_begin.size != n:
        raise ValueError("one pix_begin per observer")
    arr = (_lib.ZlObserver * n)()
    view = np.frombuffer(arr, dtype=np.uint8).reshape(n, ctypes.sizeof(_lib.ZlObserver))
    rec = np.zeros(n, dtype=[("obs", "<f8", 3), ("earth", "<f8", 3), ("pix_begin", "<i8"), ("outside", "<u4"), ("reserved", "<u4")])
    rec["obs"] = obs_xyz.T
    rec["earth"] = np.broadcast_to(earth_xyz.T, (n, 3))
    rec["pix_begin"] = pix_begin
    view[:] = rec.view(np.uint8).reshape(n, -1)
    lib = _lib.load()
    _lib.check(lib.zl_observer_flags(ctypes.byref(model), arr, n, 1 if any_mode else 0), "zl_observer_flags")
    return arr
