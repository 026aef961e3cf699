"""The model parameter vector of the adjoint, and its mapping to ``ZlModel``.

The vector follows the gradient layout of ``include/zodigb.h`` (``zl_backward``).
Kelsall models: per component, the reference's parameter-dictionary entries in
order (``zodipy/zodiacal_light_model.py:38-55``: x_0, y_0, z_0, i, Omega, n_0 and
the type's own, angles in degrees), then T_0 and delta, then per spectral set the
interpolated emissivity and albedo of every component, C1, C2, C3 and the solar
irradiance.  RRM models (``zodipy/zodiacal_light_model.py:90-102``): per
component x_0, y_0, z_0, i, Omega and the type's own fields, then T_0 of every
component, delta of every component, then the interpolated calibration of every
spectral set.  ``vector_from_model`` reads a packed ``ZlModel`` into that vector,
``model_from_vector`` writes a vector back (re-deriving sin/cos and radians as
``zodipy/component.py:39-44,87-89,133-136`` does).
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib

_OWN = {
    _lib.ZL_CLOUD: ("alpha", "beta", "gamma", "mu"),
    _lib.ZL_BAND: ("delta_zeta", "v", "p", "delta_r"),
    _lib.ZL_RING: ("R", "sigma_r", "sigma_z"),
    _lib.ZL_FEATURE: ("R", "sigma_r", "sigma_z", "theta", "sigma_theta"),
}
# own parameters that the ZlModel stores in radians but the dictionary holds in degrees
_DEG = {(_lib.ZL_BAND, 0), (_lib.ZL_FEATURE, 3), (_lib.ZL_FEATURE, 4)}


# RRM component types: the reference's dataclass fields after the geometry, each stored in
# ZlComponent as n_0 or p[j] (in radians where the dictionary holds degrees: the feature's angles)
_OWN_RRM = {
    _lib.ZL_FAN: (("gamma", 0), ("Z_0", 1), ("Q", 2), ("P", 3), ("R_outer", 4)),
    _lib.ZL_COMET: (("gamma", 0), ("Z_0", 1), ("P", 2), ("amp", 3), ("R_inner", 4), ("R_outer", 5)),
    _lib.ZL_NARROW_BAND: (("gamma", 0), ("A", 1), ("G", 2), ("R_inner", 3), ("R_outer", 4), ("beta_nb", 5)),
    _lib.ZL_BROAD_BAND: (("gamma", 0), ("A", 1), ("R_inner", 2), ("R_outer", 3), ("beta_bb", 4), ("sigma_bb", 5)),
    _lib.ZL_INTERSTELLAR: (("amp", 0),),
    _lib.ZL_RING_RRM: (("n_0", None), ("R", 0), ("sigma_r", 1), ("sigma_z", 2), ("A", 3)),
    _lib.ZL_FEATURE_RRM: (("n_0", None), ("R", 0), ("sigma_r", 1), ("sigma_z", 2), ("theta", 3), ("sigma_theta", 4),
                          ("A", 5)),
}
_DEG_RRM = {(_lib.ZL_FEATURE_RRM, 3), (_lib.ZL_FEATURE_RRM, 4)}


def _own(t) -> tuple:
    try:
        return _OWN[t]
    except KeyError:
        raise ValueError(f"component type {t} is not a Kelsall component type") from None


def _rrm(m) -> bool:
    return m.family == _lib.ZL_RRM


def names(zl_model, labels) -> list[str]:
    if _rrm(zl_model):
        out = []
        for c in range(zl_model.n_comps):
            own = [k for k, _ in _OWN_RRM[zl_model.comp[c].type]]
            out += [f"comps.{labels[c]}.{k}" for k in ("x_0", "y_0", "z_0", "i", "Omega", *own)]
        out += [f"T_0.{labels[c]}" for c in range(zl_model.n_comps)]
        out += [f"delta.{labels[c]}" for c in range(zl_model.n_comps)]
        out += [f"calibration[{s}]" if zl_model.n_spec > 1 else "calibration" for s in range(zl_model.n_spec)]
        return out
    out = []
    for c in range(zl_model.n_comps):
        t = zl_model.comp[c].type
        lab = labels[c]
        out += [f"comps.{lab}.{k}" for k in ("x_0", "y_0", "z_0", "i", "Omega", "n_0", *_own(t))]
    out += ["T_0", "delta"]
    for s in range(zl_model.n_spec):
        sfx = f"[{s}]" if zl_model.n_spec > 1 else ""
        out += [f"emissivity.{lab}{sfx}" for lab in labels[: zl_model.n_comps]]
        out += [f"albedo.{lab}{sfx}" for lab in labels[: zl_model.n_comps]]
        out += [f"C1{sfx}", f"C2{sfx}", f"C3{sfx}", f"solar_irradiance{sfx}"]
    return out


def vector_from_model(m) -> np.ndarray:
    if _rrm(m):
        v = []
        for c in range(m.n_comps):
            k = m.comp[c]
            inc = math.degrees(math.atan2(k.sin_i, k.cos_i))
            node = math.degrees(math.atan2(k.sin_Omega, k.cos_Omega))
            v += [k.offset[0], k.offset[1], k.offset[2], inc, node]
            for _, j in _OWN_RRM[k.type]:
                if j is None:
                    v.append(k.n_0)
                else:
                    v.append(math.degrees(k.p[j]) if (k.type, j) in _DEG_RRM else k.p[j])
        v += [m.comp_T_0[c] for c in range(m.n_comps)]
        v += [m.comp_delta[c] for c in range(m.n_comps)]
        v += [m.spec[s].calibration for s in range(m.n_spec)]
        return np.asarray(v, dtype=np.float64)
    v = []
    for c in range(m.n_comps):
        k = m.comp[c]
        inc = math.degrees(math.atan2(k.sin_i, k.cos_i))
        node = math.degrees(math.atan2(k.sin_Omega, k.cos_Omega))
        v += [k.offset[0], k.offset[1], k.offset[2], inc, node, k.n_0]
        for j in range(len(_own(k.type))):
            v.append(math.degrees(k.p[j]) if (k.type, j) in _DEG else k.p[j])
    v += [m.T_0, m.delta]
    for s in range(m.n_spec):
        sp = m.spec[s]
        v += [sp.emissivity[c] for c in range(m.n_comps)]
        v += [sp.albedo[c] for c in range(m.n_comps)]
        v += [sp.C1, sp.C2, sp.C3, sp.solar_irradiance]
    return np.asarray(v, dtype=np.float64)


def model_from_vector(base, vec) -> "_lib.ZlModel":
    """A copy of ``base`` with every vector parameter replaced."""
    m = _lib.ZlModel.from_buffer_copy(base)
    vec = np.asarray(vec, dtype=np.float64)
    if _rrm(m):
        return _rrm_from_vector(m, vec)
    j = 0
    for c in range(m.n_comps):
        k = m.comp[c]
        k.offset[0], k.offset[1], k.offset[2] = vec[j : j + 3]
        inc, node = math.radians(vec[j + 3]), math.radians(vec[j + 4])
        k.sin_i, k.cos_i = math.sin(inc), math.cos(inc)
        k.sin_Omega, k.cos_Omega = math.sin(node), math.cos(node)
        k.n_0 = vec[j + 5]
        j += 6
        for q in range(len(_own(k.type))):
            k.p[q] = math.radians(vec[j]) if (k.type, q) in _DEG else vec[j]
            j += 1
    m.T_0, m.delta = vec[j], vec[j + 1]
    j += 2
    for s in range(m.n_spec):
        sp = m.spec[s]
        for c in range(m.n_comps):
            sp.emissivity[c] = vec[j + c]
            sp.albedo[c] = vec[j + m.n_comps + c]
        j += 2 * m.n_comps
        sp.C1, sp.C2, sp.C3, sp.solar_irradiance = vec[j : j + 4]
        j += 4
    if j != vec.size:
        raise ValueError(f"parameter vector has {vec.size} entries, the model needs {j}")
    _lib.check(_lib.load().zl_model_check(ctypes.byref(m)), "zl_model_check")
    return m


def _rrm_from_vector(m, vec):
    j = 0
    for c in range(m.n_comps):
        k = m.comp[c]
        k.offset[0], k.offset[1], k.offset[2] = vec[j : j + 3]
        inc, node = math.radians(vec[j + 3]), math.radians(vec[j + 4])
        k.sin_i, k.cos_i = math.sin(inc), math.cos(inc)
        k.sin_Omega, k.cos_Omega = math.sin(node), math.cos(node)
        j += 5
        for _, q in _OWN_RRM[k.type]:
            if q is None:
                k.n_0 = vec[j]
            else:
                k.p[q] = math.radians(vec[j]) if (k.type, q) in _DEG_RRM else vec[j]
            j += 1
    for c in range(m.n_comps):
        m.comp_T_0[c] = vec[j + c]
        m.comp_delta[c] = vec[j + m.n_comps + c]
    j += 2 * m.n_comps
    # components share a line-of-sight range only while their cutoffs and grain temperature law
    # agree (the forward kernels take the law per range): re-derive the ranges
    keys, cut = [], []
    for c in range(m.n_comps):
        r = m.comp[c].range
        key = (m.cutoff[r][0], m.cutoff[r][1], m.comp_T_0[c], m.comp_delta[c])
        if key not in keys:
            keys.append(key)
            cut.append((m.cutoff[r][0], m.cutoff[r][1]))
        m.comp[c].range = keys.index(key)
    if len(keys) > _lib.ZL_MAX_RANGES:
        raise ValueError(f"{len(keys)} distinct line-of-sight ranges exceed the kernels' {_lib.ZL_MAX_RANGES}")
    m.n_ranges = len(keys)
    for r, (lo, hi) in enumerate(cut):
        m.cutoff[r][0], m.cutoff[r][1] = lo, hi
    for s in range(m.n_spec):
        m.spec[s].calibration = vec[j + s]
    j += m.n_spec
    if j != vec.size:
        raise ValueError(f"parameter vector has {vec.size} entries, the model needs {j}")
    _lib.check(_lib.load().zl_model_check(ctypes.byref(m)), "zl_model_check")
    return m


def size(m) -> int:
    if _rrm(m):
        return sum(5 + len(_OWN_RRM[m.comp[c].type]) for c in range(m.n_comps)) + 2 * m.n_comps + m.n_spec
    return sum(6 + len(_own(m.comp[c].type)) for c in range(m.n_comps)) + 2 + m.n_spec * (2 * m.n_comps + 4)
