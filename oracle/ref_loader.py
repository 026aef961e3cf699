"""Load ZodiPy's own numeric modules without astropy (test infrastructure only).

This module is part of the oracle: only the golden-fixture generator under
``tests/golden/`` and CPU tests that validate the oracle use it, and only in a
checkout where the ZodiPy source tree is present.  The product package never
imports it.

ZodiPy v1.1.3 imports astropy at module level (``zodipy/blackbody.py:4-5``,
``zodipy/bodies.py:5-8``, ``zodipy/source_params.py:1``,
``zodipy/zodiacal_light_model.py:8``, ``zodipy/unpack_model.py:7``) but its
line-of-sight arithmetic (``line_of_sight.py``, ``brightness.py``,
``number_density.py``, ``scattering.py``, ``component*.py``) is plain numpy.
astropy is not installed here, so a minimal stand-in is registered in
``sys.modules`` before the reference modules are executed from their own
files.  Nothing of the reference is copied: the files are executed in place.
"""

from __future__ import annotations

import importlib
import os
import sys
import types

import numpy as np

# Root of a ZodiPy v1.1.3 source tree (the directory holding ``zodipy/``); there is no built-in
# default: set ZODIPY_REF_ROOT or pass the path.
REF_ROOT_ENV = "ZODIPY_REF_ROOT"


def ref_root_from_env() -> str | None:
    return os.environ.get(REF_ROOT_ENV) or None

# (1 MJy / AU) in Jy / cm, the unit change astropy applies to the RRM calibration
# (unpack_model.py:131-132): 1e6 Jy over 1 au = 1.495978707e13 cm (IAU 2012 exact).
MJY_PER_AU_TO_JY_PER_CM = 1e6 / 1.495978707e13


class _Unit:
    def __init__(self, name: str, scale: float = 1.0) -> None:
        self.name = name
        self.scale = scale

    def __rmul__(self, other):
        return _Quantity(other, self)

    def __mul__(self, other):
        if isinstance(other, _Unit):
            return _Unit(f"{self.name}*{other.name}")
        return _Quantity(other, self)

    def __truediv__(self, other):
        return _Unit(f"{self.name}/{getattr(other, 'name', other)}")

    def __repr__(self) -> str:
        return f"Unit({self.name})"


class _Quantity(np.ndarray):
    """ndarray carrying a ``.unit``; ``.value`` returns the plain array."""

    def __new__(cls, value, unit=None, dtype=None):
        obj = np.asarray(value, dtype=dtype).view(cls)
        obj.unit = unit
        return obj

    def __array_finalize__(self, obj):
        self.unit = getattr(obj, "unit", None)

    @property
    def value(self):
        return np.asarray(self)

    def to_value(self, unit=None, equivalencies=None):
        return np.asarray(self)

    def to(self, unit=None, equivalencies=None):
        return self


def _install_astropy_stub() -> None:
    if "astropy" in sys.modules and not getattr(sys.modules["astropy"], "_zl_stub", False):
        return  # a real astropy is present; use it
    astropy = types.ModuleType("astropy")
    astropy._zl_stub = True
    astropy.__path__ = []
    units = types.ModuleType("astropy.units")
    for name in ("K", "GHz", "micron", "um", "AU", "MJy", "sr", "Jy", "cm", "Hz", "m", "deg", "s", "day", "hour"):
        setattr(units, name, _Unit(name))
    units.K = 1.0  # blackbody.py:9-10 multiplies temperatures by K before np.linspace
    units.Quantity = _Quantity
    units.UnitConversionError = type("UnitConversionError", (Exception,), {})
    units.spectral = lambda: None
    coordinates = types.ModuleType("astropy.coordinates")
    time_mod = types.ModuleType("astropy.time")
    time_mod.Time = type("Time", (), {})
    modeling = types.ModuleType("astropy.modeling")
    modeling.__path__ = []
    physical_models = types.ModuleType("astropy.modeling.physical_models")

    class BlackBody:  # the reference's module-level table object; never evaluated here
        def __init__(self, *args, **kwargs) -> None:
            pass

    physical_models.BlackBody = BlackBody
    astropy.units = units
    astropy.coordinates = coordinates
    astropy.time = time_mod
    astropy.modeling = modeling
    modeling.physical_models = physical_models
    sys.modules.update(
        {
            "astropy": astropy,
            "astropy.units": units,
            "astropy.coordinates": coordinates,
            "astropy.time": time_mod,
            "astropy.modeling": modeling,
            "astropy.modeling.physical_models": physical_models,
        }
    )


def load_reference(ref_root: str | None = None) -> types.SimpleNamespace:
    """Execute the reference's numeric modules in place and return them.

    ``ref_root`` defaults to $ZODIPY_REF_ROOT.  Raises FileNotFoundError when
    neither names a ZodiPy source tree.
    """
    ref_root = ref_root or ref_root_from_env()
    if not ref_root:
        raise FileNotFoundError(f"no reference tree: pass its path or set {REF_ROOT_ENV}")
    pkg_dir = os.path.join(ref_root, "zodipy")
    if not os.path.isdir(pkg_dir):
        raise FileNotFoundError(f"reference package not found at {pkg_dir}")
    sys.dont_write_bytecode = True  # the reference mount must stay untouched
    _install_astropy_stub()
    if "zodipy" not in sys.modules:
        pkg = types.ModuleType("zodipy")
        pkg.__path__ = [pkg_dir]  # do not run zodipy/__init__.py (it imports model.py)
        sys.modules["zodipy"] = pkg
    names = (
        "component",
        "component_params",
        "source_params",
        "scattering",
        "blackbody",
        "brightness",
        "zodiacal_light_model",
        "model_registry",
        "line_of_sight",
        "number_density",
        "unpack_model",
    )
    mods = {n: importlib.import_module(f"zodipy.{n}") for n in names}
    return types.SimpleNamespace(**mods)


def reference_available(ref_root: str | None = None) -> bool:
    ref_root = ref_root or ref_root_from_env()
    return bool(ref_root) and os.path.isdir(os.path.join(ref_root, "zodipy"))


class _V:
    """Plain holder with ``.value`` for ``interp_spectral_param`` (unpack_model.py:140-173)."""

    def __init__(self, v) -> None:
        self.value = np.asarray(v, dtype=np.float64)


def reference_evaluate(
    ref: types.SimpleNamespace,
    model_name,
    unit_vectors: np.ndarray,
    obs_xyz: np.ndarray,
    earth_xyz: np.ndarray,
    bb_table: np.ndarray,
    x_in_model_units: np.ndarray,
    weights: np.ndarray | None,
    gauss_quad_degree: int,
    bounds_error: bool = False,
    scalars: dict | None = None,
) -> np.ndarray:
    """Run the reference's own hot path exactly as ``Model._evaluate`` does.

    Follows ``zodipy/model.py:253-277`` (LOS range, density partials, per-component
    quadrature) with spectral scalars produced by the reference's
    ``interp_spectral_param`` (``unpack_model.py:140-173``) in the same way as
    ``interp_and_unpack_kelsall`` (``unpack_model.py:23-107``).  The astropy-only
    inputs (blackbody table, Earth position, unit vectors) are supplied by the
    caller.  ``x_in_model_units`` is the wavelength/frequency already converted
    to the model spectrum's unit; ``weights`` are the already-normalised weights
    (``model.py:94``) or None.
    """
    model = ref.model_registry.model_registry.get_model(model_name) if isinstance(model_name, str) else model_name
    spectrum = _V(np.asarray(model.spectrum))
    x = _V(x_in_model_units)
    w = None if weights is None else _V(weights)
    isp = ref.unpack_model.interp_spectral_param

    if type(model).__name__ == "RRM":
        # unpack_model.py:110-132; the calibration's unit change (MJy/AU -> Jy/cm) is astropy's
        # and is restated here as a factor
        comp_params = {label: {"T_0": model.T_0[label], "delta": model.delta[label]} for label in model.comps}
        cal = isp(x, w, spectrum, model.calibration, bounds_error=bounds_error)
        shared = {"calibration": float(cal) * MJY_PER_AU_TO_JY_PER_CM}
        if scalars is not None and "calibration" in scalars:
            shared["calibration"] = scalars["calibration"]
        return _run_reference_path(ref, model, unit_vectors, obs_xyz, earth_xyz, bb_table, gauss_quad_degree,
                                   comp_params, shared)

    comp_params = {}
    for label in model.comps:
        comp_params[label] = {
            "emissivity": isp(x, w, spectrum, model.emissivities[label], bounds_error=bounds_error),
            "albedo": (
                isp(x, w, spectrum, model.albedos[label], bounds_error=bounds_error)
                if model.albedos is not None
                else 0
            ),
        }
    shared = {"T_0": model.T_0, "delta": model.delta}
    for key in ("C1", "C2", "C3"):
        table = getattr(model, key)
        shared[key] = (
            isp(x, w, spectrum, table, use_nearest=True, bounds_error=bounds_error) if table is not None else 0
        )
    shared["solar_irradiance"] = (
        isp(x, w, spectrum, model.solar_irradiance, bounds_error=bounds_error)
        if model.solar_irradiance is not None
        else 0
    )

    if scalars is not None:  # explicit interpolated spectral scalars (for derivatives)
        for idx, label in enumerate(model.comps):
            comp_params[label] = {"emissivity": scalars["emissivity"][idx], "albedo": scalars["albedo"][idx]}
        for key in ("C1", "C2", "C3", "solar_irradiance"):
            shared[key] = scalars[key]
        shared["T_0"] = scalars.get("T_0", shared["T_0"])
        shared["delta"] = scalars.get("delta", shared["delta"])
    return _run_reference_path(ref, model, unit_vectors, obs_xyz, earth_xyz, bb_table, gauss_quad_degree,
                               comp_params, shared)


def _run_reference_path(ref, model, unit_vectors, obs_xyz, earth_xyz, bb_table, gauss_quad_degree, comp_params,
                        shared):
    """The reference's ``Model._evaluate`` loop (``model.py:253-277``) with unpacked parameters."""
    import functools

    obs = np.asarray(obs_xyz, dtype=np.float64)
    if obs.ndim == 1:
        obs = obs[:, np.newaxis]
    earth = np.asarray(earth_xyz, dtype=np.float64)
    if earth.ndim == 1:
        earth = earth[:, np.newaxis]
    u = np.asarray(unit_vectors, dtype=np.float64)

    start, stop = ref.line_of_sight.get_line_of_sight_range(
        components=model.comps.keys(), unit_vectors=u, obs_pos=obs
    )
    dens = ref.number_density.get_partial_number_density_func(comps=model.comps)
    dens = ref.number_density.update_partial_earth_pos(dens, earth_pos=earth)
    bright = functools.partial(
        model.brightness_at_step_callable, bp_interpolation_table=bb_table, X_obs=obs, **shared
    )
    pts, wts = np.polynomial.legendre.leggauss(gauss_quad_degree)
    out = np.zeros((model.ncomps, u.shape[-1]))
    for idx, label in enumerate(model.comps.keys()):
        f = functools.partial(
            bright,
            u_los=u,
            start=start[label],
            stop=stop[label],
            number_density_func=dens[label],
            **comp_params[label],
        )
        out[idx] = ref.line_of_sight.integrate_leggauss(f, pts, wts)
    return out


def reference_spectral_scalars(ref, model_name, x_in_model_units, weights, bounds_error=False) -> dict:
    """Spectral scalars exactly as the reference unpacks them (``unpack_model.py:23-107``)."""
    model = ref.model_registry.model_registry.get_model(model_name)
    spectrum = _V(np.asarray(model.spectrum))
    x = _V(x_in_model_units)
    w = None if weights is None else _V(weights)
    isp = ref.unpack_model.interp_spectral_param
    out = {"emissivity": [], "albedo": []}
    for label in model.comps:
        out["emissivity"].append(float(isp(x, w, spectrum, model.emissivities[label], bounds_error=bounds_error)))
        out["albedo"].append(
            float(isp(x, w, spectrum, model.albedos[label], bounds_error=bounds_error)) if model.albedos else 0.0
        )
    for key in ("C1", "C2", "C3"):
        table = getattr(model, key)
        out[key] = float(isp(x, w, spectrum, table, use_nearest=True, bounds_error=bounds_error)) if table else 0.0
    out["solar_irradiance"] = (
        float(isp(x, w, spectrum, model.solar_irradiance, bounds_error=bounds_error))
        if model.solar_irradiance
        else 0.0
    )
    return out


def reference_rrm_calibration(ref, model_name, x_in_model_units, weights, bounds_error=False) -> float:
    """RRM calibration [Jy/cm] as ``interp_and_unpack_rrm`` forms it (``unpack_model.py:110-132``)."""
    model = ref.model_registry.model_registry.get_model(model_name)
    w = None if weights is None else _V(weights)
    cal = ref.unpack_model.interp_spectral_param(
        _V(x_in_model_units), w, _V(np.asarray(model.spectrum)), model.calibration, bounds_error=bounds_error
    )
    return float(cal) * MJY_PER_AU_TO_JY_PER_CM


def reference_fd_gradient(ref, model_name, u, obs, earth, bb_table, x_model, weights, degree, a, rel_step=1e-5):
    """Central finite differences of L = sum_i a_i total_i through the reference's own code.

    Parameters are the component init parameters (``to_dict`` order, angles in
    degrees), T_0, delta, and the interpolated spectral scalars (emissivity and
    albedo per component, C1, C2, C3, solar irradiance).  The step is
    ``rel_step * max(|p|, 1)``.  Returns (names, gradient, loss).
    """
    import dataclasses

    base = ref.model_registry.model_registry.get_model(model_name)
    scal = reference_spectral_scalars(ref, model_name, x_model, weights)
    scal = {k: (list(v) if isinstance(v, list) else v) for k, v in scal.items()}
    scal["T_0"], scal["delta"] = float(base.T_0), float(base.delta)

    def loss(model, sc):
        out = reference_evaluate(ref, model, u, obs, earth, bb_table, x_model, weights, degree, scalars=sc)
        return float(np.dot(a, out.sum(axis=0)))

    names, grads = [], []
    L0 = loss(base, scal)
    for label, comp in base.comps.items():
        init = {f.name: getattr(comp, f.name) for f in dataclasses.fields(comp) if f.init}
        for key, val in init.items():
            h = rel_step * max(abs(float(val)), 1.0)
            vals = []
            for sgn in (1, -1):
                comps = dict(base.comps)
                comps[label] = type(comp)(**{**init, key: float(val) + sgn * h})
                vals.append(loss(dataclasses.replace(base, comps=comps), scal))
            names.append(f"comps.{label.value}.{key}")
            grads.append((vals[0] - vals[1]) / (2 * h))
    for key in ("T_0", "delta"):
        h = rel_step * max(abs(scal[key]), 1.0)
        vals = [loss(base, {**scal, key: scal[key] + sgn * h}) for sgn in (1, -1)]
        names.append(key)
        grads.append((vals[0] - vals[1]) / (2 * h))
    for key in ("emissivity", "albedo"):
        for idx, label in enumerate(base.comps):
            v0 = scal[key][idx]
            h = rel_step * max(abs(v0), 1.0)
            vals = []
            for sgn in (1, -1):
                lst = list(scal[key])
                lst[idx] = v0 + sgn * h
                vals.append(loss(base, {**scal, key: lst}))
            names.append(f"{key}.{label.value}")
            grads.append((vals[0] - vals[1]) / (2 * h))
    for key in ("C1", "C2", "C3", "solar_irradiance"):
        h = rel_step * max(abs(scal[key]), 1.0)
        vals = [loss(base, {**scal, key: scal[key] + sgn * h}) for sgn in (1, -1)]
        names.append(key)
        grads.append((vals[0] - vals[1]) / (2 * h))
    return names, np.asarray(grads), L0


def reference_fd_gradient_rrm(ref, model_name, u, obs, earth, bb_table, x_model, weights, degree, a,
                              rel_step=1e-5):
    """Central finite differences of L = sum_i a_i total_i through the reference's own code, for
    the Rowan-Robinson & May model (``brightness.py:59-83``, ``number_density.py:184-404``).

    Parameters: every component's init parameters (``to_dict`` order, angles in degrees), then
    the grain temperature law of every component (``T_0.<label>``, then ``delta.<label>``), then
    the interpolated calibration.  Step ``rel_step * max(|p|, 1)``.  Returns (names, gradient,
    loss).
    """
    import dataclasses

    base = ref.model_registry.model_registry.get_model(model_name)
    cal0 = reference_rrm_calibration(ref, model_name, x_model, weights)

    def loss(model, cal):
        out = reference_evaluate(ref, model, u, obs, earth, bb_table, x_model, weights, degree,
                                 scalars={"calibration": cal})
        return float(np.dot(a, out.sum(axis=0)))

    names, grads = [], []
    L0 = loss(base, cal0)
    for label, comp in base.comps.items():
        init = {f.name: getattr(comp, f.name) for f in dataclasses.fields(comp) if f.init}
        for key, val in init.items():
            h = rel_step * max(abs(float(val)), 1.0)
            vals = []
            for sgn in (1, -1):
                comps = dict(base.comps)
                comps[label] = type(comp)(**{**init, key: float(val) + sgn * h})
                vals.append(loss(dataclasses.replace(base, comps=comps), cal0))
            names.append(f"comps.{label.value}.{key}")
            grads.append((vals[0] - vals[1]) / (2 * h))
    for field in ("T_0", "delta"):
        table = getattr(base, field)
        for label in base.comps:
            v0 = float(table[label])
            h = rel_step * max(abs(v0), 1.0)
            vals = [loss(dataclasses.replace(base, **{field: {**table, label: v0 + sgn * h}}), cal0) for sgn in (1, -1)]
            names.append(f"{field}.{label.value}")
            grads.append((vals[0] - vals[1]) / (2 * h))
    h = rel_step * max(abs(cal0), 1.0)
    vals = [loss(base, cal0 + sgn * h) for sgn in (1, -1)]
    names.append("calibration")
    grads.append((vals[0] - vals[1]) / (2 * h))
    return names, np.asarray(grads), L0
