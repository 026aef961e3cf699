"""Model definitions (Kelsall, RRM) and the model registry.

Mirrors the reference's ``Kelsall`` / ``RRM`` dataclasses and ``ModelRegistry``
(``zodipy/zodiacal_light_model.py:20-142``, ``zodipy/model_registry.py:4-62``)
so that ``get_parameters()`` / ``update_parameters()`` dictionaries have the
same structure and keys.
"""

from __future__ import annotations

import copy
from dataclasses import dataclass, field
from typing import Mapping, Sequence

import numpy as np

from . import model_data as md
from .components import ComponentLabel, ZodiacalComponent
from .units import GHz, Quantity, UnitConversionError, as_quantity, micron, spectral

# Per-component (inner, outer) cutoff radii of the line of sight
# (zodipy/line_of_sight.py:14-52).
R_0 = float(np.finfo(np.float64).eps)
R_JUPITER = 5.2
R_EARTH = 1.0
_RRM = {lbl: cls(**kw) for lbl, (cls, kw) in md.RRM_COMPONENTS.items()}
COMPONENT_CUTOFFS = {
    ComponentLabel.CLOUD: (R_0, R_JUPITER),
    ComponentLabel.BAND1: (R_0, R_JUPITER),
    ComponentLabel.BAND2: (R_0, R_JUPITER),
    ComponentLabel.BAND3: (R_0, R_JUPITER),
    ComponentLabel.RING: (R_EARTH - 0.2, R_EARTH + 0.2),
    ComponentLabel.FEATURE: (R_EARTH - 0.3, R_EARTH + 0.3),
    # RRM: the cutoffs of the built-in parameters, fixed at import like the reference's
    ComponentLabel.FAN: (R_0, _RRM[ComponentLabel.FAN].R_outer),
    ComponentLabel.INNER_NARROW_BAND: (
        _RRM[ComponentLabel.INNER_NARROW_BAND].R_inner,
        _RRM[ComponentLabel.INNER_NARROW_BAND].R_outer,
    ),
    ComponentLabel.OUTER_NARROW_BAND: (
        _RRM[ComponentLabel.OUTER_NARROW_BAND].R_inner,
        _RRM[ComponentLabel.OUTER_NARROW_BAND].R_outer,
    ),
    ComponentLabel.BROAD_BAND: (_RRM[ComponentLabel.BROAD_BAND].R_inner, _RRM[ComponentLabel.BROAD_BAND].R_outer),
    ComponentLabel.COMET: (_RRM[ComponentLabel.COMET].R_inner, _RRM[ComponentLabel.COMET].R_outer),
    ComponentLabel.INTERSTELLAR: (R_0, md.R_KUIPER_BELT),
    ComponentLabel.RING_RRM: (R_EARTH - 0.2, R_EARTH + 0.2),
    ComponentLabel.FEATURE_RRM: (R_EARTH - 0.3, R_EARTH + 0.3),
}


@dataclass(repr=False)
class ZodiacalLightModel:
    """Base: components and the spectrum over which the model is valid."""

    comps: Mapping[ComponentLabel, ZodiacalComponent]
    spectrum: Quantity

    def to_dict(self) -> dict:
        """Parameter dictionary in the reference's layout (``zodiacal_light_model.py:38-55``)."""
        out: dict = {}
        for key, value in vars(self).items():
            if key == "comps":
                out[key] = {lbl.value: comp.init_dict() for lbl, comp in value.items()}
            elif isinstance(value, dict):
                out[key] = {k.value: v for k, v in value.items()}
            else:
                out[key] = value
        return out

    @property
    def ncomps(self) -> int:
        return len(self.comps)

    def is_valid_at(self, x: Quantity) -> bool:
        """All of x inside the tabulated spectrum (``zodiacal_light_model.py:62-69``)."""
        try:
            xv = as_quantity(x).to_value(self.spectrum.unit, equivalencies=spectral())
        except UnitConversionError as err:
            raise UnitConversionError("Input 'x' must have units convertible to Hz or m.") from err
        lo, hi = np.min(self.spectrum.value), np.max(self.spectrum.value)
        return bool(np.all((lo <= xv) & (xv <= hi)))


@dataclass(repr=False)
class Kelsall(ZodiacalLightModel):
    """Kelsall et al. (1998) model family."""

    T_0: float
    delta: float
    emissivities: Mapping[ComponentLabel, Sequence[float]]
    albedos: Mapping[ComponentLabel, Sequence[float]] | None = None
    solar_irradiance: Sequence[float] | None = None
    C1: Sequence[float] | None = None
    C2: Sequence[float] | None = None
    C3: Sequence[float] | None = None


@dataclass(repr=False)
class RRM(ZodiacalLightModel):
    """Rowan-Robinson & May (2013) model family: grain temperature per component, one calibration."""

    T_0: Mapping[ComponentLabel, float]
    delta: Mapping[ComponentLabel, float]
    calibration: Sequence[float]


@dataclass
class ModelRegistry:
    """Name -> model container (``zodiacal_light_model.py:105-142``)."""

    _registry: dict = field(init=False, default_factory=dict)

    @property
    def models(self) -> list[str]:
        return list(self._registry.keys())

    def register_model(self, name: str, model: ZodiacalLightModel) -> None:
        if (name := name.lower()) in self._registry:
            raise ValueError(f"a model by the name {name!s} is already registered.")
        if not isinstance(model, ZodiacalLightModel):
            raise TypeError("model must be an instance of ZodiacalLightModel.")
        self._registry[name] = model

    def get_model(self, name: str) -> ZodiacalLightModel:
        if (name := name.lower()) not in self._registry:
            raise ValueError(
                f"{name!r} is not a registered Interplanetary Dust model. "
                f"Avaliable models are: {', '.join(self._registry)}."
            )
        return self._registry[name]


def _components(spec: dict) -> dict:
    return {label: cls(**params) for label, (cls, params) in spec.items()}


def _registry() -> ModelRegistry:
    reg = ModelRegistry()
    reg.register_model(
        "dirbe",
        Kelsall(
            comps=_components(md.DIRBE_COMPONENTS),
            spectrum=Quantity(md.DIRBE_BANDS_MICRON, micron),
            T_0=md.T_0_DIRBE,
            delta=md.DELTA_DIRBE,
            emissivities=copy.deepcopy(md.DIRBE_EMISSIVITY),
            albedos=copy.deepcopy(md.DIRBE_ALBEDO),
            solar_irradiance=list(md.DIRBE_SOLAR_IRRADIANCE),
            C1=list(md.DIRBE_C1),
            C2=list(md.DIRBE_C2),
            C3=list(md.DIRBE_C3),
        ),
    )
    for name, comps, emis in (
        ("planck13", md.DIRBE_COMPONENTS, md.PLANCK13_EMISSIVITY),
        ("planck15", md.PLANCK_COMPONENTS, md.PLANCK15_EMISSIVITY),
        ("planck18", md.PLANCK_COMPONENTS, md.PLANCK18_EMISSIVITY),
        ("odegard", md.PLANCK_COMPONENTS, md.ODEGARD_EMISSIVITY),
    ):
        reg.register_model(
            name,
            Kelsall(
                comps=_components(comps),
                spectrum=Quantity(md.PLANCK_BANDS_GHZ, GHz),
                T_0=md.T_0_DIRBE,
                delta=md.DELTA_DIRBE,
                emissivities=copy.deepcopy(emis),
            ),
        )
    reg.register_model(
        "rrm-experimental",
        RRM(
            comps=_components(md.RRM_COMPONENTS),
            spectrum=Quantity(md.IRAS_BANDS_MICRON, micron),
            calibration=list(md.CALIBRATION_RRM),
            T_0=dict(md.T_0_RRM),
            delta=dict(md.DELTA_RRM),
        ),
    )
    return reg


model_registry = _registry()
