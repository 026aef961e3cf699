"""Zodiacal dust components of the Kelsall et al. (1998) model family.

The field names and their order are part of the public parameter-dict format
(``Model.get_parameters`` / ``update_parameters``), so they match
``zodipy/component.py:14-136`` of the reference.  Derived geometry (the
offset vector, sin/cos of inclination and ascending node, angles in radians)
is computed once per component like ``component.py:39-44,87-89,133-136`` and
packed into the kernel parameter block by ``zodipy_gb300.packing``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field, fields
from enum import Enum


class ComponentLabel(Enum):
    """Component labels (``component.py:207-223``; RRM labels are not modelled here)."""

    CLOUD = "cloud"
    BAND1 = "band1"
    BAND2 = "band2"
    BAND3 = "band3"
    RING = "ring"
    FEATURE = "feature"


@dataclass
class ZodiacalComponent:
    """Common geometry: offset from the Sun [AU], inclination and ascending node [deg]."""

    x_0: float
    y_0: float
    z_0: float
    i: float
    Omega: float

    X_0: tuple = field(init=False, repr=False)
    sin_i_rad: float = field(init=False, repr=False)
    cos_i_rad: float = field(init=False, repr=False)
    sin_Omega_rad: float = field(init=False, repr=False)
    cos_Omega_rad: float = field(init=False, repr=False)

    def __post_init__(self) -> None:
        self.X_0 = (float(self.x_0), float(self.y_0), float(self.z_0))
        i_rad = math.radians(self.i)
        o_rad = math.radians(self.Omega)
        self.sin_i_rad = math.sin(i_rad)
        self.cos_i_rad = math.cos(i_rad)
        self.sin_Omega_rad = math.sin(o_rad)
        self.cos_Omega_rad = math.cos(o_rad)

    def init_dict(self) -> dict:
        """The constructor arguments, in declaration order (``to_dict`` format)."""
        return {f.name: getattr(self, f.name) for f in fields(self) if f.init}


@dataclass
class Cloud(ZodiacalComponent):
    """Smooth diffuse cloud: n_0 at 1 AU, radial power law alpha, vertical beta/gamma, widening mu."""

    n_0: float
    alpha: float
    beta: float
    gamma: float
    mu: float


@dataclass
class Band(ZodiacalComponent):
    """Asteroidal dust band: n_0 at 3 AU, shape delta_zeta [deg], v, p, inner cutoff delta_r."""

    n_0: float
    delta_zeta: float
    v: float
    p: float
    delta_r: float
    delta_zeta_rad: float = field(init=False, repr=False)

    def __post_init__(self) -> None:
        super().__post_init__()
        self.delta_zeta_rad = math.radians(self.delta_zeta)


@dataclass
class Ring(ZodiacalComponent):
    """Circumsolar ring: n_0, peak radius R, radial/vertical dispersions."""

    n_0: float
    R: float
    sigma_r: float
    sigma_z: float


@dataclass
class Feature(ZodiacalComponent):
    """Earth-trailing feature: ring parameters plus longitude offset theta and spread [deg]."""

    n_0: float
    R: float
    sigma_r: float
    sigma_z: float
    theta: float
    sigma_theta: float
    theta_rad: float = field(init=False, repr=False)
    sigma_theta_rad: float = field(init=False, repr=False)

    def __post_init__(self) -> None:
        super().__post_init__()
        self.theta_rad = math.radians(self.theta)
        self.sigma_theta_rad = math.radians(self.sigma_theta)


# Numeric component type codes shared with the CUDA kernels (include/zodigb.h).
COMPONENT_TYPE_CODE = {Cloud: 0, Band: 1, Ring: 2, Feature: 3}
