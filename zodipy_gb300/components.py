"""Zodiacal dust components of the Kelsall et al. (1998) and Rowan-Robinson & May (2013) models.

The field names and their order are part of the public parameter-dict format
(``Model.get_parameters`` / ``update_parameters``), so they match
``zodipy/component.py:14-223`` of the reference.  Derived geometry (the
offset vector, sin/cos of inclination and ascending node, angles in radians)
is computed once per component like ``component.py:39-44,87-89,133-136`` and
packed into the kernel parameter block by ``zodipy_gb300.packing``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field, fields
from enum import Enum


class ComponentLabel(Enum):
    """Component labels (``component.py:207-223``)."""

    CLOUD = "cloud"
    BAND1 = "band1"
    BAND2 = "band2"
    BAND3 = "band3"
    RING = "ring"
    FEATURE = "feature"
    FAN = "fan"
    COMET = "comet"
    INTERSTELLAR = "interstellar"
    INNER_NARROW_BAND = "inner_narrow_band"
    OUTER_NARROW_BAND = "outer_narrow_band"
    BROAD_BAND = "broad_band"
    RING_RRM = "ring_rrm"
    FEATURE_RRM = "feature_rrm"


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


@dataclass
class Fan(ZodiacalComponent):
    """RRM fan: radial power law gamma, vertical shape Z_0, Q, P, inside R_outer (RRM eq. 3)."""

    gamma: float
    Z_0: float
    Q: float
    P: float
    R_outer: float


@dataclass
class Comet(ZodiacalComponent):
    """RRM cometary dust between R_inner and R_outer."""

    gamma: float
    Z_0: float
    P: float
    amp: float
    R_inner: float
    R_outer: float


@dataclass
class Interstellar(ZodiacalComponent):
    """RRM interstellar dust: a constant density amp."""

    amp: float


@dataclass
class NarrowBand(ZodiacalComponent):
    """RRM narrow asteroidal band: latitude cut beta_nb [deg] with fall-off G (RRM eq. 4)."""

    gamma: float
    A: float
    G: float
    R_inner: float
    R_outer: float
    beta_nb: float


@dataclass
class BroadBand(ZodiacalComponent):
    """RRM broad asteroidal band: Gaussians at +-beta_bb [deg] of width sigma_bb (RRM eq. 5)."""

    gamma: float
    A: float
    R_inner: float
    R_outer: float
    beta_bb: float
    sigma_bb: float


@dataclass
class RingRRM(Ring):
    """RRM circumsolar ring: the Kelsall ring scaled by A."""

    A: float


@dataclass
class FeatureRRM(Feature):
    """RRM Earth-trailing feature: the Kelsall feature scaled by A."""

    A: float


# Numeric component type codes shared with the CUDA kernels (include/zodigb.h).
COMPONENT_TYPE_CODE = {
    Cloud: 0,
    Band: 1,
    Ring: 2,
    Feature: 3,
    Fan: 4,
    Comet: 5,
    Interstellar: 6,
    NarrowBand: 7,
    BroadBand: 8,
    RingRRM: 9,
    FeatureRRM: 10,
}
