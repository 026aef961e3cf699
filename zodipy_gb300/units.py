"""A small units layer for the ``Model`` front end.

The reference takes astropy ``Quantity``/``SkyCoord``/``Time`` objects
(``zodipy/model.py:36-45,119-126``).  astropy is not a dependency here, so this
module provides the few pieces the front end needs — spectral units
(wavelength/frequency with the spectral equivalency), lengths in AU, angles,
MJy/sr — and converts real astropy objects when they are passed in.  It is
host-side glue only; nothing here runs per pixel.
"""

from __future__ import annotations

import numpy as np

C_SI = 299792458.0  # m/s
AU_M = 149597870700.0


class UnitConversionError(ValueError):
    """Raised when a value cannot be converted to the requested unit."""


class Unit:
    """A named unit: physical kind and scale to the kind's SI unit."""

    __array_ufunc__ = None  # make ``ndarray * unit`` build a Quantity

    def __init__(self, name: str, kind: str, scale: float) -> None:
        self.name = name
        self.kind = kind
        self.scale = scale

    def __rmul__(self, value):
        return Quantity(value, self)

    __mul__ = __rmul__

    def __truediv__(self, other: "Unit") -> "Unit":
        return Unit(f"{self.name} / {other.name}", f"{self.kind}/{other.kind}", self.scale / other.scale)

    def __eq__(self, other) -> bool:
        return isinstance(other, Unit) and self.kind == other.kind and self.scale == other.scale

    def __hash__(self) -> int:
        return hash((self.kind, self.scale))

    def __repr__(self) -> str:
        return self.name

    def to_string(self) -> str:
        return self.name


m = Unit("m", "length", 1.0)
cm = Unit("cm", "length", 1e-2)
mm = Unit("mm", "length", 1e-3)
micron = Unit("micron", "length", 1e-6)
um = micron
nm = Unit("nm", "length", 1e-9)
km = Unit("km", "length", 1e3)
AU = Unit("AU", "length", AU_M)
Hz = Unit("Hz", "frequency", 1.0)
kHz = Unit("kHz", "frequency", 1e3)
MHz = Unit("MHz", "frequency", 1e6)
GHz = Unit("GHz", "frequency", 1e9)
THz = Unit("THz", "frequency", 1e12)
s = Unit("s", "time", 1.0)
day = Unit("d", "time", 86400.0)
deg = Unit("deg", "angle", np.pi / 180.0)
rad = Unit("rad", "angle", 1.0)
K = Unit("K", "temperature", 1.0)
MJy = Unit("MJy", "flux", 1e-20)
Jy = Unit("Jy", "flux", 1e-26)
sr = Unit("sr", "solid_angle", 1.0)
dimensionless = Unit("", "dimensionless", 1.0)

_BY_NAME = {
    u.name: u for u in (m, cm, mm, micron, nm, km, AU, Hz, kHz, MHz, GHz, THz, s, day, deg, rad, K, MJy, Jy, sr)
}
_BY_NAME.update({"um": micron, "µm": micron, "AU": AU, "au": AU})


class Quantity:
    """An array with a unit.  Supports what the front end needs (``to``, ``value``)."""

    def __init__(self, value, unit: Unit | str = dimensionless) -> None:
        if isinstance(unit, str):
            unit = _BY_NAME[unit]
        if isinstance(value, Quantity):
            value = value.to_value(unit)
        self.value = np.asarray(value, dtype=np.float64) if not np.isscalar(value) else np.float64(value)
        self.unit = unit

    # array-like surface -------------------------------------------------
    @property
    def isscalar(self) -> bool:
        return np.ndim(self.value) == 0

    @property
    def size(self) -> int:
        return int(np.size(self.value))

    @property
    def shape(self):
        return np.shape(self.value)

    @property
    def ndim(self) -> int:
        return np.ndim(self.value)

    def __len__(self) -> int:
        return len(self.value)

    def __getitem__(self, item) -> "Quantity":
        return Quantity(np.asarray(self.value)[item], self.unit)

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self.value, dtype=dtype)

    def __repr__(self) -> str:
        return f"<Quantity {self.value!r} {self.unit.name}>"

    def min(self) -> "Quantity":
        return Quantity(np.min(self.value), self.unit)

    def max(self) -> "Quantity":
        return Quantity(np.max(self.value), self.unit)

    def sum(self, axis=None) -> "Quantity":
        return Quantity(np.sum(self.value, axis=axis), self.unit)

    def __mul__(self, other):
        if isinstance(other, Unit):
            return Quantity(self.value, Unit(f"{self.unit.name} {other.name}", self.unit.kind, self.unit.scale))
        return Quantity(self.value * np.asarray(other), self.unit)

    __rmul__ = __mul__

    def __eq__(self, other):
        return np.asarray(self.value) == np.asarray(other.to_value(self.unit) if isinstance(other, Quantity) else other)

    # conversion ----------------------------------------------------------
    def to_value(self, unit: Unit | str, equivalencies=None):
        if isinstance(unit, str):
            unit = _BY_NAME[unit]
        if unit.kind == self.unit.kind:
            return self.value * (self.unit.scale / unit.scale)
        if equivalencies == "spectral" and {unit.kind, self.unit.kind} == {"length", "frequency"}:
            si = self.value * self.unit.scale
            with np.errstate(divide="ignore"):
                return (C_SI / si) / unit.scale
        raise UnitConversionError(f"'{self.unit.name}' ({self.unit.kind}) cannot be converted to '{unit.name}'")

    def to(self, unit: Unit | str, equivalencies=None) -> "Quantity":
        if isinstance(unit, str):
            unit = _BY_NAME[unit]
        return Quantity(self.to_value(unit, equivalencies), unit)


def spectral() -> str:
    """The wavelength <-> frequency equivalency (``nu = c / lambda``)."""
    return "spectral"


def as_quantity(x) -> Quantity:
    """Accept this module's Quantity or an astropy Quantity; raise TypeError otherwise."""
    if isinstance(x, Quantity):
        return x
    unit = getattr(x, "unit", None)
    if unit is not None and hasattr(x, "value") and hasattr(unit, "to_string"):
        name = unit.to_string()
        mapped = _BY_NAME.get(name) or _BY_NAME.get(name.replace(" ", ""))
        if mapped is None:
            phys = str(getattr(unit, "physical_type", ""))
            if "length" in phys:
                return Quantity(x.to_value("m"), m)
            if "frequency" in phys:
                return Quantity(x.to_value("Hz"), Hz)
            if "time" in phys:
                return Quantity(x.to_value("s"), s)
            return Quantity(np.asarray(x.value), Unit(name, phys or "unknown", 1.0))
        return Quantity(np.asarray(x.value), mapped)
    raise TypeError("expected a Quantity (zodipy_gb300.units or astropy.units)")
