"""Light stand-ins for astropy's ``Time`` and ``SkyCoord`` (host-side glue).

``Model.evaluate`` accepts real astropy objects when astropy is installed.
Without it, these classes carry what the evaluation needs: observation
times as MJD and sky directions as heliocentric-ecliptic unit vectors.  Frame
rotations are the fixed J2000 matrices (galactic -> ICRS from the IAU 1958
definition via FK5; ICRS -> mean ecliptic of J2000 with the IAU 2006
obliquity 84381.406"), good to ~1e-7 rad — frame bias and the equinox of date
are not modelled, and need not be for sky maps of this smoothness.
"""

from __future__ import annotations

import numpy as np

from .ephemeris import iso_to_mjd
from .units import Quantity, as_quantity, deg

_EPS0 = np.radians(84381.406 / 3600.0)
# ICRS (equatorial J2000) -> ecliptic J2000
_EQ_TO_ECL = np.array(
    [[1.0, 0.0, 0.0], [0.0, np.cos(_EPS0), np.sin(_EPS0)], [0.0, -np.sin(_EPS0), np.cos(_EPS0)]]
)
# galactic -> equatorial J2000 (transpose of the standard equatorial -> galactic matrix)
_GAL_TO_EQ = np.array(
    [
        [-0.0548755604162154, -0.8734370902348850, -0.4838350155487132],
        [+0.4941094278755837, -0.4448296299600112, +0.7469822444972189],
        [-0.8676661490190047, -0.1980763734312015, +0.4559837761750669],
    ]
).T

_FRAMES = ("icrs", "galactic", "barycentricmeanecliptic", "heliocentricmeanecliptic", "ecliptic")


class Time:
    """Observation time(s) as MJD; accepts ISO strings, MJD floats or lists of them."""

    def __init__(self, value, format: str | None = None) -> None:
        if isinstance(value, Time):
            self.mjd = value.mjd
            return
        if isinstance(value, str):
            self.mjd = np.float64(iso_to_mjd(value))
        elif isinstance(value, (list, tuple)) and value and isinstance(value[0], str):
            self.mjd = np.array([iso_to_mjd(v) for v in value])
        else:
            if format not in (None, "mjd"):
                raise ValueError(f"unsupported time format {format!r}")
            arr = np.asarray(value, dtype=np.float64)
            self.mjd = arr if arr.ndim else np.float64(arr)

    @property
    def size(self) -> int:
        return int(np.size(self.mjd))

    @property
    def isscalar(self) -> bool:
        return np.ndim(self.mjd) == 0

    def __getitem__(self, item) -> "Time":
        return Time(np.asarray(self.mjd)[item], format="mjd")


class SkyCoord:
    """Directions given as longitude/latitude in one of a few fixed frames."""

    def __init__(self, lon, lat, *, unit=deg, frame: str = "icrs", obstime=None) -> None:
        frame = frame.lower()
        if frame not in _FRAMES:
            raise ValueError(f"unsupported frame {frame!r}")
        lon_q = lon if hasattr(lon, "unit") else Quantity(lon, unit)
        lat_q = lat if hasattr(lat, "unit") else Quantity(lat, unit)
        self.lon = np.radians(np.asarray(as_quantity(lon_q).to_value(deg), dtype=np.float64))
        self.lat = np.radians(np.asarray(as_quantity(lat_q).to_value(deg), dtype=np.float64))
        self.frame = frame
        self.obstime = None if obstime is None else Time(obstime)

    @property
    def isscalar(self) -> bool:
        return np.ndim(self.lon) == 0

    @property
    def size(self) -> int:
        return int(np.size(self.lon))

    def ecliptic_rotation(self) -> np.ndarray:
        """3x3 matrix from this frame's Cartesian axes to the ecliptic ones."""
        if self.frame == "icrs":
            return _EQ_TO_ECL
        if self.frame == "galactic":
            return _EQ_TO_ECL @ _GAL_TO_EQ
        return np.eye(3)

    def ecliptic_unit_vectors(self) -> np.ndarray:
        """(3, n) heliocentric-ecliptic unit vectors of the directions."""
        cl = np.cos(self.lat)
        v = np.stack([np.atleast_1d(cl * np.cos(self.lon)), np.atleast_1d(cl * np.sin(self.lon)), np.atleast_1d(np.sin(self.lat))])
        if self.frame == "icrs":
            v = _EQ_TO_ECL @ v
        elif self.frame == "galactic":
            v = _EQ_TO_ECL @ (_GAL_TO_EQ @ v)
        return v
