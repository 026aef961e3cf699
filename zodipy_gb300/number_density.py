"""``grid_number_density``: component densities tabulated on a Cartesian mesh.

Drop-in for ``zodipy.grid_number_density`` (``zodipy/number_density.py:482-536``):
same arguments, same model/TypeError handling, same output layout
(C, ny, nx, nz) — the shape of ``numpy.meshgrid(x, y, z)`` with its default
'xy' indexing.  The densities are evaluated in float64 by libzodigb's
``zl_density_grid`` kernel, which shares its density code with the float64
line-of-sight kernel.

One deliberate difference: coordinates given in a length unit other than AU
are converted to AU (the reference uses the raw numbers of whatever unit it
is given).  Plain arrays are taken as AU.
"""

from __future__ import annotations

import numpy as np

from . import engine, packing
from .coords import Time as _LiteTime
from .model import earth_xyz
from .units import AU, as_quantity
from .zodiacal_light_model import ZodiacalLightModel, model_registry


def _au(v) -> np.ndarray:
    if hasattr(v, "unit"):
        return np.asarray(as_quantity(v).to_value(AU), dtype=np.float64).reshape(-1)
    return np.asarray(v, dtype=np.float64).reshape(-1)


def _mjd(obstime) -> float:
    if isinstance(obstime, str):
        obstime = _LiteTime(obstime)
    mjd = np.asarray(obstime.mjd, dtype=np.float64).reshape(-1)
    if mjd.size != 1:
        raise ValueError("obstime must be a single time")
    return float(mjd[0])


def grid_number_density(x, y, z, obstime, model: str | ZodiacalLightModel = "dirbe", ephemeris: str = "builtin", *, device_output: bool = False):
    """Component-wise densities of the zodiacal components on ``meshgrid(x, y, z)``.

    Returns a float64 numpy array of shape (n_comps, len(y), len(x), len(z));
    with ``device_output=True`` the CUDA tensor is returned instead (no copy
    back to the host).
    """
    if isinstance(model, str):
        zodiacal_light_model = model_registry.get_model(model)
    elif isinstance(model, ZodiacalLightModel):
        zodiacal_light_model = model
    else:
        raise TypeError("model type must be a `str` or a `ZodiacalLightModel`.")

    earth = earth_xyz(np.array([_mjd(obstime)]), ephemeris).reshape(3)
    zl = packing.pack_densities(zodiacal_light_model)
    torch = engine._torch()
    xd, yd, zd = (torch.from_numpy(_au(v)).cuda() for v in (x, y, z))
    out = engine.density_grid(zl, xd, yd, zd, earth)
    if device_output:
        return out
    return out.cpu().numpy()
