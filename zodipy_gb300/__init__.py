"""zodipy_gb300: ZodiPy's line-of-sight integral on GB300 (sm_103a) CUDA kernels.

A drop-in for the path ``zodipy.Model(...).evaluate(skycoord, obspos=...)``:
same constructor, same ``evaluate`` surface, same parameter dictionaries, with
the per-pixel quadrature running in libzodigb (``include/zodigb.h``).
"""

from . import units
from .coords import SkyCoord, Time
from .fused import ModelSet
from .model import Model
from .number_density import grid_number_density
from .zodiacal_light_model import model_registry

__all__ = ("Model", "ModelSet", "grid_number_density", "model_registry", "units", "SkyCoord", "Time")
