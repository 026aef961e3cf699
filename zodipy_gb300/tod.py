"""Time-ordered inputs: body positions at every sample time, on the device.

For a call whose ``obstime`` holds one time per coordinate, the reference
evaluates the ephemeris on hourly knots spanning the first to the last sample
time (``zodipy/bodies.py:16-19``, ``zodipy/model.py:177-180``) and interpolates
with scipy's ``CubicSpline`` to every sample (``bodies.py:22-35``).  Here the
host evaluates the ephemeris on the knots and builds the same spline (its
piecewise-polynomial coefficients, O(hours) work); ``zl_spline_eval`` evaluates
it at the samples on the GPU, so per-sample work never touches the host.
"""

from __future__ import annotations

import numpy as np

from . import engine

# (1 hour).to_value(day): the knot spacing of bodies.py:18
HOUR_IN_DAYS = 1.0 / 24.0


def interp_obstimes(t0: float, t1: float) -> np.ndarray:
    """Hourly knots [MJD] from the first to the last sample time (``bodies.py:16-19``)."""
    return np.arange(t0, t1 + HOUR_IN_DAYS, HOUR_IN_DAYS)


def spline_coefficients(knots: np.ndarray, positions: np.ndarray) -> np.ndarray:
    """(4, K-1, 3) coefficients of the cubic spline through (3, K) positions (``bodies.py:33-34``)."""
    from scipy.interpolate import CubicSpline

    return np.ascontiguousarray(CubicSpline(knots, positions, axis=-1).c, dtype=np.float64)


def spline_positions(knots: np.ndarray, positions: np.ndarray, t_dev):
    """(3, N) float64 CUDA tensor: the spline through ``positions`` at knots, evaluated at ``t_dev``."""
    import torch

    coef = spline_coefficients(knots, positions)
    dev = t_dev.device
    knots_dev = torch.from_numpy(np.ascontiguousarray(knots, dtype=np.float64)).to(dev)
    coef_dev = torch.from_numpy(coef).to(dev)
    return engine.spline_eval(knots_dev, coef_dev, t_dev.to(torch.float64).contiguous())
