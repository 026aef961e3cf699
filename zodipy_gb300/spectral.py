"""Host-side spectral set-up: blackbody table and spectral model parameters.

Run once per ``Model`` (and per ``update_parameters``); the results become
scalars and a 100-entry table in the kernel parameter block.

- ``blackbody_table`` restates ``zodipy/blackbody.py:9-13,33-49``: temperatures
  ``linspace(40, 550, 100)`` K and astropy's ``BlackBody`` B_nu in MJy/sr,
  integrated over the bandpass with the trapezoid rule.
- ``interp_spectral_param`` restates ``zodipy/unpack_model.py:140-173``:
  linear (or nearest, for the phase coefficients) interpolation of a tabulated
  parameter in the model's spectral unit, then the trapezoid integral against
  the normalised weights.
"""

from __future__ import annotations

import numpy as np
from scipy import integrate, interpolate

# Exact SI 2019 constants (astropy 6 uses CODATA 2018, which has these values).
H_PLANCK = 6.62607015e-34
K_BOLTZMANN = 1.380649e-23
C_LIGHT = 299792458.0

T_MIN_K = 40.0
T_MAX_K = 550.0
N_TEMPS = 100


def table_temperatures() -> np.ndarray:
    return np.linspace(T_MIN_K, T_MAX_K, N_TEMPS)


def _freq_hz(x: np.ndarray, kind: str, scale: float) -> np.ndarray:
    if kind == "frequency":
        return x * scale
    return C_LIGHT / (x * scale)


def planck_bnu_mjysr(freq_hz: np.ndarray, temps: np.ndarray) -> np.ndarray:
    """B_nu(T) [MJy/sr] on the grid freq x temps: 2 h nu^3 / c^2 / expm1(h nu / k T)."""
    f = np.asarray(freq_hz, dtype=np.float64)[..., np.newaxis]
    with np.errstate(over="ignore"):
        boltzm1 = np.expm1(H_PLANCK * f / (K_BOLTZMANN * temps))
    return 2.0 * H_PLANCK * f**3 / (C_LIGHT**2 * boltzm1) * 1e20


def blackbody_table(x_values, kind: str, scale: float, normalized_weights=None) -> np.ndarray:
    """(2, 100) array ``[T_K, B_MJy/sr]`` for a single x or a bandpass.

    ``x_values`` are in the user's unit (``kind``/``scale`` describe it); the
    bandpass integral runs over those values, as the reference does.
    """
    temps = table_temperatures()
    x = np.asarray(x_values, dtype=np.float64)
    bnu = planck_bnu_mjysr(_freq_hz(x, kind, scale), temps)
    if normalized_weights is None:
        vals = bnu.reshape(N_TEMPS)
    else:
        vals = integrate.trapezoid(np.asarray(normalized_weights) * bnu.T, x)
    return np.asarray([temps, vals], dtype=np.float64)


def normalize_weights(weights, x_values) -> np.ndarray:
    """``weights / trapezoid(weights, x)`` in the user's unit (``zodipy/model.py:94``)."""
    w = np.asarray(weights, dtype=np.float64)
    return w / integrate.trapezoid(w, np.asarray(x_values, dtype=np.float64))


def interp_spectral_param(
    x_model_units,
    normalized_weights,
    model_spectrum,
    parameter,
    use_nearest: bool = False,
    bounds_error: bool = True,
):
    """Spectral parameter at x (or integrated over the bandpass)."""
    spectrum = np.asarray(model_spectrum, dtype=np.float64)
    param = np.asarray(parameter, dtype=np.float64)
    if not np.array_equal(spectrum, np.sort(spectrum)):
        spectrum = np.flip(spectrum)
        param = np.flip(param)
    fill_value = np.nan if bounds_error else "extrapolate"
    f = interpolate.interp1d(
        spectrum,
        param,
        bounds_error=bounds_error,
        fill_value=fill_value,
        kind="nearest" if use_nearest else "linear",
    )
    val = f(np.asarray(x_model_units, dtype=np.float64))
    if normalized_weights is not None:
        return integrate.trapezoid(np.asarray(normalized_weights) * val, x=np.asarray(x_model_units))
    return val
