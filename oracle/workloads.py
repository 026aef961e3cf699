"""Inputs of the benchmark workloads for the CPU side — TEST INFRASTRUCTURE ONLY.

The reference arm of ``bench.py`` and the CPU baseline time the oracle
(``zodi_oracle.py``, the numpy restatement of ZodiPy's path) on the same
workload as the GPU, and must do so without importing the package under test.
Everything the oracle needs is built here from committed, reference-held data:

- model parameters: ``tests/golden/ref_models.json``, the parameter
  dictionaries dumped from the reference's own model registry
  (``zodipy/model_registry.py``) by ``tests/golden/make_golden.py``;
- spectral scalars (emissivities, albedos, phase coefficients, solar
  irradiance) and the blackbody table: ``tests/golden/spectral.json``, from the
  reference's ``interp_spectral_param`` (``zodipy/unpack_model.py:140-173``)
  and the oracle's ``planck_table``;
- cutoff radii: the reference's ``COMPONENT_CUTOFFS``
  (``zodipy/line_of_sight.py:19-49``), also in ``ref_models.json``;
- pixel centres of a HEALPix RING map (Gorski et al. 2005, ApJ 622, 759,
  sec. 4), built ring by ring;
- Earth's heliocentric ecliptic position at 2022-01-01T00:00 UTC, the epoch of
  the DIRBE map workloads (Standish's approximate Keplerian elements, the
  method the package uses where astropy is absent; a CPU test keeps this
  constant equal to the package's ephemeris).
"""

from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden")

# heliocentric ecliptic Earth [AU] at 2022-01-01T00:00:00 UTC
EARTH_2022_01_01 = np.array([-0.1747230043053385, 0.9676736707443417, -4.8363258321237025e-05])
EARTH_2022_01_01_ISO = "2022-01-01T00:00:00"


def _load(name: str) -> dict:
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def oracle_desc(model: str, spectral_key: str, degree: int) -> dict:
    """Oracle description (``zodi_oracle.evaluate``) of a Kelsall model at one spectral set.

    ``model``: a key of ref_models.json ("dirbe", "planck18", ...);
    ``spectral_key``: a key of spectral.json of the same model ("dirbe_25um",
    "dirbe_bp_80_130", "planck18_857ghz", ...).
    """
    m = _load("ref_models.json")[model]
    sp = _load("spectral.json")[spectral_key]
    if sp["model"] != model:
        raise ValueError(f"spectral set {spectral_key} belongs to {sp['model']}, not {model}")
    sc = sp["scalars"]
    return {
        "labels": list(m["comps"]),
        "comps": m["comps"],
        "cutoffs": {k: tuple(v) for k, v in m["cutoffs"].items()},
        "T_0": m["T_0"],
        "delta": m["delta"],
        "emissivity": list(sc["emissivity"]),
        "albedo": list(sc["albedo"]),
        "C1": float(sc["C1"]),
        "C2": float(sc["C2"]),
        "C3": float(sc["C3"]),
        "solar_irradiance": float(sc["solar_irradiance"]),
        "bb_table": np.asarray(sp["bb_table"], dtype=np.float64),
        "gauss_quad_degree": int(degree),
    }


def healpix_ring_centres(nside: int) -> np.ndarray:
    """(3, 12 nside^2) float64 unit vectors of the RING-ordered pixel centres.

    Rings i = 1 .. 4 nside - 1 from the north pole: the polar caps hold 4 i
    pixels at 1 - z = i^2 / (3 nside^2) (mirrored in the south), the equatorial
    belt 4 nside pixels at z = (2 nside - i) 2 / (3 nside), every other belt ring
    shifted by half a pixel; phi = (j - 1/2) pi / (2 i) in the caps.
    """
    nside = int(nside)
    fact = 1.0 / (3.0 * nside * nside)
    zs, omzs, phis = [], [], []
    for i in range(1, 4 * nside):
        if i < nside:
            j = np.arange(1, 4 * i + 1, dtype=np.float64)
            omz = i * i * fact
            z, one_minus_z = 1.0 - omz, omz
            phi = (j - 0.5) * np.pi / (2.0 * i)
        elif i <= 3 * nside:
            j = np.arange(1, 4 * nside + 1, dtype=np.float64)
            s = (i - nside + 1) % 2
            z = (2.0 * nside - i) * 2.0 / (3.0 * nside)
            one_minus_z = 1.0 - z
            phi = (j - s / 2.0) * np.pi / (2.0 * nside)
        else:
            k = 4 * nside - i
            j = np.arange(1, 4 * k + 1, dtype=np.float64)
            omz = k * k * fact
            z, one_minus_z = omz - 1.0, 2.0 - omz
            phi = (j - 0.5) * np.pi / (2.0 * k)
        zs.append(np.full(j.size, z))
        omzs.append(np.full(j.size, one_minus_z))
        phis.append(phi)
    z, omz, phi = np.concatenate(zs), np.concatenate(omzs), np.concatenate(phis)
    sin_theta = np.sqrt(omz * (1.0 + z))
    return np.stack([sin_theta * np.cos(phi), sin_theta * np.sin(phi), z])
