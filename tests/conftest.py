import glob
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libzodigb.so")


def golden_cases():
    return sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "los_*.npz")))


def load_case(name):
    with np.load(os.path.join(GOLDEN, f"los_{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def ref_models():
    with open(os.path.join(GOLDEN, "ref_models.json")) as f:
        return json.load(f)


def oracle_desc(case, models=None):
    """Oracle model description for a golden case, built from the reference's own parameter dump."""
    models = models or ref_models()
    name = str(case["model"])
    m = models[name]
    labels = list(m["comps"])
    if m.get("family") == "rrm":
        return {
            "family": "rrm",
            "labels": labels,
            "comps": m["comps"],
            "cutoffs": {k: tuple(v) for k, v in m["cutoffs"].items()},
            "T_0": m["T_0"],
            "delta": m["delta"],
            "calibration": float(case["calibration"]),
            "bb_table": case["bb_table"],
            "gauss_quad_degree": int(case["degree"]),
        }
    return {
        "labels": labels,
        "comps": m["comps"],
        "cutoffs": {k: tuple(v) for k, v in m["cutoffs"].items()},
        "T_0": m["T_0"],
        "delta": m["delta"],
        "emissivity": list(case["emissivity"]),
        "albedo": list(case["albedo"]),
        "C1": float(case["C"][0]),
        "C2": float(case["C"][1]),
        "C3": float(case["C"][2]),
        "solar_irradiance": float(case["C"][3]),
        "bb_table": case["bb_table"],
        "gauss_quad_degree": int(case["degree"]),
    }


def product_model(case, precision="float64"):
    """The product Model configured like a golden case (same x / weights / degree)."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    unit = {"micron": u.micron, "GHz": u.GHz}[str(case["user_unit"])]
    if bool(case["x_is_scalar"]):
        x = float(case["x"][0]) * unit
        weights = None
    else:
        x = case["x"] * unit
        weights = case["weights"]
    return zg.Model(
        x,
        weights=weights,
        name=str(case["model"]),
        gauss_quad_degree=int(case["degree"]),
        extrapolate=True,
        precision=precision,
    )


def cuda_ok():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    from zodipy_gb300 import _build, _lib

    _build.build()
    return _lib.load()


def band_tail_share(u, obs, degree=50, warp=32):
    """Share of (warp of consecutive pixels, quadrature node) pairs at which DIRBE bands 1 and 2
    are both beyond 2.2 delta_zeta of their planes for every pixel of the warp: the nodes the
    DIRBE-layout kernels skip as exactly zero.  float64 geometry of the cloud/band LOS range
    (observer to the 5.2 AU sphere); tells a test that its inputs exercise the skip."""
    from zodipy_gb300 import model_data
    from zodipy_gb300.components import ComponentLabel as L

    x, _ = np.polynomial.legendre.leggauss(degree)
    b = u.T @ obs
    stop = -b + np.sqrt(b * b - (obs @ obs - 5.2**2))
    n_w = u.shape[1] // warp
    dead = np.ones((degree, n_w), bool)
    for lbl in (L.BAND1, L.BAND2):
        p = model_data.DIRBE_COMPONENTS[lbl][1]
        i, om = np.radians(p["i"]), np.radians(p["Omega"])
        nrm = np.array([np.sin(om) * np.sin(i), -np.cos(om) * np.sin(i), np.cos(i)])
        for k in range(degree):
            X = obs[:, None] + (0.5 * stop * (x[k] + 1.0))[None, :] * u
            zeta = np.abs(nrm @ X) / np.linalg.norm(X, axis=0)
            far = zeta > 2.2 * np.radians(p["delta_zeta"])
            dead[k] &= far[: n_w * warp].reshape(n_w, warp).all(axis=1)
    return float(dead.mean())
