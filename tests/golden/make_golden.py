"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run with the path of a ZodiPy v1.1.3 source tree (the directory that holds
``zodipy/``), given as ``--ref PATH`` or in $ZODIPY_REF_ROOT:

    python tests/golden/make_golden.py --ref PATH [grid | rrm | rrm-grad | configs]

The reference's own numeric modules are executed in place under an astropy
stand-in (oracle/ref_loader.py).  Inputs that the reference would get from
astropy — unit vectors, Earth/observer positions, the blackbody table — are
built here and stored with the outputs, so the fixtures pin the path from
those inputs to the per-component emission.  Outputs:

  ref_models.json     parameter dictionaries of the reference's Kelsall models
  spectral.json       spectral scalars from the reference's interp_spectral_param
  los_<case>.npz      inputs + reference per-component emission for one call
  dirbe_idl.npz       inputs + reference emission for the DIRBE IDL known-answer
                      points (tests/dirbe_tabulated.py of the reference)
  grid_<case>.npz     inputs + reference grid_number_density output

``... grid`` regenerates only the grid fixtures, ``... rrm`` only
ref_models.json and the RRM fixtures, ``... rrm-grad`` only the RRM gradient
fixtures, ``... configs`` only the fixtures on the
benchmark configurations' inputs (los_cfg*.npz).
"""

from __future__ import annotations

import ast
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import zodi_oracle  # noqa: E402
from oracle.ref_loader import (  # noqa: E402
    REF_ROOT_ENV,
    load_reference,
    reference_evaluate,
    reference_fd_gradient,
    reference_fd_gradient_rrm,
    reference_rrm_calibration,
    reference_spectral_scalars,
)
from zodipy_gb300.ephemeris import earth_position, iso_to_mjd  # noqa: E402
from zodipy_gb300.healpix import pix2vec_ring, random_sphere  # noqa: E402

C_UM_GHZ = 299792.458  # nu[GHz] = C / lambda[um]


def dump_models(ref) -> dict:
    out = {}
    reg = ref.model_registry.model_registry
    for name in reg.models:
        m = reg.get_model(name)
        d = m.to_dict()

        def seq(v):
            return None if v is None else [float(x) for x in v]

        cutoffs = {lbl.value: [float(v) for v in ref.line_of_sight.COMPONENT_CUTOFFS[lbl]] for lbl in m.comps}
        comps = {k: {kk: float(vv) for kk, vv in v.items()} for k, v in d["comps"].items()}
        if type(m).__name__ == "RRM":
            out[name] = {
                "family": "rrm",
                "comps": comps,
                "spectrum": seq(np.asarray(m.spectrum)),
                "spectrum_unit": "micron",
                "T_0": {k: float(v) for k, v in d["T_0"].items()},
                "delta": {k: float(v) for k, v in d["delta"].items()},
                "calibration": seq(d["calibration"]),
                "cutoffs": cutoffs,
            }
            continue

        out[name] = {
            "comps": {k: {kk: float(vv) for kk, vv in v.items()} for k, v in d["comps"].items()},
            "spectrum": seq(np.asarray(m.spectrum)),
            "spectrum_unit": "micron" if name == "dirbe" else "GHz",
            "T_0": float(d["T_0"]),
            "delta": float(d["delta"]),
            "emissivities": {k: seq(v) for k, v in d["emissivities"].items()},
            "albedos": None if d["albedos"] is None else {k: seq(v) for k, v in d["albedos"].items()},
            "solar_irradiance": seq(d["solar_irradiance"]),
            "C1": seq(d["C1"]),
            "C2": seq(d["C2"]),
            "C3": seq(d["C3"]),
            "cutoffs": cutoffs,
        }
    return out


def model_unit(name: str) -> str:
    return "micron" if name in ("dirbe", "rrm-experimental") else "GHz"


def to_model_units(x, user_unit: str, name: str) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    if user_unit == model_unit(name):
        return x
    return C_UM_GHZ / x


def make_case(ref, name, x, user_unit, weights, u, obs, earth, degree):
    """Run the reference for one call; returns the npz payload."""
    w_norm = None
    if weights is not None:
        w = np.asarray(weights, dtype=np.float64)
        w_norm = w / np.trapezoid(w, np.asarray(x, dtype=np.float64))
    bb = zodi_oracle.planck_table(x, w_norm, unit=user_unit)
    xm = to_model_units(x, user_unit, name)
    out = reference_evaluate(ref, name, u, obs, earth, bb, xm, w_norm, degree, bounds_error=False)
    if name.startswith("rrm"):
        scal = {"emissivity": [], "albedo": [], "C1": 0.0, "C2": 0.0, "C3": 0.0, "solar_irradiance": 0.0}
        scal["calibration"] = reference_rrm_calibration(ref, name, xm, w_norm)
    else:
        scal = reference_spectral_scalars(ref, name, xm, w_norm, bounds_error=False)
        scal["calibration"] = 0.0
    return dict(
        model=np.array(name),
        x=np.atleast_1d(np.asarray(x, dtype=np.float64)),
        x_is_scalar=np.array(weights is None),
        user_unit=np.array(user_unit),
        weights=np.zeros(0) if weights is None else np.asarray(weights, dtype=np.float64),
        unit_vectors=np.asarray(u, dtype=np.float64),
        obs=np.asarray(obs, dtype=np.float64),
        earth=np.asarray(earth, dtype=np.float64),
        bb_table=bb,
        degree=np.array(degree),
        emissivity=np.array(scal["emissivity"]),
        albedo=np.array(scal["albedo"]),
        C=np.array([scal["C1"], scal["C2"], scal["C3"], scal["solar_irradiance"]]),
        calibration=np.array(scal["calibration"]),
        ref_out=out,
    )


def dirbe_idl_fixture(ref_root: str):
    """DAYS/LON/LAT/TABULATED_DIRBE_EMISSION read as literals from the reference's test data."""
    path = os.path.join(ref_root, "tests", "dirbe_tabulated.py")
    tree = ast.parse(open(path).read())
    vals = {}
    for node in tree.body:
        if isinstance(node, (ast.Assign, ast.AnnAssign)):
            target = node.targets[0] if isinstance(node, ast.Assign) else node.target
            if isinstance(target, ast.Name) and target.id in ("DAYS", "LON", "LAT", "TABULATED_DIRBE_EMISSION"):
                vals[target.id] = ast.literal_eval(node.value)
    return vals


def make_grids(ref) -> None:
    """Reference ``grid_number_density`` (number_density.py:482-536) on small meshes.

    The reference asks astropy for Earth's position (bodies.py:53-62); the
    fixture fixes it instead, by replacing that lookup with the stored vector.
    """
    nd = ref.number_density
    grid_cases = {
        "dirbe_wide": ("dirbe", np.linspace(-3, 3, 13), np.linspace(-2.5, 2.5, 11), np.linspace(-1, 1, 7), "2022-01-01T00:00:00"),
        "dirbe_near_earth": ("dirbe", np.linspace(-0.9, -0.1, 17), np.linspace(-1.3, -0.5, 9), np.linspace(-0.1, 0.1, 5), "2022-06-01T00:00:00"),
        "planck13_wide": ("planck13", np.linspace(0, 5, 10), np.linspace(0, 5, 10), np.linspace(0, 2, 6), "2022-01-01T00:00:00"),
        "planck18_ring": ("planck18", np.linspace(0.7, 1.3, 8), np.linspace(-1.3, -0.7, 8), np.linspace(-0.05, 0.05, 3), "1990-06-11T00:00:00"),
    }
    saved = nd.get_earthpos_inst
    try:
        for key, (name, x, y, z, iso) in grid_cases.items():
            earth = earth_position(iso_to_mjd(iso)).reshape(3)
            nd.get_earthpos_inst = lambda obstime, ephemeris, e=earth: e.copy()
            out = nd.grid_number_density(x, y, z, obstime=None, model=name)
            np.savez_compressed(
                os.path.join(HERE, f"grid_{key}.npz"),
                model=np.array(name),
                x=x,
                y=y,
                z=z,
                obstime=np.array(iso),
                earth=earth,
                ref_out=np.asarray(out, dtype=np.float64),
            )
    finally:
        nd.get_earthpos_inst = saved


def make_rrm(ref) -> None:
    """Rowan-Robinson & May model: line-of-sight cases and density grids."""
    earth_2022 = earth_position(iso_to_mjd("2022-01-01T00:00:00"))
    earth_1990 = earth_position(iso_to_mjd("1990-06-11T00:00:00"))
    dirs_rand = random_sphere(256, seed=17)
    lam = np.linspace(10.0, 14.0, 16)
    cases = {
        # observer at 1 AU: inside every inner cutoff
        "rrm25_nside8": ("rrm-experimental", 25.0, None, pix2vec_ring(8), [0.9833, 0.0, 0.0], earth_2022, 50),
        # just outside Mars's orbit: the fan's outer and the bands' and comet's inner cutoffs collapse to eps
        "rrm60_mars": ("rrm-experimental", 60.0, None, dirs_rand, [1.2, -1.05, 0.02], earth_2022, 50),
        # beyond the asteroid belt: the bands' both cutoffs collapse
        "rrm100_belt": ("rrm-experimental", 100.0, None, dirs_rand, [2.5, 2.6, 0.1], earth_2022, 50),
        "rrm12_bandpass": ("rrm-experimental", lam, np.exp(-0.5 * ((lam - 12.0) / 1.0) ** 2), dirs_rand,
                           [0.2, 0.99, 0.0], earth_1990, 100),
    }
    for key, (name, x, w, u, obs, earth, deg) in cases.items():
        payload = make_case(ref, name, x, "micron", w, u, np.asarray(obs, dtype=np.float64), earth, deg)
        np.savez_compressed(os.path.join(HERE, f"los_{key}.npz"), **payload)
    nd = ref.number_density
    grid_cases = {
        "rrm_wide": (np.linspace(0, 5, 10), np.linspace(0, 5, 10), np.linspace(0, 2, 6), "2022-01-01T00:00:00"),
        "rrm_inner": (np.linspace(-2, 2, 21), np.linspace(-2, 2, 17), np.linspace(-0.3, 0.3, 7), "2022-06-01T00:00:00"),
    }
    saved = nd.get_earthpos_inst
    try:
        for key, (x, y, z, iso) in grid_cases.items():
            earth = earth_position(iso_to_mjd(iso)).reshape(3)
            nd.get_earthpos_inst = lambda obstime, ephemeris, e=earth: e.copy()
            out = nd.grid_number_density(x, y, z, obstime=None, model="rrm-experimental")
            np.savez_compressed(
                os.path.join(HERE, f"grid_{key}.npz"),
                model=np.array("rrm-experimental"),
                x=x,
                y=y,
                z=z,
                obstime=np.array(iso),
                earth=earth,
                ref_out=np.asarray(out, dtype=np.float64),
            )
    finally:
        nd.get_earthpos_inst = saved


def make_config_cases(ref) -> None:
    """The reference on seeded subsets of each benchmark configuration's own inputs
    (``los_cfg*.npz``): the map, observers, spectral set and degree of the five configs,
    at a size the reference runs in seconds.  The GPU tests compare the full-size runs with
    the oracle, and these fixtures pin the oracle to the reference on the same geometry."""
    from zodipy_gb300.batch import uneven_observers

    rng = np.random.default_rng(20260101)
    earth_2022 = earth_position(iso_to_mjd("2022-01-01T00:00:00"))
    lam = np.linspace(80, 130, 64)
    w_bp = np.exp(-0.5 * ((lam - 100) / 10) ** 2)

    def healpix_subset(nside, n):
        idx = np.sort(rng.choice(12 * nside * nside, n, replace=False))
        return pix2vec_ring(nside, idx)

    # config 3: per-pixel observers of the first four batch observers (one map of directions each)
    bobs, _ = uneven_observers(256, seed=2024)
    n3 = 96
    u3 = random_sphere(4 * n3, seed=2025)
    obs3 = np.repeat(bobs[:, :4], n3, axis=1)
    # config 5: three observers at 0/120/240 deg on the 1 AU circle, nside 2048
    ang = np.radians([0.0, 120.0, 240.0])
    n5 = 128
    u5 = healpix_subset(2048, 3 * n5)
    obs5 = np.repeat(np.stack([np.cos(ang), np.sin(ang), np.zeros(3)]), n5, axis=1)
    cases = {
        "cfg1_dirbe25_nside128": ("dirbe", 25.0, "micron", None, healpix_subset(128, 1024), [0.9833, 0.0, 0.0], 50),
        "cfg2_bandpass_nside512": ("dirbe", lam, "micron", w_bp, healpix_subset(512, 1024), [0.7071, 0.7071, 0.0], 50),
        "cfg3_planck18_batch": ("planck18", 857.0, "GHz", None, u3, obs3, 50),
        "cfg4_dirbe12_nside256": ("dirbe", 12.0, "micron", None, healpix_subset(256, 1024), [0.9833, 0.0, 0.0], 50),
        "cfg5_dirbe60_gl100": ("dirbe", 60.0, "micron", None, u5, obs5, 100),
    }
    for key, (name, x, unit, w, u, obs, deg) in cases.items():
        payload = make_case(ref, name, x, unit, w, u, np.asarray(obs, dtype=np.float64), earth_2022, deg)
        np.savez_compressed(os.path.join(HERE, f"los_{key}.npz"), **payload)


def make_rrm_gradients(ref) -> None:
    """Central finite differences of L = sum_i a_i total_i through the reference's own RRM code
    (grad_rrm*.npz): every component parameter, T_0 and delta of every component, the
    calibration."""
    earth_2022 = earth_position(iso_to_mjd("2022-01-01T00:00:00"))
    cases = {
        # observer at 1 AU: inside the fan, below the bands and the comet
        "rrm25": (25.0, random_sphere(24, seed=31), [0.9833, 0.0, 0.0]),
        # just outside the fan's outer cutoff: the observer sits among the bands
        "rrm60_belt": (60.0, random_sphere(24, seed=32), [1.9, -1.1, 0.04]),
    }
    for key, (x, u, obs) in cases.items():
        obs = np.asarray(obs, dtype=np.float64)
        bb = zodi_oracle.planck_table(x, None, unit="micron")
        a = np.random.default_rng(98).uniform(0.5, 1.5, u.shape[1])
        names, grad, L0 = reference_fd_gradient_rrm(ref, "rrm-experimental", u, obs, earth_2022, bb,
                                                    np.asarray(x, dtype=np.float64), None, 50, a)
        np.savez_compressed(
            os.path.join(HERE, f"grad_{key}.npz"),
            model=np.array("rrm-experimental"),
            x=np.atleast_1d(np.float64(x)),
            user_unit=np.array("micron"),
            unit_vectors=u,
            obs=obs,
            earth=np.asarray(earth_2022, dtype=np.float64),
            weights_a=a,
            names=np.array(names),
            fd_grad=grad,
            loss=np.array(L0),
        )


def parse_args(argv):
    """(reference root, remaining words): ``--ref PATH`` wins over $ZODIPY_REF_ROOT."""
    argv = list(argv)
    ref_root = os.environ.get(REF_ROOT_ENV)
    if "--ref" in argv:
        i = argv.index("--ref")
        ref_root = argv[i + 1]
        del argv[i : i + 2]
    if not ref_root:
        raise SystemExit(f"usage: make_golden.py --ref PATH [grid|rrm]  (or set {REF_ROOT_ENV})")
    return ref_root, argv


def main() -> None:
    ref_root, words = parse_args(sys.argv[1:])
    ref = load_reference(ref_root)
    sys.argv[1:] = words
    if sys.argv[1:] == ["grid"]:
        make_grids(ref)
        print("wrote grid fixtures to", HERE)
        return
    if sys.argv[1:] == ["configs"]:
        make_config_cases(ref)
        print("wrote benchmark-configuration fixtures to", HERE)
        return
    if sys.argv[1:] == ["rrm"]:
        with open(os.path.join(HERE, "ref_models.json"), "w") as f:
            json.dump(dump_models(ref), f, indent=1)
        make_rrm(ref)
        make_rrm_gradients(ref)
        print("wrote RRM fixtures to", HERE)
        return
    if sys.argv[1:] == ["rrm-grad"]:
        make_rrm_gradients(ref)
        print("wrote RRM gradient fixtures to", HERE)
        return
    make_grids(ref)
    make_rrm(ref)
    make_rrm_gradients(ref)
    make_config_cases(ref)
    models = dump_models(ref)
    with open(os.path.join(HERE, "ref_models.json"), "w") as f:
        json.dump(models, f, indent=1)

    # spectral scalars for a spread of inputs (delta, bandpass, GHz input, extrapolation)
    spec_cases = {
        "dirbe_25um": ("dirbe", 25.0, "micron", None),
        "dirbe_1p25um": ("dirbe", 1.25, "micron", None),
        "dirbe_3p1um": ("dirbe", 3.1, "micron", None),
        "dirbe_20um_as_ghz": ("dirbe", C_UM_GHZ / 20.0, "GHz", None),
        "dirbe_300um_extrap": ("dirbe", 300.0, "micron", None),
        "planck18_857ghz": ("planck18", 857.0, "GHz", None),
        "planck13_600ghz": ("planck13", 600.0, "GHz", None),
        "dirbe_bp_80_130": ("dirbe", list(np.linspace(80, 130, 64)), "micron", list(np.exp(-0.5 * ((np.linspace(80, 130, 64) - 100) / 10) ** 2))),
        "dirbe_bp_1_3": ("dirbe", list(np.linspace(1.1, 3.0, 17)), "micron", list(np.linspace(0.2, 1.0, 17))),
    }
    spectral = {}
    for key, (name, x, unit, w) in spec_cases.items():
        xa = np.asarray(x, dtype=np.float64)
        w_norm = None if w is None else np.asarray(w) / np.trapezoid(np.asarray(w), xa)
        xm = to_model_units(xa, unit, name)
        spectral[key] = {
            "model": name,
            "x": xa.tolist() if xa.ndim else float(xa),
            "unit": unit,
            "weights": w,
            "scalars": reference_spectral_scalars(ref, name, xm, w_norm, bounds_error=False),
            "bb_table": zodi_oracle.planck_table(xa, w_norm, unit=unit).tolist(),
        }
    with open(os.path.join(HERE, "spectral.json"), "w") as f:
        json.dump(spectral, f, indent=1)

    rng = np.random.default_rng(20240611)
    earth_2022 = earth_position(iso_to_mjd("2022-01-01T00:00:00"))
    earth_1990 = earth_position(iso_to_mjd("1990-06-11T00:00:00"))
    dirs_hp8 = pix2vec_ring(8)
    dirs_rand = random_sphere(256, seed=7)
    cases = {
        "dirbe25_nside8": ("dirbe", 25.0, "micron", None, dirs_hp8, [0.9833, 0.0, 0.0], earth_2022, 50),
        "dirbe1p25_scatter": ("dirbe", 1.25, "micron", None, dirs_rand, earth_1990, earth_1990, 50),
        "dirbe3p5_scatter": ("dirbe", 3.5, "micron", None, dirs_rand, [0.0, 1.01, 0.002], earth_1990, 50),
        "planck18_857": ("planck18", 857.0, "GHz", None, dirs_rand, [np.cos(2.0), np.sin(2.0), 0.013], earth_2022, 50),
        "planck13_545": ("planck13", 545.0, "GHz", None, dirs_rand, [0.3, -0.95, 0.0], earth_2022, 50),
        "odegard_353": ("odegard", 353.0, "GHz", None, dirs_rand, [-0.98, 0.2, -0.01], earth_2022, 50),
        "dirbe_bandpass": (
            "dirbe",
            np.linspace(80, 130, 64),
            "micron",
            np.exp(-0.5 * ((np.linspace(80, 130, 64) - 100) / 10) ** 2),
            dirs_rand,
            [0.7071, 0.7071, 0.0],
            earth_2022,
            50,
        ),
        "dirbe12_gl100": ("dirbe", 12.0, "micron", None, dirs_rand, [0.9833, 0.0, 0.0], earth_2022, 100),
        "dirbe25_mars": ("dirbe", 25.0, "micron", None, dirs_rand, [1.1, -1.1, 0.03], earth_2022, 50),
        "dirbe25_venus": ("dirbe", 25.0, "micron", None, dirs_rand, [0.5, 0.5, 0.01], earth_2022, 50),
        "dirbe60_gl7": ("dirbe", 60.0, "micron", None, dirs_rand, [0.2, 0.99, 0.0], earth_2022, 7),
        "dirbe25_b0": ("dirbe", 25.0, "micron", None, dirs_rand[:, :32], [0.0, 0.0, 0.4], earth_2022, 20),
        "dirbe25_single": ("dirbe", 25.0, "micron", None, dirs_rand[:, :1], [0.9833, 0.0, 0.0], earth_2022, 50),
    }
    for key, (name, x, unit, w, u, obs, earth, deg) in cases.items():
        payload = make_case(ref, name, x, unit, w, u, np.asarray(obs, dtype=np.float64), earth, deg)
        np.savez_compressed(os.path.join(HERE, f"los_{key}.npz"), **payload)

    # time-ordered data: a position per pixel (3, N), as the reference takes for obstime.size > 1
    n_tod = 128
    t = np.linspace(0.0, 2.0 * np.pi, n_tod)
    obs_tod = np.stack([np.cos(t), np.sin(t), 0.01 * np.sin(3 * t)])
    earth_tod = np.stack([np.cos(t + 0.01), np.sin(t + 0.01), np.zeros(n_tod)])
    payload = make_case(ref, "dirbe", 25.0, "micron", None, random_sphere(n_tod, seed=11), obs_tod, earth_tod, 50)
    np.savez_compressed(os.path.join(HERE, "los_dirbe25_tod.npz"), **payload)

    # DIRBE IDL known-answer points (observer = Earth, approximate ephemeris)
    kat = dirbe_idl_fixture(ref_root)
    start = iso_to_mjd("1990-01-01T00:00:00")
    lon, lat = np.radians(kat["LON"]), np.radians(kat["LAT"])
    u = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)])
    mjd = start + np.asarray(kat["DAYS"], dtype=np.float64) - 1.0
    earth = earth_position(mjd)
    bands = sorted(kat["TABULATED_DIRBE_EMISSION"])
    ref_tot = np.zeros((len(bands), len(mjd)))
    tab = np.zeros_like(ref_tot)
    for bi, band in enumerate(bands):
        for j in range(len(mjd)):
            p = make_case(ref, "dirbe", float(band), "micron", None, u[:, j : j + 1], earth[:, j], earth[:, j], 50)
            ref_tot[bi, j] = p["ref_out"].sum(axis=0)[0]
        tab[bi] = kat["TABULATED_DIRBE_EMISSION"][band]
    np.savez_compressed(
        os.path.join(HERE, "dirbe_idl.npz"),
        bands=np.asarray(bands, dtype=np.float64),
        unit_vectors=u,
        earth=earth,
        mjd=mjd,
        ref_total=ref_tot,
        tabulated=tab,
    )
    # finite-difference gradients of L = sum_i a_i total_i through the reference itself
    grad_cases = {
        "dirbe25": ("dirbe", 25.0, "micron", random_sphere(24, seed=21), [0.9833, 0.0, 0.0], earth_2022),
        "dirbe1p25": ("dirbe", 1.25, "micron", random_sphere(24, seed=22), earth_1990, earth_1990),
        "planck18_857": ("planck18", 857.0, "GHz", random_sphere(24, seed=23), [np.cos(2.0), np.sin(2.0), 0.013], earth_2022),
    }
    for key, (name, x, unit, u, obs, earth) in grad_cases.items():
        obs = np.asarray(obs, dtype=np.float64)
        bb = zodi_oracle.planck_table(x, None, unit=unit)
        xm = to_model_units(x, unit, name)
        a = np.random.default_rng(99).uniform(0.5, 1.5, u.shape[1])
        names, grad, L0 = reference_fd_gradient(ref, name, u, obs, earth, bb, xm, None, 50, a)
        np.savez_compressed(
            os.path.join(HERE, f"grad_{key}.npz"),
            model=np.array(name),
            x=np.atleast_1d(np.float64(x)),
            user_unit=np.array(unit),
            unit_vectors=u,
            obs=obs,
            earth=np.asarray(earth, dtype=np.float64),
            weights_a=a,
            names=np.array(names),
            fd_grad=grad,
            loss=np.array(L0),
        )
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
