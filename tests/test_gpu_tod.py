"""Time-ordered input on the device: spline positions, directions, SEMB-L2, per-pixel observers.

Tolerances: the spline, rotation and SEMB-L2 kernels evaluate the same float64
expressions as scipy / numpy; they may differ by FMA contraction and summation
order only, so they are held to a few ulp (rtol 1e-15 on values of order 1).
The per-pixel-observer forward and adjoint entry points must equal the
observer-record entry points bit for bit (same arithmetic, other memory
layout).  The full time-ordered Model.evaluate is held to the float64 kernel's
parity bound (1e-10) against the oracle fed with the same spline positions.
"""

import numpy as np
import pytest

from conftest import cuda_ok, ref_models

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]


def _cuda(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def test_spline_matches_scipy(lib):
    from scipy.interpolate import CubicSpline

    from zodipy_gb300 import tod
    from zodipy_gb300.ephemeris import earth_position

    t0, t1 = 59580.3, 59583.71
    knots = tod.interp_obstimes(t0, t1)
    pos = earth_position(knots)
    rng = np.random.default_rng(5)
    t = np.concatenate([rng.uniform(t0 - 0.2, t1 + 0.2, 5000), knots, [knots[0] - 1.0, knots[-1] + 1.0]])
    got = tod.spline_positions(knots, pos, _cuda(t)).cpu().numpy()
    ref = CubicSpline(knots, pos, axis=-1)(t)
    np.testing.assert_allclose(got, ref, rtol=1e-15, atol=1e-15)


def test_spline_two_and_three_knots(lib):
    from scipy.interpolate import CubicSpline

    from zodipy_gb300 import tod

    for k in (2, 3):
        knots = np.arange(k, dtype=np.float64) * tod.HOUR_IN_DAYS + 100.0
        pos = np.random.default_rng(k).standard_normal((3, k))
        t = np.linspace(99.9, 100.2, 101)
        got = tod.spline_positions(knots, pos, _cuda(t)).cpu().numpy()
        np.testing.assert_allclose(got, CubicSpline(knots, pos, axis=-1)(t), rtol=1e-14, atol=1e-14)


def test_directions_match_host_rotation(lib):
    from zodipy_gb300 import engine
    from zodipy_gb300.coords import SkyCoord

    rng = np.random.default_rng(9)
    lon = rng.uniform(0, 360, 4096)
    lat = np.degrees(np.arcsin(rng.uniform(-1, 1, 4096)))
    for frame in ("icrs", "galactic", "barycentricmeanecliptic"):
        sc = SkyCoord(lon, lat, frame=frame)
        got = engine.directions(_cuda(sc.lon), _cuda(sc.lat), sc.ecliptic_rotation()).cpu().numpy()
        np.testing.assert_allclose(got, sc.ecliptic_unit_vectors(), rtol=0, atol=2e-15, err_msg=frame)


def test_semb_l2_both_forms(lib):
    from zodipy_gb300 import engine
    from zodipy_gb300.ephemeris import MEAN_DIST_TO_L2, earth_position, semb_l2

    e = earth_position(np.linspace(59000.0, 59010.0, 777))
    got1 = engine.semb_l2(_cuda(e), MEAN_DIST_TO_L2, whole_array_norm=False).cpu().numpy()
    np.testing.assert_allclose(got1, semb_l2(e), rtol=1e-15, atol=0)
    got2 = engine.semb_l2(_cuda(e), MEAN_DIST_TO_L2, whole_array_norm=True).cpu().numpy()
    norm = np.linalg.norm(e)  # what bodies.py:46 computes for a (3, n) array
    np.testing.assert_allclose(got2, e / norm * (norm + MEAN_DIST_TO_L2), rtol=1e-14, atol=0)


def _tod_inputs(n=3000, seed=4):
    from zodipy_gb300.healpix import random_sphere

    t = np.linspace(0.0, 2.0 * np.pi, n)
    u = random_sphere(n, seed=seed)
    obs = np.stack([np.cos(t), np.sin(t), 0.01 * np.sin(3 * t)]) * 1.05
    earth = np.stack([np.cos(t + 0.01), np.sin(t + 0.01), np.zeros(n)])
    return u, obs, earth


@pytest.mark.parametrize("precision", ["float64", "float32"])
@pytest.mark.parametrize("name", ["dirbe", "rrm-experimental"])
def test_forward_tod_equals_record_mode(lib, precision, name):
    """Same pixels through zl_forward (one record per pixel, flags OR-ed on the host) and
    zl_forward_tod (SoA positions, flags OR-ed on the device): identical bits."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import engine, packing
    from zodipy_gb300 import units as u_

    m = zg.Model(25 * u_.micron, name=name)
    u, obs, earth = _tod_inputs()
    n = u.shape[1]
    table = packing.observer_table(m.zl_model, obs, earth, np.arange(n), any_mode=True)
    rec = engine.forward(m.zl_model, _cuda(u), engine.upload_observers(table), n, precision)
    tod_ = engine.forward_tod(m.zl_model, _cuda(u), _cuda(obs), _cuda(earth), precision)
    np.testing.assert_array_equal(tod_[0].cpu().numpy(), rec[0].cpu().numpy())
    np.testing.assert_array_equal(tod_[1].cpu().numpy(), rec[1].cpu().numpy())


def test_backward_tod_equals_record_mode(lib):
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import engine, packing
    from zodipy_gb300 import units as u_

    m = zg.Model(12 * u_.micron)
    u, obs, earth = _tod_inputs(n=2000)
    n = u.shape[1]
    g = torch.randn((1, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(7))
    table = packing.observer_table(m.zl_model, obs, earth, np.arange(n), any_mode=True)
    a = engine.backward(m.zl_model, _cuda(u), engine.upload_observers(table), n, g_total=g).cpu().numpy()
    b = engine.backward_tod(m.zl_model, _cuda(u), _cuda(obs), _cuda(earth), g_total=g).cpu().numpy()
    np.testing.assert_array_equal(a, b)


def test_flags_follow_any_rule(lib):
    """One sample outside the ring's outer sphere collapses the ring's range for every pixel."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import engine
    from zodipy_gb300 import units as u_

    m = zg.Model(25 * u_.micron)
    u, obs, earth = _tod_inputs(n=512)
    inside = engine.forward_tod(m.zl_model, _cuda(u), _cuda(obs * (1.1 / 1.05)), _cuda(earth), "float64")[0]
    obs2 = obs * (1.1 / 1.05)
    obs2[:, 7] = [1.25, 0.0, 0.0]  # outside the ring's 1.2 AU sphere
    outside = engine.forward_tod(m.zl_model, _cuda(u), _cuda(obs2), _cuda(earth), "float64")[0]
    ring = 4
    assert np.all(inside[0, ring].cpu().numpy() != 0)
    np.testing.assert_array_equal(outside[0, ring].cpu().numpy(), 0.0)


def test_model_evaluate_time_ordered(lib):
    """Model.evaluate with one obstime per coordinate (lite SkyCoord, galactic frame) against the
    oracle fed with the same hourly-spline Earth positions and host-rotated directions."""
    from scipy.interpolate import CubicSpline

    import zodipy_gb300 as zg
    from oracle import zodi_oracle as zo
    from zodipy_gb300 import tod
    from zodipy_gb300 import units as u_
    from zodipy_gb300.ephemeris import MEAN_DIST_TO_L2, earth_position

    n = 400
    rng = np.random.default_rng(12)
    mjd = np.sort(rng.uniform(59580.0, 59590.0, n))
    lon = rng.uniform(0, 360, n)
    lat = np.degrees(np.arcsin(rng.uniform(-1, 1, n)))
    sc = zg.SkyCoord(lon, lat, frame="galactic", obstime=zg.Time(mjd, format="mjd"))
    model = zg.Model(25 * u_.micron)
    for obspos in ("earth", "semb-l2"):
        got = model.evaluate(sc, obspos=obspos, return_comps=True)
        got = np.asarray(getattr(got, "value", got))
        knots = tod.interp_obstimes(mjd[0], mjd[-1])
        earth = CubicSpline(knots, earth_position(knots), axis=-1)(mjd)
        if obspos == "earth":
            obs = earth
        else:
            norm = np.linalg.norm(earth)
            obs = earth / norm * (norm + MEAN_DIST_TO_L2)
        m = ref_models()["dirbe"]
        desc = {
            "labels": list(m["comps"]),
            "comps": m["comps"],
            "cutoffs": {k: tuple(v) for k, v in m["cutoffs"].items()},
            "T_0": m["T_0"],
            "delta": m["delta"],
            "emissivity": model._spectrum["emissivity"],
            "albedo": model._spectrum["albedo"],
            "C1": model._spectrum["C1"],
            "C2": model._spectrum["C2"],
            "C3": model._spectrum["C3"],
            "solar_irradiance": model._spectrum["solar_irradiance"],
            "bb_table": model._b_nu_table,
            "gauss_quad_degree": 50,
        }
        ref = zo.evaluate(desc, sc.ecliptic_unit_vectors(), obs, earth)
        err = np.abs(got - ref) - 1e-10 * np.abs(ref)
        assert np.all(err <= 1e-15 * np.abs(ref.sum(axis=0))[None, :]), (obspos, np.max(np.abs(got - ref) / np.abs(ref)))
