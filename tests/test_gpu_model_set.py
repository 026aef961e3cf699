"""ModelSet: several bands of one model in one launch equal each band's own Model.

The fused launch evaluates the same expressions per band (shared geometry and
density, per-band table lookup); the float64 kernel is held to 1e-13 relative
per component, the float32 kernel to 2e-6 (its per-band Kahan sums are the
same, but the compiled schedule differs between band counts)."""

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]


def _close(a, b, rtol):
    """Per component, relative to max(|component|, 1e-3 |pixel total|) (the parity tests' metric)."""
    tot = np.abs(b.sum(axis=0)) if b.ndim == 2 else np.abs(b)
    scale = np.maximum(np.abs(b), 1e-3 * tot)
    assert np.all(np.abs(a - b) <= rtol * scale), float(np.max(np.abs(a - b) / scale))


@pytest.mark.parametrize("precision,rtol", [("float64", 1e-13), ("float32", 2e-6)])
def test_model_set_equals_single_models(lib, precision, rtol):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u
    from zodipy_gb300.healpix import random_sphere

    lam = np.linspace(80, 130, 32)
    models = [zg.Model(x * u.micron, precision=precision) for x in (1.25, 3.5, 12, 25, 60)]
    models.append(zg.Model(lam * u.micron, weights=np.exp(-0.5 * ((lam - 100) / 10) ** 2), precision=precision))
    ms = zg.ModelSet(models)
    dirs = random_sphere(5000, seed=31)
    obs, earth = np.array([0.9, 0.42, 0.003]), np.array([0.91, 0.41, 0.0])
    got = ms.evaluate_xyz(dirs, obs, earth, return_comps=True)
    assert got.shape == (6, 6, 5000)
    for k, m in enumerate(models):
        _close(got[k], m.evaluate_xyz(dirs, obs, earth, return_comps=True), rtol)
    tot = ms.evaluate_xyz(dirs, obs, earth)
    np.testing.assert_array_equal(tot, got.sum(axis=1)) if precision == "float64" else _close(tot, got.sum(axis=1), 1e-15)


def test_model_set_rrm_sky_and_time_ordered(lib):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    models = [zg.Model(x * u.micron, name="rrm-experimental") for x in (12, 25, 60)]
    ms = zg.ModelSet(models)
    rng = np.random.default_rng(2)
    lon, lat = rng.uniform(0, 360, 300), rng.uniform(-90, 90, 300)
    sc = zg.SkyCoord(lon, lat, frame="ecliptic", obstime=zg.Time("2022-03-01"))
    got = np.asarray(ms.evaluate(sc, obspos="earth").value)
    for k, m in enumerate(models):
        _close(got[k], np.asarray(m.evaluate(sc, obspos="earth").value), 1e-13)
    sc_t = zg.SkyCoord(lon, lat, frame="ecliptic", obstime=zg.Time(np.linspace(59600.0, 59603.0, 300), format="mjd"))
    got_t = np.asarray(ms.evaluate(sc_t, obspos="semb-l2", return_comps=True).value)
    for k, m in enumerate(models):
        _close(got_t[k], np.asarray(m.evaluate(sc_t, obspos="semb-l2", return_comps=True).value), 1e-13)
