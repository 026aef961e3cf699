"""Host-side set-up against the reference: model data, spectral unpacking, validation."""

import json

import numpy as np
import pytest

from conftest import GOLDEN, ref_models


def test_parameter_data_equals_reference_registry():
    from zodipy_gb300 import model_registry

    ref = ref_models()
    for name, rec in ref.items():
        m = model_registry.get_model(name)
        d = m.to_dict()
        assert d["comps"] == rec["comps"], name
        assert list(d["comps"]) == list(rec["comps"]), name  # component (output) order
        if rec.get("family") == "rrm":
            assert d["T_0"] == rec["T_0"] and d["delta"] == rec["delta"]
            assert list(d["calibration"]) == rec["calibration"]
            assert list(np.asarray(m.spectrum.value)) == rec["spectrum"]
            continue
        assert d["T_0"] == rec["T_0"] and d["delta"] == rec["delta"]
        assert list(np.asarray(m.spectrum.value)) == rec["spectrum"]
        assert {k: list(v) for k, v in d["emissivities"].items()} == rec["emissivities"]
        if rec["albedos"] is None:
            assert d["albedos"] is None
        else:
            assert {k: list(v) for k, v in d["albedos"].items()} == rec["albedos"]
        for key in ("solar_irradiance", "C1", "C2", "C3"):
            assert (None if d[key] is None else list(d[key])) == rec[key], (name, key)


def test_cutoffs_equal_reference():
    from zodipy_gb300.components import ComponentLabel
    from zodipy_gb300.zodiacal_light_model import COMPONENT_CUTOFFS

    for name, rec in ref_models().items():
        for lbl, cut in rec["cutoffs"].items():
            assert list(COMPONENT_CUTOFFS[ComponentLabel(lbl)]) == cut


def test_spectral_unpacking_and_blackbody_table_equal_reference():
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    with open(f"{GOLDEN}/spectral.json") as f:
        cases = json.load(f)
    for key, rec in cases.items():
        unit = {"micron": u.micron, "GHz": u.GHz}[rec["unit"]]
        x = rec["x"]
        if rec["weights"] is None:
            m = zg.Model(float(x) * unit, name=rec["model"], extrapolate=True)
        else:
            m = zg.Model(np.asarray(x) * unit, weights=rec["weights"], name=rec["model"], extrapolate=True)
        sc = rec["scalars"]
        np.testing.assert_allclose(m._spectrum["emissivity"], sc["emissivity"], rtol=1e-13, atol=1e-15, err_msg=key)
        np.testing.assert_allclose(m._spectrum["albedo"], sc["albedo"], rtol=1e-13, atol=1e-15, err_msg=key)
        for k in ("C1", "C2", "C3", "solar_irradiance"):
            np.testing.assert_allclose(m._spectrum[k], sc[k], rtol=1e-13, atol=1e-15, err_msg=(key, k))
        np.testing.assert_allclose(m._b_nu_table, np.asarray(rec["bb_table"]), rtol=1e-13, err_msg=key)


def test_micron_and_ghz_give_the_same_setup():
    """Reference tests/test_evaluate.py:33-45: emission equal to 12 decimals for um and GHz input."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    m1 = zg.Model(20.0 * u.micron)
    m2 = zg.Model((299792.458 / 20.0) * u.GHz)
    for k in ("emissivity", "albedo", "C1", "C2", "C3", "solar_irradiance"):
        np.testing.assert_allclose(m1._spectrum[k], m2._spectrum[k], rtol=1e-12)
    np.testing.assert_allclose(m1._b_nu_table, m2._b_nu_table, rtol=1e-12)


def test_constructor_validation_matches_reference():
    """Reference tests/test_model.py:11-51."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    with pytest.raises(u.UnitConversionError):
        zg.Model(20 * u.s)
    with pytest.raises(TypeError):
        zg.Model(20)
    with pytest.raises(ValueError):
        zg.Model(np.linspace(20, 25, 10) * u.micron)
    with pytest.raises(ValueError):
        zg.Model(20 * u.micron, weights=np.random.rand(10))
    with pytest.raises(ValueError):
        zg.Model(np.linspace(20, 25, 15) * u.micron, weights=np.random.rand(10))
    with pytest.raises(ValueError):
        zg.Model(0.5 * u.micron, name="dirbe", extrapolate=False)
    with pytest.raises(ValueError):
        zg.Model(400 * u.micron, name="dirbe", extrapolate=False)
    zg.Model(20 * u.micron, extrapolate=True)
    x = np.linspace(40, 125, 10) * u.GHz
    with pytest.raises(ValueError):
        zg.Model(x, weights=np.random.rand(10), name="planck18", extrapolate=False)
    zg.Model(x, weights=np.random.rand(10), name="planck18", extrapolate=True)
    with pytest.raises(ValueError):
        zg.model_registry.get_model("invalid")


def test_evaluate_validation_matches_reference():
    """Reference tests/test_evaluate.py:98-195 (the checks made before any GPU work)."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    m = zg.Model(20 * u.micron)
    with pytest.raises(TypeError):
        m.evaluate(20)
    with pytest.raises(ValueError):
        m.evaluate(zg.SkyCoord(20, 30, unit=u.deg))
    t = zg.Time("2021-01-01T00:00:00")
    sc = zg.SkyCoord(20, 30, unit=u.deg, obstime=t)
    with pytest.raises(ValueError):
        m.evaluate(sc, obspos="invalid")
    with pytest.raises(TypeError):
        m.evaluate(sc, obspos=[30, 40, 50])
    with pytest.raises(u.UnitConversionError):
        m.evaluate(sc, obspos=[30, 40, 50] * u.s)
    with pytest.raises(ValueError):
        m.evaluate(sc, obspos=np.array([[30, 40, 50], [30, 40, 50]]) * u.AU)
    times = zg.Time([t.mjd + i for i in range(4)], format="mjd")
    with pytest.raises(ValueError):
        m.evaluate(zg.SkyCoord([20, 30], [30, 40], unit=u.deg, obstime=times))
    with pytest.raises(ValueError):
        m.evaluate(
            zg.SkyCoord([20, 30, 40, 50], [30, 40, 30, 20], unit=u.deg, obstime=times), obspos=[1, 2, 3] * u.AU
        )


def test_parameters_round_trip_and_update():
    """get_parameters/update_parameters keep the reference's dict format (model.py:303-333)."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    m = zg.Model(25 * u.micron)
    p = m.get_parameters()
    assert set(p) == {"comps", "spectrum", "T_0", "delta", "emissivities", "albedos", "solar_irradiance", "C1", "C2", "C3"}
    before = m._zl_model.comp[4].p[0]
    p["comps"]["ring"]["R"] = 1.1
    m.update_parameters(p)
    assert m.get_parameters()["comps"]["ring"]["R"] == 1.1
    assert m._zl_model.comp[4].p[0] == 1.1 != before


def test_parameter_vector_round_trip():
    import zodipy_gb300 as zg
    from zodipy_gb300 import params, units as u

    m = zg.Model(1.25 * u.micron)
    v = params.vector_from_model(m.zl_model)
    assert v.size == params.size(m.zl_model) == 78
    m2 = params.model_from_vector(m.zl_model, v)
    np.testing.assert_allclose(params.vector_from_model(m2), v, rtol=1e-14, atol=1e-14)
    names = params.names(m.zl_model, m.comp_labels)
    assert names[:6] == ["comps.cloud.x_0", "comps.cloud.y_0", "comps.cloud.z_0", "comps.cloud.i", "comps.cloud.Omega", "comps.cloud.n_0"]
    assert names[-4:] == ["C1", "C2", "C3", "solar_irradiance"]


def test_rrm_calibration_unpacking():
    """unpack_model.py:110-132: calibration interpolated over the IRAS bands, in Jy/cm."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    for key in ("rrm25_nside8", "rrm12_bandpass"):
        z = np.load(f"{GOLDEN}/los_{key}.npz")
        x = z["x"] * u.micron if not bool(z["x_is_scalar"]) else float(z["x"][0]) * u.micron
        w = None if bool(z["x_is_scalar"]) else z["weights"]
        m = zg.Model(x, weights=w, name="rrm-experimental", extrapolate=True, gauss_quad_degree=int(z["degree"]))
        zl = m.zl_model
        assert zl.family == 1
        np.testing.assert_allclose(zl.spec[0].calibration, float(z["calibration"]), rtol=1e-15)
        assert [zl.comp_T_0[c] for c in range(zl.n_comps)] == [255.0] * 5 + [305.0] + [255.0] * 2
        np.testing.assert_allclose(m._b_nu_table, z["bb_table"], rtol=1e-13)


def test_rrm_parameters_round_trip_and_gradient_layout(lib):
    import zodipy_gb300 as zg
    from zodipy_gb300 import _lib, engine
    from zodipy_gb300 import units as u

    m = zg.Model(25 * u.micron, name="rrm-experimental")
    p = m.get_parameters()
    assert list(p) == ["comps", "spectrum", "T_0", "delta", "calibration"]
    p2 = {**p, "T_0": {**p["T_0"], "fan": 260.0}}
    p2["comps"] = {**p["comps"], "fan": {**p["comps"]["fan"], "Q": 11.0}}
    m.update_parameters(p2)
    assert m.get_parameters()["T_0"]["fan"] == 260.0 and m.get_parameters()["comps"]["fan"]["Q"] == 11.0
    assert m.zl_model.comp_T_0[0] == 260.0 and m.zl_model.comp[0].p[2] == 11.0
    # the fan no longer shares its temperature law with anything, and the bands still share one range
    assert m.zl_model.comp[2].range == m.zl_model.comp[3].range == m.zl_model.comp[4].range
    # the adjoint's gradient vector: every component's parameters, every T_0 and delta, the calibration
    from zodipy_gb300 import params

    n = engine.grad_count(m.zl_model)
    assert n == params.size(m.zl_model) == len(params.names(m.zl_model, m.comp_labels)) == 99
    v = params.vector_from_model(m.zl_model)
    np.testing.assert_array_equal(params.vector_from_model(params.model_from_vector(m.zl_model, v)), v)
    assert engine.backward_workspace_bytes(m.zl_model, 1000) == 8 * 8 * 20 * 8  # comps x tiles x slots x 8 B
    assert isinstance(_lib.ZL_RRM, int)


def test_model_set_rejects_incompatible_models(lib):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    with pytest.raises(TypeError):
        zg.ModelSet([])
    with pytest.raises(ValueError):
        zg.ModelSet([zg.Model(25 * u.micron), zg.Model(857 * u.GHz, name="planck18")])
    with pytest.raises(ValueError):
        zg.ModelSet([zg.Model(25 * u.micron), zg.Model(12 * u.micron, gauss_quad_degree=20)])
    s = zg.ModelSet([zg.Model(x * u.micron) for x in (1.25, 12, 25, 60, 100)])
    assert len(s) == 5 and [z.n_spec for z in s._zls] == [4, 1]


@pytest.mark.parametrize("degree", [1, 2, 7, 50, 100])
def test_quadrature_nodes_ascend(degree):
    """The packed Gauss-Legendre nodes ascend (numpy's leggauss order, the reference's summation
    order): the kernels' band-tail search over the node table relies on it."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    zl = zg.Model(25 * u.micron, gauss_quad_degree=degree).zl_model
    x = np.array(zl.gl_x[: zl.n_nodes])
    assert zl.n_nodes == degree
    assert np.all(np.diff(x) > 0)
