"""Config-5 shape at reduced size: three DIRBE bands fused in one launch, three
observers, Gauss-Legendre degree 100; float32 and float64 kernels against the
CPU oracle on a random subset, and the adjoint of an L2 loss against finite
differences of the float64 kernel for a few parameters."""

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]


def _setup(nside=32):
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import engine, packing
    from zodipy_gb300 import units as u
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import pix2vec_ring_torch

    models = [zg.Model(w * u.micron, name="dirbe", gauss_quad_degree=100) for w in (12.0, 25.0, 60.0)]
    zl = fuse_models(models)
    umap = pix2vec_ring_torch(nside, "cuda")
    npix = umap.shape[1]
    uu = umap.repeat(1, 3).contiguous()
    ang = np.radians([0.0, 120.0, 240.0])
    obs = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)])
    earth = np.array([-0.17, 0.97, 0.0])
    tab = packing.observer_table(zl, obs, earth, np.array([0, npix, 2 * npix]), any_mode=False)
    return models, zl, uu, npix, obs, earth, engine.upload_observers(tab)


def _desc(model):
    from zodipy_gb300.zodiacal_light_model import COMPONENT_CUTOFFS

    m = model.get_parameters()
    return {
        "labels": list(m["comps"]),
        "comps": m["comps"],
        "cutoffs": {lbl.value: COMPONENT_CUTOFFS[lbl] for lbl in model._ipd_model.comps},
        "T_0": m["T_0"],
        "delta": m["delta"],
        **{k: model._spectrum[k] for k in ("emissivity", "albedo", "C1", "C2", "C3", "solar_irradiance")},
        "bb_table": model._b_nu_table,
        "gauss_quad_degree": 100,
    }


def test_three_bands_three_observers_vs_oracle(lib):
    from oracle import zodi_oracle as zo
    from zodipy_gb300 import _lib, engine

    models, zl, uu, npix, obs, earth, obs_dev = _setup()
    _, t32 = engine.forward(zl, uu, obs_dev, 3, _lib.ZL_PREC_F32, want_comps=False)
    _, t64 = engine.forward(zl, uu, obs_dev, 3, _lib.ZL_PREC_F64, want_comps=False)
    t32, t64 = t32.cpu().numpy(), t64.cpu().numpy()
    rng = np.random.default_rng(8)
    u_host = uu.cpu().numpy()
    for o in range(3):
        idx = o * npix + np.sort(rng.choice(npix, 150, replace=False))
        for s, mod in enumerate(models):
            ref = zo.evaluate(_desc(mod), u_host[:, idx], obs[:, o], earth).sum(axis=0)
            np.testing.assert_allclose(t64[s, idx], ref, rtol=1e-10)
            np.testing.assert_allclose(t32[s, idx], ref, rtol=1e-5)


def test_three_bands_l2_adjoint_vs_float64_fd(lib):
    import torch

    from zodipy_gb300 import _lib, engine, params

    models, zl, uu, npix, obs, earth, obs_dev = _setup(nside=16)
    theta0 = params.vector_from_model(zl)
    rng = np.random.default_rng(9)
    zl_true = params.model_from_vector(zl, theta0 * (1 + 0.02 * rng.standard_normal(theta0.size)))
    _, d = engine.forward(zl_true, uu, obs_dev, 3, _lib.ZL_PREC_F64, want_comps=False)
    # upstream gradient from the float64 map, so the comparison isolates the adjoint
    # (with the float32 map, (m - d) itself differs by ~1e-6 m / 0.02 m = 5e-5 per pixel)
    _, m = engine.forward(zl, uu, obs_dev, 3, _lib.ZL_PREC_F64, want_comps=False)
    grad = engine.backward(zl, uu, obs_dev, 3, g_total=2 * (m - d)).cpu().numpy()

    def loss(vec):
        _, mm = engine.forward(params.model_from_vector(zl, vec), uu, obs_dev, 3, _lib.ZL_PREC_F64, want_comps=False)
        return float(((mm - d) ** 2).sum())

    names = params.names(zl, models[0].comp_labels)
    for key in ("comps.cloud.n_0", "comps.cloud.alpha", "comps.band2.delta_zeta", "comps.ring.sigma_r",
                "comps.feature.theta", "T_0", "delta", "emissivity.cloud[1]"):
        j = names.index(key)
        h = 1e-5 * max(abs(theta0[j]), 1.0)
        vp, vm = theta0.copy(), theta0.copy()
        vp[j] += h
        vm[j] -= h
        fd = (loss(vp) - loss(vm)) / (2 * h)
        assert abs(grad[j] - fd) <= 2e-4 * abs(fd) + 1e-9, (key, grad[j], fd)
