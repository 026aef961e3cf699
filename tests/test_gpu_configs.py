"""Parity at the full sizes of the five benchmark configurations.

The golden fixtures (``los_cfg*.npz``) pin the oracle to the reference on seeded
subsets of each configuration's own inputs.  Here the kernels run the whole
workloads and are checked against the oracle (float64, 1e-10, the bar of
tests/test_gpu_parity.py) and against the float64 kernel (float32, 1e-5), with
the maximum and median errors printed (run pytest with -s to see them):

  1  DIRBE 25 um, HEALPix nside 128 (196,608 LOS), observer (0.9833, 0, 0) AU, GL 50,
     float64 kernel vs the oracle on every pixel
  2  DIRBE over 64 wavelengths 80-130 um (Gaussian weights), nside 512 (3,145,728 LOS),
     observer (0.7071, 0.7071, 0) AU: float32 vs float64 kernel on every pixel, and the
     float64 kernel vs the oracle on 100,000 seeded pixels
  -  the headline: DIRBE 25 um, nside 512, observer (0.7071, 0.7071, 0) AU: float32 vs
     float64 on every pixel, float64 vs the oracle on 100,000 seeded pixels
  3  planck18 857 GHz, 256 observers with 10,000-500,000 random directions each (68.9 M
     LOS) in one batched launch: float32 vs float64 kernel on every LOS, float64 vs the
     oracle on 8 observers x 64 directions
  4  chi^2 of DIRBE 12 + 25 um maps at nside 256 (786,432 LOS per band) against targets
     from perturbed parameters plus 1 % noise: every gradient vs central finite
     differences of the float64 kernel
  5  DIRBE 12/25/60 um fused, 3 observers, GL 100 at nside 256 (2,359,296 LOS): float32 vs
     float64 kernel on every value, the L2-loss adjoint vs finite differences

Anchors: the per-component quadrature of zodipy/model.py:253-277, and the bit-exact
sum and partition bars of the reference's tests/test_evaluate.py:198-262 (the
total equals the component sum).
"""

import os

import numpy as np
import pytest

from conftest import cuda_ok
from oracle import workloads
from oracle import zodi_oracle as zo

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

F64_RTOL, F32_RTOL = 1e-10, 1e-5
OBS1 = np.array([0.9833, 0.0, 0.0])
OBS2 = np.array([0.7071, 0.7071, 0.0])
EARTH = workloads.EARTH_2022_01_01
NPROC = min(os.cpu_count() or 1, 16)


def oracle(desc, u, obs, earth=EARTH):
    """The oracle over a spawn pool (this process has initialised CUDA: no fork), with the
    documented finite root where the reference's intersection gives nan (b == 0 exactly, which
    HEALPix centres on the observer's perpendicular meridian hit)."""
    return zo.evaluate_chunked(desc, u, obs, earth, nprocesses=NPROC, start_method="spawn", fix_b0=True)


def same_inputs(model, desc):
    """The oracle description with the model's own spectral inputs, after checking them against
    the reference-held ones: the blackbody table is computed on the running machine (its libm
    can differ from the one that wrote the fixture by an ulp), so both sides get the same bits."""
    np.testing.assert_allclose(model._b_nu_table, desc["bb_table"], rtol=1e-14, atol=0)
    for k in ("emissivity", "albedo", "C1", "C2", "C3", "solar_irradiance"):
        np.testing.assert_allclose(model._spectrum[k], desc[k], rtol=1e-14, atol=0)
    out = dict(desc)
    out["bb_table"] = np.asarray(model._b_nu_table)
    for k in ("emissivity", "albedo", "C1", "C2", "C3", "solar_irradiance"):
        out[k] = model._spectrum[k]
    return out


def assert_f64_close(got, ref, what):
    """|got - ref| <= 1e-10 |ref| + 1e-15 |pixel total| (tests/test_gpu_parity.py)."""
    assert np.isfinite(got).all() and np.isfinite(ref).all()
    floor = np.maximum(1e-200, 1e-15 * np.abs(ref.sum(axis=0)))[None, :]
    bad = np.abs(got - ref) - F64_RTOL * np.abs(ref) > floor
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    print(f"{what}: float64 vs oracle max rel {rel.max():.3e}, median {np.median(rel):.3e} over {ref.size} values")
    assert not bad.any(), f"{what}: {bad.sum()} of {bad.size} values off, worst {rel.max():.3e}"


def f32_errors(c32, c64):
    """(total max, total median, component max): component errors relative to
    max(|component|, 1e-3 |total|), as tests/test_gpu_parity.py."""
    import torch

    t32, t64 = c32.sum(-2), c64.sum(-2)
    e_tot = ((t32 - t64).abs() / t64.abs()).flatten()
    floor = torch.maximum(c64.abs(), 1e-3 * t64.abs().unsqueeze(-2))
    e_comp = ((c32 - c64).abs() / floor).amax()
    return float(e_tot.max()), float(e_tot.median()), float(e_comp)


def _model(x, unit="micron", name="dirbe", degree=50, weights=None, precision="float64"):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    q = np.asarray(x) * {"micron": u.micron, "GHz": u.GHz}[unit]
    return zg.Model(q, weights=weights, name=name, gauss_quad_degree=degree, precision=precision)


def test_config1_nside128_float64_vs_oracle_every_pixel(lib):
    import torch

    from zodipy_gb300.healpix import pix2vec_ring_torch

    model = _model(25.0)
    desc = same_inputs(model, workloads.oracle_desc("dirbe", "dirbe_25um", 50))
    u = pix2vec_ring_torch(128, "cuda")
    assert u.shape[1] == 196_608
    got = model.evaluate_xyz(u, OBS1, EARTH, return_comps=True, precision="float64")
    tot = model.evaluate_xyz(u, OBS1, EARTH, return_comps=False, precision="float64")
    torch.cuda.synchronize()
    got, tot = got.cpu().numpy(), tot.cpu().numpy()
    np.testing.assert_array_equal(got.sum(axis=0), tot)  # total = ordered component sum, bit for bit
    ref = oracle(desc, u.cpu().numpy(), OBS1)
    assert_f64_close(got, ref, "config 1 (196,608 LOS)")


def test_config2_bandpass_nside512_float32_vs_float64_and_oracle(lib):
    import torch

    from zodipy_gb300 import engine, packing
    from zodipy_gb300.healpix import pix2vec_ring_torch

    lam = np.linspace(80, 130, 64)
    w = np.exp(-0.5 * ((lam - 100) / 10) ** 2)
    model = _model(lam, weights=w)
    desc = same_inputs(model, workloads.oracle_desc("dirbe", "dirbe_bp_80_130", 50))
    u = pix2vec_ring_torch(512, "cuda")
    n = u.shape[1]
    assert n == 3_145_728
    zl = model.zl_model
    obs = engine.upload_observers(packing.observer_table(zl, OBS2, EARTH, [0], any_mode=False))
    c64, _ = engine.forward(zl, u, obs, 1, "float64", want_total=False)
    c32, _ = engine.forward(zl, u, obs, 1, "float32", want_total=False)
    e_max, e_med, e_comp = f32_errors(c32[0], c64[0])
    print(f"config 2: float32 vs float64 total max {e_max:.3e} median {e_med:.3e}, component max {e_comp:.3e}")
    assert e_max <= F32_RTOL and e_comp <= F32_RTOL
    idx = np.sort(np.random.default_rng(2).choice(n, 100_000, replace=False))
    idx_t = torch.from_numpy(idx).cuda()
    sub = c64[0][:, idx_t].cpu().numpy()
    del c32, c64
    ref = oracle(desc, u[:, idx_t].cpu().numpy(), OBS2)
    assert_f64_close(sub, ref, "config 2 (100,000 of 3,145,728 LOS)")


def test_headline_dirbe25_nside512_float32_vs_float64_and_oracle(lib):
    """The workload the throughput is quoted on: DIRBE 25 um, nside 512, observer (0.7071,
    0.7071, 0) AU, GL 50.  The default float32 kernel (component pairs, band tails, the block's
    shared observer set-up) against the float64 kernel on every pixel, and the float64 kernel
    against the oracle on 100,000 seeded pixels."""
    import torch

    from zodipy_gb300 import engine, packing
    from zodipy_gb300.healpix import pix2vec_ring_torch

    model = _model(25.0)
    desc = same_inputs(model, workloads.oracle_desc("dirbe", "dirbe_25um", 50))
    u = pix2vec_ring_torch(512, "cuda")
    n = u.shape[1]
    zl = model.zl_model
    obs = engine.upload_observers(packing.observer_table(zl, OBS2, EARTH, [0], any_mode=False))
    c64, _ = engine.forward(zl, u, obs, 1, "float64", want_total=False)
    c32, _ = engine.forward(zl, u, obs, 1, "float32", want_total=False)
    e_max, e_med, e_comp = f32_errors(c32[0], c64[0])
    print(f"headline: float32 vs float64 total max {e_max:.3e} median {e_med:.3e}, component max {e_comp:.3e}")
    assert e_max <= F32_RTOL and e_comp <= F32_RTOL
    idx = np.sort(np.random.default_rng(5).choice(n, 100_000, replace=False))
    idx_t = torch.from_numpy(idx).cuda()
    sub = c64[0][:, idx_t].cpu().numpy()
    del c32, c64
    ref = oracle(desc, u[:, idx_t].cpu().numpy(), OBS2)
    assert_f64_close(sub, ref, "headline (100,000 of 3,145,728 LOS)")


def test_config3_batch_float32_vs_float64_every_los(lib):
    import torch

    from zodipy_gb300.batch import BatchEvaluator, random_directions_device, uneven_observers

    model = _model(857.0, unit="GHz", name="planck18")
    obs, counts = uneven_observers(256, seed=2024)
    n = int(counts.sum())
    assert 6.5e7 < n < 7.2e7
    u = random_directions_device(n, seed=2025)
    ev32 = BatchEvaluator(model.zl_model, u, obs, counts, EARTH, precision="float32")
    ev32.capture()
    ev32.replay()
    ev64 = BatchEvaluator(model.zl_model, u, obs, counts, EARTH, precision="float64")
    t64 = ev64.run()
    torch.cuda.synchronize()
    rel = ((ev32.total - t64).abs() / t64.abs()).flatten()
    e_max, e_med = float(rel.max()), float(rel.median())
    print(f"config 3 ({n} LOS): float32 vs float64 max {e_max:.3e} median {e_med:.3e}")
    assert e_max <= F32_RTOL
    del rel, ev32
    desc = same_inputs(model, workloads.oracle_desc("planck18", "planck18_857ghz", 50))
    begin = np.concatenate([[0], np.cumsum(counts)])
    rng = np.random.default_rng(3)
    for o in rng.choice(256, 8, replace=False):
        idx = begin[o] + np.sort(rng.choice(counts[o], 64, replace=False))
        idx_t = torch.from_numpy(idx).cuda()
        ref = zo.evaluate(desc, u[:, idx_t].cpu().numpy(), obs[:, o], EARTH).sum(axis=0)
        got = t64[0, idx_t].cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=F64_RTOL, atol=0, err_msg=f"observer {o}")


REL, FLOOR = 2e-4, 2e-6  # sensitivity metric of tests/test_gpu_adjoint.py


def _check_sensitivities(names, theta, g_adj, g_fd, what):
    scale = np.maximum(np.abs(theta), 1.0)
    s_adj, s_fd = g_adj * scale, g_fd * scale
    tol = REL * np.abs(s_fd) + FLOOR * np.abs(s_fd).max()
    dev = np.abs(s_adj - s_fd) / (np.abs(s_fd) + FLOOR / REL * np.abs(s_fd).max())
    print(f"{what}: {len(names)} gradients, max deviation {dev.max():.3e} of the tolerance's relative part")
    bad = np.abs(s_adj - s_fd) > tol
    if bad.any():
        rows = [f"{names[j]}: adj {g_adj[j]:.6e} fd {g_fd[j]:.6e}" for j in np.flatnonzero(bad)[:12]]
        raise AssertionError(f"{what}: {bad.sum()} parameters off\n" + "\n".join(rows))


def test_config4_chi2_nside256_every_gradient_vs_float64_fd(lib):
    import torch

    from zodipy_gb300 import engine, params
    from zodipy_gb300.autograd import ZodiAdjoint, fuse_models
    from zodipy_gb300.healpix import pix2vec_ring

    m12, m25 = _model(12.0), _model(25.0)
    zl = fuse_models([m12, m25])
    u = pix2vec_ring(256)
    assert u.shape[1] == 786_432
    adj = ZodiAdjoint(zl, u, OBS1, EARTH, labels=m12.comp_labels)
    theta0 = params.vector_from_model(zl)
    rng = np.random.default_rng(44)
    zl_true = params.model_from_vector(zl, theta0 * (1 + 0.02 * rng.standard_normal(theta0.size)))
    _, d = engine.forward(zl_true, adj.u, adj.obs_dev, 1, "float64", want_comps=False)
    d = d * (1 + 0.01 * torch.from_numpy(rng.standard_normal(tuple(d.shape))).cuda())
    sigma2 = (0.01 * d) ** 2
    theta = torch.tensor(theta0, dtype=torch.float64, device="cuda", requires_grad=True)
    loss = (((adj(theta) - d) ** 2) / sigma2).sum()
    loss.backward()
    g_adj = theta.grad.cpu().numpy()

    def chi2(vec):
        _, mm = engine.forward(params.model_from_vector(zl, vec), adj.u, adj.obs_dev, 1, "float64", want_comps=False)
        return float((((mm - d) ** 2) / sigma2).sum())

    g_fd = np.zeros_like(theta0)
    for j in range(theta0.size):
        h = 1e-5 * max(abs(theta0[j]), 1.0)
        vp, vm = theta0.copy(), theta0.copy()
        vp[j] += h
        vm[j] -= h
        g_fd[j] = (chi2(vp) - chi2(vm)) / (2 * h)
    _check_sensitivities(adj.names(), theta0, g_adj, g_fd, "config 4 (2 x 786,432 LOS)")


def test_config5_three_bands_three_observers_gl100_nside256(lib):
    import torch

    from zodipy_gb300 import _lib, engine, packing, params
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import pix2vec_ring_torch

    models = [_model(w, degree=100) for w in (12.0, 25.0, 60.0)]
    zl = fuse_models(models)
    umap = pix2vec_ring_torch(256, "cuda")
    npix = umap.shape[1]
    u = umap.repeat(1, 3).contiguous()
    ang = np.radians([0.0, 120.0, 240.0])
    obs = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)])
    obs_dev = engine.upload_observers(packing.observer_table(zl, obs, EARTH, [0, npix, 2 * npix], any_mode=False))
    c64, _ = engine.forward(zl, u, obs_dev, 3, _lib.ZL_PREC_F64, want_total=False)
    c32, _ = engine.forward(zl, u, obs_dev, 3, _lib.ZL_PREC_F32, want_total=False)
    e_max, e_med, e_comp = f32_errors(c32, c64)
    print(f"config 5 ({3 * npix} LOS x 3 bands): float32 vs float64 total max {e_max:.3e} median {e_med:.3e}, "
          f"component max {e_comp:.3e}")
    assert e_max <= F32_RTOL and e_comp <= F32_RTOL
    del c32
    # adjoint of sum (m - d)^2, d the float64 map at perturbed parameters
    theta0 = params.vector_from_model(zl)
    rng = np.random.default_rng(55)
    zl_true = params.model_from_vector(zl, theta0 * (1 + 0.02 * rng.standard_normal(theta0.size)))
    _, d = engine.forward(zl_true, u, obs_dev, 3, _lib.ZL_PREC_F64, want_comps=False)
    m = c64.sum(1)
    grad = engine.backward(zl, u, obs_dev, 3, g_total=2 * (m - d)).cpu().numpy()
    del c64, m

    def loss(vec):
        _, mm = engine.forward(params.model_from_vector(zl, vec), u, obs_dev, 3, _lib.ZL_PREC_F64, want_comps=False)
        return float(((mm - d) ** 2).sum())

    names = params.names(zl, models[0].comp_labels)
    keys = ("comps.cloud.n_0", "comps.cloud.alpha", "comps.band2.delta_zeta", "comps.ring.sigma_r",
            "comps.feature.theta", "T_0", "delta", "emissivity.cloud[2]")
    fd = np.zeros(len(keys))
    idx = [names.index(k) for k in keys]
    for a, j in enumerate(idx):
        h = 1e-5 * max(abs(theta0[j]), 1.0)
        vp, vm = theta0.copy(), theta0.copy()
        vp[j] += h
        vm[j] -= h
        fd[a] = (loss(vp) - loss(vm)) / (2 * h)
    _check_sensitivities(list(keys), theta0[idx], grad[idx], fd, "config 5 (2,359,296 LOS x 3 bands)")
    torch.cuda.synchronize()
