"""Adjoint kernel: gradients against central finite differences.

Comparison metric.  Parameters live on very different scales (n_0 ~ 1e-7,
T_0 ~ 286, offsets 0), so each derivative is compared as a sensitivity
s_j = dL/dp_j * max(|p_j|, 1): the change of L for a unit relative change of
p_j (unit absolute change where p_j is small).  The float32 adjoint must match
float64 finite differences to

    |s_adj - s_fd| <= 2e-4 |s_fd| + 2e-6 max_j |s_fd|

i.e. a relative 2e-4 per parameter, with a floor at 2e-6 of the largest
sensitivity for parameters whose effect on L is negligible (and whose finite
difference is mostly rounding noise).
"""

import numpy as np
import pytest

from conftest import GOLDEN, cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

REL, FLOOR = 2e-4, 2e-6


def _model(name, x, unit, degree=50):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u

    return zg.Model(float(x) * {"micron": u.micron, "GHz": u.GHz}[unit], name=name, gauss_quad_degree=degree)


def _check(names, theta, g_adj, g_fd, what):
    scale = np.maximum(np.abs(theta), 1.0)
    s_adj, s_fd = g_adj * scale, g_fd * scale
    tol = REL * np.abs(s_fd) + FLOOR * np.abs(s_fd).max()
    bad = np.abs(s_adj - s_fd) > tol
    if bad.any():
        rows = [f"{names[j]}: adj {g_adj[j]:.6e} fd {g_fd[j]:.6e}" for j in np.flatnonzero(bad)[:12]]
        raise AssertionError(f"{what}: {bad.sum()} parameters off\n" + "\n".join(rows))


@pytest.mark.parametrize("case", ["dirbe25", "dirbe1p25", "planck18_857"])
def test_adjoint_matches_reference_finite_differences(lib, case):
    """Gradient of L = sum_i a_i total_i vs central differences through the reference's own code."""
    import torch

    from zodipy_gb300.autograd import ZodiAdjoint

    z = np.load(f"{GOLDEN}/grad_{case}.npz")
    model = _model(str(z["model"]), z["x"][0], str(z["user_unit"]))
    adj = ZodiAdjoint(model.zl_model, z["unit_vectors"], z["obs"], z["earth"], labels=model.comp_labels)
    assert adj.names() == [str(n) for n in z["names"]]
    theta = adj.theta0().requires_grad_(True)
    a = torch.from_numpy(z["weights_a"]).cuda()
    out = adj(theta)
    loss = (out[0] * a).sum()
    loss.backward()
    assert abs(loss.item() / float(z["loss"]) - 1) < 1e-5
    _check(adj.names(), theta.detach().cpu().numpy(), theta.grad.cpu().numpy(), z["fd_grad"], case)


def _chi2_setup(nside=16, seed=3):
    """Two DIRBE bands (12, 25 um) fused in one launch; targets from perturbed float64 maps + 1 % noise."""
    import torch

    from zodipy_gb300 import engine, params
    from zodipy_gb300.autograd import ZodiAdjoint, fuse_models
    from zodipy_gb300.healpix import pix2vec_ring

    m12, m25 = _model("dirbe", 12.0, "micron"), _model("dirbe", 25.0, "micron")
    zl = fuse_models([m12, m25])
    u = pix2vec_ring(nside)
    obs = np.array([0.9833, 0.0, 0.0])
    earth = np.array([-0.17, 0.97, 0.0])
    adj = ZodiAdjoint(zl, u, obs, earth, labels=m12.comp_labels)
    theta0 = params.vector_from_model(zl)
    rng = np.random.default_rng(seed)
    theta_true = theta0 * (1 + 0.02 * rng.standard_normal(theta0.size))
    zl_true = params.model_from_vector(zl, theta_true)
    _, d = engine.forward(zl_true, adj.u, adj.obs_dev, 1, "float64", want_comps=False)
    d = d * (1 + 0.01 * torch.from_numpy(rng.standard_normal(tuple(d.shape))).cuda())
    sigma2 = (0.01 * d) ** 2
    return adj, zl, theta0, d, sigma2


def test_adjoint_chi2_two_bands_vs_float64_finite_differences(lib):
    """Config-4 style: chi^2 over 12 and 25 um maps, gradient w.r.t. every parameter
    against central differences of the plain float64 kernel (relative step 1e-5)."""
    import torch

    from zodipy_gb300 import engine, params

    adj, zl, theta0, d, sigma2 = _chi2_setup()
    theta = torch.tensor(theta0, dtype=torch.float64, device="cuda", requires_grad=True)
    m = adj(theta)
    loss = (((m - d) ** 2) / sigma2).sum()
    loss.backward()
    g_adj = theta.grad.cpu().numpy()

    def chi2(vec):
        zlp = params.model_from_vector(zl, vec)
        _, mm = engine.forward(zlp, adj.u, adj.obs_dev, 1, "float64", want_comps=False)
        return float((((mm - d) ** 2) / sigma2).sum())

    g_fd = np.zeros_like(theta0)
    for j in range(theta0.size):
        h = 1e-5 * max(abs(theta0[j]), 1.0)
        vp, vm = theta0.copy(), theta0.copy()
        vp[j] += h
        vm[j] -= h
        g_fd[j] = (chi2(vp) - chi2(vm)) / (2 * h)
    _check(adj.names(), theta0, g_adj, g_fd, "chi2 12+25um")


def test_adjoint_deterministic_across_launch_shapes(lib):
    import torch

    from zodipy_gb300 import _lib, engine

    adj, zl, theta0, d, sigma2 = _chi2_setup(nside=8)
    g = torch.randn((2, adj.u.shape[1]), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    outs = []
    for bps in (0, 1, 3, 8):
        opt = engine.launch_options(blocks_per_sm=bps)
        outs.append(engine.backward(zl, adj.u, adj.obs_dev, 1, g_total=g, launch=opt).cpu().numpy())
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])


def test_adjoint_fused_equals_sum_of_single_bands(lib):
    """A two-band launch gives the sum of the single-band gradients for shared parameters
    (to float32 accumulation accuracy: the fused pass forms sum_s g_s e_s per node) and
    each band's own block for the spectral ones.  The single-band launch forms the emissivity
    and albedo sums from the density sum (sum w n B = n_0 sum w (n / n_0) B), the fused one
    per set, so those agree to float32 rounding of each pixel's terms: the bound is 1e-6 of
    the sum of the terms' magnitudes, the gradient for |g| (every term of one sign)."""
    import torch

    from zodipy_gb300 import engine, packing

    adj, zl, theta0, d, sigma2 = _chi2_setup(nside=8)
    n = adj.u.shape[1]
    g = torch.randn((2, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(2))
    fused = engine.backward(zl, adj.u, adj.obs_dev, 1, g_total=g).cpu().numpy()
    singles, mags = [], []
    for s in range(2):
        m1 = type(zl).from_buffer_copy(zl)
        m1.n_spec = 1
        m1.spec[0] = zl.spec[s]
        tab = packing.observer_table(m1, [0.9833, 0, 0], [-0.17, 0.97, 0.0], [0], any_mode=False)
        obs1 = engine.upload_observers(tab)
        gs = g[s : s + 1].contiguous()
        singles.append(engine.backward(m1, adj.u, obs1, 1, g_total=gs).cpu().numpy())
        mags.append(np.abs(engine.backward(m1, adj.u, obs1, 1, g_total=gs.abs()).cpu().numpy()))
    n_shared = fused.size - 2 * (2 * zl.n_comps + 4)
    summed = singles[0][:n_shared] + singles[1][:n_shared]
    scale = np.abs(singles[0][:n_shared]) + np.abs(singles[1][:n_shared])
    assert np.all(np.abs(fused[:n_shared] - summed) <= 1e-5 * scale + 1e-7 * scale.max())
    per = 2 * zl.n_comps + 4
    for s, block in enumerate((fused[n_shared : n_shared + per], fused[n_shared + per :])):
        ref, mag = singles[s][n_shared:], mags[s][n_shared:]
        assert np.all(np.abs(block - ref) <= 1e-6 * mag + 1e-12), (s, np.max(np.abs(block - ref) / (mag + 1e-30)))


def test_adjoint_component_and_total_upstream_agree(lib):
    import torch

    from zodipy_gb300 import engine

    adj, zl, theta0, d, sigma2 = _chi2_setup(nside=8)
    n = adj.u.shape[1]
    g = torch.randn((2, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(3))
    a = engine.backward(zl, adj.u, adj.obs_dev, 1, g_total=g).cpu().numpy()
    gc = g[:, None, :].expand(2, zl.n_comps, n).contiguous()
    b = engine.backward(zl, adj.u, adj.obs_dev, 1, g_comps=gc).cpu().numpy()
    np.testing.assert_array_equal(a, b)


def test_backward_rejects_small_workspace(lib):
    import ctypes

    import torch

    from zodipy_gb300 import _lib, engine

    adj, zl, theta0, d, sigma2 = _chi2_setup(nside=4)
    n = adj.u.shape[1]
    g = torch.zeros((2, n), dtype=torch.float64, device="cuda")
    out = torch.empty(engine.grad_count(zl), dtype=torch.float64, device="cuda")
    ws = torch.empty(16, dtype=torch.uint8, device="cuda")
    rc = lib.zl_backward(
        ctypes.byref(zl), ctypes.c_void_p(adj.u.data_ptr()), n, ctypes.c_void_p(adj.obs_dev.data_ptr()), 1,
        None, ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()), 16, None,
    )
    assert rc == _lib.ZL_ERR_SPACE and "workspace" in _lib.last_error()


@pytest.mark.parametrize(
    "bands,per_comp",
    [((25.0,), False), ((1.25,), False), ((12.0, 25.0), False), ((1.25, 2.2, 3.5, 4.9), False), ((25.0,), True)],
)
def test_paired_adjoint_equals_scalar_kernel(lib, bands, per_comp):
    """The DIRBE layout's component-paired adjoint kernels (ring/feature and bands 1/2
    in packed lanes) against the scalar kernel on the same inputs: the same gradient to
    float32 rounding of the node sums (sensitivity metric of this file, REL 1e-5)."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import _lib, engine, packing, params
    from zodipy_gb300 import units as u_
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import random_sphere

    models = [zg.Model(b * u_.micron) for b in bands]
    zl = fuse_models(models)
    dirs = torch.from_numpy(random_sphere(5003, seed=11)).cuda()
    tab = packing.observer_table(zl, [0.75, 0.66, 0.01], [0.76, 0.65, 0.0], [0], any_mode=False)
    obs = engine.upload_observers(tab)
    gen = torch.Generator("cuda").manual_seed(4)
    n = dirs.shape[1]
    shape = (len(bands), zl.n_comps, n) if per_comp else (len(bands), n)
    g = 0.5 + torch.rand(shape, dtype=torch.float64, device="cuda", generator=gen)
    kw = {"g_comps": g} if per_comp else {"g_total": g}
    ref = engine.backward(zl, dirs, obs, 1, launch=engine.launch_options(kernel=_lib.ZL_KERNEL_ONE_PIXEL), **kw)
    ref = ref.cpu().numpy()
    got = engine.backward(zl, dirs, obs, 1, **kw).cpu().numpy()
    names = params.names(zl, models[0].comp_labels)
    theta = params.vector_from_model(zl)
    scale = np.maximum(np.abs(theta), 1.0)
    s_got, s_ref = got * scale, ref * scale
    dev = np.abs(s_got - s_ref) / (np.abs(s_ref) + 1e-7 * np.abs(s_ref).max())
    worst = int(np.argmax(dev))
    assert dev.max() <= 1e-5, f"{names[worst]}: paired {got[worst]:.9e} scalar {ref[worst]:.9e} ({dev.max():.2e})"


@pytest.mark.parametrize("bands,per_comp", [((25.0,), False), ((12.0, 25.0, 60.0), False), ((25.0,), True)])
def test_paired_adjoint_band_tails_healpix_order(lib, bands, per_comp):
    """The {cloud, bands} adjoint kernel stops evaluating the bands past the node from which
    they are zero for every pixel of a warp (about half of this HEALPix map's nodes; random
    directions almost never give such warps).  Against the scalar kernel, which evaluates
    every node; same metric and tolerance as above."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import _lib, engine, packing, params
    from zodipy_gb300 import units as u_
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import pix2vec_ring

    from conftest import band_tail_share

    models = [zg.Model(b * u_.micron) for b in bands]
    zl = fuse_models(models)
    obs_xyz = np.array([0.75, 0.66, 0.01])
    u_np = pix2vec_ring(32)
    assert band_tail_share(u_np, obs_xyz) > 0.3
    dirs = torch.from_numpy(u_np).cuda()
    tab = packing.observer_table(zl, obs_xyz, [0.76, 0.65, 0.0], [0], any_mode=False)
    obs = engine.upload_observers(tab)
    gen = torch.Generator("cuda").manual_seed(7)
    n = dirs.shape[1]
    shape = (len(bands), zl.n_comps, n) if per_comp else (len(bands), n)
    g = 0.5 + torch.rand(shape, dtype=torch.float64, device="cuda", generator=gen)
    kw = {"g_comps": g} if per_comp else {"g_total": g}
    ref = engine.backward(zl, dirs, obs, 1, launch=engine.launch_options(kernel=_lib.ZL_KERNEL_ONE_PIXEL), **kw)
    ref = ref.cpu().numpy()
    got = engine.backward(zl, dirs, obs, 1, **kw).cpu().numpy()
    names = params.names(zl, models[0].comp_labels)
    scale = np.maximum(np.abs(params.vector_from_model(zl)), 1.0)
    s_got, s_ref = got * scale, ref * scale
    dev = np.abs(s_got - s_ref) / (np.abs(s_ref) + 1e-7 * np.abs(s_ref).max())
    worst = int(np.argmax(dev))
    assert dev.max() <= 1e-5, f"{names[worst]}: paired {got[worst]:.9e} scalar {ref[worst]:.9e} ({dev.max():.2e})"


def test_adjoint_linear_in_tiny_upstream_gradient(lib):
    """The adjoint is linear in the upstream gradient, whatever its scale: a gradient 1e-22
    times smaller (below the range where the kernels convert doubles by bit operations) gives
    a parameter gradient 1e-22 times smaller, not zero."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import engine, packing
    from zodipy_gb300 import units as u_
    from zodipy_gb300.healpix import pix2vec_ring

    zl = zg.Model(25 * u_.micron).zl_model
    dirs = torch.from_numpy(pix2vec_ring(16)).cuda()
    obs = engine.upload_observers(packing.observer_table(zl, [0.9833, 0.0, 0.0], [-0.17, 0.97, 0.0], [0], any_mode=False))
    g = 0.5 + torch.rand((1, dirs.shape[1]), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(2))
    ref = engine.backward(zl, dirs, obs, 1, g_total=g).cpu().numpy()
    tiny = engine.backward(zl, dirs, obs, 1, g_total=g * 1e-22).cpu().numpy()
    big = np.abs(ref) > 1e-12 * np.abs(ref).max()
    assert big.sum() > 10
    np.testing.assert_allclose(tiny[big] * 1e22, ref[big], rtol=1e-5)
