"""Adjoint of the Rowan-Robinson & May model against central finite differences of the
reference's own code (tests/golden/grad_rrm*.npz, relative step 1e-5): every component
parameter of rrm-experimental, every component's T_0 and delta, and the calibration.

Metric: each derivative as a sensitivity s_j = dL/dp_j |p_j| (dL/dp_j where p_j = 0), the
change of L for a unit relative change of the parameter; the float32 adjoint must match the
reference's float64 differences to |s_adj - s_fd| <= 2e-4 |s_fd| + 2e-6 max |s_fd|.  The
mask edges (R_inner, R_outer where they only cut, beta_nb's cut) have zero derivative in
both: the quadrature's nodes do not move with them."""

import numpy as np
import pytest

from conftest import GOLDEN, cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

REL, FLOOR = 2e-4, 2e-6


def _check(names, theta, g_adj, g_fd, what):
    scale = np.where(np.abs(theta) > 0, np.abs(theta), 1.0)
    s_adj, s_fd = g_adj * scale, g_fd * scale
    tol = REL * np.abs(s_fd) + FLOOR * np.abs(s_fd).max()
    bad = np.abs(s_adj - s_fd) > tol
    if bad.any():
        rows = [f"{names[j]}: adj {g_adj[j]:.6e} fd {g_fd[j]:.6e}" for j in np.flatnonzero(bad)[:16]]
        raise AssertionError(f"{what}: {bad.sum()} parameters off\n" + "\n".join(rows))


@pytest.mark.parametrize("case", ["rrm25", "rrm60_belt"])
def test_rrm_adjoint_matches_reference_finite_differences(lib, case):
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u
    from zodipy_gb300.autograd import ZodiAdjoint

    z = np.load(f"{GOLDEN}/grad_{case}.npz")
    model = zg.Model(float(z["x"][0]) * u.micron, name="rrm-experimental", gauss_quad_degree=50)
    adj = ZodiAdjoint(model.zl_model, z["unit_vectors"], z["obs"], z["earth"], labels=model.comp_labels)
    assert adj.names() == [str(n) for n in z["names"]]
    theta = adj.theta0().requires_grad_(True)
    a = torch.from_numpy(z["weights_a"]).cuda()
    loss = (adj(theta)[0] * a).sum()
    loss.backward()
    assert abs(loss.item() / float(z["loss"]) - 1) < 1e-5
    _check(adj.names(), theta.detach().cpu().numpy(), theta.grad.cpu().numpy(), z["fd_grad"], case)


def test_rrm_adjoint_component_upstream_and_determinism(lib):
    """Per-component upstream gradients equal to a total's give the same gradient; launch shapes
    do not change a bit."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import engine, packing
    from zodipy_gb300 import units as u
    from zodipy_gb300.healpix import pix2vec_ring

    zl = zg.Model(25 * u.micron, name="rrm-experimental").zl_model
    dirs = torch.from_numpy(pix2vec_ring(16)).cuda()
    n = dirs.shape[1]
    obs = engine.upload_observers(packing.observer_table(zl, [0.9833, 0.0, 0.0], [-0.17, 0.97, 0.0], [0],
                                                         any_mode=False))
    g = 0.5 + torch.rand((1, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(3))
    a = engine.backward(zl, dirs, obs, 1, g_total=g).cpu().numpy()
    b = engine.backward(zl, dirs, obs, 1, g_comps=g[:, None, :].expand(1, zl.n_comps, n).contiguous()).cpu().numpy()
    np.testing.assert_array_equal(a, b)
    for bps in (1, 3, 8):
        c = engine.backward(zl, dirs, obs, 1, g_total=g, launch=engine.launch_options(blocks_per_sm=bps)).cpu().numpy()
        np.testing.assert_array_equal(c, a)
    assert np.isfinite(a).all() and np.abs(a).max() > 0
