"""The float64 warp-per-pixel forward kernel (ZL_KERNEL_WARP_PER_PIXEL): one warp per
line of sight, the quadrature nodes across its lanes, shuffle sums.

It evaluates every node with the same device functions as the one-thread-per-pixel
float64 kernel and differs only in how the node sum is associated (per-lane partial sums,
then a butterfly), so the two agree to 1e-13 relative per component (floor 1e-15 of the
pixel total, as the parity tests use for ill-conditioned terms), and it meets the same
1e-10 bar against the reference's golden outputs.
"""

import numpy as np
import pytest

from conftest import cuda_ok, golden_cases, load_case, product_model
from test_gpu_parity import _ref_fixed, assert_f64_close

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

RTOL = 1e-13


def _f64(model_zl, dirs, obs, earth, kernel, out_index=None, **launch):
    import torch

    from zodipy_gb300 import engine, packing

    tab = packing.observer_table(model_zl, obs, earth, [0], any_mode=False)
    u = torch.from_numpy(np.ascontiguousarray(dirs)).cuda()
    opt = engine.launch_options(kernel=kernel, out_index=out_index, **launch)
    comps, _ = engine.forward(model_zl, u, engine.upload_observers(tab), 1, "float64", launch=opt)
    return comps[0].cpu().numpy() if model_zl.n_spec == 1 else comps.cpu().numpy()


def _close(a, b):
    floor = 1e-15 * np.abs(b.sum(axis=-2, keepdims=True))
    assert np.all(np.abs(a - b) <= RTOL * np.abs(b) + floor), np.max(np.abs(a - b) / np.abs(b))


SINGLE_OBSERVER = [n for n in golden_cases() if load_case(n)["obs"].ndim == 1]


@pytest.mark.parametrize("name", SINGLE_OBSERVER)
def test_warp_kernel_matches_reference_and_thread_kernel(lib, name):
    from zodipy_gb300 import _lib

    case = load_case(name)
    zl = product_model(case).zl_model
    args = (zl, case["unit_vectors"], case["obs"], case["earth"])
    warp = _f64(*args, _lib.ZL_KERNEL_WARP_PER_PIXEL)
    thread = _f64(*args, _lib.ZL_KERNEL_AUTO)
    assert np.isfinite(warp).all()
    _close(warp, thread)
    assert_f64_close(warp, _ref_fixed(case), name)


@pytest.mark.parametrize("n", [1, 31, 33, 1000])
@pytest.mark.parametrize("name,bands,degree", [("dirbe", (1.25,), 50), ("planck18", (545.0, 857.0), 100),
                                               ("rrm-experimental", (25.0,), 20)])
def test_warp_kernel_ragged_groups_and_permutation(lib, n, name, bands, degree):
    """Pixel counts that leave a warp's group of 32 part-empty, degrees that leave lanes idle on
    the last pass (50, 100) or never reach the second (20), several spectral sets, and an output
    permutation: agreement with the one-thread-per-pixel kernel, column for column."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import _lib
    from zodipy_gb300 import units as u_
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import random_sphere

    unit = u_.GHz if name == "planck18" else u_.micron
    zl = fuse_models([zg.Model(b * unit, name=name, gauss_quad_degree=degree) for b in bands])
    dirs = random_sphere(n, seed=n + degree)
    obs, earth = np.array([0.75, 0.66, 0.01]), np.array([0.76, 0.65, 0.0])
    thread = _f64(zl, dirs, obs, earth, _lib.ZL_KERNEL_AUTO)
    for tpb, bps in ((128, 0), (32, 1), (64, 3)):
        _close(_f64(zl, dirs, obs, earth, _lib.ZL_KERNEL_WARP_PER_PIXEL, threads_per_block=tpb, blocks_per_sm=bps),
               thread)
    order = np.random.default_rng(n).permutation(n)
    got = _f64(zl, dirs[:, order], obs, earth, _lib.ZL_KERNEL_WARP_PER_PIXEL, out_index=torch.from_numpy(order).cuda())
    _close(got, thread)


def test_warp_kernel_options_are_checked(lib):
    import torch

    from zodipy_gb300 import _lib, engine, packing

    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u_

    zl = zg.Model(25 * u_.micron).zl_model
    dirs = torch.nn.functional.normalize(torch.ones(3, 64, dtype=torch.float64), dim=0).cuda()
    obs = engine.upload_observers(packing.observer_table(zl, np.array([1.0, 0, 0]), np.array([1.0, 0, 0]), [0],
                                                         any_mode=False))
    queue = torch.zeros(2, dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.ZodiGBError):  # no work queue
        engine.forward(zl, dirs, obs, 1, "float64",
                       launch=engine.launch_options(kernel=_lib.ZL_KERNEL_WARP_PER_PIXEL, tile=128, queue=queue))
    with pytest.raises(_lib.ZodiGBError):  # float64 only
        engine.forward(zl, dirs, obs, 1, "float32", launch=engine.launch_options(kernel=_lib.ZL_KERNEL_WARP_PER_PIXEL))
    with pytest.raises(_lib.ZodiGBError):  # no two-pixel float64 kernel
        engine.forward(zl, dirs, obs, 1, "float64", launch=engine.launch_options(kernel=_lib.ZL_KERNEL_TWO_PIXEL))
