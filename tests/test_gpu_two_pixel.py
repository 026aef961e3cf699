"""Two-pixel (packed float32) forward kernel against the one-pixel kernel.

Both evaluate the same operations per pixel; they may differ where the compiler
fuses a multiply and an add in one but not the other, i.e. by a few float32 ulp
per term.  Components are compared at 2e-6 relative to max(|component|, 1e-3
|total|), the total at 2e-6; odd pixel counts exercise the repeated last lane.
"""

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

TOL = 2e-6


def _run(model, u, obs, earth, one_pixel, tod=False):
    import torch

    from zodipy_gb300 import _lib, engine, packing

    lib = _lib.load()
    _lib.check(lib.zl_debug_one_pixel(1 if one_pixel else -1), "one_pixel")
    try:
        u_dev = torch.from_numpy(u).cuda()
        if tod:
            comps, total = engine.forward_tod(model, u_dev, obs, earth, "float32")
        else:
            tab = packing.observer_table(model, obs, earth, [0], any_mode=False)
            comps, total = engine.forward(model, u_dev, engine.upload_observers(tab), 1, "float32")
        return comps.cpu().numpy(), total.cpu().numpy()
    finally:
        _lib.check(lib.zl_debug_one_pixel(0), "one_pixel")


def _check(a, b):
    (ca, ta), (cb, tb) = a, b
    floor = np.maximum(np.abs(cb), 1e-3 * np.abs(tb)[:, None, :])
    assert np.max(np.abs(ca - cb) / floor) <= TOL
    assert np.max(np.abs(ta - tb) / np.abs(tb)) <= TOL


@pytest.mark.parametrize("name,bands", [("dirbe", (25.0,)), ("dirbe", (1.25,)), ("dirbe", (12.0, 25.0, 60.0)),
                                        ("planck18", (857.0,)), ("planck18", (545.0, 857.0))])
@pytest.mark.parametrize("n", [1, 2, 1001])
def test_two_pixel_equals_one_pixel(lib, name, bands, n):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u_
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import random_sphere

    unit = u_.micron if name == "dirbe" else u_.GHz
    models = [zg.Model(b * unit, name=name) for b in bands]
    zl = fuse_models(models)
    dirs = random_sphere(n, seed=n)
    obs, earth = np.array([0.75, 0.66, 0.01]), np.array([0.76, 0.65, 0.0])
    _check(_run(zl, dirs, obs, earth, one_pixel=False), _run(zl, dirs, obs, earth, one_pixel=True))


def test_two_pixel_time_ordered(lib):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u_
    from zodipy_gb300.healpix import random_sphere

    n = 777
    t = np.linspace(0, 2 * np.pi, n)
    obs = np.stack([np.cos(t), np.sin(t), 0.01 * np.sin(2 * t)])
    earth = np.stack([np.cos(t + 0.01), np.sin(t + 0.01), np.zeros(n)])
    zl = zg.Model(25 * u_.micron).zl_model
    dirs = random_sphere(n, seed=3)
    _check(_run(zl, dirs, obs, earth, False, tod=True), _run(zl, dirs, obs, earth, True, tod=True))


@pytest.mark.parametrize("bands", [(25.0,), (1.25,), (12.0, 25.0, 60.0)])
def test_component_paired_equals_one_pixel(lib, bands):
    """The DIRBE layout's default kernel pairs components in packed lanes; same tolerance."""
    import zodipy_gb300 as zg
    from zodipy_gb300 import _lib
    from zodipy_gb300 import units as u_
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import random_sphere

    zl = fuse_models([zg.Model(b * u_.micron) for b in bands])
    dirs = random_sphere(1001, seed=5)
    obs, earth = np.array([0.75, 0.66, 0.01]), np.array([0.76, 0.65, 0.0])
    lib_ = _lib.load()
    _lib.check(lib_.zl_debug_one_pixel(0), "default kernel")
    a = _run(zl, dirs, obs, earth, one_pixel=True)
    _lib.check(lib_.zl_debug_one_pixel(0), "default kernel")
    from zodipy_gb300 import engine, packing
    import torch

    tab = packing.observer_table(zl, obs, earth, [0], any_mode=False)
    comps, total = engine.forward(zl, torch.from_numpy(dirs).cuda(), engine.upload_observers(tab), 1, "float32")
    _check((comps.cpu().numpy(), total.cpu().numpy()), a)


@pytest.mark.parametrize("bands", [(25.0,), (1.25,), (12.0, 25.0, 60.0)])
def test_component_paired_band_tails_healpix_order(lib, bands):
    """In HEALPix RING order the 32 pixels of a warp lie on one latitude ring, so beyond some
    node every pixel of the warp is far enough from the bands' planes that their factor
    e^-(zeta/dzeta)^6 is zero in float32, and the paired kernel stops evaluating them (about
    half of this map's nodes; random directions, as above, almost never form such a warp).
    Same tolerance against the one-pixel kernel, which evaluates every node."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import _lib, engine, packing
    from zodipy_gb300 import units as u_
    from zodipy_gb300.autograd import fuse_models
    from zodipy_gb300.healpix import pix2vec_ring

    from conftest import band_tail_share

    zl = fuse_models([zg.Model(b * u_.micron) for b in bands])
    dirs = pix2vec_ring(64)
    obs, earth = np.array([0.75, 0.66, 0.01]), np.array([0.76, 0.65, 0.0])
    assert band_tail_share(dirs, obs) > 0.3
    ref = _run(zl, dirs, obs, earth, one_pixel=True)
    _lib.check(lib.zl_debug_one_pixel(0), "default kernel")
    tab = packing.observer_table(zl, obs, earth, [0], any_mode=False)
    comps, total = engine.forward(zl, torch.from_numpy(dirs).cuda(), engine.upload_observers(tab), 1, "float32")
    _check((comps.cpu().numpy(), total.cpu().numpy()), ref)
