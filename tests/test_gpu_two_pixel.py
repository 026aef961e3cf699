"""Two-pixel (packed float32) forward kernel against the one-pixel kernel, and the
launch options of zl_forward_ex (work queue, output permutation, band tails).

The two kernels evaluate the same operations per pixel; they may differ where the
compiler fuses a multiply and an add in one but not the other, i.e. by a few float32
ulp per term.  Components are compared at 2e-6 relative to max(|component|, 1e-3
|total|), the total at 2e-6; odd pixel counts exercise the repeated last lane.  Launch
options that only change which thread or block computes a pixel (work queue, tile,
output permutation, band tails) must give the same bits.
"""

import numpy as np
import pytest

from conftest import band_tail_share, cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

TOL = 2e-6


def _run(model, u, obs, earth, kernel, tod=False, **launch):
    """float32 forward through zl_forward_ex with the given kernel; a time-ordered call (a
    position per pixel) is given one observer record per pixel with the flags OR-ed over the
    call, which is what zl_forward_tod evaluates."""
    import torch

    from zodipy_gb300 import engine, packing

    u_dev = torch.from_numpy(u).cuda()
    n = u.shape[1]
    if tod:
        tab = packing.observer_table(model, obs, earth, np.arange(n), any_mode=True)
        n_obs = n
    else:
        tab = packing.observer_table(model, obs, earth, [0], any_mode=False)
        n_obs = 1
    opt = engine.launch_options(kernel=kernel, **launch)
    comps, total = engine.forward(model, u_dev, engine.upload_observers(tab), n_obs, "float32", launch=opt)
    return comps.cpu().numpy(), total.cpu().numpy()


def _check(a, b):
    (ca, ta), (cb, tb) = a, b
    floor = np.maximum(np.abs(cb), 1e-3 * np.abs(tb)[:, None, :])
    assert np.max(np.abs(ca - cb) / floor) <= TOL
    assert np.max(np.abs(ta - tb) / np.abs(tb)) <= TOL


def _models(name, bands):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u_
    from zodipy_gb300.autograd import fuse_models

    unit = u_.micron if name == "dirbe" else u_.GHz
    return fuse_models([zg.Model(b * unit, name=name) for b in bands])


OBS, EARTH = np.array([0.75, 0.66, 0.01]), np.array([0.76, 0.65, 0.0])


@pytest.mark.parametrize("name,bands", [("dirbe", (25.0,)), ("dirbe", (1.25,)), ("dirbe", (12.0, 25.0, 60.0)),
                                        ("planck18", (857.0,)), ("planck18", (545.0, 857.0))])
@pytest.mark.parametrize("n", [1, 2, 255, 257, 1001])
def test_two_pixel_equals_one_pixel(lib, name, bands, n):
    from zodipy_gb300 import _lib
    from zodipy_gb300.healpix import random_sphere

    zl = _models(name, bands)
    dirs = random_sphere(n, seed=n)
    _check(_run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_TWO_PIXEL), _run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_ONE_PIXEL))


def test_two_pixel_time_ordered(lib):
    """A position per pixel: the default kernel of zl_forward_tod (two-pixel for the Planck
    layout) against the one-pixel kernel on the same per-pixel observers."""
    import torch

    from zodipy_gb300 import _lib, engine
    from zodipy_gb300.healpix import random_sphere

    n = 777
    t = np.linspace(0, 2 * np.pi, n)
    obs = np.stack([np.cos(t), np.sin(t), 0.01 * np.sin(2 * t)])
    earth = np.stack([np.cos(t + 0.01), np.sin(t + 0.01), np.zeros(n)])
    for zl in (_models("planck18", (857.0,)), _models("dirbe", (25.0,))):
        dirs = random_sphere(n, seed=3)
        c, tot = engine.forward_tod(zl, torch.from_numpy(dirs).cuda(), obs, earth, "float32")
        _check((c.cpu().numpy(), tot.cpu().numpy()), _run(zl, dirs, obs, earth, _lib.ZL_KERNEL_ONE_PIXEL, tod=True))


@pytest.mark.parametrize("bands", [(25.0,), (1.25,), (12.0, 25.0, 60.0)])
def test_component_paired_equals_one_pixel(lib, bands):
    """The DIRBE layout's default kernel pairs components in packed lanes; same tolerance."""
    from zodipy_gb300 import _lib
    from zodipy_gb300.healpix import random_sphere

    zl = _models("dirbe", bands)
    dirs = random_sphere(1001, seed=5)
    _check(_run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_AUTO), _run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_ONE_PIXEL))


@pytest.mark.parametrize("bands", [(25.0,), (1.25,), (12.0, 25.0, 60.0)])
def test_component_paired_band_tails_healpix_order(lib, bands):
    """In HEALPix RING order the 32 pixels of a warp lie on one latitude ring, so beyond some
    node every pixel of the warp is far enough from the bands' planes that their factor
    e^-(zeta/dzeta)^6 is zero in float32, and the paired kernel stops evaluating them (about
    half of this map's nodes; random directions, as above, almost never form such a warp).
    Same tolerance against the one-pixel kernel, which evaluates every node."""
    from zodipy_gb300 import _lib
    from zodipy_gb300.healpix import pix2vec_ring

    zl = _models("dirbe", bands)
    dirs = pix2vec_ring(64)
    assert band_tail_share(dirs, OBS) > 0.3
    _check(_run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_AUTO), _run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_ONE_PIXEL))


@pytest.mark.parametrize("name,bands", [("planck18", (857.0,)), ("dirbe", (25.0,)), ("planck18", (545.0, 857.0))])
def test_two_pixel_band_tails_same_bits(lib, name, bands):
    """Band tails in the two-pixel kernel skip exactly-zero terms: the same bits with and
    without them, on a HEALPix map (coherent warps) and on random directions sorted by
    latitude (the batched evaluator's order), where a large share of the nodes is skipped."""
    from zodipy_gb300 import _lib
    from zodipy_gb300.healpix import pix2vec_ring, random_sphere

    zl = _models(name, bands)
    hp = pix2vec_ring(64)
    rnd = random_sphere(50_001, seed=9)
    rnd = rnd[:, np.argsort(rnd[2], kind="stable")]
    for dirs in (hp, rnd):
        assert band_tail_share(dirs, OBS, warp=64) > 0.2
        a = _run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_TWO_PIXEL, band_tails=True)
        b = _run(zl, dirs, OBS, EARTH, _lib.ZL_KERNEL_TWO_PIXEL, band_tails=False)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("name,bands,kernel", [("planck18", (857.0,), 0), ("dirbe", (25.0,), 0),
                                                ("dirbe", (25.0,), 1), ("dirbe", (25.0,), 2),
                                                ("planck18", (545.0, 857.0), 1)])
@pytest.mark.parametrize("n", [1, 129, 20_011])
def test_work_queue_and_permutation_same_bits(lib, name, bands, kernel, n):
    """A work-queue launch (tiles pulled from a device counter, several tile sizes and grid
    caps, replayed on the same queue) and a permuted output order give the static launch's
    bits, column for column; the queue is back at zero after every call."""
    import torch

    from zodipy_gb300.healpix import random_sphere

    zl = _models(name, bands)
    dirs = random_sphere(n, seed=n + 1)
    ref = _run(zl, dirs, OBS, EARTH, kernel)
    queue = torch.zeros(2, dtype=torch.int32, device="cuda")
    # the DIRBE layout's paired kernel is compiled once per schedule (its static form keeps 96
    # registers), and the compiler may fuse a multiply and an add differently in the two: the
    # two-pixel tolerance; every other kernel serves both schedules from one build: the same bits
    separate_builds = name == "dirbe" and kernel == 0
    first_queued = None
    for tpb, tile, bps in ((128, 128, 1), (64, 256, 3), (128, 1024, 8), (96, 96, 0)):
        got = _run(zl, dirs, OBS, EARTH, kernel, threads_per_block=tpb, tile=tile, blocks_per_sm=bps, queue=queue)
        torch.cuda.synchronize()
        assert queue.cpu().tolist() == [0, 0]
        if separate_builds:
            _check(got, ref)
            first_queued = got if first_queued is None else first_queued
            np.testing.assert_array_equal(got[0], first_queued[0])  # queued launches agree among themselves
            continue
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])
    order = np.random.default_rng(n).permutation(n)  # evaluate pixel order[i] i-th
    cols = torch.from_numpy(order).cuda()  # ... and write it to its own column order[i]
    got = _run(zl, dirs[:, order], OBS, EARTH, kernel, out_index=cols)
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])


def test_float64_queue_and_permutation_same_bits(lib):
    import torch

    from zodipy_gb300 import engine, packing
    from zodipy_gb300.healpix import random_sphere

    zl = _models("dirbe", (25.0,))
    n = 3001
    dirs = random_sphere(n, seed=4)
    obs = engine.upload_observers(packing.observer_table(zl, OBS, EARTH, [0], any_mode=False))
    u = torch.from_numpy(dirs).cuda()
    ref = engine.forward(zl, u, obs, 1, "float64")[0].cpu().numpy()
    queue = torch.zeros(2, dtype=torch.int32, device="cuda")
    order = np.random.default_rng(1).permutation(n)
    opt = engine.launch_options(tile=256, queue=queue, out_index=torch.from_numpy(order).cuda())
    got = engine.forward(zl, torch.from_numpy(dirs[:, order]).cuda(), obs, 1, "float64", launch=opt)[0]
    np.testing.assert_array_equal(got.cpu().numpy(), ref)
    assert queue.cpu().tolist() == [0, 0]


def test_launch_options_are_checked(lib):
    import torch

    from zodipy_gb300 import _lib, engine
    from zodipy_gb300.healpix import random_sphere

    zl = _models("dirbe", (25.0,))
    dirs = random_sphere(64, seed=1)
    bad = [dict(threads_per_block=48), dict(threads_per_block=256), dict(blocks_per_sm=-1), dict(kernel=7),
           dict(tile=100), dict(tile=128)]  # tile 100: not a multiple of 128; tile 128: no queue
    for kw in bad:
        with pytest.raises(_lib.ZodiGBError):
            _run(zl, dirs, OBS, EARTH, kw.pop("kernel", 0), **kw)
    assert torch.cuda.is_available()
