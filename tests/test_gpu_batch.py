"""Batched observers: one graph-captured launch over uneven pixel counts."""

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]


def _setup(n_obs=7, seed=4, lo=50, hi=900, name="planck18", x=857.0, unit="GHz"):
    import zodipy_gb300 as zg
    from zodipy_gb300 import units as u
    from zodipy_gb300.batch import random_directions_device, uneven_observers

    model = zg.Model(x * {"GHz": u.GHz, "micron": u.micron}[unit], name=name)
    obs, counts = uneven_observers(n_obs, seed, lo, hi)
    uu = random_directions_device(int(counts.sum()), seed + 1)
    earth = np.array([-0.17, 0.97, 0.0])
    return model, obs, counts, uu, earth


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_batch_equals_separate_calls(lib, precision):
    from zodipy_gb300.batch import BatchEvaluator

    model, obs, counts, uu, earth = _setup()
    ev = BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision=precision, comps=True)
    ev.run()
    got = ev.comps[0].cpu().numpy()
    begin = np.concatenate([[0], np.cumsum(counts)])
    for o in range(len(counts)):
        part = uu[:, begin[o] : begin[o + 1]]
        ref = model.evaluate_xyz(part, obs[:, o], earth, return_comps=True, precision=precision)
        np.testing.assert_array_equal(got[:, begin[o] : begin[o + 1]], ref.cpu().numpy())


def test_batch_matches_oracle(lib):
    """float32 batched result vs the CPU oracle on every observer (a few pixels each)."""
    from oracle import zodi_oracle as zo
    from zodipy_gb300.batch import BatchEvaluator
    from zodipy_gb300.zodiacal_light_model import COMPONENT_CUTOFFS

    model, obs, counts, uu, earth = _setup(n_obs=5)
    ev = BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32")
    tot = ev.run()[0].cpu().numpy()
    m = model.get_parameters()
    desc = {
        "labels": list(m["comps"]),
        "comps": m["comps"],
        "cutoffs": {lbl.value: COMPONENT_CUTOFFS[lbl] for lbl in model._ipd_model.comps},
        "T_0": m["T_0"],
        "delta": m["delta"],
        **{k: model._spectrum[k] for k in ("emissivity", "albedo", "C1", "C2", "C3", "solar_irradiance")},
        "bb_table": model._b_nu_table,
        "gauss_quad_degree": 50,
    }
    begin = np.concatenate([[0], np.cumsum(counts)])
    u_host = uu.cpu().numpy()
    for o in range(len(counts)):
        sl = slice(begin[o], begin[o] + 40)
        ref = zo.evaluate(desc, u_host[:, sl], obs[:, o], earth).sum(axis=0)
        np.testing.assert_allclose(tot[sl], ref, rtol=1e-5)


def test_graph_replay_equals_eager_and_launch_shape_does_not_matter(lib):
    """Static and work-queue launches, tile sizes, sorted or input order, eager or replayed
    from a CUDA graph (several replays on the same self-resetting queue): the same bits."""
    import torch

    from zodipy_gb300.batch import BatchEvaluator

    model, obs, counts, uu, earth = _setup(n_obs=9, lo=2000, hi=9000)
    plain = BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32", sort=False)
    plain.set_launch(64, 0, 0, False)
    ref = plain.run().clone()
    ev = BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32")
    for launch in ((64, 3, 64, True), (128, 0, 0, False), (128, 8, 512, True), (96, 0, 0, True)):
        ev.set_launch(*launch)
        np.testing.assert_array_equal(ev.run().cpu().numpy(), ref.cpu().numpy())
    ev.capture()
    for _ in range(3):
        ev.total.zero_()
        ev.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ev.total.cpu().numpy(), ref.cpu().numpy())
    assert ev.queue.cpu().tolist() == [0, 0]


def test_sorted_batch_skips_band_tails(lib):
    """Sorting each observer's directions by latitude makes warps coherent: the share of
    (warp, node) pairs at which the bands are zero for the whole warp goes from ~0 to a
    large fraction (the kernel then skips them, with the same results)."""
    from conftest import band_tail_share
    from zodipy_gb300.batch import BatchEvaluator

    model, obs, counts, uu, earth = _setup(n_obs=2, lo=40000, hi=40000)
    ev = BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32")
    u0 = uu[:, : counts[0]].cpu().numpy()
    s0 = ev.u[:, : counts[0]].cpu().numpy()
    assert band_tail_share(u0, obs[:, 0], warp=64) < 0.02
    assert band_tail_share(s0, obs[:, 0], warp=64) > 0.2
    np.testing.assert_array_equal(np.sort(s0[2]), s0[2])


def test_tuning_one_evaluator_leaves_other_calls_alone(lib, tmp_path, monkeypatch):
    """The autotuner picks a candidate shape and keeps it in its own evaluator: a Model
    evaluated meanwhile, and another evaluator, keep their launches and results."""
    from zodipy_gb300 import batch

    monkeypatch.setattr(batch, "CACHE_PATH", str(tmp_path / "tune.json"))
    model, obs, counts, uu, earth = _setup(n_obs=4, lo=20000, hi=40000)
    other = batch.BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32")
    other.set_launch(96, 0, 0, True)
    before = other.run().cpu().numpy().copy()
    probe = uu[:, :500]
    m_before = model.evaluate_xyz(probe, obs[:, 0], earth, return_comps=True, precision="float32").cpu().numpy()
    ev = batch.BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32")
    tpb, bps, tile, tails, ms = ev.autotune(sample=1 << 16, reps=1)
    assert (tpb, bps, tile, tails) in batch.STATIC_CHOICES + batch.QUEUE_CHOICES and ms > 0
    assert ev.launch == (tpb, bps, tile, tails) and other.launch == (96, 0, 0, True)
    again = ev.autotune(sample=1 << 16, reps=1)  # from the cache
    assert tuple(again[:4]) == (tpb, bps, tile, tails)
    np.testing.assert_array_equal(other.run().cpu().numpy(), before)
    m_after = model.evaluate_xyz(probe, obs[:, 0], earth, return_comps=True, precision="float32").cpu().numpy()
    np.testing.assert_array_equal(m_after, m_before)
    np.testing.assert_array_equal(ev.run().cpu().numpy(), before)
