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
    import torch

    from zodipy_gb300.batch import BatchEvaluator

    model, obs, counts, uu, earth = _setup(n_obs=9, lo=2000, hi=9000)
    ev = BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32")
    ev.set_launch(64, 3)
    eager = ev.run().clone()
    ev.set_launch(128, 8)
    ev.capture()
    ev.total.zero_()
    ev.replay()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ev.total.cpu().numpy(), eager.cpu().numpy())


def test_autotuner_picks_a_valid_shape(lib, tmp_path, monkeypatch):
    from zodipy_gb300 import batch

    monkeypatch.setattr(batch, "CACHE_PATH", str(tmp_path / "tune.json"))
    model, obs, counts, uu, earth = _setup(n_obs=4, lo=20000, hi=40000)
    ev = batch.BatchEvaluator(model.zl_model, uu, obs, counts, earth, precision="float32")
    tpb, bps, ms = ev.autotune(sample=1 << 16, reps=1)
    assert tpb in batch.TPB_CHOICES and bps in batch.BPS_CHOICES and ms > 0
    again = ev.autotune(sample=1 << 16, reps=1)  # from the cache
    assert tuple(again[:2]) == (tpb, bps)
    ev.set_launch(0, 0)
