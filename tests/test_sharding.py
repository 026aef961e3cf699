"""Sharding of the pixel work over ranks: bounds, observer re-basing and the rank-ordered
gradient sum, the last over a real two-process gloo group on CPU."""

import os
import socket

import numpy as np
import pytest


def test_shard_bounds_cover_and_align():
    from zodipy_gb300.sharding import TILE, shard_bounds

    for n in (0, 1, 127, 128, 129, 1000, 3 * 128 + 5, 786432):
        for world in (1, 2, 3, 4, 7, 8):
            bounds = [shard_bounds(n, r, world) for r in range(world)]
            assert bounds[0][0] == 0 and bounds[-1][1] == n
            for (b0, e0), (b1, e1) in zip(bounds, bounds[1:]):
                assert e0 == b1 and b0 <= e0
            assert all(b % TILE == 0 or b == n for b, _ in bounds)
    with pytest.raises(ValueError):
        shard_bounds(10, 2, 2)


def test_shard_observer_table_rebases():
    from zodipy_gb300.sharding import shard_observer_table

    obs = np.arange(12, dtype=float).reshape(3, 4)
    pb = np.array([0, 100, 250, 400])
    o, e, p = shard_observer_table(obs, obs[:, :1], pb, 128, 384)
    np.testing.assert_array_equal(p, [0, 122])  # observer 1 covers 128..249, observer 2 250..
    np.testing.assert_array_equal(o, obs[:, 1:3])
    assert e.shape == (3, 2)
    o, e, p = shard_observer_table(obs, obs, pb, 0, 100)
    np.testing.assert_array_equal(p, [0])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from zodipy_gb300.sharding import combine_in_rank_order

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        local = np.sin(np.arange(16) * (rank + 1.3)) * 10.0 ** (-3 * rank)  # values of mixed size
        np.save(os.path.join(out_dir, f"r{rank}.npy"), combine_in_rank_order(local))
    finally:
        dist.destroy_process_group()


def test_rank_ordered_sum_over_gloo(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r0, r1 = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    expect = np.sin(np.arange(16) * 1.3) + np.sin(np.arange(16) * 2.3) * 1e-3
    np.testing.assert_array_equal(r0, r1)
    np.testing.assert_array_equal(r0, expect)


def _oracle_block(desc, u, observers, earth, pix_begin, b, e):
    """The oracle's per-component map of pixels [b, e) of a batched call: each observer
    overlapping the block evaluates its own pixels (one reference call per observer)."""
    from oracle import zodi_oracle as zo
    from zodipy_gb300.sharding import shard_observer_table

    o, ea, pb = shard_observer_table(observers, earth, pix_begin, b, e)
    ends = list(pb[1:]) + [e - b]
    parts = [zo.evaluate(desc, u[:, b + s : b + t], o[:, j], ea[:, j]) for j, (s, t) in enumerate(zip(pb, ends))]
    return np.concatenate(parts, axis=-1)


def _batch_case():
    from conftest import load_case, oracle_desc

    case = load_case("cfg3_planck18_batch")  # 4 observers x 96 directions, the reference's own output
    u = case["unit_vectors"]
    n = u.shape[1]
    pix_begin = np.arange(0, n, 96)
    observers = case["obs"][:, pix_begin]
    a = np.random.default_rng(5).uniform(0.5, 1.5, n)  # weights of a linear loss sum_i a_i total_i
    return oracle_desc(case), u, observers, case["earth"], pix_begin, a, case["ref_out"]


def _shard_worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from zodipy_gb300.sharding import combine_in_rank_order, shard_bounds

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        desc, u, observers, earth, pix_begin, a, _ = _batch_case()
        b, e = shard_bounds(u.shape[1], rank, world)
        block = _oracle_block(desc, u, observers, earth, pix_begin, b, e)
        local = block @ a[b:e]  # per-component loss of this rank's pixels
        blocks = [None] * world
        dist.all_gather_object(blocks, (rank, block))
        np.save(os.path.join(out_dir, f"loss{rank}.npy"), combine_in_rank_order(local))
        np.save(os.path.join(out_dir, f"local{rank}.npy"), local)
        np.save(os.path.join(out_dir, f"map{rank}.npy"), np.concatenate([blk for _, blk in sorted(blocks)], axis=-1))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_batch_over_gloo_ranks(tmp_path, world):
    """A batched call (4 observers) split over 2 and 3 gloo ranks on CPU with the package's
    shard bounds and observer re-basing, each rank evaluating its block with the oracle: the
    ranks' blocks concatenate to the unsharded map bit for bit (and to the reference's own
    output at 1e-13), and the per-rank loss vectors combine in rank order to the same bits on
    every rank, within 1e-12 of the unsharded sum."""
    import torch.multiprocessing as mp

    mp.start_processes(_shard_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    desc, u, observers, earth, pix_begin, a, ref = _batch_case()
    whole = _oracle_block(desc, u, observers, earth, pix_begin, 0, u.shape[1])
    np.testing.assert_allclose(whole, ref, rtol=1e-13, atol=0)
    maps = [np.load(tmp_path / f"map{r}.npy") for r in range(world)]
    losses = [np.load(tmp_path / f"loss{r}.npy") for r in range(world)]
    for r in range(world):
        np.testing.assert_array_equal(maps[r], whole)
        np.testing.assert_array_equal(losses[r], losses[0])
    ordered = np.load(tmp_path / "local0.npy").copy()
    for r in range(1, world):
        ordered += np.load(tmp_path / f"local{r}.npy")
    np.testing.assert_array_equal(losses[0], ordered)
    np.testing.assert_allclose(losses[0], whole @ a, rtol=1e-12, atol=0)
