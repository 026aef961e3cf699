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
