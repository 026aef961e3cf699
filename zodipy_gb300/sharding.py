"""Data-parallel sharding of the line-of-sight work over ranks (one GPU per rank).

Every line of sight is independent, so the forward pass partitions pixels into
contiguous blocks and needs no collective: each rank evaluates its block.  The
adjoint has one exchange step: the per-shard gradient vectors (a few dozen
float64 values) are summed.  To keep that sum deterministic -- the same bits on
every rank, whatever the backend's all-reduce order -- the vectors are
all-gathered and added in rank order.

Shards start on multiples of the adjoint's 128-pixel tile, so each shard's tiles
are tiles of the unsharded call.
"""

from __future__ import annotations

import numpy as np

TILE = 128


def shard_bounds(n: int, rank: int, world: int, align: int = TILE) -> tuple[int, int]:
    """[begin, end) of rank's contiguous block of n items; blocks start on multiples of align."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    n_units = -(-int(n) // align)
    lo = n_units * rank // world
    hi = n_units * (rank + 1) // world
    return min(lo * align, n), min(hi * align, n)


def shard_observer_table(obs_xyz, earth_xyz, pix_begin, begin: int, end: int):
    """Observer records for pixels [begin, end): the observers overlapping it, re-based to begin.

    Arrays follow ``packing.observer_table``: obs/earth (3, n_obs), pix_begin (n_obs,)
    sorted with pix_begin[0] == 0.
    """
    obs = np.asarray(obs_xyz, dtype=np.float64).reshape(3, -1)
    earth = np.asarray(earth_xyz, dtype=np.float64).reshape(3, -1)
    pb = np.asarray(pix_begin, dtype=np.int64).reshape(-1)
    if earth.shape[1] == 1 and obs.shape[1] > 1:
        earth = np.repeat(earth, obs.shape[1], axis=1)
    first = int(np.searchsorted(pb, begin, side="right")) - 1
    last = int(np.searchsorted(pb, max(end - 1, begin), side="right")) - 1
    sel = slice(max(first, 0), last + 1)
    new_pb = np.maximum(pb[sel] - begin, 0)
    return obs[:, sel], earth[:, sel], new_pb


def combine_in_rank_order(local, group=None) -> np.ndarray:
    """Sum of every rank's float64 vector, added in rank order (identical bits on all ranks)."""
    import torch
    import torch.distributed as dist

    vec = torch.as_tensor(np.asarray(local, dtype=np.float64))
    if not dist.is_available() or not dist.is_initialized():
        return vec.numpy().copy()
    world = dist.get_world_size(group)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    vec = vec.to(dev)
    parts = [torch.empty_like(vec) for _ in range(world)]
    dist.all_gather(parts, vec, group=group)
    total = parts[0].clone()
    for p in parts[1:]:
        total += p
    return total.cpu().numpy()


def sharded_backward(zl_model, u_host, obs_xyz, earth_xyz, pix_begin, g_total, rank: int, world: int, group=None):
    """Adjoint of this rank's block of pixels, summed over ranks in rank order.

    ``u_host`` (3, N) and ``g_total`` (n_spec, N) cover the whole call; each rank
    uploads and differentiates only its block.  Returns the gradient vector
    (float64 numpy array), the same on every rank.
    """
    import torch

    from . import engine, packing

    n = np.asarray(u_host).shape[-1]
    b, e = shard_bounds(n, rank, world)
    g = np.asarray(g_total, dtype=np.float64).reshape(zl_model.n_spec, n)
    if e > b:
        o, ea, pb = shard_observer_table(obs_xyz, earth_xyz, pix_begin, b, e)
        tab = packing.observer_table(zl_model, o, ea, pb, any_mode=False)
        u = torch.from_numpy(np.ascontiguousarray(np.asarray(u_host, dtype=np.float64)[:, b:e])).cuda()
        gd = torch.from_numpy(np.ascontiguousarray(g[:, b:e])).cuda()
        local = engine.backward(zl_model, u, engine.upload_observers(tab), len(pb), g_total=gd).cpu().numpy()
    else:
        local = np.zeros(engine.grad_count(zl_model))
    return combine_in_rank_order(local, group)
