"""Sharded adjoint on one GPU: k tile-aligned shards, summed in order, against the unsharded call.

Shards start on 128-pixel tile boundaries, so every tile's float32 accumulation is the
unsharded one; only the float64 sum over tiles is associated differently (rtol 1e-12).
The same k gives the same bits.  Forward sharding needs no collective and is covered by
the partition-independence test of test_gpu_parity.py.
"""

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]


def test_sharded_adjoint_matches_unsharded(lib):
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import engine, packing
    from zodipy_gb300 import units as u_
    from zodipy_gb300.healpix import random_sphere
    from zodipy_gb300.sharding import sharded_backward

    m = zg.Model(25 * u_.micron).zl_model
    n = 20000
    u = random_sphere(n, seed=8)
    obs = np.array([[0.98, 0.3], [0.1, 0.9], [0.0, 0.01]])  # two observers: pixels [0, 7000) and [7000, n)
    earth = np.array([0.97, 0.2, 0.0])
    pb = np.array([0, 7000])
    g = np.random.default_rng(1).standard_normal((1, n))
    tab = packing.observer_table(m, obs, earth, pb, any_mode=False)
    ref = engine.backward(m, torch.from_numpy(u).cuda(), engine.upload_observers(tab), 2,
                          g_total=torch.from_numpy(g).cuda()).cpu().numpy()
    for k in (1, 2, 3, 5):
        parts = [sharded_backward(m, u, obs, earth, pb, g, r, k) for r in range(k)]
        total = parts[0].copy()
        for p in parts[1:]:
            total += p
        np.testing.assert_allclose(total, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
        again = [sharded_backward(m, u, obs, earth, pb, g, r, k) for r in range(k)]
        for a, b in zip(parts, again):
            np.testing.assert_array_equal(a, b)
