"""Host-array calls -- zero copy on mapped host memory, or pipelined through two copy streams --
give the same bits as the device-array call: neither changes any pixel's arithmetic."""

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]


@pytest.mark.parametrize("zero_copy", [True, False])
def test_host_call_equals_device_call(lib, zero_copy, monkeypatch):
    """Host arrays through zero copy (mapped host memory) and through the copy pipeline."""
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import model as model_mod
    from zodipy_gb300 import units as u_
    from zodipy_gb300.healpix import random_sphere

    monkeypatch.setattr(model_mod, "_ZERO_COPY", zero_copy)
    n = 2 * model_mod._PIPE_CHUNK + 12345  # three chunks, the last one short
    dirs = random_sphere(n, seed=21)
    obs, earth = np.array([0.7071, 0.7071, 0.0]), np.array([0.70, 0.71, 0.0])
    m = zg.Model(25 * u_.micron, precision="float32")
    dev = m.evaluate_xyz(torch.from_numpy(dirs).cuda(), obs, earth).cpu().numpy()
    out = torch.empty(n, dtype=torch.float64).pin_memory()
    host = m.evaluate_xyz(torch.from_numpy(dirs).pin_memory(), obs, earth, out=out)
    np.testing.assert_array_equal(host.numpy(), dev)
    comps_dev = m.evaluate_xyz(torch.from_numpy(dirs).cuda(), obs, earth, return_comps=True).cpu().numpy()
    comps_host = m.evaluate_xyz(dirs, obs, earth, return_comps=True)
    np.testing.assert_array_equal(comps_host, comps_dev)
    ms = zg.ModelSet([m, zg.Model(12 * u_.micron, precision="float32")])
    both = ms.evaluate_xyz(dirs, obs, earth)
    np.testing.assert_array_equal(both[0], dev)


def test_mapped_pointer_of_pinned_and_pageable(lib):
    import torch

    from zodipy_gb300 import engine

    assert engine.mapped_pointer(torch.empty(16, dtype=torch.float64).pin_memory()) is not None
    assert engine.mapped_pointer(torch.empty(16, dtype=torch.float64)) is None
