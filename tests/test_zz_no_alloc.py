"""zl_backward_static: the adjoint for callers that cannot allocate device memory.

Such callers (a host that owns all device memory through its own pool, an
allocation-free real-time loop, a binding without a CUDA allocator) cannot
provide zl_backward's workspace.  zl_backward_static runs the same kernels on
a fixed scratch array built into the library.  This test calls it through the
C ABI twice in a row and checks both results against zl_backward with a
caller-allocated workspace, then checks that a problem larger than the
built-in scratch is refused.  It is its own file, collected last, so that a
run stopping at the first failure has run every other test first.
"""

import ctypes

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]

STATIC_SCRATCH_BYTES = 32 << 20


def _problem(nside=64):
    import torch

    import zodipy_gb300 as zg
    from zodipy_gb300 import engine, packing
    from zodipy_gb300 import units as u
    from zodipy_gb300.healpix import pix2vec_ring

    model = zg.Model(25 * u.micron)
    zl = model.zl_model
    uu = torch.from_numpy(pix2vec_ring(nside)).cuda()
    tab = packing.observer_table(zl, [0.9833, 0.0, 0.0], [-0.17, 0.97, 0.0], [0], any_mode=False)
    obs = engine.upload_observers(tab)
    g = torch.randn((1, uu.shape[1]), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(11))
    return zl, uu, obs, g


def _static(lib, zl, uu, n, obs, g, out):
    import torch

    return lib.zl_backward_static(
        ctypes.byref(zl),
        ctypes.c_void_p(uu.data_ptr()),
        n,
        ctypes.c_void_p(obs.data_ptr()),
        1,
        None,
        ctypes.c_void_p(g.data_ptr()),
        ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
    )


def test_static_scratch_backward_matches_workspace_backward(lib):
    import torch

    from zodipy_gb300 import _lib, engine

    zl, uu, obs, g = _problem()
    n = uu.shape[1]
    ref = engine.backward(zl, uu, obs, 1, g_total=g).cpu().numpy()
    for _ in range(2):  # two calls in a row share (and reuse) the built-in scratch
        out = torch.full((engine.grad_count(zl),), np.nan, dtype=torch.float64, device="cuda")
        rc = _static(lib, zl, uu, n, obs, g, out)
        assert rc == _lib.ZL_OK, _lib.last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        # same kernels, same fixed-order reduction: equal to the tolerance of the
        # determinism tests (they are in fact bit-identical)
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0)


def test_static_scratch_refuses_problems_beyond_its_size(lib):
    import torch

    from zodipy_gb300 import _lib, engine

    zl, uu, obs, g = _problem(nside=4)
    n_big = 4 << 20  # a DIRBE band at 4.2 million pixels needs ~39 MB of scratch
    assert engine.backward_workspace_bytes(zl, n_big) > STATIC_SCRATCH_BYTES
    out = torch.empty(engine.grad_count(zl), dtype=torch.float64, device="cuda")
    rc = _static(lib, zl, uu, n_big, obs, g, out)  # refused before any device access
    assert rc == _lib.ZL_ERR_SPACE
    msg = _lib.last_error()
    assert "scratch" in msg and "zl_backward" in msg
