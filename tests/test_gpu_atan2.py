"""The float32 kernels' branch-free atan2 (per-node feature longitude and scattering
angle) against the correctly rounded atan2 (numpy, float64) and CUDA's atan2f.

Bound: 4 ulp of the float32 result (the fit is 1.1 ulp on [0, 1]; the reciprocal
and the octant identities add the rest), and at most 4 ulp from CUDA's atan2f
(itself within 2 ulp of the correctly rounded value)."""

import ctypes

import numpy as np
import pytest

from conftest import cuda_ok

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not cuda_ok(), reason="needs CUDA")]


def _points():
    rng = np.random.default_rng(12)
    y = rng.standard_normal(1 << 20).astype(np.float32)
    x = rng.standard_normal(1 << 20).astype(np.float32)
    # axes, diagonals, octant boundaries, tiny and large magnitudes, the node coordinates' range
    a = np.array([0.0, 1.0, -1.0, 1e-30, -1e-30, 1e30, 3.0, -2.5, 0.5], dtype=np.float32)
    yy, xx = np.meshgrid(a, a)
    ang = rng.uniform(-np.pi, np.pi, 1 << 16)
    rad = 10.0 ** rng.uniform(-3, 1, 1 << 16)
    y = np.concatenate([y, yy.ravel(), (rad * np.sin(ang)).astype(np.float32)])
    x = np.concatenate([x, xx.ravel(), (rad * np.cos(ang)).astype(np.float32)])
    return y, x


def test_atan2_poly_within_4_ulp(lib):
    import torch

    from zodipy_gb300 import _lib

    y, x = _points()
    yd, xd = torch.from_numpy(y).cuda(), torch.from_numpy(x).cuda()
    out = torch.empty_like(yd)
    _lib.check(
        lib.zl_diag_atan2(ctypes.c_void_p(yd.data_ptr()), ctypes.c_void_p(xd.data_ptr()),
                          ctypes.c_void_p(out.data_ptr()), y.size, None),
        "zl_diag_atan2",
    )
    got = out.cpu().numpy().astype(np.float64)
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    err = np.abs(got - ref) / ulp
    both_zero = (x == 0) & (y == 0)
    assert np.all(got[both_zero] == 0.0)
    w = int(np.argmax(np.where(both_zero, 0, err)))
    assert err[~both_zero].max() <= 4.0, f"y={y[w]!r} x={x[w]!r}: {got[w]!r} vs {ref[w]!r} ({err[w]:.2f} ulp)"
    cuda = torch.atan2(yd, xd).cpu().numpy().astype(np.float64)
    dc = np.abs(got - cuda) / ulp
    assert dc[~both_zero].max() <= 4.0
