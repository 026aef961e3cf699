"""Device execution: calls into libzodigb on torch CUDA tensors.

PyTorch provides device memory and streams; every kernel that touches pixels
is libzodigb's own.  There is no CPU path: without a CUDA device or without
the library these functions raise.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

PRECISIONS = {"float64": _lib.ZL_PREC_F64, "f64": _lib.ZL_PREC_F64, "float32": _lib.ZL_PREC_F32, "f32": _lib.ZL_PREC_F32}


def precision_code(precision) -> int:
    if isinstance(precision, int) and precision in (_lib.ZL_PREC_F64, _lib.ZL_PREC_F32):
        return precision
    try:
        return PRECISIONS[str(precision).lower()]
    except KeyError as err:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, got {precision!r}") from err


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise _lib.ZodiGBError("a CUDA device is required: zodipy_gb300 has no CPU evaluation path")
    return torch


def upload_observers(observers, device=None):
    """Copy a ctypes ``ZlObserver`` array to a uint8 device tensor."""
    torch = _torch()
    raw = np.frombuffer(observers, dtype=np.uint8).copy()
    return torch.from_numpy(raw).to(device or "cuda")


def current_stream_handle(device=None) -> int:
    torch = _torch()
    return int(torch.cuda.current_stream(device).cuda_stream)


def forward(
    zl_model: _lib.ZlModel,
    u_dev,
    observers_dev,
    n_obs: int,
    precision,
    want_comps: bool = True,
    want_total: bool = True,
    out_comps=None,
    out_total=None,
    stream: int | None = None,
    launch: _lib.ZlLaunch | None = None,
):
    """Run ``zl_forward`` (``zl_forward_ex`` when ``launch`` options are given); returns
    (comps [n_spec, C, N] or None, total [n_spec, N] or None)."""
    torch = _torch()
    if u_dev.dtype != torch.float64 or not u_dev.is_cuda or u_dev.dim() != 2 or u_dev.shape[0] != 3:
        raise ValueError("unit vectors must be a float64 CUDA tensor of shape (3, N)")
    u_dev = u_dev.contiguous()
    n = u_dev.shape[1]
    ns, nc = zl_model.n_spec, zl_model.n_comps
    dev = u_dev.device
    if want_comps and out_comps is None:
        out_comps = torch.empty((ns, nc, n), dtype=torch.float64, device=dev)
    if want_total and out_total is None:
        out_total = torch.empty((ns, n), dtype=torch.float64, device=dev)
    lib = _lib.load()
    rc = lib.zl_forward_ex(
        ctypes.byref(zl_model),
        ctypes.c_void_p(u_dev.data_ptr()),
        n,
        ctypes.c_void_p(observers_dev.data_ptr()),
        n_obs,
        precision_code(precision),
        ctypes.c_void_p(out_comps.data_ptr() if out_comps is not None else 0),
        ctypes.c_void_p(out_total.data_ptr() if out_total is not None else 0),
        ctypes.byref(launch) if launch is not None else None,
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(dev)),
    )
    _lib.check(rc, "zl_forward")
    return (out_comps if want_comps else None), (out_total if want_total else None)


def launch_options(threads_per_block: int = 0, blocks_per_sm: int = 0, kernel: int = _lib.ZL_KERNEL_AUTO,
                   band_tails: bool = False, tile: int = 0, queue=None, out_index=None) -> _lib.ZlLaunch:
    """A ``ZlLaunch`` for one call; ``queue`` (two int32 words, zero) and ``out_index`` (int64, a
    permutation of the call's pixel indices) are CUDA tensors.  The struct holds references to
    both, so they stay allocated as long as it does (it carries only their addresses to the
    library)."""
    if out_index is not None and (out_index.dtype != _torch().int64 or not out_index.is_cuda):
        raise ValueError("out_index must be an int64 CUDA tensor")
    if queue is not None and (queue.numel() < 2 or queue.element_size() != 4 or not queue.is_cuda):
        raise ValueError("queue must be a CUDA tensor of two 32-bit words")
    opt = _lib.ZlLaunch()
    opt._keep = (queue, out_index)
    opt.threads_per_block = int(threads_per_block)
    opt.blocks_per_sm = int(blocks_per_sm)
    opt.kernel = int(kernel)
    opt.band_tails = 1 if band_tails else 0
    opt.tile = int(tile)
    opt.queue_dev = queue.data_ptr() if queue is not None else None
    opt.out_index_dev = out_index.data_ptr() if out_index is not None else None
    return opt


def grad_count(zl_model: _lib.ZlModel) -> int:
    n = ctypes.c_int32(0)
    _lib.check(_lib.load().zl_grad_count(ctypes.byref(zl_model), ctypes.byref(n)), "zl_grad_count")
    return int(n.value)


def backward_workspace_bytes(zl_model: _lib.ZlModel, n_pix: int) -> int:
    b = ctypes.c_size_t(0)
    _lib.check(
        _lib.load().zl_backward_workspace_bytes(ctypes.byref(zl_model), int(n_pix), ctypes.byref(b)),
        "zl_backward_workspace_bytes",
    )
    return int(b.value)


def backward(
    zl_model: _lib.ZlModel,
    u_dev,
    observers_dev,
    n_obs: int,
    g_comps=None,
    g_total=None,
    grad_out=None,
    workspace=None,
    stream: int | None = None,
    launch: _lib.ZlLaunch | None = None,
):
    """Run ``zl_backward`` (``zl_backward_ex`` with ``launch`` options): gradient (float64 CUDA
    tensor) of the loss w.r.t. the parameter vector."""
    torch = _torch()
    if (g_comps is None) == (g_total is None):
        raise ValueError("pass exactly one of g_comps (n_spec, C, N) or g_total (n_spec, N)")
    u_dev = u_dev.contiguous()
    n = u_dev.shape[1]
    dev = u_dev.device
    g = (g_comps if g_comps is not None else g_total).to(device=dev, dtype=torch.float64).contiguous()
    want = (zl_model.n_spec, zl_model.n_comps, n) if g_comps is not None else (zl_model.n_spec, n)
    if tuple(g.shape) != want:
        raise ValueError(f"upstream gradient must have shape {want}, got {tuple(g.shape)}")
    if grad_out is None:
        grad_out = torch.empty(grad_count(zl_model), dtype=torch.float64, device=dev)
    need = backward_workspace_bytes(zl_model, n)
    if workspace is None or workspace.numel() * workspace.element_size() < need:
        workspace = torch.empty(max(need, 8), dtype=torch.uint8, device=dev)
    rc = _lib.load().zl_backward_ex(
        ctypes.byref(zl_model),
        ctypes.c_void_p(u_dev.data_ptr()),
        n,
        ctypes.c_void_p(observers_dev.data_ptr()),
        n_obs,
        ctypes.c_void_p(g.data_ptr() if g_comps is not None else 0),
        ctypes.c_void_p(g.data_ptr() if g_total is not None else 0),
        ctypes.c_void_p(grad_out.data_ptr()),
        ctypes.c_void_p(workspace.data_ptr()),
        workspace.numel() * workspace.element_size(),
        ctypes.byref(launch) if launch is not None else None,
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(dev)),
    )
    _lib.check(rc, "zl_backward")
    return grad_out


def density_grid(zl_model: _lib.ZlModel, x_dev, y_dev, z_dev, earth_xyz, out=None, stream: int | None = None):
    """Run ``zl_density_grid``: float64 (C, ny, nx, nz) densities on the mesh of x, y, z (CUDA tensors)."""
    torch = _torch()
    for v in (x_dev, y_dev, z_dev):
        if v.dtype != torch.float64 or not v.is_cuda or v.dim() != 1:
            raise ValueError("grid coordinates must be 1-D float64 CUDA tensors")
    x_dev, y_dev, z_dev = x_dev.contiguous(), y_dev.contiguous(), z_dev.contiguous()
    nx, ny, nz = x_dev.numel(), y_dev.numel(), z_dev.numel()
    shape = (zl_model.n_comps, ny, nx, nz)
    if out is None:
        out = torch.empty(shape, dtype=torch.float64, device=x_dev.device)
    elif tuple(out.shape) != shape or out.dtype != torch.float64 or not out.is_contiguous():
        raise ValueError(f"out must be a contiguous float64 tensor of shape {shape}")
    earth = (ctypes.c_double * 3)(*[float(v) for v in np.asarray(earth_xyz, dtype=np.float64).reshape(3)])
    rc = _lib.load().zl_density_grid(
        ctypes.byref(zl_model),
        ctypes.c_void_p(x_dev.data_ptr()),
        nx,
        ctypes.c_void_p(y_dev.data_ptr()),
        ny,
        ctypes.c_void_p(z_dev.data_ptr()),
        nz,
        earth,
        ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(x_dev.device)),
    )
    _lib.check(rc, "zl_density_grid")
    return out


def _soa3(x, n, dev, what):
    torch = _torch()
    if x is None:
        return None
    if not isinstance(x, torch.Tensor):
        x = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64)))
    x = x.to(device=dev, dtype=torch.float64)
    if x.dim() == 1:
        x = x.reshape(3, 1)
    if x.shape[0] != 3 or x.shape[-1] not in (1, n):
        raise ValueError(f"{what} must be (3,) or (3, {n})")
    return x.expand(3, n).contiguous() if x.shape[-1] != n else x.contiguous()


def forward_tod(zl_model, u_dev, obs_xyz, earth_xyz, precision, want_comps=True, want_total=True, out_comps=None,
                out_total=None, flags=None, stream: int | None = None):
    """Run ``zl_forward_tod``: one observer / Earth position per pixel ((3, N) each, device or host)."""
    torch = _torch()
    if u_dev.dtype != torch.float64 or not u_dev.is_cuda or u_dev.dim() != 2 or u_dev.shape[0] != 3:
        raise ValueError("unit vectors must be a float64 CUDA tensor of shape (3, N)")
    u_dev = u_dev.contiguous()
    n, dev = u_dev.shape[1], u_dev.device
    obs = _soa3(obs_xyz, n, dev, "observer positions")
    earth = _soa3(earth_xyz, n, dev, "Earth positions")
    ns, nc = zl_model.n_spec, zl_model.n_comps
    if want_comps and out_comps is None:
        out_comps = torch.empty((ns, nc, n), dtype=torch.float64, device=dev)
    if want_total and out_total is None:
        out_total = torch.empty((ns, n), dtype=torch.float64, device=dev)
    if flags is None:
        flags = torch.empty(1, dtype=torch.int32, device=dev)
    rc = _lib.load().zl_forward_tod(
        ctypes.byref(zl_model),
        ctypes.c_void_p(u_dev.data_ptr()),
        n,
        ctypes.c_void_p(obs.data_ptr()),
        ctypes.c_void_p(earth.data_ptr() if earth is not None else 0),
        ctypes.c_void_p(flags.data_ptr()),
        precision_code(precision),
        ctypes.c_void_p(out_comps.data_ptr() if out_comps is not None else 0),
        ctypes.c_void_p(out_total.data_ptr() if out_total is not None else 0),
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(dev)),
    )
    _lib.check(rc, "zl_forward_tod")
    return (out_comps if want_comps else None), (out_total if want_total else None)


def backward_tod(zl_model, u_dev, obs_xyz, earth_xyz, g_comps=None, g_total=None, grad_out=None, workspace=None,
                 flags=None, stream: int | None = None):
    """Run ``zl_backward_tod``: gradient w.r.t. the parameter vector for time-ordered positions."""
    torch = _torch()
    if (g_comps is None) == (g_total is None):
        raise ValueError("pass exactly one of g_comps (n_spec, C, N) or g_total (n_spec, N)")
    u_dev = u_dev.contiguous()
    n, dev = u_dev.shape[1], u_dev.device
    obs = _soa3(obs_xyz, n, dev, "observer positions")
    earth = _soa3(earth_xyz, n, dev, "Earth positions")
    g = (g_comps if g_comps is not None else g_total).to(device=dev, dtype=torch.float64).contiguous()
    want = (zl_model.n_spec, zl_model.n_comps, n) if g_comps is not None else (zl_model.n_spec, n)
    if tuple(g.shape) != want:
        raise ValueError(f"upstream gradient must have shape {want}, got {tuple(g.shape)}")
    if grad_out is None:
        grad_out = torch.empty(grad_count(zl_model), dtype=torch.float64, device=dev)
    need = backward_workspace_bytes(zl_model, n)
    if workspace is None or workspace.numel() * workspace.element_size() < need:
        workspace = torch.empty(max(need, 8), dtype=torch.uint8, device=dev)
    if flags is None:
        flags = torch.empty(1, dtype=torch.int32, device=dev)
    rc = _lib.load().zl_backward_tod(
        ctypes.byref(zl_model),
        ctypes.c_void_p(u_dev.data_ptr()),
        n,
        ctypes.c_void_p(obs.data_ptr()),
        ctypes.c_void_p(earth.data_ptr() if earth is not None else 0),
        ctypes.c_void_p(flags.data_ptr()),
        ctypes.c_void_p(g.data_ptr() if g_comps is not None else 0),
        ctypes.c_void_p(g.data_ptr() if g_total is not None else 0),
        ctypes.c_void_p(grad_out.data_ptr()),
        ctypes.c_void_p(workspace.data_ptr()),
        workspace.numel() * workspace.element_size(),
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(dev)),
    )
    _lib.check(rc, "zl_backward_tod")
    return grad_out


def spline_eval(knots_dev, coef_dev, t_dev, out=None, stream: int | None = None):
    """Run ``zl_spline_eval``: (3, n) positions of a piecewise cubic (coef (4, K-1, 3)) at times t."""
    torch = _torch()
    k = knots_dev.numel()
    if tuple(coef_dev.shape) != (4, k - 1, 3):
        raise ValueError(f"coefficients must have shape (4, {k - 1}, 3)")
    n = t_dev.numel()
    if out is None:
        out = torch.empty((3, n), dtype=torch.float64, device=t_dev.device)
    rc = _lib.load().zl_spline_eval(
        ctypes.c_void_p(knots_dev.data_ptr()),
        k,
        ctypes.c_void_p(coef_dev.data_ptr()),
        ctypes.c_void_p(t_dev.data_ptr()),
        n,
        ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(t_dev.device)),
    )
    _lib.check(rc, "zl_spline_eval")
    return out


def semb_l2(earth_dev, l2_distance: float, whole_array_norm: bool, out=None, stream: int | None = None):
    """Run ``zl_semb_l2`` on (3, n) Earth positions."""
    torch = _torch()
    earth_dev = earth_dev.contiguous()
    n = earth_dev.shape[1]
    if out is None:
        out = torch.empty_like(earth_dev)
    scratch = torch.empty(_lib.ZL_SEMB_L2_SCRATCH, dtype=torch.float64, device=earth_dev.device)
    rc = _lib.load().zl_semb_l2(
        ctypes.c_void_p(earth_dev.data_ptr()),
        n,
        float(l2_distance),
        1 if whole_array_norm else 0,
        ctypes.c_void_p(scratch.data_ptr()),
        scratch.numel(),
        ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(earth_dev.device)),
    )
    _lib.check(rc, "zl_semb_l2")
    return out


def directions(lon_dev, lat_dev, rotation=None, out=None, stream: int | None = None):
    """Run ``zl_directions``: (3, n) ecliptic unit vectors of (lon, lat) [rad] under a 3x3 rotation."""
    torch = _torch()
    lon_dev, lat_dev = lon_dev.contiguous(), lat_dev.contiguous()
    n = lon_dev.numel()
    if lat_dev.numel() != n:
        raise ValueError("lon and lat must have the same size")
    if out is None:
        out = torch.empty((3, n), dtype=torch.float64, device=lon_dev.device)
    rot = None
    if rotation is not None:
        r = np.ascontiguousarray(np.asarray(rotation, dtype=np.float64).reshape(9))
        rot = (ctypes.c_double * 9)(*r.tolist())
    rc = _lib.load().zl_directions(
        ctypes.c_void_p(lon_dev.data_ptr()),
        ctypes.c_void_p(lat_dev.data_ptr()),
        n,
        rot,
        ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(stream if stream is not None else current_stream_handle(lon_dev.device)),
    )
    _lib.check(rc, "zl_directions")
    return out


def mapped_pointer(host_tensor) -> int | None:
    """Device address of a page-locked CPU tensor (``zl_mapped_pointer``), or None if unmapped."""
    if not host_tensor.is_pinned():
        return None
    p = ctypes.c_void_p()
    rc = _lib.load().zl_mapped_pointer(ctypes.c_void_p(host_tensor.data_ptr()), ctypes.byref(p))
    return p.value if rc == _lib.ZL_OK and p.value else None


def forward_ptr(zl_model, u_ptr: int, n: int, observers_dev, n_obs: int, precision, out_comps_ptr, out_total_ptr,
                stream: int | None = None) -> None:
    """``zl_forward`` on raw addresses (device buffers or mapped host memory).  ``observers_dev``
    is a device tensor or the integer address of the records (e.g. mapped host memory)."""
    _torch()
    obs_ptr = observers_dev if isinstance(observers_dev, int) else observers_dev.data_ptr()
    if stream is None:
        stream = current_stream_handle(None if isinstance(observers_dev, int) else observers_dev.device)
    rc = _lib.load().zl_forward(
        ctypes.byref(zl_model),
        ctypes.c_void_p(u_ptr),
        int(n),
        ctypes.c_void_p(obs_ptr),
        n_obs,
        precision_code(precision),
        ctypes.c_void_p(out_comps_ptr or 0),
        ctypes.c_void_p(out_total_ptr or 0),
        ctypes.c_void_p(stream),
    )
    _lib.check(rc, "zl_forward")
