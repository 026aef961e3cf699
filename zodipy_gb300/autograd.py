"""Differentiable evaluation: ``torch.autograd`` over the model parameter vector.

``ZodiAdjoint(model)`` binds a model (or several fused spectral sets) to a set
of lines of sight; calling it with a parameter vector ``theta`` (the layout of
``zodipy_gb300.params``) returns the float32-kernel maps as a tensor that
autograd can differentiate.  The backward pass is libzodigb's adjoint kernel:
it recomputes the integrand per node and reduces over pixels in a fixed
order, so gradients are deterministic.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib, engine, packing, params
from .fused import fuse_models  # noqa: F401  (one ZlModel for several spectral sets)


class _Emission(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, state, return_comps):
        zl = params.model_from_vector(state.base, theta.detach().to("cpu", torch.float64).numpy())
        comps, total = engine.forward(
            zl, state.u, state.obs_dev, state.n_obs, _lib.ZL_PREC_F32, want_comps=return_comps, want_total=not return_comps
        )
        ctx.zl = zl
        ctx.state = state
        ctx.return_comps = return_comps
        ctx.theta_device = theta.device
        return comps if return_comps else total

    @staticmethod
    def backward(ctx, grad_out):
        st = ctx.state
        g = grad_out.to(torch.float64)
        if ctx.return_comps:
            grad = engine.backward(ctx.zl, st.u, st.obs_dev, st.n_obs, g_comps=g, workspace=st.workspace())
        else:
            grad = engine.backward(ctx.zl, st.u, st.obs_dev, st.n_obs, g_total=g, workspace=st.workspace())
        return grad.to(ctx.theta_device), None, None


class ZodiAdjoint:
    """A model bound to lines of sight, differentiable in its parameter vector.

    ``zl_model``: a packed ``ZlModel`` (``Model.zl_model`` or ``fuse_models``).
    ``unit_vectors``: (3, N) float64 (numpy or CUDA tensor); ``obs_pos`` /
    ``earth_pos``: (3,) for one observer, or (3, n_obs) with ``counts``
    (pixels per observer, summing to N) for several.
    """

    def __init__(self, zl_model, unit_vectors, obs_pos, earth_pos, counts=None, labels=None):
        self.base = _lib.ZlModel.from_buffer_copy(zl_model)
        u = unit_vectors if isinstance(unit_vectors, torch.Tensor) else torch.from_numpy(np.asarray(unit_vectors, dtype=np.float64))
        self.u = u.to("cuda", torch.float64).contiguous()
        n = self.u.shape[1]
        obs = np.asarray(obs_pos, dtype=np.float64).reshape(3, -1)
        earth = np.asarray(earth_pos, dtype=np.float64).reshape(3, -1)
        if counts is None:
            if obs.shape[1] != 1:
                raise ValueError("several observers need `counts`")
            begin = np.zeros(1, dtype=np.int64)
        else:
            counts = np.asarray(counts, dtype=np.int64)
            if counts.sum() != n or counts.size != obs.shape[1]:
                raise ValueError("counts must give one pixel count per observer, summing to N")
            begin = np.concatenate([[0], np.cumsum(counts)[:-1]])
        table = packing.observer_table(self.base, obs, earth if earth.shape[1] in (1, obs.shape[1]) else earth, begin, any_mode=False)
        self.obs_dev = engine.upload_observers(table, self.u.device)
        self.n_obs = obs.shape[1]
        self._ws = None
        self.labels = labels or [f"c{c}" for c in range(self.base.n_comps)]

    def workspace(self):
        need = engine.backward_workspace_bytes(self.base, self.u.shape[1])
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(max(need, 8), dtype=torch.uint8, device=self.u.device)
        return self._ws

    def theta0(self, device="cuda") -> torch.Tensor:
        return torch.tensor(params.vector_from_model(self.base), dtype=torch.float64, device=device)

    def names(self) -> list[str]:
        return params.names(self.base, self.labels)

    def __call__(self, theta: torch.Tensor, return_comps: bool = False) -> torch.Tensor:
        return _Emission.apply(theta, self, return_comps)


