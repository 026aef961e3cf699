"""Several wavelengths or bandpasses of one model in one launch.

ZodiPy evaluates one ``Model`` (one wavelength or bandpass) per call, so a
multi-band simulation repeats the whole line-of-sight integral per band.  The
geometry -- cutoff intersections, node positions, densities, temperatures --
does not depend on the band; only the blackbody table and the spectral scalars
do.  ``ModelSet`` packs up to ``ZL_MAX_SPEC`` models into one ``ZlModel`` and
the kernels evaluate every band at each node from the same density (the
per-band work is one table lookup and one multiply-add per component).  More
models are split into groups of ``ZL_MAX_SPEC``.

This API has no counterpart in the reference; each band's result equals that
band's ``Model.evaluate``.
"""

from __future__ import annotations

import numpy as np

from . import _lib, engine, packing


def _geometry_key(model) -> tuple:
    p = model.get_parameters()
    return (type(model._ipd_model), repr(p["comps"]), repr(p.get("T_0")), repr(p.get("delta")))


def fuse_models(models) -> _lib.ZlModel:
    """One ``ZlModel`` evaluating up to ``ZL_MAX_SPEC`` ``Model``s that share geometry in one launch.

    The models must share components, grain temperature law and quadrature
    degree; they may differ in wavelength / bandpass (each keeps its own
    blackbody table and spectral parameters).
    """
    models = list(models)
    if not 1 <= len(models) <= _lib.ZL_MAX_SPEC:
        raise ValueError(f"1..{_lib.ZL_MAX_SPEC} models can share one launch, got {len(models)}")
    first = models[0]
    key = _geometry_key(first)
    for m in models[1:]:
        if _geometry_key(m) != key:
            raise ValueError("fused models must share their components and grain temperature law")
        if m._gauss_quad_degree != first._gauss_quad_degree:
            raise ValueError("fused models must share the quadrature degree")
    return packing.pack_model(
        first._ipd_model,
        [m._spectrum for m in models],
        [m._b_nu_table for m in models],
        first._quad_points,
        first._quad_weights,
    )


class ModelSet:
    """Evaluate several ``Model``s (same components, different wavelengths/bandpasses) together.

    ``evaluate`` and ``evaluate_xyz`` take the arguments of ``Model.evaluate`` /
    ``Model.evaluate_xyz`` and return the models' results stacked on a new
    leading axis: (n_models, N) or, with ``return_comps``, (n_models, C, N).
    """

    def __init__(self, models, *, precision=None) -> None:
        from .model import Model

        models = list(models)
        if not models or not all(isinstance(m, Model) for m in models):
            raise TypeError("ModelSet takes a non-empty sequence of Model instances")
        self.models = models
        self._lead = models[0]
        self._precision = self._lead.precision if precision is None else engine.precision_code(precision)
        step = _lib.ZL_MAX_SPEC
        self._zls = [fuse_models(models[i : i + step]) for i in range(0, len(models), step)]

    def __len__(self) -> int:
        return len(self.models)

    def evaluate(self, skycoord, *, obspos="earth", return_comps: bool = False, nprocesses: int = 1):
        """Emission [MJy/sr] of every model, stacked: (n_models, N) or (n_models, C, N)."""
        lead = self._lead
        parts = [
            lead._evaluate_sky(skycoord, obspos, return_comps, zl=zl, all_spec=True, precision=self._precision)
            for zl in self._zls
        ]
        return lead._as_output_quantity(np.concatenate(parts, axis=0), skycoord)

    def evaluate_xyz(self, unit_vectors, obs_pos, earth_pos=None, *, return_comps: bool = False, precision=None):
        """``Model.evaluate_xyz`` for every model, stacked on a leading axis."""
        import torch

        prec = self._precision if precision is None else precision
        if earth_pos is None:
            earth_pos = np.asarray(obs_pos, dtype=np.float64)
        parts = [
            self._lead._evaluate(unit_vectors, obs_pos, earth_pos, return_comps, prec, zl=zl, all_spec=True)
            for zl in self._zls
        ]
        if isinstance(parts[0], torch.Tensor):
            return torch.cat(parts, dim=0)
        return np.concatenate(parts, axis=0)
