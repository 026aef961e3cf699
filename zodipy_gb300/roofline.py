"""Algorithmic work counts of the line-of-sight integral (roofline numerators).

The path is bound by transcendental throughput (the MUFU/XU pipe) and FP32
arithmetic, not by memory: a line of sight reads 24 B of unit vector and
writes 8 B per output.  The unit of work is one integrand evaluation -- one
(line of sight, component, node) -- and its cost is counted at formula level,
as the reference writes each term (a power = log2 + exp2, a division =
reciprocal + multiply, an atan2 = one transcendental plus ~10 FMA), not as any
implementation schedules it:

  term                                              XU ops   FP32 (FMA-pipe) ops
  shared per evaluation (position, |X|, T = T_0 R^-delta,
      table interpolation, weight and accumulation)    3        14
  cloud                                                 7        15
  each band                                             8        16
  ring                                                  2        10
  feature                                               3        20
  scattering, per evaluation with albedo != 0           4        10

For DIRBE (6 components) that is 6 x 3 + 7 + 3 x 8 + 2 + 3 = 54 XU and
6 x 14 + 15 + 48 + 10 + 20 = 177 FP32 operations per node, 2700 and 8850 per
line of sight at 50 nodes.  The roofline rate is the smaller of
(XU peak / XU ops) and (FMA peak / FP32 ops) per line of sight.

The Rowan-Robinson & May components follow the same rules: fan 9 XU
(power, asin, cos^Q, |beta|^eps, sin, exp), comet 7, narrow band 4, broad
band 5, interstellar 0, and the RRM ring / feature as the Kelsall ones.

``implemented_xu_ops_per_node`` counts the MUFU instructions the float32 kernel
actually issues (components share their range's position and temperature;
integer powers by squaring); it describes the implementation, not the work.
"""

from __future__ import annotations

from . import _lib

# (XU, FP32) per evaluation of each component type
_TERM = {
    _lib.ZL_CLOUD: (7, 15),
    _lib.ZL_BAND: (8, 16),
    _lib.ZL_RING: (2, 10),
    _lib.ZL_FEATURE: (3, 20),
    _lib.ZL_FAN: (9, 20),
    _lib.ZL_COMET: (7, 15),
    _lib.ZL_INTERSTELLAR: (0, 2),
    _lib.ZL_NARROW_BAND: (4, 12),
    _lib.ZL_BROAD_BAND: (5, 15),
    _lib.ZL_RING_RRM: (2, 11),
    _lib.ZL_FEATURE_RRM: (3, 21),
}
_SHARED = (3, 14)
_SCAT = (4, 10)


def _scatters(m, c) -> bool:
    return m.family == _lib.ZL_KELSALL and any(m.spec[s].albedo[c] != 0.0 for s in range(m.n_spec))


def ops_per_node(zl_model) -> tuple[int, int]:
    """(XU, FP32) operations per node for one line of sight, formula level."""
    m = zl_model
    xu = fp = 0
    for c in range(m.n_comps):
        t = _TERM[m.comp[c].type]
        xu += _SHARED[0] + t[0]
        fp += _SHARED[1] + t[1]
        if _scatters(m, c):
            xu += _SCAT[0]
            fp += _SCAT[1]
    return xu, fp


def xu_ops_per_los(zl_model) -> int:
    return ops_per_node(zl_model)[0] * zl_model.n_nodes


def fp32_ops_per_los(zl_model) -> int:
    return ops_per_node(zl_model)[1] * zl_model.n_nodes


def implemented_xu_ops_per_node(zl_model) -> int:
    """MUFU instructions the float32 kernel issues per node (DIRBE: 23)."""
    m = zl_model
    ranges = set()
    ops = 0
    scat = any(_scatters(m, c) for c in range(m.n_comps))
    for c in range(m.n_comps):
        k = m.comp[c]
        ranges.add(k.range)
        offset = any(v != 0.0 for v in k.offset)
        if k.type == _lib.ZL_CLOUD:
            ops += 3 + (2 if offset else 0)
        elif k.type == _lib.ZL_BAND:
            ops += 2 + (2 if k.p[2] != 4.0 else 0) + (2 if offset else 0)
        elif k.type == _lib.ZL_RING:
            ops += 1 + (2 if offset else 0)
        else:
            ops += 2 + (2 if offset else 0)
    ops += 3 * len(ranges)
    if scat:
        ops += (1 + m.n_spec) * len(ranges)
    return ops


def evaluations_per_los(zl_model) -> int:
    """Integrand evaluations (component x node) per line of sight."""
    return zl_model.n_comps * zl_model.n_nodes


def io_bytes_per_los(zl_model, comps: bool, total: bool) -> int:
    """Algorithmic HBM bytes per line of sight: float64 unit vector in, float64 outputs."""
    return 24 + 8 * zl_model.n_spec * ((zl_model.n_comps if comps else 0) + (1 if total else 0))
