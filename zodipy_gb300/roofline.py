"""Algorithmic work counts of the line-of-sight integral (roofline numerators).

The path is bound by transcendental throughput (the MUFU/XU pipe) and FP32
arithmetic, not by memory: a line of sight reads 24 B of unit vector and
writes 8 B per output.  The unit of work is one integrand evaluation — one
(pixel, component, node) — and the numerator of the XU roofline is the number
of MUFU operations the Kelsall formulas need per node, counted with the
cheapest exact formulation of each term:

  per LOS range (position shared by its components):
      1/sqrt(R^2), log2 R, 2^(-delta log2 R) for T(R)           3
      scattering (albedo != 0): atan2 -> 1 reciprocal, e^(C3 Theta)  2
  cloud       log2 g, 2^(gamma log2 g), 2^(density exponent)   3
              (+ 1/sqrt, log2 for its own distance when offset) +2
  band        e^(-zeta^6), e^(-(R/dr)^20); zeta^4 and (R/dr)^20 by squaring  2
              (+ 2 for a non-integer p, + 2 when offset)
  ring        e^(density exponent)                              1
  feature     atan2 -> 1 reciprocal, e^(density exponent)      2

For DIRBE (3 ranges; cloud offset; 3 bands with p = 4; ring; feature) this is
9 + 5 + 6 + 1 + 2 = 23 per node, 1150 per line of sight at 50 nodes.
"""

from __future__ import annotations

from . import _lib


def xu_ops_per_node(zl_model) -> int:
    m = zl_model
    ranges = set()
    ops = 0
    scat = any(m.spec[s].albedo[c] != 0.0 for s in range(m.n_spec) for c in range(m.n_comps))
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


def xu_ops_per_los(zl_model) -> int:
    return xu_ops_per_node(zl_model) * zl_model.n_nodes


def evaluations_per_los(zl_model) -> int:
    """Integrand evaluations (component x node) per line of sight."""
    return zl_model.n_comps * zl_model.n_nodes


def io_bytes_per_los(zl_model, comps: bool, total: bool) -> int:
    """Algorithmic HBM bytes per line of sight: float64 unit vector in, float64 outputs."""
    return 24 + 8 * zl_model.n_spec * ((zl_model.n_comps if comps else 0) + (1 if total else 0))
