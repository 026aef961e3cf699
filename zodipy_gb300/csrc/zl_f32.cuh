// Float32-path helpers shared by the forward and adjoint kernels.
#pragma once

#include "zl_common.cuh"

namespace zl {

// Compile-time component layouts.  Nibble c: bit0 present, bit1 first component
// of a new LOS range, bits 2-3 component type.  LAYOUT 0 = generic (runtime).
constexpr uint32_t kLayoutDirbe = 0xFB5553u;   // cloud | band band band (same range) | ring | feature
constexpr uint32_t kLayoutPlanck = 0x5553u;    // cloud | band band band
constexpr uint32_t kLayoutGeneric = 0u;

template <uint32_t LAYOUT>
struct Lay {
  static constexpr bool generic = (LAYOUT == 0u);
  static constexpr bool rrm = false;  // grain temperature per component (ZL_RRM), not shared
  __host__ __device__ static constexpr int ncomp() {
    if (generic) return ZL_MAX_COMPS;
    int n = 0;
    for (int c = 0; c < ZL_MAX_COMPS; ++c)
      if ((LAYOUT >> (4 * c)) & 1u) n = c + 1;
    return n;
  }
  __host__ __device__ static constexpr int type(int c) { return (int)((LAYOUT >> (4 * c + 2)) & 3u); }
  __host__ __device__ static constexpr bool first(int c) { return ((LAYOUT >> (4 * c + 1)) & 1u) != 0; }
  // LOS-range index of component c: ranges are numbered in order of first use
  __host__ __device__ static constexpr int range(int c) {
    int r = -1;
    for (int j = 0; j <= c; ++j)
      if (first(j)) ++r;
    return r;
  }
  // first band of component c's range (c itself if none precedes it)
  __host__ __device__ static constexpr int first_band(int c) {
    for (int j = 0; j < c; ++j)
      if (range(j) == range(c) && type(j) == ZL_BAND) return j;
    return c;
  }
};

// The registry's RRM model (zodipy/model_registry.py:64-73, rrm-experimental): fan | comet |
// narrow band, narrow band, broad band (one LOS range) | interstellar | ring | feature.  Its
// component types and LOS ranges are compiled in; every parameter (offsets, scattering) is read
// at run time (kFlagsRuntime), and each component has its own grain temperature law.
constexpr uint32_t kLayoutRRM = 0x80000000u;

template <>
struct Lay<kLayoutRRM> {
  static constexpr bool generic = false;
  static constexpr bool rrm = true;
  __host__ __device__ static constexpr int ncomp() { return 8; }
  __host__ __device__ static constexpr int type(int c) {
    return c == 0 ? ZL_FAN : c == 1 ? ZL_COMET : c <= 3 ? ZL_NARROW_BAND : c == 4 ? ZL_BROAD_BAND
         : c == 5 ? ZL_INTERSTELLAR : c == 6 ? ZL_RING_RRM : ZL_FEATURE_RRM;
  }
  __host__ __device__ static constexpr int range(int c) { return c <= 1 ? c : c <= 4 ? 2 : c - 2; }
  __host__ __device__ static constexpr bool first(int c) { return c == 0 || range(c) != range(c - 1); }
  __host__ __device__ static constexpr int first_band(int c) { return c; }
};

// Compile-time properties of a model for the built-in layouts (FLAGS); bit 0 set = read them
// from the parameter block at run time instead (any model, the generic layout):
//   bit 1        some component scatters sunlight (albedo != 0)
//   bit 8 + c    component c is offset from the Sun
//   bit 16 + c   band c has p == 4 (its (zeta/dzeta)^p is a square of a square)
//   bit 24 + c   band c reuses the first band's 1 - e^-(R/delta_r)^20 (equal delta_r and offset)
constexpr uint32_t kFlagsRuntime = 1u;

template <uint32_t F>
struct KFlags {
  static constexpr bool runtime = (F & 1u) != 0;
  __device__ static __forceinline__ bool scat(const KParamsF32& P) {
    return runtime ? P.has_scat != 0 : ((F >> 1) & 1u) != 0;
  }
  __device__ static __forceinline__ bool offset(const KCompF32& C, int c) {
    return runtime ? C.zero_offset == 0 : ((F >> (8 + c)) & 1u) != 0;
  }
  __device__ static __forceinline__ bool p4(const KCompF32& C, int c) {
    return runtime ? C.c[5] != 0.f : ((F >> (16 + c)) & 1u) != 0;
  }
  __device__ static __forceinline__ bool share_first(int c) { return ((F >> (24 + c)) & 1u) != 0; }
};

// The flag set of the built-in Kelsall models (cloud offset, bands with p = 4, band 3 reusing
// band 1's inner-cutoff term) for the DIRBE and Planck layouts.
constexpr uint32_t kFlagsKelsall = (1u << 8) | (7u << 17) | (1u << 27);

// Flag set of a model for a layout (1 = DIRBE, 2 = Planck), or kFlagsRuntime (zl_fwd_f32.cu).
uint32_t f32_flags(const KParamsF32& P, int layout);

// Root of |obs + s u| = cutoff (line_of_sight.py:80-85) in float-float; b omits
// z_obs u_z like the reference.  At b == 0 the root is taken with sign(+0).
// c = |X_obs|^2 - cutoff^2 is formed exactly (it cancels for an observer near the sphere;
// sphere_distance_ff below, or once per observer); the other sums need accuracy relative to
// their operands only (ff_add_fast).
// SHORT: ff_sqrt and ff_div (three-addition residuals), else ff_sqrt_sum and ff_div_ieee.
template <bool SHORT = true>
__device__ __forceinline__ ff sphere_distance_ffc(ff b, ff c) {
  const ff D = ff_add_fast(ff_mul(b, b), ff_scale(c, -4.0f));
  const ff sq = SHORT ? ff_sqrt(D) : ff_sqrt_sum(D);
  const ff q = ff_scale(ff_add_fast(b, (b.hi < 0.f || (b.hi == 0.f && signbit(b.hi))) ? ff_neg(sq) : sq), -0.5f);
  const ff cq = SHORT ? ff_div(c, q) : ff_div_ieee(c, q);
  if (isnan(q.hi) || isnan(cq.hi)) return {q.hi + cq.hi, 0.f};
  return (q.hi > cq.hi || (q.hi == cq.hi && q.lo >= cq.lo)) ? q : cq;
}

template <bool SHORT = true>
__device__ __forceinline__ ff sphere_distance_ff(ff b, ff r2, ff cut2) {
  return sphere_distance_ffc<SHORT>(b, ff_add(r2, ff_neg(cut2)));
}

__device__ __forceinline__ float bb_lookup(const float4* __restrict__ tab, float T, float t_min, float t_max,
                                           float inv_dt, int nT) {
  const float Tc = fminf(fmaxf(T, t_min), t_max);
  int j = __float2int_rd(fmaf(Tc, inv_dt, -t_min * inv_dt));  // segment index; the offset is loop-invariant
  j = min(j, nT - 2);
  const float4 e = tab[j];  // (T_j, B_j, slope_j, -)
  return fmaf(e.z, Tc - e.x, e.y);
}

// Table value and its derivative dB/dT: the slope of the segment holding T, and
// 0 where numpy.interp clamps (T outside the table).
__device__ __forceinline__ float2 bb_lookup_d(const float4* __restrict__ tab, float T, float t_min, float t_max,
                                              float inv_dt, int nT) {
  const float Tc = fminf(fmaxf(T, t_min), t_max);
  int j = __float2int_rd((Tc - t_min) * inv_dt);
  j = min(j, nT - 2);
  const float4 e = tab[j];
  const float slope = (T > t_min && T < t_max) ? e.z : 0.f;
  return make_float2(fmaf(e.z, Tc - e.x, e.y), slope);
}

// Quadrature nodes summed in plain float32 before each compensated addition: the
// relative error of a block sum stays below (kSumBlock - 1) 2^-24 (positive terms).
constexpr int kSumBlock = 8;

__device__ __forceinline__ void kahan_add(float& s, float& c, float t) {
  const float y = t - c;
  const float s1 = s + y;
  c = (s1 - s) - y;
  s = s1;
}

// float32 value of a * x + b from float-float parts, within ~1 ulp of the result
// even when the two terms cancel: the FMA forms a.hi x.hi + b.hi exactly before
// its single rounding, and the low-part terms are first-order corrections.
__device__ __forceinline__ float lin_ff(ff a, ff x, ff b) {
  const float r = fmaf(a.hi, x.hi, b.hi);
  return r + fmaf(a.hi, x.lo, fmaf(a.lo, x.hi, b.lo));
}

__device__ __forceinline__ float node_position(ff hs, ff x, ff mid) { return lin_ff(hs, x, mid); }

// a * x + b as an unevaluated float-float sum (exact TwoProd of the high parts,
// TwoSum with b.hi, low-part terms added once)
__device__ __forceinline__ ff lin_ff2(ff a, ff x, ff b) {
  const float p = a.hi * x.hi;
  const float pe = fmaf(a.hi, x.hi, -p);
  const ff s = ff_two_sum(p, b.hi);
  return ff_quick(s.hi, s.lo + (pe + fmaf(a.hi, x.lo, fmaf(a.lo, x.hi, b.lo))));
}

// w^2 + c to ~1 ulp of the result: the FMA squares w.hi exactly
__device__ __forceinline__ float sq_plus_ff(ff w, ff c) {
  return fmaf(w.hi, w.hi, c.hi) + fmaf(2.f * w.hi, w.lo, c.lo);
}

// w^2 + c as a float-float (exact square of w.hi, first-order low parts)
__device__ __forceinline__ ff sq_plus_ff2(ff w, ff c) {
  const float p = w.hi * w.hi;
  const float pe = fmaf(w.hi, w.hi, -p);
  const ff s = ff_two_sum(p, c.hi);
  return ff_quick(s.hi, s.lo + (pe + fmaf(2.f * w.hi, w.lo, c.lo)));
}

// a < b for normalised float-float values
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// Where a band stops contributing (Kelsall bands, number_density.py:99-110).  A band's
// factor e^-(zeta/dzeta)^6 is evaluated as ex2(-log2(e) (zeta/dzeta)^6), and
// ex2.approx.ftz returns +0 once its result 2^x falls
// below the smallest normal float (x < -126, i.e. zeta > 2.11 dzeta): from there on the
// node adds exactly nothing.  Along a line of sight, zeta = |Z|/R with Z = a1 x + a0 and
// R^2 = (h x + m)^2 + b^2 in the node abscissa x, so zeta > c for
//   (a1 x + a0)^2 - c^2 ((h x + m)^2 + b^2) > 0,
// a quadratic whose leading coefficient a1^2 - c^2 h^2 is positive when the direction
// itself leaves the band (|u . n| > c).  Then every node beyond the larger root is zero.
// Returns that root for c = 2.2 dzeta (4 % inside the flush threshold, which absorbs the
// float32 rounding of this estimate, its approximate divisions and square root, and the node
// loop's zeta), -inf when the whole line of sight is beyond it, +inf when no tail is
// guaranteed (and for NaN input).  Called by every lane of the warp together: unless every
// pixel's direction leaves the band (A > 0), the warp has no common tail and all lanes return
// +inf at once (random directions almost never pass this, and skip the rest).
__device__ __forceinline__ float band_zero_tail(float a1, float a0, float h, float m, float b2h, float inv_dzeta) {
  const float c = __fdividef(2.2f, inv_dzeta);
  const float c2 = c * c;
  const float A = a1 * a1 - c2 * (h * h);
  if (!__all_sync(__activemask(), A > 0.f)) return INFINITY;
  const float B = 2.f * (a1 * a0 - c2 * (h * m));
  const float C = a0 * a0 - c2 * (m * m + b2h);
  const float disc = B * B - 4.f * A * C;
  if (disc < 0.f) return -INFINITY;
  const float q = -0.5f * (B + copysignf(disc * rsqrt_ftz(fmaxf(disc, 1e-30f)), B));
  const float r = fmaxf(__fdividef(q, A), __fdividef(C, q));  // the two roots (q != 0 unless B = disc = 0)
  return isnan(r) ? INFINITY : r;
}

// Number of quadrature nodes at or below abscissa xs, for an xs the whole warp shares:
// the warp's maximum of its pixels' tail starts, so that every lane's tail covers the
// nodes from the returned index on.
__device__ __forceinline__ int warp_tail_index(const KParamsF32& P, float xs) {
  // order-preserving map of floats to unsigned integers, so the warp maximum is an integer one
  const uint32_t bits = __float_as_uint(xs);
  const uint32_t key = (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
  const uint32_t kmax = __reduce_max_sync(__activemask(), key);
  const float xw = __uint_as_float((kmax & 0x80000000u) ? (kmax & 0x7fffffffu) : ~kmax);
  if (!(xw < INFINITY)) return P.n_nodes;  // no tail (warp-uniform)
  int lo = 0, hi = P.n_nodes;  // nodes ascend in x
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (P.gl_x_hi[mid] <= xw) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Abscissa interval of the nodes at which a band's inner-cutoff factor 1 - e^-y, y = (R/delta_r)^20
// (number_density.py:109), may differ from 1.0f: R < 1.26 delta_r.  Beyond it y > 101, e^-y
// (ex2.approx.ftz of -y log2(e) < -126) is zero and 1 - e^-y is exactly 1.0f, as is the adjoint's
// y e^-y / (1 - e^-y); 1 - e^-y rounds to 1.0f from R = 1.162 delta_r on, so the bound leaves 8 %
// of R for the float32 rounding of this estimate.  R^2 = (h x + w)^2 + b2 along the line of sight
// (h, w, b2: the pixel's set-up); returns (x1, x2), x1 > x2 when no point is that close.
__device__ __forceinline__ float2 cutoff_interval(float h, float w, float b2, float inv_dr2) {
  const float D = __fdividef(1.5876f, inv_dr2) - b2;  // (1.26 delta_r)^2 - b^2
  if (!(D > 0.f)) return make_float2(INFINITY, -INFINITY);
  const float sq = sqrtf(D);
  if (!(h > 0.f)) return fabsf(w) < sq ? make_float2(-INFINITY, INFINITY) : make_float2(INFINITY, -INFINITY);
  const float ih = __fdividef(1.f, h);
  return make_float2((-w - sq) * ih, (sq - w) * ih);
}

// Order-preserving map of floats to unsigned integers (warp minima and maxima as integer ones).
__device__ __forceinline__ uint32_t float_key(float x) {
  const uint32_t b = __float_as_uint(x);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Node indices [lo, hi) covering the abscissa interval (x1, x2) of every active lane of the warp
// (lo == hi: none).  Warp-uniform.
__device__ __forceinline__ int2 warp_node_range(const KParamsF32& P, float x1, float x2) {
  const uint32_t m = __activemask();
  const float x1w = key_float(__reduce_min_sync(m, float_key(x1)));
  const float x2w = key_float(__reduce_max_sync(m, float_key(x2)));
  if (!(x1w <= x2w)) return make_int2(0, 0);
  int lo = 0, hi = P.n_nodes;  // first node at or above x1w (nodes ascend in x)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (P.gl_x_hi[mid] < x1w) lo = mid + 1;
    else hi = mid;
  }
  const int first = lo;
  hi = P.n_nodes;  // first node above x2w
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (P.gl_x_hi[mid] <= x2w) lo = mid + 1;
    else hi = mid;
  }
  return make_int2(first, lo);
}

// Fan, comet, narrow and broad band of the RRM model (number_density.py:184-342) in float32,
// without the amplitude C.c[0] (the caller applies it).
// The radial mask R_inner <= |X - X_0| <= R_outer and the narrow band's cut |beta| < beta_nb are
// decided on float-float squares (|X - X_0|^2 = w^2 + b^2, Z^2 < sin^2(beta_nb) R^2), so float32
// rounding cannot move a node across them; the values inside are plain float32.
// (hs, x, wm, b2): the distance terms of the node; (z1, z0): Z = z1 x + z0; Z, rinv, lg2R: float32
// height above the symmetry plane, 1/R and log2 R of the same node.
__device__ __forceinline__ float rrm_masked_density(const KCompF32& C, int type, ff hs, ff x, ff wm, ff b2, ff z1,
                                                    ff z0, float Z, float rinv, float lg2R) {
  const ff R2 = sq_plus_ff2(lin_ff2(hs, x, wm), b2);
  if (ff_lt(R2, ff{C.c[8], C.c[9]}) || ff_lt(ff{C.c[10], C.c[11]}, R2)) return 0.f;
  const float s = fminf(fmaxf(Z * rinv, -1.f), 1.f);  // sin(beta)
  const float beta = asinf(s);
  if (type == ZL_FAN || type == ZL_COMET) {
    const float za = fabsf(Z) * C.c[4];  // |Z| / Z_0
    const float eps = za < 1.f ? 2.f - za : 1.f;
    float f = ex2_ftz(C.c[3] * sinf(ex2_ftz(eps * lg2_ftz(fabsf(beta)))));  // exp(-P sin(|beta|^eps))
    if (type == ZL_FAN && C.c[2] != 0.f) f *= ex2_ftz(C.c[2] * lg2_ftz(fmaxf(1.f - s * s, 0.f)));  // cos^Q
    return ex2_ftz(C.c[1] * lg2R) * f;
  }
  const float bdeg = beta * 57.29577951308232f;
  const float radial = ex2_ftz(fmaf(C.c[1], lg2R, C.c[5]));  // (R / R_outer)^-gamma
  if (type == ZL_NARROW_BAND) {
    const ff Zf = lin_ff2(z1, x, z0);
    if (!ff_lt(ff_mul(Zf, Zf), ff_mul(ff{C.c[6], C.c[7]}, R2))) return 0.f;
    return radial * ex2_ftz(C.c[2] * (fabsf(bdeg) - C.c[3]));
  }
  const float a = (bdeg - C.c[2]) * C.c[3], b = (bdeg + C.c[2]) * C.c[3];
  return radial * (ex2_ftz(-0.5f * kLog2e * (a * a)) + ex2_ftz(-0.5f * kLog2e * (b * b)));
}

}  // namespace zl
