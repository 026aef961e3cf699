// Device-side building blocks shared by the forward and adjoint kernels.
//
// The kernels evaluate ZodiPy's line-of-sight integral (zodipy/model.py:253-277):
// for every pixel and component, a Gauss-Legendre sum over the Kelsall integrand
// (zodipy/brightness.py:21-56) between the cutoff-sphere intersections
// (zodipy/line_of_sight.py:64-105).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/zodigb.h"

namespace zl {

constexpr double kEps = 2.220446049250313e-16;  // np.finfo(float64).eps (line_of_sight.py:14)
constexpr double kPi = 3.141592653589793;
constexpr float kLog2e = 1.4426950408889634f;
constexpr float kPiF = 3.14159265358979f;
constexpr float kTwoPiF = 6.28318530717959f;
constexpr float kInvTwoPiF = 0.159154943091895f;

// ---------------------------------------------------------------------------
// Host-derived kernel parameter blocks.  They are built once per launch from a
// ZlModel by the host code in zl_api.cu and passed by value (__grid_constant__),
// so concurrent launches with different models never share state.
// ---------------------------------------------------------------------------

// float64 plain kernel: the model itself plus slopes of the blackbody table.
struct KParamsF64 {
  ZlModel m;
  double slope[ZL_MAX_SPEC][ZL_MAX_TEMPS];  // (fp[j+1]-fp[j])/(xp[j+1]-xp[j]) as np.interp forms it
  double phase_norm[ZL_MAX_SPEC];           // scattering.py:53-59
  int32_t first_in_range[ZL_MAX_COMPS];     // component starts a new LOS range group
  int32_t range_scat[ZL_MAX_RANGES];        // some component of the range has albedo != 0
  double range_T0[ZL_MAX_RANGES], range_delta[ZL_MAX_RANGES];  // T = T_0 R^-delta of the range's components
};

// Component-type predicates shared by the kernels.
__host__ __device__ constexpr bool ringlike(int t) {
  return t == ZL_RING || t == ZL_FEATURE || t == ZL_RING_RRM || t == ZL_FEATURE_RRM;
}
__host__ __device__ constexpr bool featurelike(int t) { return t == ZL_FEATURE || t == ZL_FEATURE_RRM; }
// RRM densities that are zero outside [R_inner, R_outer] (number_density.py:184-342)
__host__ __device__ constexpr bool masked(int t) {
  return t == ZL_FAN || t == ZL_COMET || t == ZL_NARROW_BAND || t == ZL_BROAD_BAND;
}

// Per-component constants of the float32 kernel.
struct KCompF32 {
  int32_t type, range, first_in_range, zero_offset;
  int32_t share_t4;  // band: index of an earlier band with the same delta_r (reuse its 1 - e^-y), else -1
  int32_t same_plane_prev;  // 1: same symmetry plane and centre as component c - 1
  float T0, neg_delta;     // T = T_0 R^-delta of this component's range (generic layout)
  float nx, ny, nz;        // unit normal of the symmetry plane (sinO sini, -cosO sini, cosi)
  float nx_lo, ny_lo, nz_lo;  // low parts of the normal for float-float heights
  float ox, oy, oz;        // offset X_0 [AU]
  float ox_lo, oy_lo, oz_lo;  // low parts of X_0 for float-float geometry
  // type constants:
  //  cloud:   c0=n_0, c1=alpha, c2=beta*log2(e), c3=gamma, c4=mu, c5=1/(2 mu), c6=mu/2, c7=-alpha/2
  //  band:    c0=3 n_0, c1=1/delta_zeta_rad, c2=1/v, c3=p, c4=1/delta_r^2, c5=(p==4)
  //  ring:    c0=n_0, c1=R, c2=log2(e)/sigma_r^2, c3=log2(e)/sigma_z, c4=R^2 (hi), c5=R^2 (lo)
  //  feature: c0=n_0, c1=R, c2=log2(e)/sigma_r^2, c3=log2(e)/sigma_z, c4=R^2 (hi), c5=R^2 (lo),
  //           c6=theta_rad, c7=log2(e)/sigma_theta_rad^2
  //  RRM ring / feature: as ring / feature with c0 = A n_0
  //  fan:     c1=-gamma, c2=Q/2, c3=-P log2(e), c4=1/Z_0
  //  comet:   c0=amp, c1=-gamma, c3=-P log2(e), c4=1/Z_0
  //  interstellar: c0=amp
  //  narrow band: c0=A, c1=-gamma, c2=G log2(e), c3=beta_nb [deg], c5=gamma log2(R_outer),
  //           c6,c7=sin^2(beta_nb) (hi, lo)
  //  broad band:  c0=A, c1=-gamma, c2=beta_bb [deg], c3=1/sigma_bb, c5=gamma log2(R_outer)
  //  masked RRM types: c8,c9 = R_inner^2 (hi, lo), c10,c11 = R_outer^2 (hi, lo)
  float c[12];
};

struct KSpecF32 {
  float em1[ZL_MAX_COMPS];  // (1 - albedo) * emissivity
  // forward: the component's density prefactor times em1 (times the albedo): the node loop sums
  // the prefactor-free density and these constants scale each block sum once
  float outer[ZL_MAX_COMPS], outer_alb[ZL_MAX_COMPS];
  float alb[ZL_MAX_COMPS];  // albedo
  float C1, C2, C3l2e, S, N;  // phase function (C3 pre-multiplied by log2 e), solar flux, normalisation
  float pad[3];
};

struct KParamsF32 {
  int32_t n_comps, n_ranges, n_spec, n_nodes, n_temps, has_scat;
  float T0, neg_delta, t_min, t_max, inv_dt, neg_half_delta;  // neg_half_delta = -delta / 2 (T from lg2 R^2)
  double cut_in[ZL_MAX_RANGES], cut_out[ZL_MAX_RANGES];
  float cut_in_hi[ZL_MAX_RANGES], cut_in_lo[ZL_MAX_RANGES];
  float cut_out_hi[ZL_MAX_RANGES], cut_out_lo[ZL_MAX_RANGES];
  float gl_x_hi[ZL_MAX_NODES], gl_x_lo[ZL_MAX_NODES], gl_w[ZL_MAX_NODES];
  KCompF32 comp[ZL_MAX_COMPS];
  KSpecF32 spec[ZL_MAX_SPEC];
  float4 table[ZL_MAX_SPEC][ZL_MAX_TEMPS];  // (T_j, B_j, slope_j, 0), staged to shared memory
};

// Host-derived constants for the derivatives.
struct KGradAux {
  float dni[ZL_MAX_COMPS][3];  // d n_hat / d i   [per degree]
  float dnO[ZL_MAX_COMPS][2];  // d n_hat / d Omega [per degree] (z component is 0)
  float q[ZL_MAX_COMPS][8];    // type constants in natural units (see zl_api.cu)
  float n0[ZL_MAX_COMPS];      // density prefactor: n_0, or 3 n_0 for a band (densities are evaluated without it)
  float eps[ZL_MAX_SPEC][ZL_MAX_COMPS], one_m_alb[ZL_MAX_SPEC][ZL_MAX_COMPS];  // per spectral set
  float dN[ZL_MAX_SPEC][3];    // d N / d C1, C2, C3 of the phase normalisation, per spectral set
};

// ---------------------------------------------------------------------------
// Float-float ("double-single") arithmetic on the FP32 pipe.  GB300 runs FP64
// at a small fraction of its FP32 rate, so the few quantities that need more
// than 24 bits (cutoff intersections, node positions near the ring and the
// feature) carry a (hi, lo) pair with ~48-bit significand instead.
// Algorithms: Dekker (1971) / Knuth TwoSum, FMA-based TwoProd.
// ---------------------------------------------------------------------------
struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

__device__ __forceinline__ ff ff_quick(float a, float b) {  // |a| >= |b|
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = ff_two_sum(a.hi, b.hi);
  ff t = ff_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = ff_quick(s.hi, s.lo);
  s.lo += t.lo;
  return ff_quick(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return ff_quick(p, e);
}

__device__ __forceinline__ ff ff_mulf(ff a, float b) {
  float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return ff_quick(p, e);
}

// Faster sum: exact TwoSum of the high parts, low parts added once.  Its error is
// a few units of 2^-48 of the larger operand even under cancellation, which is
// what the callers need (an absolute accuracy, not a relative one).
__device__ __forceinline__ ff ff_add_fast(ff a, ff b) {
  ff s = ff_two_sum(a.hi, b.hi);
  return ff_quick(s.hi, s.lo + (a.lo + b.lo));
}

// a * b + c, all float-float
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

__device__ __forceinline__ ff ff_scale(ff a, float pow2) { return {a.hi * pow2, a.lo * pow2}; }

// A double as a float-float pair, without float64 instructions.  GB300 runs float64
// (conversions included) at a small fraction of its float32 rate, and each pixel's set-up
// splits nine doubles, so this works on the bits: the top 24 significand bits (truncated) and
// the next 23 (made a float by setting them as the significand of 2^(E-23) and subtracting
// 2^(E-23) exactly), renormalised so that hi is the rounded float value of d (as (float)d
// gives it); |hi + lo - d| < 2^-45 |d|.  The 6 significand bits below those 47 are not kept, but they
// stick to the lowest kept bit (set it when any of them is set), so that a value just above a
// halfway point between two floats still rounds up when the pair is renormalised, as
// round-to-nearest of the double does; an exact halfway point rounds to even in both.
// |d| < 2^-70 (zero, subnormals) gives (+-0, 0), an absolute error below 2^-70; doubles
// beyond the float range, inf and NaN take the conversion.
__device__ __forceinline__ ff ff_split(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned int hw = (unsigned int)(b >> 32), lw = (unsigned int)b;
  const int e = (int)((hw >> 20) & 0x7ffu);  // biased exponent: |d| in [2^(e-1023), 2^(e-1022))
  const unsigned int sign = hw & 0x80000000u;
  if (e < 1023 - 70) return {__uint_as_float(sign), 0.f};
  if (e > 1023 + 127) return {__double2float_rn(d), 0.f};
  const float hi = __uint_as_float(sign | ((unsigned int)(e - 1023 + 127) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29));
  const unsigned int base = sign | ((unsigned int)(e - 1023 - 23 + 127) << 23);  // +-2^(e-1023-23)
  const unsigned int low23 = ((lw & 0x1fffffffu) >> 6) | ((lw & 0x3fu) != 0u ? 1u : 0u);  // sticky
  const float lo = __uint_as_float(base | low23) - __uint_as_float(base);
  return ff_quick(hi, lo);
}

// (float)d from the bit split (no float64 instruction) where |d| is in [2^-70, 2^128); outside
// that range (zero, tiny or huge values, inf, NaN) the conversion instruction, so that no
// value is flushed: d here is an upstream gradient, whose scale is the caller's.
__device__ __forceinline__ float d2f_bits(double d) {
  const int e = (__double2hiint(d) >> 20) & 0x7ff;
  if (e < 1023 - 70 || e > 1023 + 127) return __double2float_rn(d);
  return ff_split(d).hi;  // the rounded value: ff_split renormalises its pair
}

// (double)f by bit operations, without a float64 instruction (GB300's FP64 pipe takes a
// warp's conversion over tens of cycles, and every pixel converts each of its results): the
// sign, the exponent re-biased from 127 to 1023 and the significand shifted into place; every
// float is a double, so the value is the same.  Zero keeps its sign; subnormal floats, inf and
// NaN take the conversion instruction.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int e = (b >> 23) & 0xffu;
  if ((b & 0x7fffffffu) != 0u && e - 1u >= 254u) return (double)f;
  const unsigned int hi = (b & 0x7fffffffu) ? (b & 0x80000000u) | ((e + (1023u - 127u)) << 20) | ((b & 0x7fffffu) >> 3)
                                            : (b & 0x80000000u);
  return __hiloint2double((int)hi, (int)(b << 29));
}

// ff_mul without the final renormalisation: (p, e) with |e| <= ulp(p); the fast sums below
// accept it as an operand
__device__ __forceinline__ ff ff_mul_nr(ff a, ff b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return {p, e};
}

// sqrt of a positive float-float (one Newton correction of the FP32 root), the residual
// a - s^2 as a float-float sum; ff_div_ieee: a / b from IEEE divisions.  Kept for the Planck
// layout's kernels, where the shorter forms below measured slower (different schedules).
__device__ __forceinline__ ff ff_sqrt_sum(ff a) {
  if (!(a.hi > 0.f)) return {sqrtf(a.hi), 0.f};
  float r = rsqrtf(a.hi);
  float s = a.hi * r;
  ff s2 = {s * s, fmaf(s, s, -s * s)};
  ff d = ff_add(a, ff_neg(s2));
  return ff_quick(s, d.hi * 0.5f * r);
}

__device__ __forceinline__ ff ff_div_ieee(ff a, ff b) {
  float q = a.hi / b.hi;
  ff p = ff_mulf(b, q);
  ff r = ff_add(a, ff_neg(p));
  return ff_quick(q, r.hi / b.hi);
}

// sqrt of a positive float-float (one Newton correction of the FP32 root).  The root s is
// within a few ulps of sqrt(a.hi), so s^2 = p + pe (exact, by an FMA) lies within a factor 2 of
// a.hi and a.hi - p is exact (Sterbenz): the residual a - s^2 takes three additions.
__device__ __forceinline__ ff ff_sqrt(ff a) {
  if (!(a.hi > 0.f)) return {sqrtf(a.hi), 0.f};
  const float r = rsqrtf(a.hi);
  const float s = a.hi * r;
  const float p = s * s, pe = fmaf(s, s, -p);
  const float d = ((a.hi - p) - pe) + a.lo;
  return ff_quick(s, d * 0.5f * r);
}

// a / b (one Newton correction).  q = a.hi / b.hi to a few ulps (reciprocal approximation), so
// b.hi q = p + pe (exact, by an FMA) lies within a factor 2 of a.hi and a.hi - p is exact
// (Sterbenz): the residual a - b q takes three additions and the low part's product.  Relative
// error below 2^-42 (the reciprocal's error times the residual's; 2^-45 with IEEE divisions, at
// four times the instructions).  A zero divisor gives an infinite or NaN quotient, as the
// division does.
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float rb = __fdividef(1.f, b.hi);
  const float q = a.hi * rb;
  const float p = b.hi * q, pe = fmaf(b.hi, q, -p);
  const float r = fmaf(-b.lo, q, ((a.hi - p) - pe) + a.lo);
  return ff_quick(q, r * rb);
}

// Single MUFU instructions (flush-to-zero): the integrands never need subnormal
// results, so the range fix-ups that exp2f/__log2f/rsqrtf wrap around them are skipped.
__device__ __forceinline__ float ex2_ftz(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float lg2_ftz(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_ftz(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// atan2(y, x) without branches, for the per-node angles of the float32 kernels (the
// feature's longitude offset, the scattering angle).  Octant reduction: with
// t = min(|x|, |y|) / max(|x|, |y|) in [0, 1] (one rcp.approx), atan t = t + t^3 Q(t^2)
// with Q of degree 7, its coefficients fitted for this library by iteratively reweighted
// least squares (Lawson's method) on the relative error of atan over [0, 1] (1.1 ulp
// there in float32; tests/atan2_fit.py reproduces them); then atan2 = pi/2 - atan t where |y| > |x|, pi - (that) where
// x < 0, and the sign of y.  About 3 ulp from the correctly rounded atan2 for finite
// arguments; (0, 0) gives 0.
__device__ __forceinline__ float atan2_poly(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(fmaxf(ax, ay), 1e-37f), mn = fminf(ax, ay);
  const float t = mn * rcp_ftz(mx);
  const float s = t * t;
  float q = 0.0029206655f;
  q = fmaf(q, s, -0.016367827f);
  q = fmaf(q, s, 0.043211706f);
  q = fmaf(q, s, -0.07552202f);
  q = fmaf(q, s, 0.10665999f);
  q = fmaf(q, s, -0.14211054f);
  q = fmaf(q, s, 0.19993773f);
  q = fmaf(q, s, -0.33333153f);
  float r = fmaf(t * s, q, t);
  r = ay > ax ? 1.5707964f - r : r;
  r = x < 0.f ? 3.1415927f - r : r;
  return copysignf(r, y);
}

// ---------------------------------------------------------------------------
// Binary search of the observer that owns pixel `i` (records sorted by pix_begin).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_observer(const ZlObserver* __restrict__ obs, int n_obs, int64_t i) {
  int lo = 0, hi = n_obs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&obs[mid].pix_begin) <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Where a kernel finds pixel i's observer: sorted ZlObserver records (one per
// instant, rec != NULL), or time-ordered positions, one per pixel, as float64
// [3][n_pix] arrays with a single cutoff-flag word for the whole call.
struct ObsArgs {
  const ZlObserver* rec;
  int32_t n_rec;
  const double* obs;     // [3][n_pix] (time-ordered) or NULL
  const double* earth;   // [3][n_pix] or NULL (then Earth is only needed by no component)
  const uint32_t* flags; // time-ordered: the OR of every sample's cutoff flags
};

struct PixObs {
  double ox, oy, oz, ex, ey;
  uint32_t outside;
};

// Observer record o as a pixel's observer.
__device__ __forceinline__ PixObs record_observer(const ObsArgs& OA, int o) {
  const ZlObserver& O = OA.rec[o];
  return PixObs{O.obs[0], O.obs[1], O.obs[2], O.earth[0], O.earth[1], O.outside};
}

__device__ __forceinline__ PixObs pixel_observer(const ObsArgs& A, int64_t i, int64_t n_pix) {
  PixObs p;
  if (A.rec) {
    const ZlObserver& O = A.rec[find_observer(A.rec, A.n_rec, i)];
    p.ox = O.obs[0];
    p.oy = O.obs[1];
    p.oz = O.obs[2];
    p.ex = O.earth[0];
    p.ey = O.earth[1];
    p.outside = O.outside;
  } else {
    p.ox = A.obs[i];
    p.oy = A.obs[n_pix + i];
    p.oz = A.obs[2 * n_pix + i];
    p.ex = A.earth ? A.earth[i] : 0.0;
    p.ey = A.earth ? A.earth[n_pix + i] : 0.0;
    p.outside = __ldg(A.flags);
  }
  return p;
}

// ---------------------------------------------------------------------------
// How the blocks of a forward launch find their work (ZlLaunch of the C ABI).
// A launch covers n_items items (pixels; pixel pairs for the two-pixel kernel) in
// tiles of consecutive items:
//  - static schedule (queue == NULL): tiles of blockDim.x items, block b taking tiles
//    b, b + gridDim.x, ... -- the grid-stride loop;
//  - work queue (queue != NULL): tiles of `tile` items pulled from a device counter,
//    queue[0], by one atomic add per tile, until the items run out, so blocks that
//    draw cheap tiles take more of them.  The blocks that find the queue empty count
//    themselves out in queue[1]; the last one puts both words back to zero, so the
//    next launch on the same queue (a CUDA-graph replay, say) starts from tile 0.
//    No block ever waits for another, and results never depend on which block ran
//    which tile.
// out_index: output column of each pixel (NULL: the pixel's own index); lets a caller
// run its pixels in another order (sorted for coherence) and still get its layout.
// ---------------------------------------------------------------------------
struct Sched {
  unsigned int* queue;
  int32_t tile;
  const int64_t* out_index;
};

__device__ __forceinline__ int64_t out_col(const Sched& S, int64_t i) { return S.out_index ? S.out_index[i] : i; }

// Items per tile of a launch.
__device__ __forceinline__ int64_t sched_tile(const Sched& S) { return S.queue ? (int64_t)S.tile : (int64_t)blockDim.x; }

// Schedules a kernel is compiled for: both (chosen by S.queue at run time), or one of them
// (a kernel whose register count is tight compiles one instantiation per schedule).
enum { kSchedAny = 0, kSchedStatic = 1, kSchedQueue = 2 };

template <int MODE>
__device__ __forceinline__ bool sched_queued(const Sched& S) {
  return MODE == kSchedQueue || (MODE == kSchedAny && S.queue != nullptr);
}

// Next tile from the queue, the same for every thread of the block.
__device__ __forceinline__ int64_t sched_fetch(const Sched& S) {
  __shared__ unsigned int s_next;
  __syncthreads();  // every thread has read s_next for the previous tile
  if (threadIdx.x == 0) s_next = atomicAdd(S.queue, 1u);
  __syncthreads();
  return (int64_t)s_next;
}

// After a block's last tile: count the block out; the last one resets the queue.
template <int MODE>
__device__ __forceinline__ void sched_finish(const Sched& S) {
  if (!sched_queued<MODE>(S) || threadIdx.x != 0) return;
  __threadfence();
  if (atomicAdd(S.queue + 1, 1u) == gridDim.x - 1) {
    atomicExch(S.queue + 1, 0u);
    atomicExch(S.queue, 0u);
  }
}

// The loop of ZL_SCHED_LOOP.  Static: the grid-stride loop over items.  Queue: tb is the
// first item of the block's current tile; every thread steps through the tile in blockDim
// strides (tiles are a multiple of blockDim, so all threads reach the tile's end at the same
// iteration) and the block fetches the next tile together.
template <int MODE>
__device__ __forceinline__ int64_t sched_base0(const Sched& S) {
  return sched_queued<MODE>(S) ? sched_fetch(S) * (int64_t)S.tile : 0;
}
template <int MODE>
__device__ __forceinline__ int64_t sched_i0(const Sched& S, int64_t tb) {
  return (sched_queued<MODE>(S) ? tb : (int64_t)blockIdx.x * blockDim.x) + threadIdx.x;
}
template <int MODE>
__device__ __forceinline__ bool sched_more(const Sched& S, int64_t i, int64_t tb, int64_t n_items) {
  return sched_queued<MODE>(S) ? tb < n_items : i < n_items;
}
template <int MODE>
__device__ __forceinline__ int64_t sched_next(const Sched& S, int64_t i, int64_t& tb) {
  if (!sched_queued<MODE>(S)) return i + (int64_t)gridDim.x * blockDim.x;
  i += blockDim.x;
  if (i >= tb + S.tile) {
    tb = sched_fetch(S) * (int64_t)S.tile;
    i = tb + threadIdx.x;
  }
  return i;
}

// for (each item i of this block's tiles) { ... }: a plain loop rather than a function taking
// the body as a lambda, whose closure cost the DIRBE forward kernel 17 registers.  With the queue,
// every thread of the block runs the same iterations (items past n_items skip the body), since
// the tile fetch synchronises the block.  Call sched_finish<MODE>(S) after the loop.
#define ZL_SCHED_LOOP(MODE, S, n_items, i)                                                                 \
  for (int64_t _zl_tb = ::zl::sched_base0<MODE>(S), i = ::zl::sched_i0<MODE>(S, _zl_tb);                \
       ::zl::sched_more<MODE>(S, i, _zl_tb, (n_items)); i = ::zl::sched_next<MODE>(S, i, _zl_tb))        \
    if (::zl::sched_queued<MODE>(S) && i >= (n_items)) continue;                                         \
    else

// First item of the tile that item i of a ZL_SCHED_LOOP belongs to (inside the loop only): the
// fetched tile's base with the queue, else the block's share of this grid-stride pass.
#define ZL_SCHED_TILE_BASE(MODE, S, i) (::zl::sched_queued<MODE>(S) ? _zl_tb : (i) - (int64_t)threadIdx.x)

// Host side of a forward launch: block shape, grid sizing and the schedule.
struct LaunchArgs {
  int tpb;      // threads per block
  int bps;      // blocks per SM the grid is capped at
  int num_sms;
  Sched sched;
};

// Grid of a launch over n_items: one block per tile, capped at num_sms x bps.
inline int64_t fwd_grid(const LaunchArgs& L, int64_t n_items) {
  const int64_t T = L.sched.queue ? (int64_t)L.sched.tile : (int64_t)L.tpb;
  int64_t grid = (n_items + T - 1) / T;
  const int64_t cap = (int64_t)L.num_sms * L.bps;
  if (grid > cap) grid = cap;
  return grid < 1 ? 1 : grid;
}

}  // namespace zl
