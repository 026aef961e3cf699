// Packed float32 primitives (fma/mul/add.rn.f32x2 on sm_100-class GPUs) and
// float-float pairs held as two lanes.  A packed operation rounds each lane
// exactly as its scalar counterpart; subtractions a - b are written as
// fma(b, -1, a), which rounds like a - b.  MUFU operations have no packed form
// and run per lane.
#pragma once

#include "zl_f32.cuh"

namespace zl {

struct ff2 {
  float2 hi, lo;
};

__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, bc2(-1.f), a); }  // a - b
__device__ __forceinline__ float2 abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ float2 ex2_2(float2 a) { return make_float2(ex2_ftz(a.x), ex2_ftz(a.y)); }
__device__ __forceinline__ float2 lg2_2(float2 a) { return make_float2(lg2_ftz(a.x), lg2_ftz(a.y)); }
__device__ __forceinline__ float2 rsqrt_2(float2 a) { return make_float2(rsqrt_ftz(a.x), rsqrt_ftz(a.y)); }
__device__ __forceinline__ ff2 pack_ff(ff a, ff b) { return {make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }

// lin_ff per lane: a x + b with x the node abscissa shared by both lanes
__device__ __forceinline__ float2 lin_ff_x2(const ff2& a, ff x, const ff2& b) {
  const float2 r = fma2(a.hi, bc2(x.hi), b.hi);
  return add2(r, fma2(a.hi, bc2(x.lo), fma2(a.lo, bc2(x.hi), b.lo)));
}

__device__ __forceinline__ ff2 two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  const float2 bb = sub2(s, a);
  return {s, add2(sub2(a, sub2(s, bb)), sub2(b, bb))};
}

__device__ __forceinline__ ff2 quick2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  return {s, sub2(b, sub2(s, a))};
}

// lin_ff2 per lane (float-float result)
__device__ __forceinline__ ff2 lin_ff2_x2(const ff2& a, ff x, const ff2& b) {
  const float2 p = mul2(a.hi, bc2(x.hi));
  const float2 pe = fma2(a.hi, bc2(x.hi), mul2(p, bc2(-1.f)));
  const ff2 s = two_sum2(p, b.hi);
  return quick2(s.hi, add2(s.lo, add2(pe, fma2(a.hi, bc2(x.lo), fma2(a.lo, bc2(x.hi), b.lo)))));
}

// sq_plus_ff per lane
__device__ __forceinline__ float2 sq_plus_ff_x2(const ff2& w, const ff2& c) {
  return add2(fma2(w.hi, w.hi, c.hi), fma2(mul2(bc2(2.f), w.hi), w.lo, c.lo));
}

__device__ __forceinline__ void kahan_add2(float2& s, float2& c, float2 t) {
  const float2 y = sub2(t, c);
  const float2 s1 = add2(s, y);
  c = sub2(sub2(s1, s), y);
  s = s1;
}

}  // namespace zl
