// Fast forward kernel: the line-of-sight integrand in float32 on the FP32/MUFU pipes
// (Kelsall, zodipy/brightness.py:21-56; RRM, zodipy/brightness.py:59-83, through the
// generic layout).
//
// Same integral as the float64 kernel (zodipy/model.py:253-277); what changes is
// the arithmetic, chosen for GB300 where FP64 runs at a small fraction of FP32:
//  - the cutoff-sphere intersections (zodipy/line_of_sight.py:64-85) are solved
//    per pixel in float-float (~48-bit) arithmetic;
//  - for the ring and the feature (zodipy/number_density.py:113-181), whose
//    radial profiles are narrow (sigma_r = 0.025 AU), R^2 - R0^2 at each node is
//    w^2 + c' with w = R_los + u.(X_obs - X_0) carried in float-float and c' a
//    per-pixel float-float constant, and R - R0 is recovered from it with one
//    Newton step, so the Gaussian exponent keeps float32 relative accuracy;
//  - heights above each symmetry plane are linear in the node abscissa with
//    float-float per-pixel coefficients, evaluated to ~1 ulp with one FMA on
//    the high parts plus first-order low-part corrections;
//  - distances are never formed from the position vector: |X - X_0|^2 =
//    w^2 + b^2 with w = R_los + u.(X_obs - X_0) (linear in the node abscissa,
//    evaluated as above) and b^2 the squared impact parameter (a per-pixel
//    constant), two non-negative terms, so lines of sight that graze the Sun
//    keep float32 relative accuracy where R^-alpha is steepest;
//  - everything else runs in float32 with single MUFU instructions (ex2, lg2,
//    rsqrt), integer powers by squaring and 1 - e^-y by its series where it
//    would cancel; the per-node angles (the feature's longitude offset, the
//    scattering angle) use a branch-free polynomial atan2 (atan2_poly, ~3 ulp);
//  - each component's quadrature sum is Kahan-compensated in float32 and
//    written as float64.
// One thread integrates one pixel over all nodes and components in node order,
// so a pixel's result never depends on how pixels are partitioned.
#pragma once

#include "zl_f32.cuh"

namespace zl {

// Per-pixel constants of the node loop: intersections of the line of sight with the
// cutoff spheres, node-position and plane-height coefficients, impact parameters and the
// feature's rotated frame (float-float where the node loop needs more than 24 bits).
template <int NC>
struct PixSetupF32 {
  ff hs[NC], mh[NC], z1[NC], z0[NC], wm[NC], cw[NC];
  // ring/feature: w -/+ w0 offsets and residual of R^2 - R0^2 = (w - w0)(w + w0) + rr
  ff wa[NC], wb[NC];
  float rr[NC];
  float b2[NC], fx1[NC], fx0[NC], fy1[NC], fy0[NC];
  float b2h, bperp;
};

// What a pixel's set-up derives from its observer (and Earth) alone: the same for every
// pixel of one observer, so a block derives it once and shares it (see obs_cache_index).
// The operations are those of the per-pixel set-up, so the bits are the same either way.
template <int NC>
struct ObsSetupF32 {
  ff ox, oy, oz;                                 // observer position
  ff r2;                                         // |X_obs|^2
  ff c_in[ZL_MAX_RANGES], c_out[ZL_MAX_RANGES];  // |X_obs|^2 - cutoff^2 of each range's spheres
  ff dx[NC], dy[NC], dz[NC];                     // X_obs - X_0
  ff on[NC];                                     // (X_obs - X_0) . n
  ff d2[NC];                                     // |X_obs - X_0|^2
  float rox[NC], roy[NC], cph[NC], sph[NC];      // features: X_obs - X_0 in the frame rotated by phi
  uint32_t outside;
};

template <uint32_t LAYOUT, uint32_t FLAGS, int NC>
__device__ __forceinline__ void observer_setup(const KParamsF32& P, const PixObs& O, ObsSetupF32<NC>& Q) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<LAYOUT == kLayoutGeneric ? kFlagsRuntime : FLAGS>;
  const int nc = L::generic ? P.n_comps : NC;
  const int nr = P.n_ranges;
  const ff ox = ff_split(O.ox), oy = ff_split(O.oy), oz = ff_split(O.oz);
  Q.ox = ox;
  Q.oy = oy;
  Q.oz = oz;
  Q.outside = O.outside;
  const ff r2 = ff_add(ff_add(ff_mul(ox, ox), ff_mul(oy, oy)), ff_mul(oz, oz));
  Q.r2 = r2;
#pragma unroll
  for (int r = 0; r < ZL_MAX_RANGES; ++r) {
    if (r < nr) {
      Q.c_in[r] = ff_add(r2, ff_neg(ff{P.cut_in_hi[r], P.cut_in_lo[r]}));
      Q.c_out[r] = ff_add(r2, ff_neg(ff{P.cut_out_hi[r], P.cut_out_lo[r]}));
    }
  }
  ff on = {0.f, 0.f};  // (X_obs - X_0) . n of the previous component
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    if (c >= nc) break;
    const KCompF32& C = P.comp[c];
    const int type = L::generic ? C.type : L::type(c);
    const bool off = Fl::offset(C, c);
    // X_obs - X_0 (exact for the components centred on the Sun)
    const ff dx = ff_add_fast(ox, ff{-C.ox, -C.ox_lo}), dy = ff_add_fast(oy, ff{-C.oy, -C.oy_lo}),
             dz = ff_add_fast(oz, ff{-C.oz, -C.oz_lo});
    Q.dx[c] = dx;
    Q.dy[c] = dy;
    Q.dz[c] = dz;
    // kept from the previous component when it has the same plane and centre
    if (!(c > 0 && C.same_plane_prev)) {
      const ff nx = {C.nx, C.nx_lo}, ny = {C.ny, C.ny_lo}, nz = {C.nz, C.nz_lo};
      on = ff_add_fast(ff_add_fast(ff_mul_nr(dx, nx), ff_mul_nr(dy, ny)), ff_mul_nr(dz, nz));
    }
    Q.on[c] = on;
    Q.d2[c] = !off ? r2 : ff_add_fast(ff_add_fast(ff_mul_nr(dx, dx), ff_mul_nr(dy, dy)), ff_mul_nr(dz, dz));
    Q.rox[c] = Q.roy[c] = Q.cph[c] = Q.sph[c] = 0.f;
    if (featurelike(type)) {
      // longitude relative to Earth's, minus theta (number_density.py:167-173): rotate the
      // frame by phi = atan2(earth - X_0) + theta so the wrapped difference is one atan2 of
      // two coordinates that are linear in the node abscissa
      const ff ex = ff_add_fast(ff_split(O.ex), ff{-C.ox, -C.ox_lo}), ey = ff_add_fast(ff_split(O.ey), ff{-C.oy, -C.oy_lo});
      const float phi = atan2f(ey.hi + ey.lo, ex.hi + ex.lo) + C.c[6];
      float sp, cp;
      sincosf(phi, &sp, &cp);
      const float ocx = dx.hi + dx.lo, ocy = dy.hi + dy.lo;
      Q.cph[c] = cp;
      Q.sph[c] = sp;
      Q.rox[c] = cp * ocx + sp * ocy;
      Q.roy[c] = cp * ocy - sp * ocx;
    }
  }
}

// Pixel i's set-up from its observer's (Q).
template <uint32_t LAYOUT, uint32_t FLAGS, bool PRECISE, int NC>
__device__ __forceinline__ void pixel_setup_obs(const KParamsF32& P, const double* __restrict__ u, int64_t n_pix,
                                                int64_t i, const ObsSetupF32<NC>& Q, PixSetupF32<NC>& S) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<LAYOUT == kLayoutGeneric ? kFlagsRuntime : FLAGS>;
  const int nc = L::generic ? P.n_comps : NC;
  const int nr = P.n_ranges;
  // the Planck layout's kernels keep the IEEE-division roots (measured faster there)
  constexpr bool kShortRoots = LAYOUT != kLayoutPlanck;
  // float-float values of the doubles by bit operations (no float64 instruction); the sums
  // below are ff_add_fast (accurate to a few 2^-48 of their operands: the geometry needs
  // absolute, not relative, accuracy); only |X_obs|^2 - cutoff^2, per observer, is an exact sum
  const ff ux = ff_split(u[i]), uy = ff_split(u[n_pix + i]), uz = ff_split(u[2 * n_pix + i]);
  const ff ox = Q.ox, oy = Q.oy, oz = Q.oz;
  const uint32_t outside = Q.outside;
  const float uxf = ux.hi, uyf = uy.hi;

  const ff oxux = ff_mul_nr(ox, ux), oyuy = ff_mul_nr(oy, uy);
  const ff b = ff_scale(ff_add_fast(oxux, oyuy), 2.0f);
  const ff r2 = Q.r2;
  const ff beta_h = ff_add_fast(ff_add_fast(oxux, oyuy), ff_mul_nr(oz, uz));  // u . X_obs

  ff hs_r[ZL_MAX_RANGES], mid_r[ZL_MAX_RANGES];
#pragma unroll
  for (int r = 0; r < ZL_MAX_RANGES; ++r) {
    if (r < nr) {
      const ff st = ((outside >> (2 * r)) & 1u) ? ff{(float)kEps, 0.f} : sphere_distance_ffc<kShortRoots>(b, Q.c_in[r]);
      const ff sp = ((outside >> (2 * r + 1)) & 1u) ? ff{(float)kEps, 0.f} : sphere_distance_ffc<kShortRoots>(b, Q.c_out[r]);
      hs_r[r] = ff_scale(ff_add_fast(sp, ff_neg(st)), 0.5f);
      mid_r[r] = ff_scale(ff_add_fast(sp, st), 0.5f);
    } else {
      hs_r[r] = ff{0.f, 0.f};
      mid_r[r] = ff{0.f, 0.f};
    }
  }

  // squared impact parameter of the line of sight about the Sun, |X_obs|^2 - (u . X_obs)^2 >= 0
  const ff b2h_ff = ff_add_fast(r2, ff_neg(ff_mul(beta_h, beta_h)));
  const float b2h = fmaxf(b2h_ff.hi + b2h_ff.lo, 0.f);
  // scattering angle pi - atan2(|u x X_obs|, R_los + u . X_obs) (scattering.py:26-31)
  S.b2h = b2h;
  S.bperp = Fl::scat(P) ? sqrtf(b2h) : 0.f;

  // per-component set-up
  ff un = {0.f, 0.f};  // u . n of the previous component
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    if (c >= nc) break;
    const KCompF32& C = P.comp[c];
    const int type = L::generic ? C.type : L::type(c);
    ff hs = {0.f, 0.f}, md = {0.f, 0.f};
    if (!L::generic) {
      hs = hs_r[L::range(c)];
      md = mid_r[L::range(c)];
    } else {
#pragma unroll
      for (int r = 0; r < ZL_MAX_RANGES; ++r)
        if (r == C.range) {
          hs = hs_r[r];
          md = mid_r[r];
        }
    }
    S.hs[c] = hs;
    S.mh[c] = ff_add_fast(md, beta_h);  // R_los + u . X_obs = hs x + mh
    const bool off = Fl::offset(C, c);
    // height above the symmetry plane, linear in the node abscissa x:
    //   Z = (hs x + mid)(u . n) + (X_obs - X_0) . n = z1 x + z0
    // (u . n is kept from the previous component when it has the same plane, as the ring and
    // the Earth-trailing feature do)
    if (!(c > 0 && C.same_plane_prev)) {
      const ff nx = {C.nx, C.nx_lo}, ny = {C.ny, C.ny_lo}, nz = {C.nz, C.nz_lo};
      un = ff_add_fast(ff_add_fast(ff_mul_nr(ux, nx), ff_mul_nr(uy, ny)), ff_mul_nr(uz, nz));
    }
    S.z1[c] = ff_mul(hs, un);
    S.z0[c] = ff_add_fast(ff_mul_nr(md, un), Q.on[c]);
    // |X - X_0|^2 = w^2 + b^2,  w = hs x + (mid + beta),  beta = u . (X_obs - X_0),
    // b^2 = |X_obs - X_0|^2 - beta^2;  the ring/feature use w^2 + c' with c' = b^2 - R0^2
    S.wm[c] = S.mh[c];
    S.b2[c] = b2h;
    S.cw[c] = ff{0.f, 0.f};
    S.wa[c] = S.wb[c] = ff{0.f, 0.f};
    S.rr[c] = 0.f;
    if (off || (PRECISE && ringlike(type)) || masked(type)) {
      const ff dx = Q.dx[c], dy = Q.dy[c], dz = Q.dz[c];
      const ff beta =
          !off ? beta_h : ff_add_fast(ff_add_fast(ff_mul_nr(dx, ux), ff_mul_nr(dy, uy)), ff_mul_nr(dz, uz));
      const ff bb = ff_add_fast(Q.d2[c], ff_neg(ff_mul_nr(beta, beta)));
      S.wm[c] = ff_add_fast(md, beta);
      S.b2[c] = fmaxf(bb.hi + bb.lo, 0.f);
      S.cw[c] = masked(type) ? bb : ff_add_fast(bb, ff_neg(ff{C.c[4], C.c[5]}));
      if (ringlike(type)) {
        // R^2 - R0^2 = w^2 + c' = (w - w0)(w + w0) + (w0^2 + c'),  w0 = sqrt(max(-c', 0)):
        // each factor is linear in the node abscissa and evaluated to ~1 ulp near its zero
        const ff w0 = S.cw[c].hi < 0.f ? ff_sqrt(ff_neg(S.cw[c])) : ff{0.f, 0.f};
        S.wa[c] = ff_add_fast(S.wm[c], ff_neg(w0));
        S.wb[c] = ff_add_fast(S.wm[c], w0);
        const ff res = ff_add_fast(ff_mul_nr(w0, w0), S.cw[c]);
        S.rr[c] = res.hi + res.lo;
      }
    }
    S.fx1[c] = S.fx0[c] = S.fy1[c] = S.fy0[c] = 0.f;
    if (featurelike(type)) {
      const float cp = Q.cph[c], sp = Q.sph[c];
      const float rux = cp * uxf + sp * uyf, ruy = cp * uyf - sp * uxf;
      const float h = hs.hi + hs.lo, m = md.hi + md.lo;
      S.fx1[c] = h * rux;
      S.fx0[c] = fmaf(m, rux, Q.rox[c]);
      S.fy1[c] = h * ruy;
      S.fy0[c] = fmaf(m, ruy, Q.roy[c]);
    }
  }
}

// Pixel i's set-up with its observer's part evaluated in place (the same operations as
// observer_setup + pixel_setup_obs, interleaved so that each observer quantity is consumed
// where it is formed: splitting them kept the generic layout's eighty-odd observer values
// alive at once and spilled).
template <uint32_t LAYOUT, uint32_t FLAGS, bool PRECISE, int NC>
__device__ __forceinline__ void pixel_setup(const KParamsF32& P, const double* __restrict__ u, int64_t n_pix,
                                            const ObsArgs& OA, int64_t i, PixSetupF32<NC>& S) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<LAYOUT == kLayoutGeneric ? kFlagsRuntime : FLAGS>;
  const int nc = L::generic ? P.n_comps : NC;
  const int nr = P.n_ranges;
  // the Planck layout's kernels keep the IEEE-division roots (measured faster there)
  constexpr bool kShortRoots = LAYOUT != kLayoutPlanck;
  // float-float values of the doubles by bit operations (no float64 instruction); the sums
  // below are ff_add_fast (accurate to a few 2^-48 of their operands: the geometry needs
  // absolute, not relative, accuracy); only |X_obs|^2 - cutoff^2, per observer, is an exact sum
  const ff ux = ff_split(u[i]), uy = ff_split(u[n_pix + i]), uz = ff_split(u[2 * n_pix + i]);
  const PixObs O = pixel_observer(OA, i, n_pix);
  const ff ox = ff_split(O.ox), oy = ff_split(O.oy), oz = ff_split(O.oz);
  const uint32_t outside = O.outside;
  const float uxf = ux.hi, uyf = uy.hi, uzf = uz.hi;
  const float oxf = ox.hi, oyf = oy.hi, ozf = oz.hi;

  const ff oxux = ff_mul_nr(ox, ux), oyuy = ff_mul_nr(oy, uy);
  const ff b = ff_scale(ff_add_fast(oxux, oyuy), 2.0f);
  const ff r2 = ff_add(ff_add(ff_mul(ox, ox), ff_mul(oy, oy)), ff_mul(oz, oz));
  const ff beta_h = ff_add_fast(ff_add_fast(oxux, oyuy), ff_mul_nr(oz, uz));  // u . X_obs

  ff hs_r[ZL_MAX_RANGES], mid_r[ZL_MAX_RANGES];
#pragma unroll
  for (int r = 0; r < ZL_MAX_RANGES; ++r) {
    if (r < nr) {
      const ff st = ((outside >> (2 * r)) & 1u) ? ff{(float)kEps, 0.f}
                                                : sphere_distance_ff<kShortRoots>(b, r2, ff{P.cut_in_hi[r], P.cut_in_lo[r]});
      const ff sp = ((outside >> (2 * r + 1)) & 1u) ? ff{(float)kEps, 0.f}
                                                    : sphere_distance_ff<kShortRoots>(b, r2, ff{P.cut_out_hi[r], P.cut_out_lo[r]});
      hs_r[r] = ff_scale(ff_add_fast(sp, ff_neg(st)), 0.5f);
      mid_r[r] = ff_scale(ff_add_fast(sp, st), 0.5f);
    } else {
      hs_r[r] = ff{0.f, 0.f};
      mid_r[r] = ff{0.f, 0.f};
    }
  }

  // squared impact parameter of the line of sight about the Sun, |X_obs|^2 - (u . X_obs)^2 >= 0
  const ff b2h_ff = ff_add_fast(r2, ff_neg(ff_mul(beta_h, beta_h)));
  const float b2h = fmaxf(b2h_ff.hi + b2h_ff.lo, 0.f);
  // scattering angle pi - atan2(|u x X_obs|, R_los + u . X_obs) (scattering.py:26-31)
  S.b2h = b2h;
  S.bperp = Fl::scat(P) ? sqrtf(b2h) : 0.f;

  // per-component set-up
  ff* hs_c = S.hs;
  ff* mh_c = S.mh;
  ff* z1_c = S.z1;
  ff* z0_c = S.z0;
  ff* wm_c = S.wm;
  ff* cw_c = S.cw;
  float* b2_c = S.b2;
  float* fx1 = S.fx1;
  float* fx0 = S.fx0;
  float* fy1 = S.fy1;
  float* fy0 = S.fy0;
  ff un = {0.f, 0.f}, on = {0.f, 0.f};  // u . n and (X_obs - X_0) . n of the previous component
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    if (c >= nc) break;
    const KCompF32& C = P.comp[c];
    const int type = L::generic ? C.type : L::type(c);
    ff hs = {0.f, 0.f}, md = {0.f, 0.f};
    if (!L::generic) {
      hs = hs_r[L::range(c)];
      md = mid_r[L::range(c)];
    } else {
#pragma unroll
      for (int r = 0; r < ZL_MAX_RANGES; ++r)
        if (r == C.range) {
          hs = hs_r[r];
          md = mid_r[r];
        }
    }
    hs_c[c] = hs;
    mh_c[c] = ff_add_fast(md, beta_h);  // R_los + u . X_obs = hs x + mh
    const bool off = Fl::offset(C, c);
    // X_obs - X_0 (exact for the components centred on the Sun; selecting X_obs for them
    // instead raised the forward kernel's register count past five blocks per SM)
    const ff dx = ff_add_fast(ox, ff{-C.ox, -C.ox_lo}), dy = ff_add_fast(oy, ff{-C.oy, -C.oy_lo}),
             dz = ff_add_fast(oz, ff{-C.oz, -C.oz_lo});
    // height above the symmetry plane, linear in the node abscissa x:
    //   Z = (hs x + mid)(u . n) + (X_obs - X_0) . n = z1 x + z0
    // (u . n and (X_obs - X_0) . n are kept from the previous component when it has the same
    // plane and centre, as the ring and the Earth-trailing feature do)
    if (!(c > 0 && C.same_plane_prev)) {
      const ff nx = {C.nx, C.nx_lo}, ny = {C.ny, C.ny_lo}, nz = {C.nz, C.nz_lo};
      un = ff_add_fast(ff_add_fast(ff_mul_nr(ux, nx), ff_mul_nr(uy, ny)), ff_mul_nr(uz, nz));
      on = ff_add_fast(ff_add_fast(ff_mul_nr(dx, nx), ff_mul_nr(dy, ny)), ff_mul_nr(dz, nz));
    }
    z1_c[c] = ff_mul(hs, un);
    z0_c[c] = ff_add_fast(ff_mul_nr(md, un), on);
    // |X - X_0|^2 = w^2 + b^2,  w = hs x + (mid + beta),  beta = u . (X_obs - X_0),
    // b^2 = |X_obs - X_0|^2 - beta^2;  the ring/feature use w^2 + c' with c' = b^2 - R0^2
    wm_c[c] = mh_c[c];
    b2_c[c] = b2h;
    cw_c[c] = ff{0.f, 0.f};
    S.wa[c] = S.wb[c] = ff{0.f, 0.f};
    S.rr[c] = 0.f;
    if (off || (PRECISE && ringlike(type)) || masked(type)) {
      const ff beta =
          !off ? beta_h : ff_add_fast(ff_add_fast(ff_mul_nr(dx, ux), ff_mul_nr(dy, uy)), ff_mul_nr(dz, uz));
      const ff d2 = !off ? r2 : ff_add_fast(ff_add_fast(ff_mul_nr(dx, dx), ff_mul_nr(dy, dy)), ff_mul_nr(dz, dz));
      const ff bb = ff_add_fast(d2, ff_neg(ff_mul_nr(beta, beta)));
      wm_c[c] = ff_add_fast(md, beta);
      b2_c[c] = fmaxf(bb.hi + bb.lo, 0.f);
      cw_c[c] = masked(type) ? bb : ff_add_fast(bb, ff_neg(ff{C.c[4], C.c[5]}));
      if (ringlike(type)) {
        // R^2 - R0^2 = w^2 + c' = (w - w0)(w + w0) + (w0^2 + c'),  w0 = sqrt(max(-c', 0)):
        // each factor is linear in the node abscissa and evaluated to ~1 ulp near its zero
        const ff w0 = cw_c[c].hi < 0.f ? ff_sqrt(ff_neg(cw_c[c])) : ff{0.f, 0.f};
        S.wa[c] = ff_add_fast(wm_c[c], ff_neg(w0));
        S.wb[c] = ff_add_fast(wm_c[c], w0);
        const ff res = ff_add_fast(ff_mul_nr(w0, w0), cw_c[c]);
        S.rr[c] = res.hi + res.lo;
      }
    }
    fx1[c] = fx0[c] = fy1[c] = fy0[c] = 0.f;
    if (featurelike(type)) {
      // longitude relative to Earth's, minus theta (number_density.py:167-173): rotate the
      // frame by phi = atan2(earth - X_0) + theta so the wrapped difference is one atan2 of
      // two coordinates that are linear in the node abscissa
      const ff ex = ff_add_fast(ff_split(O.ex), ff{-C.ox, -C.ox_lo}), ey = ff_add_fast(ff_split(O.ey), ff{-C.oy, -C.oy_lo});
      const float phi = atan2f(ey.hi + ey.lo, ex.hi + ex.lo) + C.c[6];
      float sp, cp;
      sincosf(phi, &sp, &cp);
      const float ocx = dx.hi + dx.lo, ocy = dy.hi + dy.lo;
      const float rux = cp * uxf + sp * uyf, ruy = cp * uyf - sp * uxf;
      const float rox = cp * ocx + sp * ocy, roy = cp * ocy - sp * ocx;
      const float h = hs.hi + hs.lo, m = md.hi + md.lo;
      fx1[c] = h * rux;
      fx0[c] = fmaf(m, rux, rox);
      fy1[c] = h * ruy;
      fy0[c] = fmaf(m, ruy, roy);
    }
  }

}

// The observer record whose set-up a block derives once and shares (-1: none, every pixel
// derives its own): the only record of a one-observer call, else the record of the block's first
// pixel on the static schedule (a batch's observers own long runs of pixels); none with the
// work queue, whose tiles come in any order, or for time-ordered calls.  Block-uniform.
template <int MODE>
__device__ __forceinline__ int obs_cache_index(const ObsArgs& OA, int64_t first_pixel, int64_t n_pix) {
  if (!OA.rec) return -1;
  if (OA.n_rec == 1) return 0;
  if (MODE != kSchedStatic || first_pixel >= n_pix) return -1;
  return find_observer(OA.rec, OA.n_rec, first_pixel);
}

// Whether pixel i takes its block's shared observer set-up.
__device__ __forceinline__ bool obs_cache_hit(const ObsArgs& OA, int cached, int64_t i) {
  return cached >= 0 && (OA.n_rec == 1 || find_observer(OA.rec, OA.n_rec, i) == cached);
}

// Pixel i's own observer set-up, out of line: a second inlined copy of the set-up next to the
// shared one raised the DIRBE forward kernel from 95 to 121 registers (four instead of five
// blocks per SM).  Q is the caller's local memory; only the pixels that do not share their
// block's observer (and time-ordered calls) come here.
template <uint32_t LAYOUT, uint32_t FLAGS, int NC>
__device__ __noinline__ void observer_setup_own(const KParamsF32& P, const ObsArgs& OA, int64_t i, int64_t n_pix,
                                                ObsSetupF32<NC>* Q) {
  observer_setup<LAYOUT, FLAGS, NC>(P, pixel_observer(OA, i, n_pix), *Q);
}

// Pixel i's set-up: from its block's shared observer set-up when it has the same observer,
// else from its own.
template <uint32_t LAYOUT, uint32_t FLAGS, bool PRECISE, int NC>
__device__ __forceinline__ void pixel_setup_cached(const KParamsF32& P, const double* __restrict__ u, int64_t n_pix,
                                                   const ObsArgs& OA, int64_t i, int cached,
                                                   const ObsSetupF32<NC>& shared, PixSetupF32<NC>& S) {
  ObsSetupF32<NC> own;
  const ObsSetupF32<NC>* q = &shared;
  if (!obs_cache_hit(OA, cached, i)) {
    observer_setup_own<LAYOUT, FLAGS, NC>(P, OA, i, n_pix, &own);
    q = &own;
  }
  pixel_setup_obs<LAYOUT, FLAGS, PRECISE, NC>(P, u, n_pix, i, *q, S);
}

// MODE: the schedule the kernel is compiled for (kSchedStatic or kSchedQueue); one build
// serving both ran the two-pixel kernel 7 % slower on the static schedule.
template <int NSPEC, uint32_t LAYOUT, bool PRECISE, uint32_t FLAGS, int MODE>
__global__ void __launch_bounds__(128) fwd_f32_kernel(const __grid_constant__ KParamsF32 P,
                                                      const double* __restrict__ u, int64_t n_pix,
                                                      const ObsArgs OA,
                                                      double* __restrict__ out_comps, double* __restrict__ out_total,
                                                      const Sched SC) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<LAYOUT == kLayoutGeneric ? kFlagsRuntime : FLAGS>;
  constexpr int NC = L::ncomp();
  extern __shared__ float4 tab_sm[];  // [NSPEC][nT]
  // the observer set-up the block's pixels share; not for the RRM model's eight components, which
  // measured slower with it (generic layout 1.6 %, the compiled RRM layout 0.7 %, same bits)
  constexpr bool kShared = !L::generic && !L::rrm;
  __shared__ ObsSetupF32<NC> s_obs;
  const int nT = P.n_temps;
  for (int t = threadIdx.x; t < nT * NSPEC; t += blockDim.x) tab_sm[t] = P.table[t / nT][t % nT];
  const int cached = kShared ? obs_cache_index<MODE>(OA, (int64_t)blockIdx.x * blockDim.x, n_pix) : -1;
  if (kShared && threadIdx.x == 0 && cached >= 0)
    observer_setup<LAYOUT, FLAGS, NC>(P, record_observer(OA, cached), s_obs);
  __syncthreads();

  const int nc = L::generic ? P.n_comps : NC;
  const int nr = P.n_ranges;

  ZL_SCHED_LOOP(MODE, SC, n_pix, i) {
    // ---- per-pixel set-up -------------------------------------------------
    PixSetupF32<NC> PS;
    if (kShared)
      pixel_setup_cached<LAYOUT, FLAGS, PRECISE, NC>(P, u, n_pix, OA, i, cached, s_obs, PS);
    else
      pixel_setup<LAYOUT, FLAGS, PRECISE, NC>(P, u, n_pix, OA, i, PS);
    const ff* hs_c = PS.hs;
    const ff* mh_c = PS.mh;
    const ff* z1_c = PS.z1;
    const ff* z0_c = PS.z0;
    const ff* wm_c = PS.wm;
    const ff* cw_c = PS.cw;
    const float* b2_c = PS.b2;
    const float* fx1 = PS.fx1;
    const float* fx0 = PS.fx0;
    const float* fy1 = PS.fy1;
    const float* fy0 = PS.fy0;
    const float b2h = PS.b2h, bperp = PS.bperp;

    // quadrature sums: plain float32 over blocks of kSumBlock nodes, Kahan-compensated across blocks
    // (the density prefactor and emissivity / albedo multiply each block sum: S.outer, S.outer_alb)
    float acc_s[NC][NSPEC], acc_c[NC][NSPEC], part[NC][NSPEC], partS[NC][NSPEC];
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) acc_s[c][s] = acc_c[c][s] = part[c][s] = partS[c][s] = 0.f;

    // ---- quadrature nodes ------------------------------------------------
#pragma unroll 1
    for (int k = 0; k < P.n_nodes; ++k) {
      const ff xk = {P.gl_x_hi[k], P.gl_x_lo[k]};
      const float wk = P.gl_w[k];
      float wh = 0.f, R2 = 1.f, rinv = 1.f, R = 1.f, lg2R = 0.f;
      float wB[NSPEC], wS[NSPEC], t4s[NC];  // w_k B(T) and w_k x the scattering term of the range
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) wB[s] = wS[s] = 0.f;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        t4s[c] = 0.f;
        if (c >= nc) break;
        const KCompF32& C = P.comp[c];
        const int type = L::generic ? C.type : L::type(c);
        const bool first = L::generic ? (C.first_in_range != 0) : L::first(c);
        const bool precise = PRECISE && ringlike(type);
        if (first) {
          // brightness.py:27-33 — heliocentric distance of the node, R^2 = w^2 + b^2, and temperature
          wh = lin_ff(hs_c[c], xk, mh_c[c]);
          R2 = fmaf(wh, wh, b2h);
          rinv = rsqrt_ftz(R2);
          // one Newton step where 1/R feeds the bands' e^-(zeta/dzeta)^6 (sensitivity 6 x^6);
          // the ring/feature distance is corrected from R^2 - R0^2 below instead
          if (type == ZL_CLOUD || type == ZL_BAND || masked(type)) rinv = rinv * fmaf(-0.5f * R2, rinv * rinv, 1.5f);
          R = R2 * rinv;
          lg2R = lg2_ftz(R);
          const float T = (L::generic || L::rrm ? C.T0 : P.T0) *
                          ex2_ftz((L::generic || L::rrm ? C.neg_delta : P.neg_delta) * lg2R);  // blackbody.py:16-30
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) wB[s] = wk * bb_lookup(tab_sm + s * nT, T, P.t_min, P.t_max, P.inv_dt, nT);
          if (Fl::scat(P)) {  // scattering.py:11-59
            const float theta = atan2_poly(bperp, -wh);
            const float flux = rinv * rinv;
#pragma unroll
            for (int s = 0; s < NSPEC; ++s) {
              const KSpecF32& S = P.spec[s];
              wS[s] = wk * (S.S * flux * (S.N * (S.C1 + S.C2 * theta + ex2_ftz(S.C3l2e * theta))));
            }
          }
        }
        // own distance when the component is offset from the Sun
        float Rc2 = R2, rcinv = rinv, Rc = R, lg2Rc = lg2R;
        if (Fl::offset(C, c)) {
          const float wc = lin_ff(hs_c[c], xk, wm_c[c]);
          Rc2 = fmaf(wc, wc, b2_c[c]);
          rcinv = rsqrt_ftz(Rc2);
          if (type == ZL_BAND || masked(type)) rcinv = rcinv * fmaf(-0.5f * Rc2, rcinv * rcinv, 1.5f);
          Rc = Rc2 * rcinv;
          lg2Rc = 0.5f * lg2_ftz(Rc2);
        }
        const float Z = lin_ff(z1_c[c], xk, z0_c[c]);
        float dens;
        if (type == ZL_CLOUD) {  // number_density.py:60-73
          const float zeta = fabsf(Z) * rcinv;
          const float g = zeta < C.c[4] ? zeta * zeta * C.c[5] : zeta - C.c[6];
          const float gg = ex2_ftz(C.c[3] * lg2_ftz(g));
          dens = ex2_ftz(-C.c[1] * lg2Rc - C.c[2] * gg);
        } else if (type == ZL_BAND) {  // number_density.py:99-110
          const float zz = fabsf(Z) * rcinv * C.c[1];
          const float z2 = zz * zz;
          const float t2 = ex2_ftz(-kLog2e * (z2 * z2 * z2));
          const float zp = Fl::p4(C, c) ? z2 * z2 : ex2_ftz(C.c[3] * lg2_ftz(zz));
          const float t3 = fmaf(zp, C.c[2], 1.0f);
          float t4 = 0.f;
          bool shared = false;
          if (Fl::runtime) {
#pragma unroll
            for (int j = 0; j < NC; ++j)
              if (j < c && C.share_t4 == j) {
                t4 = t4s[j];
                shared = true;
              }
          } else if (Fl::share_first(c)) {
            t4 = t4s[L::first_band(c)];
            shared = true;
          }
          if (!shared) {
            const float q = Rc2 * C.c[4];  // (R/delta_r)^2
            const float q2 = q * q, q4 = q2 * q2, q8 = q4 * q4;
            const float y = q8 * q2;  // (R/delta_r)^20
            // 1 - e^-y; below 1/4 by its series (relative error < 1e-7) instead of a cancelling difference
            t4 = y < 0.25f ? y * (1.f - y * (0.5f - y * (1.f / 6.f - y * (1.f / 24.f - y * (1.f / 120.f - y * (1.f / 720.f))))))
                           : 1.0f - ex2_ftz(-kLog2e * y);
          }
          t4s[c] = t4;
          dens = rcinv * t2 * t3 * t4;
        } else if (ringlike(type)) {  // ring (number_density.py:136-139) and feature (:167-181), RRM: x A
          float dR = Rc - C.c[1];
          if (precise) {
            // R^2 - R0^2 = w^2 + c' to ~1 ulp; one Newton step on R
            const float D2 = fmaf(lin_ff(hs_c[c], xk, PS.wa[c]), lin_ff(hs_c[c], xk, PS.wb[c]), PS.rr[c]);
            dR = dR + (D2 - dR * (Rc + C.c[1])) * (0.5f * rcinv);
          }
          float arg = dR * dR * C.c[2] + fabsf(Z) * C.c[3];
          if (featurelike(type)) {
            const float dth = atan2_poly(fmaf(fy1[c], xk.hi, fy0[c]), fmaf(fx1[c], xk.hi, fx0[c]));
            arg = fmaf(dth * dth, C.c[7], arg);
          }
          dens = ex2_ftz(-arg);
        } else if (type == ZL_INTERSTELLAR) {  // number_density.py:259-264
          dens = 1.f;
        } else {
          dens = rrm_masked_density(C, type, hs_c[c], xk, wm_c[c], cw_c[c], z1_c[c], z0_c[c], Z, rcinv, lg2Rc);
        }
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          const KSpecF32& S = P.spec[s];
          part[c][s] = fmaf(wB[s], dens, part[c][s]);
          if (Fl::scat(P)) partS[c][s] = fmaf(wS[s], dens, partS[c][s]);
        }
      }
      if ((k % kSumBlock) == kSumBlock - 1 || k == P.n_nodes - 1) {
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) {
            const KSpecF32& S = P.spec[s];
            const float blk = Fl::scat(P) ? fmaf(part[c][s], S.outer[c], partS[c][s] * S.outer_alb[c])
                                          : part[c][s] * S.outer[c];
            kahan_add(acc_s[c][s], acc_c[c][s], blk);
            part[c][s] = partS[c][s] = 0.f;
          }
      }
    }

    // ---- outputs: x (stop - start)/2, component order total ----------------
    const int64_t col = out_col(SC, i);
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      double tot = 0.0;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if (c >= nc) break;
        // the compensated sum times (stop - start)/2 in float32 (GB300's FP64 pipe is narrow);
        // the total is the float64 sum of the stored components, so it equals their sum exactly
        const double v = (double)((acc_s[c][s] - acc_c[c][s]) * (hs_c[c].hi + hs_c[c].lo));
        if (out_comps) out_comps[((int64_t)s * nc + c) * n_pix + col] = v;
        tot = (c == 0) ? v : __dadd_rn(tot, v);
      }
      if (out_total) out_total[(int64_t)s * n_pix + col] = tot;
    }
  }
  sched_finish<MODE>(SC);
}

template <int NSPEC, uint32_t LAYOUT, bool PRECISE, uint32_t FLAGS>
static cudaError_t launch_f32_t(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs,
                                double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  const size_t smem = sizeof(float4) * P.n_temps * NSPEC;
  if (L.sched.queue)
    fwd_f32_kernel<NSPEC, LAYOUT, PRECISE, FLAGS, kSchedQueue>
        <<<(unsigned)fwd_grid(L, n), L.tpb, smem, st>>>(P, u, n, obs, oc, ot, L.sched);
  else
    fwd_f32_kernel<NSPEC, LAYOUT, PRECISE, FLAGS, kSchedStatic>
        <<<(unsigned)fwd_grid(L, n), L.tpb, smem, st>>>(P, u, n, obs, oc, ot, L.sched);
  return cudaGetLastError();
}

// One layout and flag set, every supported number of spectral sets.
template <uint32_t LAYOUT, uint32_t FLAGS>
static cudaError_t launch_f32_flags(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                    double* ot, cudaStream_t st, const LaunchArgs& L) {
  switch (P.n_spec) {
    case 1: return launch_f32_t<1, LAYOUT, true, FLAGS>(P, u, n, obs, oc, ot, st, L);
    case 2: return launch_f32_t<2, LAYOUT, true, FLAGS>(P, u, n, obs, oc, ot, st, L);
    case 3: return launch_f32_t<3, LAYOUT, true, FLAGS>(P, u, n, obs, oc, ot, st, L);
    default: return launch_f32_t<4, LAYOUT, true, FLAGS>(P, u, n, obs, oc, ot, st, L);
  }
}

// Per-layout launchers (zl_fwd_f32_dirbe.cu, zl_fwd_f32_planck.cu, zl_fwd_f32_generic.cu).
cudaError_t launch_fwd_f32_dirbe(const KParamsF32& P, uint32_t flags, bool plain_geometry, const double* u, int64_t n,
                                 const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L);
cudaError_t launch_fwd_f32_planck(const KParamsF32& P, uint32_t flags, const double* u, int64_t n, const ObsArgs& obs,
                                  double* oc, double* ot, cudaStream_t st, const LaunchArgs& L);
cudaError_t launch_fwd_f32_generic(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                   double* ot, cudaStream_t st, const LaunchArgs& L);
cudaError_t launch_fwd_f32_rrm(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                               double* ot, cudaStream_t st, const LaunchArgs& L);

}  // namespace zl
