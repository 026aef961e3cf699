// Adjoint (reverse-mode) kernel: gradient of a per-pixel loss with respect to
// every model parameter, recomputing the integrand instead of storing
// pixels x nodes x components.
//
// For out[s, c, i] = hs_c(i) * sum_k w_k e_sc(X_ik) n_c(X_ik)
// (zodipy/brightness.py:21-56 summed as zodipy/line_of_sight.py:55-61) and an
// upstream gradient g[s, c, i] = dL/d out[s, c, i], each thread evaluates one
// pixel and accumulates, per node,
//   dL/dp += sum_s g[s,c] hs w * d(e_sc n_c)/dp
// with analytic derivatives of the Kelsall-98 densities
// (zodipy/number_density.py:47-181), of T(R) = T0 R^-delta through the
// blackbody table's segment slope (numpy.interp's derivative; 0 where it
// clamps), and of the scattering term (zodipy/scattering.py:34-59).  All
// spectral sets of a fused model share one pass: geometry and densities are
// evaluated once per node and weighted by E_c = sum_s g[s,c] e_sc.
//
// Parameters follow the reference's parameter dictionary
// (zodipy/zodiacal_light_model.py:38-55): per component, in order,
// x_0, y_0, z_0, i, Omega, n_0 and the type's own (cloud: alpha, beta, gamma,
// mu; band: delta_zeta, v, p, delta_r; ring: R, sigma_r, sigma_z; feature:
// R, sigma_r, sigma_z, theta, sigma_theta) with angles in degrees; then T_0,
// delta; then per spectral set the interpolated emissivity[c], albedo[c], C1,
// C2, C3 and solar irradiance.
//
// Determinism: pixels are cut into fixed 128-pixel tiles; one block reduces a
// tile with a fixed shuffle tree and writes its partial vector to
// partials[tile]; a second kernel sums the tiles in a fixed order.  The result
// depends neither on the grid size nor on which SM ran which tile.
#pragma once

#include "zl_f32.cuh"

namespace zl {

constexpr float kLn2 = 0.6931471805599453f;
constexpr float kDeg = 0.017453292519943295f;  // d(rad)/d(deg)
constexpr int kTile = 128;

template <uint32_t LAYOUT, int NSPEC>
struct GradLay {
  using L = Lay<LAYOUT>;
  static constexpr int NC = L::ncomp();
  __host__ __device__ static constexpr int npar(int t) {
    return t == ZL_CLOUD ? 10 : (t == ZL_BAND ? 10 : (t == ZL_RING ? 9 : 11));
  }
  __host__ __device__ static constexpr int off(int c) {
    int o = 0;
    for (int j = 0; j < c; ++j) o += npar(L::type(j));
    return o;
  }
  static constexpr int NCP = off(NC);
  static constexpr int T0 = NCP, DELTA = NCP + 1;
  static constexpr int PER_SPEC = 2 * NC + 4;
  __host__ __device__ static constexpr int spec0(int s) { return NCP + 2 + s * PER_SPEC; }
  __host__ __device__ static constexpr int eps(int c, int s) { return spec0(s) + c; }
  __host__ __device__ static constexpr int alb(int c, int s) { return spec0(s) + NC + c; }
  __host__ __device__ static constexpr int C(int j, int s) { return spec0(s) + 2 * NC + j; }  // C1, C2, C3, S
  static constexpr int NG = NCP + 2 + NSPEC * PER_SPEC;
};

// True when component c is the last component of its LOS range among those in MASK.
template <uint32_t LAYOUT, uint32_t MASK>
__host__ __device__ constexpr bool last_of_range(int c) {
  for (int j = c + 1; j < Lay<LAYOUT>::ncomp(); ++j)
    if ((MASK >> j) & 1u) return Lay<LAYOUT>::range(j) != Lay<LAYOUT>::range(c);
  return true;
}

// Entries of the gradient vector a launch with component mask MASK writes: its
// components' own parameters, T_0 and delta, its components' emissivities and
// albedos, and with scattering the phase function and irradiance of every set.
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT>
__host__ __device__ constexpr bool grad_used(int j) {
  using G = GradLay<LAYOUT, NSPEC>;
  if (j == G::T0 || j == G::DELTA) return true;
  for (int c = 0; c < Lay<LAYOUT>::ncomp(); ++c) {
    if (!((MASK >> c) & 1u)) continue;
    if (j >= G::off(c) && j < G::off(c) + G::npar(Lay<LAYOUT>::type(c))) return true;
    for (int s = 0; s < NSPEC; ++s)
      if (j == G::eps(c, s) || j == G::alb(c, s)) return true;
  }
  if (SCAT)
    for (int s = 0; s < NSPEC; ++s)
      for (int k = 0; k < 4; ++k)
        if (j == G::C(k, s)) return true;
  return false;
}

// Per-pixel quantities of the adjoint (constant over the quadrature nodes).
template <int NC, int NSPEC>
struct BwdPix {
  ff hs_r[ZL_MAX_RANGES], mid_r[ZL_MAX_RANGES];  // (stop - start)/2 and (stop + start)/2 per LOS range
  ff beta_h;                                     // obs . u
  float uxf, uyf, uzf, oxf, oyf, ozf, bperp;
  // squared impact parameters: |X|^2 = (R_los + obs . u)^2 + b2h about the Sun, and
  // |X - X_0|^2 = (R_los + bc)^2 + b2c about an offset component's centre (bc = (obs - X_0) . u;
  // set with compiled flags only: with run-time flags comp_terms forms X - X_0 itself)
  float b2h;
  float bc[NC], b2c[NC];
  float un_c[NC], on_c[NC];                      // u . n_c and (obs - X_0,c) . n_c
  float rux[NC], ruy[NC], rox[NC], roy[NC];      // the feature's rotated u and obs - X_0
  float eqx[NC], eqy[NC];                        // d atan2(E - X_0) / d x_0, d y_0
  float gup[NC][NSPEC];                          // upstream gradient times (stop - start)/2
  ff wa_c[NC], wb_c[NC];                         // ring/feature: R^2 - R0^2 = (w - w0)(w + w0) + rr_c
  float rr_c[NC];
};

// What the adjoint's pixel set-up derives from the observer (and Earth) alone, for the
// components in MASK: shared by the pixels of a block that have the same observer
// (bwd_obs_setup once per block, bwd_pixel_setup_obs per pixel; pixels of another observer
// derive their own, bwd_obs_setup_own).
template <int NC>
struct BwdObs {
  ff ox, oy, oz, r2;
  ff c_in[ZL_MAX_RANGES], c_out[ZL_MAX_RANGES];  // |X_obs|^2 - cutoff^2
  ff dx[NC], dy[NC], dz[NC], d2[NC];             // X_obs - X_0 and its square
  float on_c[NC];                                // (X_obs - X_0) . n
  float cph[NC], sph[NC], rox[NC], roy[NC], eqx[NC], eqy[NC];  // the feature's frame
  uint32_t outside;
};

template <uint32_t LAYOUT, uint32_t MASK, uint32_t FLAGS>
__device__ __forceinline__ void bwd_obs_setup(const KParamsF32& P, const PixObs& O,
                                              BwdObs<Lay<LAYOUT>::ncomp()>& Q) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<FLAGS>;
  constexpr int NC = L::ncomp();
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
    bool used = false;
#pragma unroll
    for (int c = 0; c < NC; ++c) used = used || (((MASK >> c) & 1u) && L::range(c) == r);
    if (used && r < nr) {
      Q.c_in[r] = ff_add(r2, ff_neg(ff{P.cut_in_hi[r], P.cut_in_lo[r]}));
      Q.c_out[r] = ff_add(r2, ff_neg(ff{P.cut_out_hi[r], P.cut_out_lo[r]}));
    }
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    Q.on_c[c] = Q.cph[c] = Q.sph[c] = Q.rox[c] = Q.roy[c] = Q.eqx[c] = Q.eqy[c] = 0.f;
    if (!((MASK >> c) & 1u)) continue;
    const KCompF32& C = P.comp[c];
    const int type = L::type(c);
    const bool off = Fl::offset(C, c);
    const ff dx = ff_add_fast(ox, ff{-C.ox, -C.ox_lo}), dy = ff_add_fast(oy, ff{-C.oy, -C.oy_lo}),
             dz = ff_add_fast(oz, ff{-C.oz, -C.oz_lo});
    Q.dx[c] = dx;
    Q.dy[c] = dy;
    Q.dz[c] = dz;
    if (c > 0 && ((MASK >> (c - 1)) & 1u) && C.same_plane_prev) {
      Q.on_c[c] = Q.on_c[c - 1];
    } else {
      const ff nx = {C.nx, C.nx_lo}, ny = {C.ny, C.ny_lo}, nz = {C.nz, C.nz_lo};
      const ff on = ff_add_fast(ff_add_fast(ff_mul_nr(dx, nx), ff_mul_nr(dy, ny)), ff_mul_nr(dz, nz));
      Q.on_c[c] = on.hi + on.lo;
    }
    Q.d2[c] = !off ? r2 : ff_add_fast(ff_add_fast(ff_mul_nr(dx, dx), ff_mul_nr(dy, dy)), ff_mul_nr(dz, dz));
    if (type == ZL_FEATURE) {
      const ff exf = ff_add_fast(ff_split(O.ex), ff{-C.ox, -C.ox_lo}), eyf = ff_add_fast(ff_split(O.ey), ff{-C.oy, -C.oy_lo});
      const float ex = exf.hi + exf.lo, ey = eyf.hi + eyf.lo;
      const float phi = atan2f(ey, ex) + C.c[6];
      float sp, cp;
      sincosf(phi, &sp, &cp);
      const float ocx = dx.hi + dx.lo, ocy = dy.hi + dy.lo;
      Q.cph[c] = cp;
      Q.sph[c] = sp;
      Q.rox[c] = cp * ocx + sp * ocy;
      Q.roy[c] = cp * ocy - sp * ocx;
      const float e2 = ex * ex + ey * ey;
      Q.eqx[c] = ey / e2;
      Q.eqy[c] = -ex / e2;
    }
  }
}

// Pixel i's adjoint set-up from its observer's (Q), for the components in MASK.
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, uint32_t FLAGS>
__device__ __forceinline__ void bwd_pixel_setup_obs(const KParamsF32& P, const double* __restrict__ u, int64_t n_pix,
                                                    const double* __restrict__ g_comps,
                                                    const double* __restrict__ g_total, int64_t i,
                                                    const BwdObs<Lay<LAYOUT>::ncomp()>& Q,
                                                    BwdPix<Lay<LAYOUT>::ncomp(), NSPEC>& B) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<FLAGS>;
  constexpr int NC = L::ncomp();
  const int nr = P.n_ranges;
  const ff ux = ff_split(u[i]), uy = ff_split(u[n_pix + i]), uz = ff_split(u[2 * n_pix + i]);
  const ff ox = Q.ox, oy = Q.oy, oz = Q.oz;
  const uint32_t outside = Q.outside;
  B.uxf = ux.hi, B.uyf = uy.hi, B.uzf = uz.hi;
  B.oxf = ox.hi, B.oyf = oy.hi, B.ozf = oz.hi;
  const ff oxux = ff_mul_nr(ox, ux), oyuy = ff_mul_nr(oy, uy);
  const ff b = ff_scale(ff_add_fast(oxux, oyuy), 2.0f);
  B.beta_h = ff_add_fast(ff_add_fast(oxux, oyuy), ff_mul_nr(oz, uz));
  // |X_obs|^2 - (u . X_obs)^2 >= 0, as the forward forms it
  const ff b2h_ff = ff_add_fast(Q.r2, ff_neg(ff_mul(B.beta_h, B.beta_h)));
  B.b2h = fmaxf(b2h_ff.hi + b2h_ff.lo, 0.f);
#pragma unroll
  for (int r = 0; r < ZL_MAX_RANGES; ++r) {
    bool used = false;
#pragma unroll
    for (int c = 0; c < NC; ++c) used = used || (((MASK >> c) & 1u) && L::range(c) == r);
    if (used && r < nr) {
      const ff st = ((outside >> (2 * r)) & 1u) ? ff{(float)kEps, 0.f} : sphere_distance_ffc(b, Q.c_in[r]);
      const ff sp = ((outside >> (2 * r + 1)) & 1u) ? ff{(float)kEps, 0.f} : sphere_distance_ffc(b, Q.c_out[r]);
      B.hs_r[r] = ff_scale(ff_add_fast(sp, ff_neg(st)), 0.5f);
      B.mid_r[r] = ff_scale(ff_add_fast(sp, st), 0.5f);
    } else {
      B.hs_r[r] = B.mid_r[r] = ff{0.f, 0.f};
    }
  }
  B.bperp = 0.f;
  if (SCAT) {
    const float cx = B.uyf * B.ozf - B.uzf * B.oyf, cy = B.uzf * B.oxf - B.uxf * B.ozf,
                cz = B.uxf * B.oyf - B.uyf * B.oxf;
    B.bperp = sqrtf(cx * cx + cy * cy + cz * cz);
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    B.un_c[c] = B.on_c[c] = 0.f;
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) B.gup[c][s] = 0.f;
    B.wa_c[c] = B.wb_c[c] = ff{0.f, 0.f};
    B.rr_c[c] = 0.f;
    B.rux[c] = B.ruy[c] = B.rox[c] = B.roy[c] = B.eqx[c] = B.eqy[c] = 0.f;
    B.bc[c] = B.b2c[c] = 0.f;
    if (!((MASK >> c) & 1u)) continue;
    const KCompF32& C = P.comp[c];
    const int type = L::type(c);
    const ff hs = B.hs_r[L::range(c)], md = B.mid_r[L::range(c)];
    const bool off = Fl::offset(C, c);
    if (off && !Fl::runtime) {  // (X_obs - X_0) . u and |X_obs - X_0|^2 - ((X_obs - X_0) . u)^2 >= 0
      const ff dx = Q.dx[c], dy = Q.dy[c], dz = Q.dz[c];
      const ff beta = ff_add_fast(ff_add_fast(ff_mul_nr(dx, ux), ff_mul_nr(dy, uy)), ff_mul_nr(dz, uz));
      const ff bb = ff_add_fast(Q.d2[c], ff_neg(ff_mul_nr(beta, beta)));
      B.bc[c] = beta.hi + beta.lo;
      B.b2c[c] = fmaxf(bb.hi + bb.lo, 0.f);
    }
    if (c > 0 && ((MASK >> (c - 1)) & 1u) && C.same_plane_prev) {  // the ring's plane, for the feature
      B.un_c[c] = B.un_c[c - 1];
    } else {
      const ff nx = {C.nx, C.nx_lo}, ny = {C.ny, C.ny_lo}, nz = {C.nz, C.nz_lo};
      const ff un = ff_add_fast(ff_add_fast(ff_mul_nr(ux, nx), ff_mul_nr(uy, ny)), ff_mul_nr(uz, nz));
      B.un_c[c] = un.hi + un.lo;
    }
    B.on_c[c] = Q.on_c[c];
    const float hsf = hs.hi + hs.lo;
#pragma unroll
    for (int s = 0; s < NSPEC; ++s)
      B.gup[c][s] =
          d2f_bits(g_comps ? g_comps[((int64_t)s * NC + c) * n_pix + i] : g_total[(int64_t)s * n_pix + i]) * hsf;
    if (type == ZL_RING || type == ZL_FEATURE) {
      const ff dx = Q.dx[c], dy = Q.dy[c], dz = Q.dz[c];
      const ff beta =
          !off ? B.beta_h : ff_add_fast(ff_add_fast(ff_mul_nr(dx, ux), ff_mul_nr(dy, uy)), ff_mul_nr(dz, uz));
      const ff wm = ff_add_fast(md, beta);
      const ff cw = ff_add_fast(ff_add_fast(Q.d2[c], ff_neg(ff_mul_nr(beta, beta))), ff_neg(ff{C.c[4], C.c[5]}));
      const ff w0 = cw.hi < 0.f ? ff_sqrt(ff_neg(cw)) : ff{0.f, 0.f};
      B.wa_c[c] = ff_add_fast(wm, ff_neg(w0));
      B.wb_c[c] = ff_add_fast(wm, w0);
      const ff res = ff_add_fast(ff_mul_nr(w0, w0), cw);
      B.rr_c[c] = res.hi + res.lo;
    }
    if (type == ZL_FEATURE) {
      const float cp = Q.cph[c], sp = Q.sph[c];
      B.rux[c] = cp * B.uxf + sp * B.uyf;
      B.ruy[c] = cp * B.uyf - sp * B.uxf;
      B.rox[c] = Q.rox[c];
      B.roy[c] = Q.roy[c];
      B.eqx[c] = Q.eqx[c];
      B.eqy[c] = Q.eqy[c];
    }
  }
}

// The adjoint's observer set-up of pixel i, out of line (see observer_setup_own).
template <uint32_t LAYOUT, uint32_t MASK, uint32_t FLAGS>
__device__ __noinline__ void bwd_obs_setup_own(const KParamsF32& P, const ObsArgs& OA, int64_t i, int64_t n_pix,
                                               BwdObs<Lay<LAYOUT>::ncomp()>* Q) {
  bwd_obs_setup<LAYOUT, MASK, FLAGS>(P, pixel_observer(OA, i, n_pix), *Q);
}

// Pixel i's adjoint set-up: from its block's shared observer set-up when it has the same
// observer (obs_cache_hit), else from its own.
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, uint32_t FLAGS>
__device__ __forceinline__ void bwd_pixel_setup_cached(const KParamsF32& P, const double* __restrict__ u,
                                                       int64_t n_pix, const ObsArgs& OA,
                                                       const double* __restrict__ g_comps,
                                                       const double* __restrict__ g_total, int64_t i, int cached,
                                                       const BwdObs<Lay<LAYOUT>::ncomp()>& shared,
                                                       BwdPix<Lay<LAYOUT>::ncomp(), NSPEC>& B) {
  BwdObs<Lay<LAYOUT>::ncomp()> own;
  const BwdObs<Lay<LAYOUT>::ncomp()>* q = &shared;
  if (!(cached >= 0 && (OA.n_rec == 1 || find_observer(OA.rec, OA.n_rec, i) == cached))) {
    bwd_obs_setup_own<LAYOUT, MASK, FLAGS>(P, OA, i, n_pix, &own);
    q = &own;
  }
  bwd_pixel_setup_obs<LAYOUT, MASK, NSPEC, SCAT, FLAGS>(P, u, n_pix, g_comps, g_total, i, *q, B);
}

// The observer record a block of the adjoint shares (-1: none): a one-observer call's record,
// or the record of the block's first tile's first pixel.  Block-uniform.
__device__ __forceinline__ int bwd_obs_cache_index(const ObsArgs& OA, int64_t first_pixel, int64_t n_pix) {
  if (!OA.rec) return -1;
  if (OA.n_rec == 1) return 0;
  if (first_pixel >= n_pix) return -1;
  return find_observer(OA.rec, OA.n_rec, first_pixel);
}

// One LOS range at one quadrature node: position, distance from the Sun, grain
// temperature, blackbody value and slope per spectral set, scattering terms.
template <int NSPEC>
struct NodeR {
  float Rl, R2, rinv, R, lg2R, Tn, T, flux, theta;
  float Bv[NSPEC], dB[NSPEC], sf[NSPEC], base[NSPEC], eC3[NSPEC];
};

// NEWTON: one Newton step on 1/R (the cloud and the bands use R^-1 directly).
template <int NSPEC, bool SCAT, int NC>
__device__ __forceinline__ void node_range(const KParamsF32& P, const BwdPix<NC, NSPEC>& B, int r, bool newton, ff xk,
                                           const float4* __restrict__ tab_sm, int nT, NodeR<NSPEC>& N) {
  N.Rl = node_position(B.hs_r[r], xk, B.mid_r[r]);
  const float w = N.Rl + B.beta_h.hi;  // |X|^2 = w^2 + b^2 without forming X (no cancellation)
  N.R2 = fmaf(w, w, B.b2h);
  N.rinv = rsqrt_ftz(N.R2);
  if (newton) N.rinv = N.rinv * fmaf(-0.5f * N.R2, N.rinv * N.rinv, 1.5f);
  N.R = N.R2 * N.rinv;
  N.lg2R = lg2_ftz(N.R);
  N.Tn = ex2_ftz(P.neg_delta * N.lg2R);
  N.T = P.T0 * N.Tn;
#pragma unroll
  for (int s = 0; s < NSPEC; ++s) {
    const float2 bd = bb_lookup_d(tab_sm + s * nT, N.T, P.t_min, P.t_max, P.inv_dt, nT);
    N.Bv[s] = bd.x;
    N.dB[s] = bd.y;
  }
  N.theta = N.flux = 0.f;
#pragma unroll
  for (int s = 0; s < NSPEC; ++s) N.sf[s] = N.base[s] = N.eC3[s] = 0.f;
  if (SCAT) {
    N.theta = atan2_poly(B.bperp, -(N.Rl + B.beta_h.hi));
    N.flux = N.rinv * N.rinv;
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      const KSpecF32& S = P.spec[s];
      N.eC3[s] = ex2_ftz(S.C3l2e * N.theta);
      N.base[s] = S.C1 + S.C2 * N.theta + N.eC3[s];
      N.sf[s] = S.S * N.flux * (S.N * N.base[s]);
    }
  }
}

// Density of one component at a node (without n_0) and its log-derivatives:
// GR = d ln n / d R_c, GZ = d ln n / d Z, p6.. = d ln n / d (own parameters) without
// their pixel-constant factors, which multiply the node sums once (comp_pfactors).
struct CompTerms {
  float du, GR, GZ, rcinv, p6, p7, p8, p9, p10, dthx, dthy;
};

// t4s / y4s: a band's 1 - e^-y and y d ln(1 - e^-y)/dy, reused by equal bands.  in4 false: the
// node lies outside the warp's inner-cutoff range (cutoff_interval), where they are 1.0f and +0.
template <uint32_t LAYOUT, uint32_t MASK, uint32_t FLAGS, int NC, int NSPEC>
__device__ __forceinline__ CompTerms comp_terms(int c, const KParamsF32& P, const KGradAux& A,
                                                const BwdPix<NC, NSPEC>& B, ff xk, const NodeR<NSPEC>& N,
                                                float* t4s, float* y4s, bool in4 = true) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<FLAGS>;
  const KCompF32& C = P.comp[c];
  const int type = L::type(c);
  CompTerms t;
  t.p6 = t.p7 = t.p8 = t.p9 = t.p10 = t.dthx = t.dthy = 0.f;
  // component frame: |X - X_0|, height above the symmetry plane
  float Rc2 = N.R2, rcinv = N.rinv, Rc = N.R, lg2Rc = N.lg2R;
  if (Fl::offset(C, c)) {
    if (Fl::runtime) {  // any component may be offset: X - X_0 from the node position (fewer registers)
      const float Xc0 = fmaf(N.Rl, B.uxf, B.oxf - C.ox), Xc1 = fmaf(N.Rl, B.uyf, B.oyf - C.oy),
                  Xc2 = fmaf(N.Rl, B.uzf, B.ozf - C.oz);
      Rc2 = fmaf(Xc0, Xc0, fmaf(Xc1, Xc1, Xc2 * Xc2));
    } else {
      const float wc = N.Rl + B.bc[c];
      Rc2 = fmaf(wc, wc, B.b2c[c]);
    }
    rcinv = rsqrt_ftz(Rc2);
    if (type == ZL_BAND) rcinv = rcinv * fmaf(-0.5f * Rc2, rcinv * rcinv, 1.5f);
    Rc = Rc2 * rcinv;
    lg2Rc = 0.5f * lg2_ftz(Rc2);
  }
  t.rcinv = rcinv;
  const float Z = fmaf(N.Rl, B.un_c[c], B.on_c[c]);
  const float aZ = fabsf(Z);
  const float* q = A.q[c];
  if (type == ZL_CLOUD) {
    // q: alpha, beta, gamma, mu, 1/mu
    const float zeta = aZ * rcinv;
    const bool in = zeta < q[3];
    const float g = in ? zeta * zeta * C.c[5] : zeta - C.c[6];
    const float lgg = lg2_ftz(g);
    const float gg = ex2_ftz(q[2] * lgg);
    t.du = ex2_ftz(-q[0] * lg2Rc - C.c[2] * gg);
    const float bgg = q[1] * q[2] * gg;
    // one reciprocal: 2 / zeta inside the widening (in), 1 / g outside (g > 0 where used)
    const float rg = __fdividef(1.f, in ? 0.5f * zeta : g);
    const float Az = zeta > 0.f ? bgg * rg : 0.f;
    t.GR = (-q[0] + Az * zeta) * rcinv;
    t.GZ = -copysignf(Az, Z) * rcinv;
    // outside the widening g = zeta - mu/2 > 0 and zeta > 0, so d/dmu there is Az / 2
    t.p6 = lg2Rc;                            // d/d alpha = -ln 2 lg2 R
    t.p7 = gg;                               // d/d beta = -g^gamma
    t.p8 = g > 0.f ? gg * lgg : 0.f;         // d/d gamma = -beta ln 2 g^gamma lg2 g
    t.p9 = in ? bgg * (2.f * q[4]) : Az;     // d/d mu (x 1/2)
  } else if (type == ZL_BAND) {
    // q: delta_zeta [deg], v, p, delta_r, 1/delta_zeta [deg], -20/delta_r
    const float x = aZ * rcinv * C.c[1];
    const float x2 = x * x, x6 = x2 * x2 * x2;
    const float t2 = ex2_ftz(-kLog2e * x6);
    const float lgx = lg2_ftz(x);
    const float xp = Fl::p4(C, c) ? x2 * x2 : ex2_ftz(q[2] * lgx);
    const float xpv = xp * C.c[2];
    const float t3 = 1.f + xpv;
    float t4 = 0.f, Y4 = 0.f;
    bool shared = false;
    if (Fl::runtime) {
#pragma unroll
      for (int j = 0; j < NC; ++j)
        if (j < c && C.share_t4 == j && ((MASK >> j) & 1u)) {
          t4 = t4s[j];
          Y4 = y4s[j];
          shared = true;
        }
    } else if (Fl::share_first(c) && ((MASK >> L::first_band(c)) & 1u)) {
      t4 = t4s[L::first_band(c)];
      Y4 = y4s[L::first_band(c)];
      shared = true;
    }
    if (!shared && !in4) {
      t4 = 1.f;
      Y4 = 0.f;
    } else if (!shared) {
      const float qq = Rc2 * C.c[4];
      const float qq2 = qq * qq, qq4 = qq2 * qq2, qq8 = qq4 * qq4;
      const float y = qq8 * qq2;
      const float emy = ex2_ftz(-kLog2e * y);
      t4 = y < 0.25f ? y * (1.f - y * (0.5f - y * (1.f / 6.f - y * (1.f / 24.f - y * (1.f / 120.f - y * (1.f / 720.f))))))
                     : 1.f - emy;
      Y4 = t4 > 0.f ? y * emy * __fdividef(1.f, t4) : 1.f;  // y d ln(1 - e^-y) / d y
    }
    t4s[c] = t4;
    y4s[c] = Y4;
    t.du = rcinv * t2 * t3 * t4;  // the factor 3 of 3 n_0 is in A.n0 (and in d/dn_0 below)
    const float it3 = __fdividef(1.f, t3);
    const float xit = xpv * it3;
    const float Sx = -6.f * x6 + q[2] * xit;  // x d ln n / d x
    t.GR = (-1.f - Sx + 20.f * Y4) * rcinv;
    t.GZ = aZ > 0.f ? __fdividef(Sx, Z) : 0.f;  // Sx sign(Z) / |Z|
    t.p6 = Sx;                                   // d/d delta_zeta = -Sx / delta_zeta
    t.p7 = xit;                                  // d/d v = -xit / v
    t.p8 = x > 0.f ? xit * lgx : 0.f;            // d/d p = ln 2 xit lg2 x
    t.p9 = Y4;                                   // d/d delta_r = -20 Y4 / delta_r
  } else {
    // q: R, 1/sigma_r^2, 1/sigma_z, 2/sigma_r^3, 1/sigma_z^2, 1/sigma_theta^2, 2 deg/sigma_theta^3
    float dR = Rc - q[0];
    const ff hs = B.hs_r[L::range(c)];
    const float D2 = fmaf(lin_ff(hs, xk, B.wa_c[c]), lin_ff(hs, xk, B.wb_c[c]), B.rr_c[c]);
    dR = dR + (D2 - dR * (Rc + q[0])) * (0.5f * rcinv);
    float arg = dR * dR * q[1] + aZ * q[2];
    t.GR = -2.f * dR * q[1];
    t.GZ = Z != 0.f ? -copysignf(q[2], Z) : 0.f;
    t.p6 = t.GR;             // d/d R = -GR
    t.p7 = dR * dR;          // d/d sigma_r = 2 dR^2 / sigma_r^3
    t.p8 = aZ;               // d/d sigma_z = |Z| / sigma_z^2
    if (type == ZL_FEATURE) {
      const float dth = atan2_poly(fmaf(N.Rl, B.ruy[c], B.roy[c]), fmaf(N.Rl, B.rux[c], B.rox[c]));
      arg = fmaf(dth * dth, q[5], arg);
      const float gth = -2.f * dth * q[5];  // d ln n / d dtheta
      t.p9 = dth;                           // d/d theta = -gth pi/180 = 2 dth pi/180 / sigma_theta^2
      t.p10 = dth * dth;                    // d/d sigma_theta = 2 dth^2 / sigma_theta^3 per degree
      const float Xc0 = fmaf(N.Rl, B.uxf, B.oxf - C.ox), Xc1 = fmaf(N.Rl, B.uyf, B.oyf - C.oy);  // X - X_0
      const float rr = __fdividef(1.f, Xc0 * Xc0 + Xc1 * Xc1);
      t.dthx = gth * (Xc1 * rr - B.eqx[c]);
      t.dthy = gth * (-Xc0 * rr - B.eqy[c]);
    }
    t.du = ex2_ftz(-kLog2e * arg);
  }
  return t;
}

// The T_0 / delta sums of a LOS range: wq (sum over the range's components of w n E_T, or
// of w n K with one spectral set and no scattering) times dT/dT_0 and dT/d delta.
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, int NG>
__device__ __forceinline__ void range_flush(const NodeR<NSPEC>& N, float& wq, float (&acc)[NG]) {
  using G = GradLay<LAYOUT, NSPEC>;
  constexpr bool KF = NSPEC == 1 && !SCAT;
  if (KF) wq *= N.dB[0];
  acc[G::T0] = fmaf(wq, N.Tn, acc[G::T0]);
  acc[G::DELTA] = fmaf(-wq * N.T, N.lg2R * kLn2, acc[G::DELTA]);
  wq = 0.f;
}

// Node sums of one component.  The emission per spectral set and its upstream-weighted
// sums E = sum_s g_s e_s and Q = sum_s g_s em1_s dB_s/dT: with one spectral set and no
// scattering (KF) both are K B and K dB/dT with K = g em1 constant over the pixel's
// nodes; the sums then run without K and the pixel's K scales them after the loop.
// wq: sum over a range's components of w n E_T (the T_0 / delta derivatives), flushed
// into acc by the range's last component.
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, int NC, int NG>
__device__ __forceinline__ void comp_accumulate(int c, const KParamsF32& P, const KGradAux& A,
                                                const BwdPix<NC, NSPEC>& B, float wk, const NodeR<NSPEC>& N,
                                                const CompTerms& t, const float* kpix, float& wq, float* fthx,
                                                float* fthy, float (&acc)[NG]) {
  using L = Lay<LAYOUT>;
  using G = GradLay<LAYOUT, NSPEC>;
  constexpr bool KF = NSPEC == 1 && !SCAT;
  const int type = L::type(c);
  float E = 0.f, Q = 0.f;
  if (!KF) {
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      const KSpecF32& S = P.spec[s];
      const float ev = SCAT ? fmaf(S.alb[c], N.sf[s], S.em1[c] * N.Bv[s]) : S.em1[c] * N.Bv[s];
      E = fmaf(B.gup[c][s], ev, E);
      Q = fmaf(B.gup[c][s] * S.em1[c], N.dB[s], Q);
    }
  }
  const float wdu = wk * t.du;      // w * density / n_0
  const float wd = wdu * A.n0[c];  // w * density; the upstream gradient is in E and Q
  const float coef = KF ? wd * N.Bv[0] : wd * E;
  const int o = G::off(c);
  const float gRr = t.GR * t.rcinv;
  const float cG = coef * gRr, cZ = coef * t.GZ;
  acc[o + 0] = fmaf(cG, N.Rl, acc[o + 0]);  // sum coef g_R R_los
  acc[o + 1] += cG;                         // sum coef g_R
  acc[o + 2] += cZ;                         // sum coef g_Z
  acc[o + 3] = fmaf(cZ, N.Rl, acc[o + 3]);  // sum coef g_Z R_los
  if (type == ZL_FEATURE) {
    fthx[c] = fmaf(coef, t.dthx, fthx[c]);
    fthy[c] = fmaf(coef, t.dthy, fthy[c]);
  }
  acc[o + 5] = fmaf(wdu, KF ? N.Bv[0] : E, acc[o + 5]);
  acc[o + 6] += coef * t.p6;
  acc[o + 7] += coef * t.p7;
  acc[o + 8] += coef * t.p8;
  if (type != ZL_RING) acc[o + 9] += coef * t.p9;
  if (type == ZL_FEATURE) acc[o + 10] += coef * t.p10;
  wq = KF ? fmaf(wd, kpix[c], wq) : fmaf(wd, Q, wq);
  if (last_of_range<LAYOUT, MASK>(c)) range_flush<LAYOUT, MASK, NSPEC, SCAT>(N, wq, acc);
#pragma unroll
  for (int s = 0; s < NSPEC; ++s) {
    const KSpecF32& S = P.spec[s];
    // per node only sum w n B and w n S_flux; the pixel's constant factors follow the loop
    // (with KF, sum w n B = n_0 acc[o + 5]: bwd_finalize forms it from that sum)
    if (!KF) acc[G::eps(c, s)] = fmaf(wd, N.Bv[s], acc[G::eps(c, s)]);
    if (SCAT) acc[G::alb(c, s)] = fmaf(wd, N.sf[s], acc[G::alb(c, s)]);
    if (SCAT) {
      const float wg = wd * B.gup[c][s];
      const float af = wg * S.alb[c] * N.flux;
      acc[G::C(3, s)] += af * S.N * N.base[s];
      const float as = af * S.S;
      acc[G::C(0, s)] += as * (S.N + N.base[s] * A.dN[s][0]);
      acc[G::C(1, s)] += as * (S.N * N.theta + N.base[s] * A.dN[s][1]);
      acc[G::C(2, s)] += as * (S.N * N.theta * N.eC3[s] + N.base[s] * A.dN[s][2]);
    }
  }
}

// Pixel-constant factors of the node sums acc[off + 6 ..] (comp_terms returns the
// log-derivatives without them).
// q: cloud alpha, beta, gamma, mu, 1/mu; band delta_zeta [deg], v, p, delta_r,
// 1/delta_zeta [deg], -20/delta_r; ring/feature R, 1/sigma_r^2, 1/sigma_z,
// 2/sigma_r^3, 1/sigma_z^2, 1/sigma_theta^2, 2 deg/sigma_theta^3.
__device__ __forceinline__ void comp_pfactors(int type, const float* q, const KCompF32& C, float (&f)[5]) {
  if (type == ZL_CLOUD) {
    f[0] = -kLn2, f[1] = -1.f, f[2] = -q[1] * kLn2, f[3] = 0.5f, f[4] = 0.f;
  } else if (type == ZL_BAND) {
    f[0] = -q[4], f[1] = -C.c[2], f[2] = kLn2, f[3] = q[5], f[4] = 0.f;
  } else {
    f[0] = -1.f, f[1] = q[3], f[2] = q[4], f[3] = 2.f * q[5] * kDeg, f[4] = q[6];
  }
}

// After the node loop: d/dx_0..z_0 = -sum coef g_R (X - X_0)/R - n sum coef g_Z (+ the
// feature's longitude term); d/di, d/dOmega = sum coef g_Z (X - X_0) . dn;
// d/d eps = g (1 - A) sum w n B,  d/d A = g (sum w n S_flux - eps sum w n B).
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, int NC, int NG>
__device__ __forceinline__ void bwd_finalize(const KParamsF32& P, const KGradAux& A, const BwdPix<NC, NSPEC>& B,
                                             const float* kpix, float* fthx, float* fthy, float (&acc)[NG]) {
  using L = Lay<LAYOUT>;
  using G = GradLay<LAYOUT, NSPEC>;
  constexpr bool KF = NSPEC == 1 && !SCAT;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    if (!((MASK >> c) & 1u)) continue;
    const KCompF32& C = P.comp[c];
    const int o = G::off(c);
    {
      float f[5];
      comp_pfactors(L::type(c), A.q[c], C, f);
#pragma unroll
      for (int j = 6; j < G::npar(L::type(c)); ++j) acc[o + j] *= f[j - 6];
    }
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      // sum w n B: with KF it is n_0 sum w (n / n_0) B, the node sum acc[o + 5] (not yet scaled)
      const float sB = KF ? A.n0[c] * acc[o + 5] : acc[G::eps(c, s)], sS = SCAT ? acc[G::alb(c, s)] : 0.f;
      acc[G::eps(c, s)] = B.gup[c][s] * A.one_m_alb[s][c] * sB;
      acc[G::alb(c, s)] = B.gup[c][s] * fmaf(-A.eps[s][c], sB, sS);
    }
    // with KF the coefficient sums lack the pixel factor K = g em1 (see the node loop)
    const float kf = KF ? kpix[c] : 1.f;
    if (KF) {
#pragma unroll
      for (int j = 5; j < G::npar(L::type(c)); ++j) acc[o + j] *= kf;
      fthx[c] *= kf;
      fthy[c] *= kf;
    }
    if (L::type(c) == ZL_BAND) acc[o + 5] *= 3.f;  // d/dn_0 of 3 n_0 (...)
    const float s1 = kf * acc[o + 0], s2 = kf * acc[o + 1], s3 = kf * acc[o + 2], s4 = kf * acc[o + 3];
    const float dxc = B.oxf - C.ox, dyc = B.oyf - C.oy, dzc = B.ozf - C.oz;
    acc[o + 0] = -fmaf(B.uxf, s1, dxc * s2) - C.nx * s3 + fthx[c];
    acc[o + 1] = -fmaf(B.uyf, s1, dyc * s2) - C.ny * s3 + fthy[c];
    acc[o + 2] = -fmaf(B.uzf, s1, dzc * s2) - C.nz * s3;
    const float ui = B.uxf * A.dni[c][0] + B.uyf * A.dni[c][1] + B.uzf * A.dni[c][2];
    const float di = dxc * A.dni[c][0] + dyc * A.dni[c][1] + dzc * A.dni[c][2];
    const float uO = B.uxf * A.dnO[c][0] + B.uyf * A.dnO[c][1];
    const float dO = dxc * A.dnO[c][0] + dyc * A.dnO[c][1];
    acc[o + 3] = fmaf(ui, s4, di * s3);
    acc[o + 4] = fmaf(uO, s4, dO * s3);
  }
}

// The entries of the gradient vector a launch writes (grad_used), in order, as a
// compile-time list: the tile reduction's slots.
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT>
struct UsedGrads {
  static constexpr int NG = GradLay<LAYOUT, NSPEC>::NG;
  int idx[NG];
  int n;
  __host__ __device__ constexpr UsedGrads() : idx{}, n(0) {
    for (int j = 0; j < NG; ++j)
      if (grad_used<LAYOUT, MASK, NSPEC, SCAT>(j)) idx[n++] = j;
  }
};

// Block start: the blackbody tables into shared memory; the reduction rows zeroed
// (entries the launch never writes stay zero); the list of written entries (used_sm).
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, int NG>
__device__ __forceinline__ void bwd_block_init(const KParamsF32& P, float4* tab_sm, float (*red_sm)[NG],
                                               int* used_sm) {
  constexpr UsedGrads<LAYOUT, MASK, NSPEC, SCAT> U{};
  const int nT = P.n_temps;
  for (int t = threadIdx.x; t < nT * NSPEC; t += blockDim.x) tab_sm[t] = P.table[t / nT][t % nT];
  for (int t = threadIdx.x; t < (kTile / 32) * NG; t += blockDim.x) red_sm[t / NG][t % NG] = 0.f;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int t = 0; t < U.n; ++t) used_sm[t] = U.idx[t];
  }
  __syncthreads();
}

// One level of the warp's transposed reduction: each lane holds 2H partial sums; the lanes with
// (lane & M) keep the upper H, the others the lower H, and each adds its partner's copy of the
// slots it keeps (one shuffle per kept slot instead of one per slot and level).  Slot j's
// partner slot H + j is padding on every lane when H + j >= K: then only the lower lane's sum
// is needed, and the upper lane's (a padding slot) is left as whatever it adds up to.
template <int M, int H, int K>
__device__ __forceinline__ void warp_halve(float* v, bool up) {
#pragma unroll
  for (int j = 0; j < H; ++j) {
    if (H + j >= K) {
      v[j] += __shfl_xor_sync(0xffffffffu, v[j], M);
    } else {
      const float send = up ? v[j] : v[H + j];
      const float keep = up ? v[H + j] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, M);
    }
  }
}

// Tile reduction: the written entries, packed into 32 W slots per lane, summed over the warp by
// recursive halving (lane L ends with the warp's sums of slots L W .. L W + W - 1), then the
// warps in order.
template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, int NG>
__device__ __forceinline__ void bwd_tile_reduce(const float (&acc)[NG], float (*red_sm)[NG], const int* used_sm,
                                                double* __restrict__ partials, int64_t tile) {
  constexpr UsedGrads<LAYOUT, MASK, NSPEC, SCAT> U{};
  constexpr int K = U.n, W = (K + 31) / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float v[32 * W];
#pragma unroll
  for (int t = 0; t < 32 * W; ++t) v[t] = t < K ? acc[U.idx[t]] : 0.f;
  warp_halve<16, 16 * W, K>(v, lane & 16);
  warp_halve<8, 8 * W, K>(v, lane & 8);
  warp_halve<4, 4 * W, K>(v, lane & 4);
  warp_halve<2, 2 * W, K>(v, lane & 2);
  warp_halve<1, W, K>(v, lane & 1);
#pragma unroll
  for (int t = 0; t < W; ++t) {
    const int g = lane * W + t;
    if (g < K) red_sm[warp][used_sm[g]] = v[t];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < NG; j += blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kTile / 32; ++w) s += (double)red_sm[w][j];
    partials[tile * NG + j] = s;
  }
  __syncthreads();
}

// MASK selects the components this launch differentiates (bit c = component c).
// A model's components are split into groups that each own their LOS ranges, so
// every group launch carries only its own accumulators; parameters shared by
// all components (T_0, delta, C1..C3, S) are summed over the groups' partials.
// SCAT: some component has a non-zero albedo (scattering terms are evaluated).
// The scalar adjoint takes inner-cutoff ranges with compiled flags, no scattering and every band of
// the launch centred on the Sun (the range is estimated from the range's heliocentric geometry).
template <uint32_t LAYOUT, uint32_t MASK, uint32_t FLAGS, bool SCAT>
__host__ __device__ constexpr bool kCutRanges() {
  if (SCAT || FLAGS == kFlagsRuntime) return false;
  bool any = false;
  for (int c = 0; c < Lay<LAYOUT>::ncomp(); ++c)
    if (((MASK >> c) & 1u) && Lay<LAYOUT>::type(c) == ZL_BAND) {
      if ((FLAGS >> (8 + c)) & 1u) return false;
      any = true;
    }
  return any;
}

template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, bool SCAT, uint32_t FLAGS>
__global__ void __launch_bounds__(kTile) bwd_f32_kernel(const __grid_constant__ KParamsF32 P,
                                                        const __grid_constant__ KGradAux A,
                                                        const double* __restrict__ u, int64_t n_pix,
                                                        const ObsArgs OA,
                                                        const double* __restrict__ g_comps,
                                                        const double* __restrict__ g_total,
                                                        double* __restrict__ partials, int64_t n_tiles) {
  using L = Lay<LAYOUT>;
  using G = GradLay<LAYOUT, NSPEC>;
  constexpr bool KF = NSPEC == 1 && !SCAT;  // the upstream factor K = g em1 leaves the node loop
  constexpr int NC = L::ncomp();
  constexpr int NG = G::NG;
  __shared__ float4 tab_sm[NSPEC * ZL_MAX_TEMPS];
  __shared__ float red_sm[kTile / 32][NG];
  __shared__ int used_sm[NG];
  __shared__ BwdObs<NC> s_obs;  // the observer set-up the block's pixels share
  const int cached = bwd_obs_cache_index(OA, (int64_t)blockIdx.x * kTile, n_pix);
  if (threadIdx.x == 0 && cached >= 0) bwd_obs_setup<LAYOUT, MASK, FLAGS>(P, record_observer(OA, cached), s_obs);
  bwd_block_init<LAYOUT, MASK, NSPEC, SCAT>(P, tab_sm, red_sm, used_sm);  // its barrier also publishes s_obs
  const int nT = P.n_temps;

  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t i = tile * kTile + threadIdx.x;
    float acc[NG];
#pragma unroll
    for (int j = 0; j < NG; ++j) acc[j] = 0.f;

    if (i < n_pix) {
      BwdPix<NC, NSPEC> B;
      bwd_pixel_setup_cached<LAYOUT, MASK, NSPEC, SCAT, FLAGS>(P, u, n_pix, OA, g_comps, g_total, i, cached, s_obs, B);
      // Offset and orientation derivatives: with X - X_0 = R_los u + (X_obs - X_0) they are
      // combinations of four per-node sums per component, completed after the node loop.
      float fthx[NC], fthy[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) fthx[c] = fthy[c] = 0.f;
      float wq = 0.f;
      float kpix[NC];  // K = g em1 per component (one spectral set, no scattering)
#pragma unroll
      for (int c = 0; c < NC; ++c) kpix[c] = KF ? B.gup[c][0] * P.spec[0].em1[c] : 0.f;
      // nodes at which the bands' inner-cutoff factor and its log-derivative may differ from 1.0f
      // and +0 for some pixel of the warp (compiled flags, bands centred on the Sun, no scattering)
      int2 r4 = make_int2(0, P.n_nodes);
      if (kCutRanges<LAYOUT, MASK, FLAGS, SCAT>()) {
        const float bt = B.beta_h.hi, b2h = B.b2h;
        float x1 = INFINITY, x2 = -INFINITY;
#pragma unroll
        for (int c = 0; c < NC; ++c)
          if (((MASK >> c) & 1u) && L::type(c) == ZL_BAND) {
            const int r = L::range(c);
            const float2 iv = cutoff_interval(B.hs_r[r].hi, B.mid_r[r].hi + bt, b2h, P.comp[c].c[4]);
            x1 = fminf(x1, iv.x);
            x2 = fmaxf(x2, iv.y);
          }
        r4 = warp_node_range(P, x1, x2);
      }

#pragma unroll 1
      for (int k = 0; k < P.n_nodes; ++k) {
        const ff xk = {P.gl_x_hi[k], P.gl_x_lo[k]};
        const float wk = P.gl_w[k];
        const bool in4 = k >= r4.x && k < r4.y;
        NodeR<NSPEC> N;
        float t4s[NC], y4s[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) t4s[c] = y4s[c] = 0.f;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if (!((MASK >> c) & 1u)) continue;
          const int type = L::type(c);
          if (L::first(c))
            node_range<NSPEC, SCAT>(P, B, L::range(c), type == ZL_CLOUD || type == ZL_BAND, xk, tab_sm, nT, N);
          const CompTerms t = comp_terms<LAYOUT, MASK, FLAGS>(c, P, A, B, xk, N, t4s, y4s, in4);
          comp_accumulate<LAYOUT, MASK, NSPEC, SCAT>(c, P, A, B, wk, N, t, kpix, wq, fthx, fthy, acc);
        }
      }
      bwd_finalize<LAYOUT, MASK, NSPEC, SCAT>(P, A, B, kpix, fthx, fthy, acc);
    }
    bwd_tile_reduce<LAYOUT, MASK, NSPEC, SCAT>(acc, red_sm, used_sm, partials, tile);
  }
}

template <uint32_t LAYOUT, uint32_t MASK, int NSPEC, uint32_t FLAGS>
static void launch_one(bool scat, const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                       const ObsArgs& obs, const double* g_comps, const double* g_total,
                       double* partials, int64_t n_tiles, cudaStream_t st, int64_t grid) {
  if (scat)
    bwd_f32_kernel<LAYOUT, MASK, NSPEC, true, FLAGS>
        <<<(unsigned)grid, kTile, 0, st>>>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles);
  else
    bwd_f32_kernel<LAYOUT, MASK, NSPEC, false, FLAGS>
        <<<(unsigned)grid, kTile, 0, st>>>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles);
}

template <uint32_t LAYOUT, int NSPEC, uint32_t FLAGS>
static cudaError_t launch_groups(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                 const ObsArgs& obs, const double* g_comps, const double* g_total,
                                 double* partials, int64_t n_tiles, cudaStream_t st, int64_t grid) {
  const bool scat = P.has_scat != 0;
  launch_one<LAYOUT, 0x0Fu, NSPEC, FLAGS>(scat, P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  if constexpr (LAYOUT == kLayoutDirbe) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    constexpr int NG = GradLay<LAYOUT, NSPEC>::NG;
    launch_one<LAYOUT, 0x30u, NSPEC, FLAGS>(scat, P, A, u, n, obs, g_comps, g_total,
                                     partials + (size_t)n_tiles * NG, n_tiles, st, grid);
  }
  return cudaGetLastError();
}

template <uint32_t LAYOUT, uint32_t FLAGS>
static cudaError_t launch_bwd_nspec(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                    const ObsArgs& obs, const double* g_comps, const double* g_total,
                                    double* partials, int64_t n_tiles, cudaStream_t st, int64_t grid) {
  switch (P.n_spec) {
    case 1: return launch_groups<LAYOUT, 1, FLAGS>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
    case 2: return launch_groups<LAYOUT, 2, FLAGS>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
    case 3: return launch_groups<LAYOUT, 3, FLAGS>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
    default: return launch_groups<LAYOUT, 4, FLAGS>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  }
}

// The backward reads every flag but scattering (that is its SCAT parameter).
constexpr uint32_t kBwdFlagsMask = ~2u;

cudaError_t launch_bwd_f32_dirbe(const KParamsF32& P, const KGradAux& A, uint32_t flags, bool unpaired, const double* u,
                                 int64_t n, const ObsArgs& obs, const double* g_comps, const double* g_total,
                                 double* partials, int64_t n_tiles, cudaStream_t st, int64_t grid);
cudaError_t launch_bwd_f32_planck(const KParamsF32& P, const KGradAux& A, uint32_t flags, const double* u, int64_t n,
                                  const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                  int64_t n_tiles, cudaStream_t st, int64_t grid);

}  // namespace zl
