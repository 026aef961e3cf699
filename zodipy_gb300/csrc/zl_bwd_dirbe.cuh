// DIRBE-layout adjoint kernels with component pairs on packed FP32 instructions.
//
// The adjoint is bound by instruction issue like the forward.  Components whose
// per-node derivative arithmetic is the same sequence on different constants
// share packed float2 instructions (fma/mul/add.rn.f32x2), lanes .x and .y:
//   - {ring, feature} launch: the ring and the feature each run their own LOS
//     range, so the node position, distance, temperature, blackbody value and
//     slope, R - R0 and its Newton correction, Gaussian exponent, derivative
//     coefficients and every node sum pair up; the feature's longitude term
//     (atan2 and its derivatives) runs on lane .y alone;
//   - {cloud, bands} launch: bands 1 and 2 pair (plane height, e^-(zeta/dzeta)^6,
//     the (zeta/dzeta)^4 term, the inner-cutoff factor and their derivatives); the
//     cloud and band 3 (which reuses band 1's inner-cutoff term) run the scalar
//     component code of zl_bwd_f32.cuh on the shared LOS range.
// MUFU operations, table lookups and comparisons run per lane.  Each lane
// computes the quantities of the scalar kernel (bwd_f32_kernel) for its
// component; a few products are associated differently, so sums agree to float32
// rounding, not bit for bit.  Both kernels write the scalar kernel's partial-sum
// layout, so the tile reduction and the host side are shared.
//
// Built for the DIRBE layout with the built-in models' flags (cloud offset from
// the Sun, bands with p = 4, band 3 reusing band 1's inner-cutoff term).
#pragma once

#include "zl_bwd_f32.cuh"
#include "zl_packed.cuh"

namespace zl {

constexpr uint32_t kBwdFlagsKelsall = kFlagsKelsall & kBwdFlagsMask;

__device__ __forceinline__ float2 qpair(const KGradAux& A, int a, int b, int k) {
  return make_float2(A.q[a][k], A.q[b][k]);
}

// ---------------------------------------------------------------------------
// {ring, feature}: lane .x = ring (component 4), lane .y = feature (component 5)
// ---------------------------------------------------------------------------
template <int NSPEC, bool SCAT>
__global__ void __launch_bounds__(kTile) bwd_dirbe_rf_kernel(const __grid_constant__ KParamsF32 P,
                                                             const __grid_constant__ KGradAux A,
                                                             const double* __restrict__ u, int64_t n_pix,
                                                             const ObsArgs OA, const double* __restrict__ g_comps,
                                                             const double* __restrict__ g_total,
                                                             double* __restrict__ partials, int64_t n_tiles) {
  constexpr uint32_t LAYOUT = kLayoutDirbe, MASK = 0x30u, FLAGS = kBwdFlagsKelsall;
  using L = Lay<LAYOUT>;
  using G = GradLay<LAYOUT, NSPEC>;
  constexpr bool KF = NSPEC == 1 && !SCAT;
  constexpr int NC = L::ncomp(), NG = G::NG;
  constexpr int CR = 4, CF = 5, RR = L::range(CR), RF = L::range(CF);
  static_assert(L::type(CR) == ZL_RING && L::type(CF) == ZL_FEATURE && RR != RF, "DIRBE ring and feature");
  static_assert(((FLAGS >> (8 + CR)) & 3u) == 0u, "ring and feature centred on the Sun");
  __shared__ float4 tab_sm[NSPEC * ZL_MAX_TEMPS];
  __shared__ float red_sm[kTile / 32][NG];
  __shared__ int used_sm[NG];
  __shared__ BwdObs<NC> s_obs;  // the observer set-up the block's pixels share
  const int cached = bwd_obs_cache_index(OA, (int64_t)blockIdx.x * kTile, n_pix);
  if (threadIdx.x == 0 && cached >= 0) bwd_obs_setup<LAYOUT, MASK, FLAGS>(P, record_observer(OA, cached), s_obs);
  bwd_block_init<LAYOUT, MASK, NSPEC, SCAT>(P, tab_sm, red_sm, used_sm);  // its barrier also publishes s_obs
  const int nT = P.n_temps;
  const KCompF32& Cf = P.comp[CF];

  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t i = tile * kTile + threadIdx.x;
    float acc[NG];
#pragma unroll
    for (int j = 0; j < NG; ++j) acc[j] = 0.f;

    if (i < n_pix) {
      BwdPix<NC, NSPEC> B;
      bwd_pixel_setup_cached<LAYOUT, MASK, NSPEC, SCAT, FLAGS>(P, u, n_pix, OA, g_comps, g_total, i, cached, s_obs, B);
      const ff2 hsP = pack_ff(B.hs_r[RR], B.hs_r[RF]), mdP = pack_ff(B.mid_r[RR], B.mid_r[RF]);
      const ff2 waP = pack_ff(B.wa_c[CR], B.wa_c[CF]), wbP = pack_ff(B.wb_c[CR], B.wb_c[CF]);
      const float2 rrP = make_float2(B.rr_c[CR], B.rr_c[CF]);
      const float2 unP = make_float2(B.un_c[CR], B.un_c[CF]), onP = make_float2(B.on_c[CR], B.on_c[CF]);
      // q: R, 1/sigma_r^2, 1/sigma_z, 2/sigma_r^3, 1/sigma_z^2, 1/sigma_theta^2, 2 deg/sigma_theta^3
      const float2 q0 = qpair(A, CR, CF, 0), q1 = qpair(A, CR, CF, 1), q2 = qpair(A, CR, CF, 2);
      const float2 nq0 = mul2(q0, bc2(-1.f)), m2q1 = mul2(q1, bc2(-2.f));
      const float2 n0P = make_float2(A.n0[CR], A.n0[CF]);
      // per spectral set: g em1 and g alb of each lane (E and Q below)
      float2 gq[NSPEC], ga[NSPEC];
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        const KSpecF32& S = P.spec[s];
        const float2 g = make_float2(B.gup[CR][s], B.gup[CF][s]);
        gq[s] = mul2(g, make_float2(S.em1[CR], S.em1[CF]));
        ga[s] = mul2(g, make_float2(S.alb[CR], S.alb[CF]));
      }
      float kpix[NC];  // K = g em1 per component (one spectral set, no scattering)
#pragma unroll
      for (int c = 0; c < NC; ++c) kpix[c] = KF ? B.gup[c][0] * P.spec[0].em1[c] : 0.f;

      // node sums: the scalar kernel's acc[off + j] per lane (before comp_pfactors); T_0 and
      // delta per lane without the factor K (KF) and -ln 2 (delta)
      float2 s0 = bc2(0.f), s1 = bc2(0.f), s2 = bc2(0.f), s3 = bc2(0.f), s5 = bc2(0.f), s6 = bc2(0.f);
      float2 s7 = bc2(0.f), s8 = bc2(0.f), sT0 = bc2(0.f), sD = bc2(0.f);
      float s9 = 0.f, s10 = 0.f, fx = 0.f, fy = 0.f;
      float2 sE[NSPEC], sA[NSPEC], sC[4][NSPEC];
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        sE[s] = sA[s] = bc2(0.f);
#pragma unroll
        for (int j = 0; j < 4; ++j) sC[j][s] = bc2(0.f);
      }

#pragma unroll(SCAT ? 2 : 1)  // two nodes per iteration with scattering: 1.6 % faster; without, 2.5 % slower
      for (int k = 0; k < P.n_nodes; ++k) {
        const ff xk = {P.gl_x_hi[k], P.gl_x_lo[k]};
        const float wk = P.gl_w[k];
        // ---- each lane's LOS range: position, distance, temperature -----------
        const float2 Rl = lin_ff_x2(hsP, xk, mdP);
        const float2 wl = add2(Rl, bc2(B.beta_h.hi));  // |X|^2 = w^2 + b^2 (node_range)
        const float2 R2 = fma2(wl, wl, bc2(B.b2h));
        const float2 rinv = rsqrt_2(R2);
        const float2 R = mul2(R2, rinv);
        const float2 lg2R = lg2_2(R);
        const float2 Tn = ex2_2(mul2(bc2(P.neg_delta), lg2R));
        const float2 T = mul2(bc2(P.T0), Tn);
        float2 Bv[NSPEC], dB[NSPEC];
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          const float2 bx = bb_lookup_d(tab_sm + s * nT, T.x, P.t_min, P.t_max, P.inv_dt, nT);
          const float2 by = bb_lookup_d(tab_sm + s * nT, T.y, P.t_min, P.t_max, P.inv_dt, nT);
          Bv[s] = make_float2(bx.x, by.x);
          dB[s] = make_float2(bx.y, by.y);
        }
        float2 theta = bc2(0.f), flux = bc2(0.f), eC3[NSPEC], base[NSPEC], sf[NSPEC];
        if (SCAT) {  // scattering.py:11-59
          theta = make_float2(atan2_poly(B.bperp, -(Rl.x + B.beta_h.hi)),
                              atan2_poly(B.bperp, -(Rl.y + B.beta_h.hi)));
          flux = mul2(rinv, rinv);
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) {
            const KSpecF32& S = P.spec[s];
            eC3[s] = ex2_2(mul2(bc2(S.C3l2e), theta));
            base[s] = add2(fma2(bc2(S.C2), theta, bc2(S.C1)), eC3[s]);
            sf[s] = mul2(mul2(bc2(S.S), flux), mul2(bc2(S.N), base[s]));
          }
        }

        // ---- ring / feature density and log-derivatives (number_density.py:113-181)
        const float2 Z = fma2(Rl, unP, onP);
        const float2 aZ = abs2(Z);
        float2 dR = sub2(R, q0);
        const float2 D2 = fma2(lin_ff_x2(hsP, xk, waP), lin_ff_x2(hsP, xk, wbP), rrP);  // R^2 - R0^2
        dR = fma2(fma2(dR, fma2(R, bc2(-1.f), nq0), D2), mul2(bc2(0.5f), rinv), dR);
        const float2 dR2 = mul2(dR, dR);
        float2 arg = fma2(dR2, q1, mul2(aZ, q2));
        const float2 GR = mul2(dR, m2q1);  // d ln n / d R; d/d R0 is -GR
        const float2 GZ = make_float2(Z.x != 0.f ? -copysignf(q2.x, Z.x) : 0.f, Z.y != 0.f ? -copysignf(q2.y, Z.y) : 0.f);
        // the feature's longitude term (lane .y)
        const float dth = atan2_poly(fmaf(Rl.y, B.ruy[CF], B.roy[CF]), fmaf(Rl.y, B.rux[CF], B.rox[CF]));
        const float dth2 = dth * dth;
        arg.y = fmaf(dth2, A.q[CF][5], arg.y);
        const float gth = -2.f * dth * A.q[CF][5];  // d ln n / d dtheta
        const float Xc0 = fmaf(Rl.y, B.uxf, B.oxf - Cf.ox), Xc1 = fmaf(Rl.y, B.uyf, B.oyf - Cf.oy);  // X - X_0
        const float rr = __fdividef(1.f, Xc0 * Xc0 + Xc1 * Xc1);
        const float dthx = gth * (Xc1 * rr - B.eqx[CF]), dthy = gth * (-Xc0 * rr - B.eqy[CF]);
        const float2 du = ex2_2(mul2(bc2(-kLog2e), arg));

        // ---- node sums -------------------------------------------------------
        float2 E = bc2(0.f), Q = bc2(0.f);
        if (!KF) {
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) {
            E = fma2(gq[s], Bv[s], E);
            if (SCAT) E = fma2(ga[s], sf[s], E);
            Q = fma2(gq[s], dB[s], Q);
          }
        }
        const float2 wdu = mul2(bc2(wk), du);
        const float2 wd = mul2(wdu, n0P);
        const float2 coef = mul2(wd, KF ? Bv[0] : E);
        const float2 cGR = mul2(coef, GR);
        s6 = add2(s6, cGR);
        const float2 cG = mul2(cGR, rinv), cZ = mul2(coef, GZ);
        s0 = fma2(cG, Rl, s0);
        s1 = add2(s1, cG);
        s2 = add2(s2, cZ);
        s3 = fma2(cZ, Rl, s3);
        s5 = fma2(wdu, KF ? Bv[0] : E, s5);
        s7 = fma2(coef, dR2, s7);
        s8 = fma2(coef, aZ, s8);
        s9 = fmaf(coef.y, dth, s9);
        s10 = fmaf(coef.y, dth2, s10);
        fx = fmaf(coef.y, dthx, fx);
        fy = fmaf(coef.y, dthy, fy);
        const float2 wq = mul2(wd, KF ? dB[0] : Q);
        sT0 = fma2(wq, Tn, sT0);
        sD = fma2(mul2(wq, T), lg2R, sD);
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          if (!KF) sE[s] = fma2(wd, Bv[s], sE[s]);  // with KF, n_0 s5 (bwd_finalize)
          if (SCAT) {
            const KSpecF32& S = P.spec[s];
            sA[s] = fma2(wd, sf[s], sA[s]);
            const float2 af = mul2(mul2(wd, ga[s]), flux);
            sC[3][s] = fma2(mul2(af, bc2(S.N)), base[s], sC[3][s]);
            const float2 as = mul2(af, bc2(S.S));
            const float2 Nth = mul2(bc2(S.N), theta);
            sC[0][s] = fma2(as, fma2(base[s], bc2(A.dN[s][0]), bc2(S.N)), sC[0][s]);
            sC[1][s] = fma2(as, fma2(base[s], bc2(A.dN[s][1]), Nth), sC[1][s]);
            sC[2][s] = fma2(as, fma2(base[s], bc2(A.dN[s][2]), mul2(Nth, eC3[s])), sC[2][s]);
          }
        }
      }

      // ---- the scalar kernel's accumulator layout ------------------------------
      constexpr int oR = G::off(CR), oF = G::off(CF);
      acc[oR + 0] = s0.x, acc[oF + 0] = s0.y;
      acc[oR + 1] = s1.x, acc[oF + 1] = s1.y;
      acc[oR + 2] = s2.x, acc[oF + 2] = s2.y;
      acc[oR + 3] = s3.x, acc[oF + 3] = s3.y;
      acc[oR + 5] = s5.x, acc[oF + 5] = s5.y;
      acc[oR + 6] = s6.x, acc[oF + 6] = s6.y;
      acc[oR + 7] = s7.x, acc[oF + 7] = s7.y;
      acc[oR + 8] = s8.x, acc[oF + 8] = s8.y;
      acc[oF + 9] = s9, acc[oF + 10] = s10;
      const float kR = KF ? kpix[CR] : 1.f, kFe = KF ? kpix[CF] : 1.f;
      acc[G::T0] = fmaf(kR, sT0.x, kFe * sT0.y);
      acc[G::DELTA] = -kLn2 * fmaf(kR, sD.x, kFe * sD.y);
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        acc[G::eps(CR, s)] = sE[s].x, acc[G::eps(CF, s)] = sE[s].y;
        if (SCAT) {
          acc[G::alb(CR, s)] = sA[s].x, acc[G::alb(CF, s)] = sA[s].y;
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[G::C(j, s)] = sC[j][s].x + sC[j][s].y;
        }
      }
      float fthx[NC], fthy[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) fthx[c] = fthy[c] = 0.f;
      fthx[CF] = fx, fthy[CF] = fy;
      bwd_finalize<LAYOUT, MASK, NSPEC, SCAT>(P, A, B, kpix, fthx, fthy, acc);
    }
    bwd_tile_reduce<LAYOUT, MASK, NSPEC, SCAT>(acc, red_sm, used_sm, partials, tile);
  }
}

// Band 1's 1 - e^-y and y d ln(1 - e^-y)/dy (y = (R/delta_r)^20) as lane .x of the packed
// bands 1/2 code below forms them, operation for operation: band 3 reuses them at nodes where
// bands 1 and 2 are not evaluated.
__device__ __forceinline__ void band1_cutoff(float R2, float inv_dr2, float& t4, float& Y4) {
  const float qq = R2 * inv_dr2;
  const float qq2 = qq * qq, qq4 = qq2 * qq2, qq8 = qq4 * qq4;
  const float y = qq8 * qq2;
  const float emy = ex2_ftz(-kLog2e * y);
  const float ny = -y;
  float ser = fmaf(ny, 1.f / 720.f, 1.f / 120.f);
  ser = fmaf(ny, ser, 1.f / 24.f);
  ser = fmaf(ny, ser, 1.f / 6.f);
  ser = fmaf(ny, ser, 0.5f);
  ser = y * fmaf(ny, ser, 1.f);
  const float om = 1.f - emy;
  t4 = y < 0.25f ? ser : om;
  const float ye = (y * emy) * __fdividef(1.f, t4);
  Y4 = t4 > 0.f ? ye : 1.f;
}

// ---------------------------------------------------------------------------
// {cloud, bands}: cloud and band 3 scalar, bands 1 and 2 in lanes .x / .y
// ---------------------------------------------------------------------------
template <int NSPEC, bool SCAT>
__global__ void __launch_bounds__(kTile) bwd_dirbe_cb_kernel(const __grid_constant__ KParamsF32 P,
                                                             const __grid_constant__ KGradAux A,
                                                             const double* __restrict__ u, int64_t n_pix,
                                                             const ObsArgs OA, const double* __restrict__ g_comps,
                                                             const double* __restrict__ g_total,
                                                             double* __restrict__ partials, int64_t n_tiles) {
  constexpr uint32_t LAYOUT = kLayoutDirbe, MASK = 0x0Fu, FLAGS = kBwdFlagsKelsall;
  using L = Lay<LAYOUT>;
  using G = GradLay<LAYOUT, NSPEC>;
  constexpr bool KF = NSPEC == 1 && !SCAT;
  constexpr int NC = L::ncomp(), NG = G::NG;
  constexpr int CC = 0, C1 = 1, C2 = 2, C3 = 3;
  static_assert(L::type(CC) == ZL_CLOUD && L::type(C1) == ZL_BAND && L::type(C2) == ZL_BAND &&
                    L::type(C3) == ZL_BAND && L::range(C3) == 0 && last_of_range<LAYOUT, MASK>(C3),
                "DIRBE cloud and bands on one LOS range, band 3 last");
  static_assert(((FLAGS >> 9) & 7u) == 0u && ((FLAGS >> 17) & 3u) == 3u && ((FLAGS >> 25) & 3u) == 0u,
                "bands 1 and 2 centred on the Sun, with p = 4 and their own inner-cutoff terms");
  __shared__ float4 tab_sm[NSPEC * ZL_MAX_TEMPS];
  __shared__ float red_sm[kTile / 32][NG];
  __shared__ int used_sm[NG];
  __shared__ BwdObs<NC> s_obs;  // the observer set-up the block's pixels share
  const int cached = bwd_obs_cache_index(OA, (int64_t)blockIdx.x * kTile, n_pix);
  if (threadIdx.x == 0 && cached >= 0) bwd_obs_setup<LAYOUT, MASK, FLAGS>(P, record_observer(OA, cached), s_obs);
  bwd_block_init<LAYOUT, MASK, NSPEC, SCAT>(P, tab_sm, red_sm, used_sm);  // its barrier also publishes s_obs
  const int nT = P.n_temps;
  const KCompF32& K1 = P.comp[C1];
  const KCompF32& K2 = P.comp[C2];

  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t i = tile * kTile + threadIdx.x;
    float acc[NG];
#pragma unroll
    for (int j = 0; j < NG; ++j) acc[j] = 0.f;

    if (i < n_pix) {
      BwdPix<NC, NSPEC> B;
      bwd_pixel_setup_cached<LAYOUT, MASK, NSPEC, SCAT, FLAGS>(P, u, n_pix, OA, g_comps, g_total, i, cached, s_obs, B);
      const float2 unP = make_float2(B.un_c[C1], B.un_c[C2]), onP = make_float2(B.on_c[C1], B.on_c[C2]);
      // q: delta_zeta [deg], v, p, delta_r, 1/delta_zeta [deg], -20/delta_r
      const float2 c1P = make_float2(K1.c[1], K2.c[1]), c2P = make_float2(K1.c[2], K2.c[2]);
      const float2 c4P = make_float2(K1.c[4], K2.c[4]);
      const float2 q2P = qpair(A, C1, C2, 2);
      const float2 n0P = make_float2(A.n0[C1], A.n0[C2]);
      float2 gq[NSPEC], ga[NSPEC];
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        const KSpecF32& S = P.spec[s];
        const float2 g = make_float2(B.gup[C1][s], B.gup[C2][s]);
        gq[s] = mul2(g, make_float2(S.em1[C1], S.em1[C2]));
        ga[s] = mul2(g, make_float2(S.alb[C1], S.alb[C2]));
      }
      float fthx[NC], fthy[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) fthx[c] = fthy[c] = 0.f;
      float wq = 0.f;
      float kpix[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) kpix[c] = KF ? B.gup[c][0] * P.spec[0].em1[c] : 0.f;
      const float2 kP = make_float2(kpix[C1], kpix[C2]);

      // nodes from k12 (bands 1 and 2) and k3 (band 3) on add exactly nothing for any pixel of
      // the warp (band_zero_tail); Z = u_n R_los + o_n and R^2 = (R_los + u . X_obs)^2 + b^2.
      // With scattering the bands' share of the work is too small for the branches to pay.
      constexpr bool TAIL = !SCAT;
      int k12 = P.n_nodes, k3 = P.n_nodes;
      // and the nodes at which bands 1 and 2 (and band 3, which reuses band 1's) evaluate the
      // inner-cutoff factor 1 - e^-y and y e^-y / (1 - e^-y); at the others they are 1.0f and +0
      // for every pixel of the warp, the same bits (cutoff_interval)
      int2 r4 = make_int2(0, P.n_nodes);
      if (TAIL) {
        const float bt = B.beta_h.hi, b2h = B.b2h;
        const float h0 = B.hs_r[0].hi, m0 = B.mid_r[0].hi;
        auto tail = [&](int c) {
          return band_zero_tail(B.un_c[c] * h0, fmaf(B.un_c[c], m0, B.on_c[c]), h0, m0 + bt, b2h, P.comp[c].c[1]);
        };
        k12 = warp_tail_index(P, fmaxf(tail(C1), tail(C2)));
        k3 = warp_tail_index(P, tail(C3));
        const float2 cut1 = cutoff_interval(h0, m0 + bt, b2h, K1.c[4]);
        const float2 cut2 = cutoff_interval(h0, m0 + bt, b2h, K2.c[4]);
        r4 = warp_node_range(P, fminf(cut1.x, cut2.x), fmaxf(cut1.y, cut2.y));
      }

      // bands 1 and 2: the scalar kernel's acc[off + j] per lane (before comp_pfactors)
      float2 b0 = bc2(0.f), b1 = bc2(0.f), b2 = bc2(0.f), b3 = bc2(0.f), b5 = bc2(0.f);
      float2 b6 = bc2(0.f), b7 = bc2(0.f), b8 = bc2(0.f), b9 = bc2(0.f);
      float2 bE[NSPEC], bA[NSPEC];
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) bE[s] = bA[s] = bc2(0.f);

#pragma unroll(SCAT ? 2 : 1)  // two nodes per iteration with scattering: 1.6 % faster; without, 2.5 % slower
      for (int k = 0; k < P.n_nodes; ++k) {
        const ff xk = {P.gl_x_hi[k], P.gl_x_lo[k]};
        const float wk = P.gl_w[k];
        NodeR<NSPEC> N;
        node_range<NSPEC, SCAT>(P, B, 0, true, xk, tab_sm, nT, N);
        float t4s[NC], y4s[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) t4s[c] = y4s[c] = 0.f;

        // ---- cloud -------------------------------------------------------------
        {
          const CompTerms t = comp_terms<LAYOUT, MASK, FLAGS>(CC, P, A, B, xk, N, t4s, y4s);
          comp_accumulate<LAYOUT, MASK, NSPEC, SCAT>(CC, P, A, B, wk, N, t, kpix, wq, fthx, fthy, acc);
        }

        // ---- bands 1 and 2 (number_density.py:99-110) ----------------------------
        if (!TAIL || k < k12) {
          const float2 Z = fma2(bc2(N.Rl), unP, onP);
          const float2 aZ = abs2(Z);
          const float2 x = mul2(mul2(aZ, bc2(N.rinv)), c1P);
          const float2 x2 = mul2(x, x), x4 = mul2(x2, x2), x6 = mul2(x4, x2);
          const float2 t2 = ex2_2(mul2(bc2(-kLog2e), x6));
          const float2 lgx = lg2_2(x);
          const float2 xpv = mul2(x4, c2P);
          const float2 t3 = add2(bc2(1.f), xpv);
          float2 t4 = bc2(1.f), Y4 = bc2(0.f);
          if (!TAIL || (k >= r4.x && k < r4.y)) {
            const float2 qq = mul2(bc2(N.R2), c4P);
            const float2 qq2 = mul2(qq, qq), qq4 = mul2(qq2, qq2), qq8 = mul2(qq4, qq4);
            const float2 y = mul2(qq8, qq2);
            const float2 emy = ex2_2(mul2(bc2(-kLog2e), y));
            // 1 - e^-y: its series below y = 1/4, the difference above
            const float2 ny = mul2(y, bc2(-1.f));
            float2 ser = fma2(ny, bc2(1.f / 720.f), bc2(1.f / 120.f));
            ser = fma2(ny, ser, bc2(1.f / 24.f));
            ser = fma2(ny, ser, bc2(1.f / 6.f));
            ser = fma2(ny, ser, bc2(0.5f));
            ser = mul2(y, fma2(ny, ser, bc2(1.f)));
            const float2 om = sub2(bc2(1.f), emy);
            t4 = make_float2(y.x < 0.25f ? ser.x : om.x, y.y < 0.25f ? ser.y : om.y);
            const float2 ye = mul2(mul2(y, emy), make_float2(__fdividef(1.f, t4.x), __fdividef(1.f, t4.y)));
            Y4 = make_float2(t4.x > 0.f ? ye.x : 1.f, t4.y > 0.f ? ye.y : 1.f);
          }
          t4s[C1] = t4.x;  // band 3's inner-cutoff term
          y4s[C1] = Y4.x;
          const float2 du = mul2(mul2(mul2(bc2(N.rinv), t2), t3), t4);
          const float2 it3 = make_float2(__fdividef(1.f, t3.x), __fdividef(1.f, t3.y));
          const float2 xit = mul2(xpv, it3);
          const float2 Sx = fma2(bc2(-6.f), x6, mul2(q2P, xit));  // x d ln n / d x
          const float2 GR = mul2(sub2(fma2(Y4, bc2(20.f), bc2(-1.f)), Sx), bc2(N.rinv));
          const float2 sz = mul2(Sx, make_float2(__fdividef(1.f, Z.x), __fdividef(1.f, Z.y)));
          const float2 GZ = make_float2(aZ.x > 0.f ? sz.x : 0.f, aZ.y > 0.f ? sz.y : 0.f);
          const float2 p8r = mul2(xit, lgx);
          const float2 p8 = make_float2(x.x > 0.f ? p8r.x : 0.f, x.y > 0.f ? p8r.y : 0.f);

          float2 E = bc2(0.f), Q = bc2(0.f);
          if (!KF) {
#pragma unroll
            for (int s = 0; s < NSPEC; ++s) {
              E = fma2(gq[s], bc2(N.Bv[s]), E);
              if (SCAT) E = fma2(ga[s], bc2(N.sf[s]), E);
              Q = fma2(gq[s], bc2(N.dB[s]), Q);
            }
          }
          const float2 wdu = mul2(bc2(wk), du);
          const float2 wd = mul2(wdu, n0P);
          const float2 coef = mul2(wd, KF ? bc2(N.Bv[0]) : E);
          const float2 cG = mul2(coef, mul2(GR, bc2(N.rinv))), cZ = mul2(coef, GZ);
          b0 = fma2(cG, bc2(N.Rl), b0);
          b1 = add2(b1, cG);
          b2 = add2(b2, cZ);
          b3 = fma2(cZ, bc2(N.Rl), b3);
          b5 = fma2(wdu, KF ? bc2(N.Bv[0]) : E, b5);
          b6 = fma2(coef, Sx, b6);
          b7 = fma2(coef, xit, b7);
          b8 = fma2(coef, p8, b8);
          b9 = fma2(coef, Y4, b9);
          const float2 wqp = mul2(wd, KF ? kP : Q);
          wq += wqp.x + wqp.y;
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) {
            if (!KF) bE[s] = fma2(wd, bc2(N.Bv[s]), bE[s]);  // with KF, n_0 b5 (bwd_finalize)
            if (SCAT) {
              const KSpecF32& S = P.spec[s];
              bA[s] = fma2(wd, bc2(N.sf[s]), bA[s]);
              const float2 af2 = mul2(mul2(wd, ga[s]), bc2(N.flux));
              const float af = af2.x + af2.y;
              acc[G::C(3, s)] += af * S.N * N.base[s];
              const float as = af * S.S;
              acc[G::C(0, s)] += as * (S.N + N.base[s] * A.dN[s][0]);
              acc[G::C(1, s)] += as * (S.N * N.theta + N.base[s] * A.dN[s][1]);
              acc[G::C(2, s)] += as * (S.N * N.theta * N.eC3[s] + N.base[s] * A.dN[s][2]);
            }
          }
        }

        // ---- band 3 (band 1's inner-cutoff term; flushes the range's T_0 / delta sums)
        if (!TAIL || k < k3) {
          if (TAIL && k >= k12) {
            if (k >= r4.x && k < r4.y) {
              band1_cutoff(N.R2, K1.c[4], t4s[C1], y4s[C1]);
            } else {
              t4s[C1] = 1.f;
              y4s[C1] = 0.f;
            }
          }
          const CompTerms t = comp_terms<LAYOUT, MASK, FLAGS>(C3, P, A, B, xk, N, t4s, y4s);
          comp_accumulate<LAYOUT, MASK, NSPEC, SCAT>(C3, P, A, B, wk, N, t, kpix, wq, fthx, fthy, acc);
        } else {
          range_flush<LAYOUT, MASK, NSPEC, SCAT>(N, wq, acc);
        }
      }

      constexpr int o1 = G::off(C1), o2 = G::off(C2);
      acc[o1 + 0] = b0.x, acc[o2 + 0] = b0.y;
      acc[o1 + 1] = b1.x, acc[o2 + 1] = b1.y;
      acc[o1 + 2] = b2.x, acc[o2 + 2] = b2.y;
      acc[o1 + 3] = b3.x, acc[o2 + 3] = b3.y;
      acc[o1 + 5] = b5.x, acc[o2 + 5] = b5.y;
      acc[o1 + 6] = b6.x, acc[o2 + 6] = b6.y;
      acc[o1 + 7] = b7.x, acc[o2 + 7] = b7.y;
      acc[o1 + 8] = b8.x, acc[o2 + 8] = b8.y;
      acc[o1 + 9] = b9.x, acc[o2 + 9] = b9.y;
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        acc[G::eps(C1, s)] = bE[s].x, acc[G::eps(C2, s)] = bE[s].y;
        if (SCAT) acc[G::alb(C1, s)] = bA[s].x, acc[G::alb(C2, s)] = bA[s].y;
      }
      bwd_finalize<LAYOUT, MASK, NSPEC, SCAT>(P, A, B, kpix, fthx, fthy, acc);
    }
    bwd_tile_reduce<LAYOUT, MASK, NSPEC, SCAT>(acc, red_sm, used_sm, partials, tile);
  }
}

}  // namespace zl
