// DIRBE-layout forward kernel with component pairs on packed FP32 instructions.
//
// One thread integrates one pixel, as zl_fwd_f32.cuh does, but the components
// whose per-node arithmetic is the same sequence on different constants share
// packed float2 instructions (fma/mul/add.rn.f32x2):
//   - band 1 and band 2 (lanes .x, .y): plane height, e^-(zeta/dzeta)^6, the
//     (zeta/dzeta)^4 term and the inner-cutoff factor;
//   - the ring and the feature (lanes .x, .y): each runs its own line-of-sight
//     range, so their node distance, temperature, R^2 - R0^2, Newton step,
//     plane height and Gaussian exponent pair up.
// The cloud, band 3 and the per-lane MUFU operations, table lookups,
// comparisons and the feature's atan2 stay scalar.  Unlike the two-pixel
// kernel, no per-pixel value is duplicated, so the register footprint stays
// that of the one-pixel kernel.  Every lane computes exactly what the one-pixel
// kernel computes for that component.
//
// Built for the DIRBE layout with the built-in models' flags (cloud offset from
// the Sun, bands with p = 4, band 3 reusing band 1's inner-cutoff term).
//
// Band tails: past the node from which a band's factor e^-(zeta/dzeta)^6 is zero in
// float32 for every pixel of the warp (band_zero_tail, warp_tail_index), the band adds
// exactly nothing, and a warp-uniform branch skips it; the maps are the same bits as
// evaluating every node.
#pragma once

#include "zl_fwd_f32x2.cuh"

namespace zl {

// (C_a.c[k], C_b.c[k]) as one packed constant
__device__ __forceinline__ float2 cpair(const KCompF32& a, const KCompF32& b, int k) {
  return make_float2(a.c[k], b.c[k]);
}

// 1 - e^-y per lane: the series below 1/4, ex2 above (as the one-pixel kernel)
__device__ __forceinline__ float2 one_minus_emy2(float2 y) {
  const float2 ny = mul2(y, bc2(-1.f));
  float2 ser = fma2(ny, bc2(1.f / 720.f), bc2(1.f / 120.f));
  ser = fma2(ny, ser, bc2(1.f / 24.f));
  ser = fma2(ny, ser, bc2(1.f / 6.f));
  ser = fma2(ny, ser, bc2(0.5f));
  ser = mul2(y, fma2(ny, ser, bc2(1.f)));
  const float2 alt = sub2(bc2(1.f), ex2_2(mul2(bc2(-kLog2e), y)));
  return make_float2(y.x < 0.25f ? ser.x : alt.x, y.y < 0.25f ? ser.y : alt.y);
}

// One lane of one_minus_emy2, operation for operation (a packed operation rounds each lane as
// its scalar counterpart does): band 1's inner-cutoff factor where bands 1 and 2 are not
// evaluated but band 3, which reuses it, is.
__device__ __forceinline__ float one_minus_emy1(float y) {
  const float ny = -y;
  float ser = fmaf(ny, 1.f / 720.f, 1.f / 120.f);
  ser = fmaf(ny, ser, 1.f / 24.f);
  ser = fmaf(ny, ser, 1.f / 6.f);
  ser = fmaf(ny, ser, 0.5f);
  ser = y * fmaf(ny, ser, 1.f);
  const float alt = 1.f - ex2_ftz(-kLog2e * y);
  return y < 0.25f ? ser : alt;
}

// (R / delta_r)^20 of a band from q = R^2 / delta_r^2, as the packed lanes form it
__device__ __forceinline__ float band_y1(float R2, float inv_dr2) {
  const float q = R2 * inv_dr2;
  const float q2 = q * q, q4 = q2 * q2, q8 = q4 * q4;
  return q8 * q2;
}

// QUEUE: compiled for the work-queue schedule, else the static grid-stride loop (which keeps
// the one-band kernel at 96 registers: five blocks per SM).
template <int NSPEC, uint32_t FLAGS, bool QUEUE>
__global__ void __launch_bounds__(128, (QUEUE && NSPEC == 1 && !((FLAGS >> 1) & 1u)) ? 5 : 0) fwd_dirbe_cp_kernel(const __grid_constant__ KParamsF32 P,
                                                           const double* __restrict__ u, int64_t n_pix,
                                                           const ObsArgs OA, double* __restrict__ out_comps,
                                                           double* __restrict__ out_total, const Sched SC) {
  using Fl = KFlags<FLAGS>;
  static_assert(!Fl::runtime, "compiled flags only");
  static_assert(((FLAGS >> 8) & 0x3Fu) == 1u, "only the cloud is offset from the Sun");
  static_assert(((FLAGS >> 17) & 7u) == 7u, "bands with p = 4");
  static_assert(((FLAGS >> 25) & 7u) == 4u, "band 3 (only) reuses band 1's inner-cutoff term");
  constexpr int NC = 6;
  constexpr int MODE = QUEUE ? kSchedQueue : kSchedStatic;
  extern __shared__ float4 tab_sm[];  // [NSPEC][nT]
  __shared__ ObsSetupF32<NC> s_obs;   // the observer set-up the block's pixels share
  const int nT = P.n_temps;
  for (int t = threadIdx.x; t < nT * NSPEC; t += blockDim.x) tab_sm[t] = P.table[t / nT][t % nT];
  const int cached = obs_cache_index<MODE>(OA, (int64_t)blockIdx.x * blockDim.x, n_pix);
  if (threadIdx.x == 0 && cached >= 0) observer_setup<kLayoutDirbe, FLAGS, NC>(P, record_observer(OA, cached), s_obs);
  __syncthreads();

  const KCompF32& Cc = P.comp[0];
  const KCompF32& C1 = P.comp[1];
  const KCompF32& C2 = P.comp[2];
  const KCompF32& C3 = P.comp[3];
  const KCompF32& Cr = P.comp[4];
  const KCompF32& Cf = P.comp[5];

  ZL_SCHED_LOOP(MODE, SC, n_pix, i) {
    PixSetupF32<NC> PS;
    pixel_setup_cached<kLayoutDirbe, FLAGS, true, NC>(P, u, n_pix, OA, i, cached, s_obs, PS);
    const ff2 z1b = pack_ff(PS.z1[1], PS.z1[2]), z0b = pack_ff(PS.z0[1], PS.z0[2]);
    const ff2 hsq = pack_ff(PS.hs[4], PS.hs[5]), mhq = pack_ff(PS.mh[4], PS.mh[5]);
    const ff2 z1q = pack_ff(PS.z1[4], PS.z1[5]), z0q = pack_ff(PS.z0[4], PS.z0[5]);
    const ff2 waq = pack_ff(PS.wa[4], PS.wa[5]), wbq = pack_ff(PS.wb[4], PS.wb[5]);
    const float2 rrq = make_float2(PS.rr[4], PS.rr[5]);
    // nodes from k12 (bands 1 and 2) and k3 (band 3) on add nothing for any pixel of the warp
    auto tail = [&](int c) {
      return band_zero_tail(PS.z1[c].hi, PS.z0[c].hi, PS.hs[0].hi, PS.mh[0].hi, PS.b2h, P.comp[c].c[1]);
    };
    const int k12 = warp_tail_index(P, fmaxf(tail(1), tail(2)));
    const int k3 = warp_tail_index(P, tail(3));
    // nodes at which bands 1 and 2 (and band 3, which reuses band 1's) evaluate their inner-cutoff
    // factor 1 - e^-(R/delta_r)^20; at the others it is 1.0f for every pixel of the warp, the same
    // bits (cutoff_interval).  Without scattering: 0.9 % faster; with it 0.4 % slower, so that
    // instantiation evaluates the factor at every node
    constexpr bool kCutAll = (FLAGS >> 1) & 1u;  // scattering: every node
    int2 r4 = make_int2(0, P.n_nodes);
    if (!kCutAll) {
      const float2 cut1 = cutoff_interval(PS.hs[1].hi, PS.wm[1].hi, PS.b2[1], C1.c[4]);
      const float2 cut2 = cutoff_interval(PS.hs[2].hi, PS.wm[2].hi, PS.b2[2], C2.c[4]);
      r4 = warp_node_range(P, fminf(cut1.x, cut2.x), fmaxf(cut1.y, cut2.y));
    }

    // quadrature sums per component (pairs in float2), blocks of kSumBlock nodes, Kahan across blocks
    float ps0[NSPEC], ps3[NSPEC], pS0[NSPEC], pS3[NSPEC], as0[NSPEC], ac0[NSPEC], as3[NSPEC], ac3[NSPEC];
    float2 ps12[NSPEC], psq[NSPEC], pS12[NSPEC], pSq[NSPEC], as12[NSPEC], ac12[NSPEC], asq[NSPEC], acq[NSPEC];
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      ps0[s] = ps3[s] = pS0[s] = pS3[s] = as0[s] = ac0[s] = as3[s] = ac3[s] = 0.f;
      ps12[s] = psq[s] = pS12[s] = pSq[s] = as12[s] = ac12[s] = asq[s] = acq[s] = bc2(0.f);
    }

    // one node: each component's term into its block sum
    const auto node = [&](const int k) {
      const ff xk = {P.gl_x_hi[k], P.gl_x_lo[k]};
      const float wk = P.gl_w[k];

      // ---- range 0 (cloud, bands): distance of the node, temperature ------------
      const float wh = lin_ff(PS.hs[0], xk, PS.mh[0]);
      const float R2 = fmaf(wh, wh, PS.b2h);
      float rinv = rsqrt_ftz(R2);
      rinv = rinv * fmaf(-0.5f * R2, rinv * rinv, 1.5f);
      const float T0 = P.T0 * ex2_ftz(P.neg_half_delta * lg2_ftz(R2));  // R^-delta, blackbody.py:16-30
      float wB0[NSPEC], wS0[NSPEC];
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        wB0[s] = wk * bb_lookup(tab_sm + s * nT, T0, P.t_min, P.t_max, P.inv_dt, nT);
        wS0[s] = 0.f;
      }
      if (Fl::scat(P)) {  // scattering.py:11-59
        const float theta = atan2_poly(PS.bperp, -wh);
        const float flux = rinv * rinv;
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          const KSpecF32& S = P.spec[s];
          wS0[s] = wk * (S.S * flux * (S.N * (S.C1 + S.C2 * theta + ex2_ftz(S.C3l2e * theta))));
        }
      }

      // ---- cloud (offset): own distance, number_density.py:60-73 ----------------
      {
        const float wc = lin_ff(PS.hs[0], xk, PS.wm[0]);
        const float Rc2 = fmaf(wc, wc, PS.b2[0]);
        const float rcinv = rsqrt_ftz(Rc2);
        const float Z = lin_ff(PS.z1[0], xk, PS.z0[0]);
        const float zeta = fabsf(Z) * rcinv;
        const float g = zeta < Cc.c[4] ? zeta * zeta * Cc.c[5] : zeta - Cc.c[6];
        const float gg = ex2_ftz(Cc.c[3] * lg2_ftz(g));
        const float dens = ex2_ftz(Cc.c[7] * lg2_ftz(Rc2) - Cc.c[2] * gg);  // Rc^-alpha e^(-beta g^gamma)
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          ps0[s] = fmaf(wB0[s], dens, ps0[s]);
          if (Fl::scat(P)) pS0[s] = fmaf(wS0[s], dens, pS0[s]);
        }
      }

      // ---- bands 1 and 2 (packed), number_density.py:99-110 ---------------------
      float t4_band1 = 0.f;
      if (k < k12) {
        const float2 Z = lin_ff_x2(z1b, xk, z0b);
        const float2 zz = mul2(mul2(Z, bc2(rinv)), cpair(C1, C2, 1));  // only its square is used: no |Z|
        const float2 z2 = mul2(zz, zz);
        const float2 t2 = ex2_2(mul2(bc2(-kLog2e), mul2(mul2(z2, z2), z2)));
        const float2 t3 = fma2(mul2(z2, z2), cpair(C1, C2, 2), bc2(1.f));
        float2 t4 = bc2(1.f);
        if (kCutAll || (k >= r4.x && k < r4.y)) {
          const float2 q = mul2(bc2(R2), cpair(C1, C2, 4));  // (R/delta_r)^2
          const float2 q2 = mul2(q, q), q4 = mul2(q2, q2), q8 = mul2(q4, q4);
          t4 = one_minus_emy2(mul2(q8, q2));
        }
        t4_band1 = t4.x;
        const float2 dens = mul2(mul2(mul2(bc2(rinv), t2), t3), t4);
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          ps12[s] = fma2(bc2(wB0[s]), dens, ps12[s]);
          if (Fl::scat(P)) pS12[s] = fma2(bc2(wS0[s]), dens, pS12[s]);
        }
      }

      // ---- band 3 (inner-cutoff factor of band 1) -------------------------------
      if (k < k3) {
        if (k >= k12) t4_band1 = (kCutAll || (k >= r4.x && k < r4.y)) ? one_minus_emy1(band_y1(R2, C1.c[4])) : 1.f;
        const float Z = lin_ff(PS.z1[3], xk, PS.z0[3]);
        const float zz = Z * rinv * C3.c[1];  // only its square is used
        const float z2 = zz * zz;
        const float t2 = ex2_ftz(-kLog2e * (z2 * z2 * z2));
        const float t3 = fmaf(z2 * z2, C3.c[2], 1.0f);
        const float dens = rinv * t2 * t3 * t4_band1;
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          ps3[s] = fmaf(wB0[s], dens, ps3[s]);
          if (Fl::scat(P)) pS3[s] = fmaf(wS0[s], dens, pS3[s]);
        }
      }


      // ---- ring (.x) and feature (.y): ranges 1 and 2, number_density.py:136-181 ----
      {
        const float2 whq = lin_ff_x2(hsq, xk, mhq);
        const float2 R2q = fma2(whq, whq, bc2(PS.b2h));
        const float2 rinvq = rsqrt_2(R2q);
        const float2 Rq = mul2(R2q, rinvq);
        const float2 Tq = mul2(bc2(P.T0), ex2_2(mul2(bc2(P.neg_delta), lg2_2(Rq))));
        float2 wBq[NSPEC], wSq[NSPEC];
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          wBq[s] = mul2(bc2(wk), make_float2(bb_lookup(tab_sm + s * nT, Tq.x, P.t_min, P.t_max, P.inv_dt, nT),
                                             bb_lookup(tab_sm + s * nT, Tq.y, P.t_min, P.t_max, P.inv_dt, nT)));
          wSq[s] = bc2(0.f);
        }
        if (Fl::scat(P)) {
          const float2 theta = make_float2(atan2_poly(PS.bperp, -whq.x), atan2_poly(PS.bperp, -whq.y));
          const float2 flux = mul2(rinvq, rinvq);
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) {
            const KSpecF32& S = P.spec[s];
            const float2 ph = add2(fma2(bc2(S.C2), theta, bc2(S.C1)), ex2_2(mul2(bc2(S.C3l2e), theta)));
            wSq[s] = mul2(bc2(wk), mul2(mul2(bc2(S.S), flux), mul2(bc2(S.N), ph)));
          }
        }
        // R - R0 from R^2 - R0^2 = (w - w0)(w + w0) + rr and one Newton step
        float2 dR = sub2(Rq, cpair(Cr, Cf, 1));
        const float2 D2 = fma2(lin_ff_x2(hsq, xk, waq), lin_ff_x2(hsq, xk, wbq), rrq);
        const float2 nt = fma2(Rq, bc2(-1.f), make_float2(-Cr.c[1], -Cf.c[1]));  // -(R + R0)
        dR = fma2(fma2(dR, nt, D2), mul2(bc2(0.5f), rinvq), dR);
        const float2 Z = lin_ff_x2(z1q, xk, z0q);
        float2 arg = fma2(mul2(dR, dR), cpair(Cr, Cf, 2), mul2(abs2(Z), cpair(Cr, Cf, 3)));
        const float dth = atan2_poly(fmaf(PS.fy1[5], xk.hi, PS.fy0[5]), fmaf(PS.fx1[5], xk.hi, PS.fx0[5]));
        arg.y = fmaf(dth * dth, Cf.c[7], arg.y);
        const float2 dens = make_float2(ex2_ftz(-arg.x), ex2_ftz(-arg.y));
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          psq[s] = fma2(wBq[s], dens, psq[s]);
          if (Fl::scat(P)) pSq[s] = fma2(wSq[s], dens, pSq[s]);
        }
      }
    };
    // the block sums into the compensated totals
    const auto block_sum = [&]() {
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        const KSpecF32& S = P.spec[s];
        const float2 o12 = make_float2(S.outer[1], S.outer[2]), oq = make_float2(S.outer[4], S.outer[5]);
        const float2 a12 = make_float2(S.outer_alb[1], S.outer_alb[2]), aq = make_float2(S.outer_alb[4], S.outer_alb[5]);
        kahan_add(as0[s], ac0[s], Fl::scat(P) ? fmaf(ps0[s], S.outer[0], pS0[s] * S.outer_alb[0]) : ps0[s] * S.outer[0]);
        kahan_add(as3[s], ac3[s], Fl::scat(P) ? fmaf(ps3[s], S.outer[3], pS3[s] * S.outer_alb[3]) : ps3[s] * S.outer[3]);
        kahan_add2(as12[s], ac12[s], Fl::scat(P) ? fma2(ps12[s], o12, mul2(pS12[s], a12)) : mul2(ps12[s], o12));
        kahan_add2(asq[s], acq[s], Fl::scat(P) ? fma2(psq[s], oq, mul2(pSq[s], aq)) : mul2(psq[s], oq));
        ps0[s] = ps3[s] = pS0[s] = pS3[s] = 0.f;
        ps12[s] = psq[s] = pS12[s] = pSq[s] = bc2(0.f);
      }
    };
    if (Fl::scat(P)) {  // a compile-time constant here
      // with scattering: one loop over the nodes, two per iteration (1.5 % faster than one)
#pragma unroll 2
      for (int k = 0; k < P.n_nodes; ++k) {
        node(k);
        if ((k % kSumBlock) == kSumBlock - 1 || k == P.n_nodes - 1) block_sum();
      }
    } else {
      // without: blocks of kSumBlock nodes, so no node tests for the end of its block (1.5 % faster
      // than one loop with that test; with scattering 0.7 % slower)
      for (int k0 = 0; k0 < P.n_nodes; k0 += kSumBlock) {
        const int k1 = min(k0 + kSumBlock, P.n_nodes);
#pragma unroll 1
        for (int k = k0; k < k1; ++k) node(k);
        block_sum();
      }
    }

    // ---- outputs: x (stop - start)/2, component order total ------------------
    const int64_t col = out_col(SC, i);
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      const float sums[NC] = {as0[s] - ac0[s], as12[s].x - ac12[s].x, as12[s].y - ac12[s].y,
                              as3[s] - ac3[s], asq[s].x - acq[s].x,   asq[s].y - acq[s].y};
      // (stop - start)/2: range 0 for the cloud and bands, the packed lanes for the ring and feature
      const float hsr0 = PS.hs[0].hi + PS.hs[0].lo;
      const float hsc[NC] = {hsr0, hsr0, hsr0, hsr0, hsq.hi.x + hsq.lo.x, hsq.hi.y + hsq.lo.y};
      double tot = 0.0;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        // the bit conversion measured 1.5 % faster without scattering and 5 % slower with
        // it (the compiler schedules the two instantiations differently); same value either way
        const double v = Fl::scat(P) ? (double)(sums[c] * hsc[c]) : f2d_bits(sums[c] * hsc[c]);
        if (out_comps) out_comps[((int64_t)s * NC + c) * n_pix + col] = v;
        tot = (c == 0) ? v : __dadd_rn(tot, v);
      }
      if (out_total) out_total[(int64_t)s * n_pix + col] = tot;
    }
  }
  sched_finish<MODE>(SC);
}

template <int NSPEC, uint32_t FLAGS>
static cudaError_t launch_dirbe_cp_t(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                     double* ot, cudaStream_t st, const LaunchArgs& L) {
  const size_t smem = sizeof(float4) * P.n_temps * NSPEC;
  if (L.sched.queue)
    fwd_dirbe_cp_kernel<NSPEC, FLAGS, true><<<(unsigned)fwd_grid(L, n), L.tpb, smem, st>>>(P, u, n, obs, oc, ot, L.sched);
  else
    fwd_dirbe_cp_kernel<NSPEC, FLAGS, false><<<(unsigned)fwd_grid(L, n), L.tpb, smem, st>>>(P, u, n, obs, oc, ot, L.sched);
  return cudaGetLastError();
}

// Launcher (zl_fwd_dirbe_cp.cu); cudaErrorNotSupported for a flag set it is not compiled for.
cudaError_t launch_fwd_dirbe_cp(const KParamsF32& P, uint32_t flags, const double* u, int64_t n, const ObsArgs& obs,
                                double* oc, double* ot, cudaStream_t st, const LaunchArgs& L);

}  // namespace zl
