// Two-pixel forward kernel on Blackwell's packed FP32 instructions.
//
// The float32 forward kernel is bound by instruction issue, and most of what it
// issues goes to the FMA pipes.  sm_100-class GPUs execute fma/mul/add on a pair
// of float32 values as one instruction (fma.rn.f32x2 and friends), so a thread
// that integrates two pixels at once -- lanes .x and .y of every float2 below --
// issues one packed instruction where the one-pixel kernel issues two.  MUFU
// operations (ex2, lg2, rsqrt), the blackbody table lookup, comparisons and the
// feature's atan2 have no packed form and run per lane.
//
// Every lane performs exactly the one-pixel kernel's arithmetic (zl_fwd_f32.cuh):
// the per-pixel set-up is the same function, run once per lane, and each packed
// operation rounds as its scalar counterpart.  Subtractions a - b are written as
// fma(b, -1, a), which rounds like a - b.
//
// Lanes: on the static schedule without band tails, item j integrates pixels j and
// j + ceil(n/2); otherwise the work is cut into tiles of T items (pixel pairs) covering 2T
// consecutive pixels, item j of tile t integrating pixels 2Tt + j and 2Tt + T + j, so that
// the two lanes hold neighbours of the input order.  Loads and stores of the [3][n] and
// [.][n] arrays stay coalesced either way.  Past the end of the pixels the second lane
// repeats the first pixel and is not stored.
//
// Band tails (TAILS): as in the DIRBE paired kernel (zl_fwd_dirbe.cuh), past the node
// from which a band's factor e^-(zeta/dzeta)^6 is zero in float32 for both lanes of every
// thread of the warp, the band adds exactly nothing and a warp-uniform branch skips it.
// That pays where a warp's pixels are coherent (a HEALPix ring, directions sorted by
// latitude) and costs the per-pixel estimate and per-node branches where they are not
// (unsorted random directions), so the caller chooses.
#pragma once

#include "zl_fwd_f32.cuh"
#include "zl_packed.cuh"

namespace zl {

// Band c of a layout: whether a later band reuses its inner-cutoff term 1 - e^-(R/delta_r)^20
template <uint32_t LAYOUT, uint32_t FLAGS>
__host__ __device__ constexpr bool t4_shared_later(int c) {
  for (int j = c + 1; j < Lay<LAYOUT>::ncomp(); ++j)
    if (Lay<LAYOUT>::type(j) == ZL_BAND && ((FLAGS >> (24 + j)) & 1u) && Lay<LAYOUT>::first_band(j) == c) return true;
  return false;
}

// Every band of the layout is centred on the Sun (the band-tail estimate measures from it)
template <uint32_t LAYOUT, uint32_t FLAGS>
__host__ __device__ constexpr bool bands_centred() {
  for (int c = 0; c < Lay<LAYOUT>::ncomp(); ++c)
    if (Lay<LAYOUT>::type(c) == ZL_BAND && ((FLAGS >> (8 + c)) & 1u)) return false;
  return true;
}

// MODE: the schedule the kernel is compiled for (kSchedStatic or kSchedQueue): one build serving
// both (kSchedAny) ran 7 % slower on the static schedule (batched random directions, 15.61 ms
// against 14.54 ms).
template <int NSPEC, uint32_t LAYOUT, uint32_t FLAGS, bool TAILS, int MODE>
__global__ void __launch_bounds__(128, (NSPEC == 1 && LAYOUT == kLayoutPlanck) ? 4 : 0) fwd_f32x2_kernel(const __grid_constant__ KParamsF32 P,
                                                        const double* __restrict__ u, int64_t n_pix,
                                                        int64_t n_items, const ObsArgs OA,
                                                        double* __restrict__ out_comps,
                                                        double* __restrict__ out_total, const Sched SC) {
  using L = Lay<LAYOUT>;
  using Fl = KFlags<FLAGS>;
  static_assert(LAYOUT != kLayoutGeneric && !Fl::runtime, "the two-pixel kernel serves the built-in layouts");
  constexpr int NC = L::ncomp();
  extern __shared__ float4 tab_sm[];  // [NSPEC][nT]
  const int nT = P.n_temps;
  for (int t = threadIdx.x; t < nT * NSPEC; t += blockDim.x) tab_sm[t] = P.table[t / nT][t % nT];
  // Halves (static schedule without band tails): item j evaluates pixels j and j + n_items,
  // n_items = ceil(n_pix / 2).  Tiles (otherwise): n_items = TL x the number of 2 TL-pixel
  // tiles (TL: the schedule's tile), item j of tile k evaluates pixels 2 TL k + j and
  // 2 TL k + j + TL, so that both lanes of a thread hold neighbours of the input order (band
  // tails need coherent lanes; a queued tile must hold both of its pixels).  The halves ran
  // 1.6 % faster on the batched random-direction workload.
  constexpr bool kHalves = MODE == kSchedStatic && !TAILS;
  const int64_t TL = sched_tile(SC);
  // the observer set-ups the block's first lanes .x and .y share (the two halves of a batch
  // usually belong to different observers): warps 0 and 1 derive one each.  The Planck layout
  // only: the DIRBE layout's two-pixel kernel (not its default) spilled with them at 168
  // registers and keeps the per-pixel set-up.
  constexpr bool kShared = LAYOUT == kLayoutPlanck;
  __shared__ ObsSetupF32<NC> s_obs[kShared ? 2 : 1];
  const int64_t first_a = kHalves ? (int64_t)blockIdx.x * blockDim.x : 2 * (int64_t)blockIdx.x * blockDim.x;
  const int64_t first_b = kHalves ? first_a + n_items : first_a + TL;
  const int cached_a = kShared ? obs_cache_index<MODE>(OA, first_a, n_pix) : -1;
  const int cached_b = kShared ? obs_cache_index<MODE>(OA, first_b, n_pix) : -1;
  if (kShared && threadIdx.x == 0 && cached_a >= 0)
    observer_setup<LAYOUT, FLAGS, NC>(P, record_observer(OA, cached_a), s_obs[0]);
  if (kShared && threadIdx.x == (blockDim.x > 32 ? 32u : 0u) && cached_b >= 0)
    observer_setup<LAYOUT, FLAGS, NC>(P, record_observer(OA, cached_b), s_obs[kShared ? 1 : 0]);
  __syncthreads();
  ZL_SCHED_LOOP(MODE, SC, n_items, item) {
    const int64_t ia = kHalves ? item : item + ZL_SCHED_TILE_BASE(MODE, SC, item);
    if (ia >= n_pix) continue;
    const int64_t ib = kHalves ? (ia + n_items < n_pix ? ia + n_items : ia) : (ia + TL < n_pix ? ia + TL : ia);

    // ---- per-pixel set-up, one lane at a time, then packed ---------------
    ff2 hs[NC], mh[NC], z1[NC], z0[NC], wm[NC], wa[NC], wb[NC];
    float2 b2[NC], rr[NC], fx1[NC], fx0[NC], fy1[NC], fy0[NC];
    float2 b2h, bperp;
    {
      PixSetupF32<NC> A, B;
      if (kShared) {
        pixel_setup_cached<LAYOUT, FLAGS, true, NC>(P, u, n_pix, OA, ia, cached_a, s_obs[0], A);
        pixel_setup_cached<LAYOUT, FLAGS, true, NC>(P, u, n_pix, OA, ib, cached_b, s_obs[kShared ? 1 : 0], B);
      } else {
        pixel_setup<LAYOUT, FLAGS, true, NC>(P, u, n_pix, OA, ia, A);
        pixel_setup<LAYOUT, FLAGS, true, NC>(P, u, n_pix, OA, ib, B);
      }
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        hs[c] = pack_ff(A.hs[c], B.hs[c]);
        mh[c] = pack_ff(A.mh[c], B.mh[c]);
        z1[c] = pack_ff(A.z1[c], B.z1[c]);
        z0[c] = pack_ff(A.z0[c], B.z0[c]);
        wm[c] = pack_ff(A.wm[c], B.wm[c]);
        wa[c] = pack_ff(A.wa[c], B.wa[c]);
        wb[c] = pack_ff(A.wb[c], B.wb[c]);
        b2[c] = make_float2(A.b2[c], B.b2[c]);
        rr[c] = make_float2(A.rr[c], B.rr[c]);
        fx1[c] = make_float2(A.fx1[c], B.fx1[c]);
        fx0[c] = make_float2(A.fx0[c], B.fx0[c]);
        fy1[c] = make_float2(A.fy1[c], B.fy1[c]);
        fy0[c] = make_float2(A.fy0[c], B.fy0[c]);
      }
      b2h = make_float2(A.b2h, B.b2h);
      bperp = make_float2(A.bperp, B.bperp);
    }

    // band tails: kt[c] = first node from which band c is zero for the whole warp; kt4[c] = first
    // node from which its inner-cutoff term is needed by no band of the warp
    int kt[NC], kt4[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) kt[c] = kt4[c] = P.n_nodes;
    if (TAILS) {
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (L::type(c) == ZL_BAND) {
          const float ta = band_zero_tail(z1[c].hi.x, z0[c].hi.x, hs[c].hi.x, mh[c].hi.x, b2h.x, P.comp[c].c[1]);
          const float tb = band_zero_tail(z1[c].hi.y, z0[c].hi.y, hs[c].hi.y, mh[c].hi.y, b2h.y, P.comp[c].c[1]);
          kt[c] = kt4[c] = warp_tail_index(P, fmaxf(ta, tb));
        }
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (L::type(c) == ZL_BAND && Fl::share_first(c)) {
          const int f = L::first_band(c);
          kt4[f] = max(kt4[f], kt[c]);
        }
    }

    // quadrature sums: plain float32 over blocks of kSumBlock nodes, Kahan-compensated across blocks
    // (the density prefactor and emissivity / albedo multiply each block sum: S.outer, S.outer_alb)
    float2 acc_s[NC][NSPEC], acc_c[NC][NSPEC], part[NC][NSPEC], partS[NC][NSPEC];
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) acc_s[c][s] = acc_c[c][s] = part[c][s] = partS[c][s] = bc2(0.f);

    // ---- quadrature nodes ------------------------------------------------
#pragma unroll 1
    for (int k = 0; k < P.n_nodes; ++k) {
      const ff xk = {P.gl_x_hi[k], P.gl_x_lo[k]};
      const float wk = P.gl_w[k];
      float2 wh = bc2(0.f), R2 = bc2(1.f), rinv = bc2(1.f), R = bc2(1.f), lg2R = bc2(0.f);
      float2 wB[NSPEC], wS[NSPEC], t4s[NC];  // w_k B(T) and w_k x the scattering term of the range
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) wB[s] = wS[s] = bc2(0.f);
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        t4s[c] = bc2(0.f);
        const KCompF32& C = P.comp[c];
        const int type = L::type(c);
        if (L::first(c)) {
          // brightness.py:27-33 -- heliocentric distance of the node, R^2 = w^2 + b^2, and temperature
          wh = lin_ff_x2(hs[c], xk, mh[c]);
          R2 = fma2(wh, wh, b2h);
          rinv = rsqrt_2(R2);
          if (type == ZL_CLOUD || type == ZL_BAND)
            rinv = mul2(rinv, fma2(mul2(bc2(-0.5f), R2), mul2(rinv, rinv), bc2(1.5f)));
          R = mul2(R2, rinv);
          lg2R = lg2_2(R);
          const float2 T = mul2(bc2(P.T0), ex2_2(mul2(bc2(P.neg_delta), lg2R)));  // blackbody.py:16-30
#pragma unroll
          for (int s = 0; s < NSPEC; ++s)
            wB[s] = mul2(bc2(wk), make_float2(bb_lookup(tab_sm + s * nT, T.x, P.t_min, P.t_max, P.inv_dt, nT),
                                              bb_lookup(tab_sm + s * nT, T.y, P.t_min, P.t_max, P.inv_dt, nT)));
          if (Fl::scat(P)) {  // scattering.py:11-59
            const float2 theta = make_float2(atan2_poly(bperp.x, -wh.x), atan2_poly(bperp.y, -wh.y));
            const float2 flux = mul2(rinv, rinv);
#pragma unroll
            for (int s = 0; s < NSPEC; ++s) {
              const KSpecF32& S = P.spec[s];
              const float2 ph = add2(fma2(bc2(S.C2), theta, bc2(S.C1)), ex2_2(mul2(bc2(S.C3l2e), theta)));
              wS[s] = mul2(bc2(wk), mul2(mul2(bc2(S.S), flux), mul2(bc2(S.N), ph)));
            }
          }
        }
        // own distance when the component is offset from the Sun
        float2 Rc2 = R2, rcinv = rinv, Rc = R, lg2Rc = lg2R;
        if (Fl::offset(C, c)) {
          const float2 wc = lin_ff_x2(hs[c], xk, wm[c]);
          Rc2 = fma2(wc, wc, b2[c]);
          rcinv = rsqrt_2(Rc2);
          if (type == ZL_BAND) rcinv = mul2(rcinv, fma2(mul2(bc2(-0.5f), Rc2), mul2(rcinv, rcinv), bc2(1.5f)));
          Rc = mul2(Rc2, rcinv);
          lg2Rc = mul2(bc2(0.5f), lg2_2(Rc2));
        }
        const float2 Z = lin_ff_x2(z1[c], xk, z0[c]);
        float2 dens;
        if (type == ZL_CLOUD) {  // number_density.py:60-73
          const float2 zeta = mul2(abs2(Z), rcinv);
          const float2 gin = mul2(mul2(zeta, zeta), bc2(C.c[5]));
          const float2 gout = sub2(zeta, bc2(C.c[6]));
          const float2 g = make_float2(zeta.x < C.c[4] ? gin.x : gout.x, zeta.y < C.c[4] ? gin.y : gout.y);
          const float2 gg = ex2_2(mul2(bc2(C.c[3]), lg2_2(g)));
          dens = ex2_2(fma2(bc2(-C.c[1]), lg2Rc, mul2(bc2(-C.c[2]), gg)));
        } else if (type == ZL_BAND) {  // number_density.py:99-110
          if (TAILS && k >= kt[c]) {
            // zero for every pixel of the warp from here on; a later band may still need the
            // inner-cutoff term
            if (t4_shared_later<LAYOUT, FLAGS>(c) && k < kt4[c]) {
              const float2 q = mul2(Rc2, bc2(C.c[4]));
              const float2 q2 = mul2(q, q), q4 = mul2(q2, q2), q8 = mul2(q4, q4);
              const float2 y = mul2(q8, q2);
              const float2 ny = mul2(y, bc2(-1.f));
              float2 ser = fma2(ny, bc2(1.f / 720.f), bc2(1.f / 120.f));
              ser = fma2(ny, ser, bc2(1.f / 24.f));
              ser = fma2(ny, ser, bc2(1.f / 6.f));
              ser = fma2(ny, ser, bc2(0.5f));
              ser = mul2(y, fma2(ny, ser, bc2(1.f)));
              const float2 alt = sub2(bc2(1.f), ex2_2(mul2(bc2(-kLog2e), y)));
              t4s[c] = make_float2(y.x < 0.25f ? ser.x : alt.x, y.y < 0.25f ? ser.y : alt.y);
            }
            continue;
          }
          const float2 zz = mul2(mul2(abs2(Z), rcinv), bc2(C.c[1]));
          const float2 z2 = mul2(zz, zz);
          const float2 t2 = ex2_2(mul2(bc2(-kLog2e), mul2(mul2(z2, z2), z2)));
          const float2 zp = Fl::p4(C, c) ? mul2(z2, z2) : ex2_2(mul2(bc2(C.c[3]), lg2_2(zz)));
          const float2 t3 = fma2(zp, bc2(C.c[2]), bc2(1.f));
          float2 t4;
          if (Fl::share_first(c)) {
            t4 = t4s[L::first_band(c)];
          } else {
            const float2 q = mul2(Rc2, bc2(C.c[4]));  // (R/delta_r)^2
            const float2 q2 = mul2(q, q), q4 = mul2(q2, q2), q8 = mul2(q4, q4);
            const float2 y = mul2(q8, q2);  // (R/delta_r)^20
            // 1 - e^-y: below 1/4 by its series, above from ex2
            const float2 ny = mul2(y, bc2(-1.f));
            float2 ser = fma2(ny, bc2(1.f / 720.f), bc2(1.f / 120.f));
            ser = fma2(ny, ser, bc2(1.f / 24.f));
            ser = fma2(ny, ser, bc2(1.f / 6.f));
            ser = fma2(ny, ser, bc2(0.5f));
            ser = mul2(y, fma2(ny, ser, bc2(1.f)));
            const float2 alt = sub2(bc2(1.f), ex2_2(mul2(bc2(-kLog2e), y)));
            t4 = make_float2(y.x < 0.25f ? ser.x : alt.x, y.y < 0.25f ? ser.y : alt.y);
          }
          t4s[c] = t4;
          dens = mul2(mul2(mul2(rcinv, t2), t3), t4);
        } else {  // ring (number_density.py:136-139) and feature (:167-181)
          float2 dR = sub2(Rc, bc2(C.c[1]));
          // R^2 - R0^2 = (w - w0)(w + w0) + rr to ~1 ulp; one Newton step on R
          const float2 D2 = fma2(lin_ff_x2(hs[c], xk, wa[c]), lin_ff_x2(hs[c], xk, wb[c]), rr[c]);
          const float2 nt = fma2(Rc, bc2(-1.f), bc2(-C.c[1]));  // -(R + R0)
          dR = fma2(fma2(dR, nt, D2), mul2(bc2(0.5f), rcinv), dR);
          float2 arg = fma2(mul2(dR, dR), bc2(C.c[2]), mul2(abs2(Z), bc2(C.c[3])));
          if (featurelike(type)) {
            const float2 yy = fma2(fy1[c], bc2(xk.hi), fy0[c]);
            const float2 xx = fma2(fx1[c], bc2(xk.hi), fx0[c]);
            const float2 dth = make_float2(atan2_poly(yy.x, xx.x), atan2_poly(yy.y, xx.y));
            arg = fma2(mul2(dth, dth), bc2(C.c[7]), arg);
          }
          dens = make_float2(ex2_ftz(-arg.x), ex2_ftz(-arg.y));
        }
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          const KSpecF32& S = P.spec[s];
          part[c][s] = fma2(wB[s], dens, part[c][s]);
          if (Fl::scat(P)) partS[c][s] = fma2(wS[s], dens, partS[c][s]);
        }
      }
      if ((k % kSumBlock) == kSumBlock - 1 || k == P.n_nodes - 1) {
#pragma unroll
        for (int c = 0; c < NC; ++c)
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) {
            const KSpecF32& S = P.spec[s];
            const float2 blk = Fl::scat(P) ? fma2(part[c][s], bc2(S.outer[c]), mul2(partS[c][s], bc2(S.outer_alb[c])))
                                           : mul2(part[c][s], bc2(S.outer[c]));
            kahan_add2(acc_s[c][s], acc_c[c][s], blk);
            part[c][s] = partS[c][s] = bc2(0.f);
          }
      }
    }

    // ---- outputs: x (stop - start)/2, component order total ----------------
#pragma unroll
    for (int lane = 0; lane < 2; ++lane) {
      if (lane == 1 && ib == ia) break;
      const int64_t i = out_col(SC, lane ? ib : ia);
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        double tot = 0.0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const float as = lane ? acc_s[c][s].y : acc_s[c][s].x;
          const float ac = lane ? acc_c[c][s].y : acc_c[c][s].x;
          const float hh = lane ? hs[c].hi.y : hs[c].hi.x;
          const float hl = lane ? hs[c].lo.y : hs[c].lo.x;
          // as the one-pixel kernel: float32 product, float64 total of the stored components
          const double v = (double)((as - ac) * (hh + hl));
          if (out_comps) out_comps[((int64_t)s * NC + c) * n_pix + i] = v;
          tot = (c == 0) ? v : __dadd_rn(tot, v);
        }
        if (out_total) out_total[(int64_t)s * n_pix + i] = tot;
      }
    }
  }
  sched_finish<MODE>(SC);
}

template <int NSPEC, uint32_t LAYOUT, uint32_t FLAGS, bool TAILS>
static cudaError_t launch_f32x2_t(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                  double* ot, cudaStream_t st, const LaunchArgs& L) {
  const size_t smem = sizeof(float4) * P.n_temps * NSPEC;
  const int64_t T = L.sched.queue ? L.sched.tile : L.tpb;
  const int64_t items = (L.sched.queue || TAILS) ? ((n + 2 * T - 1) / (2 * T)) * T : (n + 1) / 2;
  if (L.sched.queue)
    fwd_f32x2_kernel<NSPEC, LAYOUT, FLAGS, TAILS, kSchedQueue>
        <<<(unsigned)fwd_grid(L, items), L.tpb, smem, st>>>(P, u, n, items, obs, oc, ot, L.sched);
  else
    fwd_f32x2_kernel<NSPEC, LAYOUT, FLAGS, TAILS, kSchedStatic>
        <<<(unsigned)fwd_grid(L, items), L.tpb, smem, st>>>(P, u, n, items, obs, oc, ot, L.sched);
  return cudaGetLastError();
}

template <uint32_t LAYOUT, uint32_t FLAGS, bool TAILS>
static cudaError_t launch_f32x2_flags(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs,
                                      double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  switch (P.n_spec) {
    case 1: return launch_f32x2_t<1, LAYOUT, FLAGS, TAILS>(P, u, n, obs, oc, ot, st, L);
    case 2: return launch_f32x2_t<2, LAYOUT, FLAGS, TAILS>(P, u, n, obs, oc, ot, st, L);
    case 3: return launch_f32x2_t<3, LAYOUT, FLAGS, TAILS>(P, u, n, obs, oc, ot, st, L);
    default: return launch_f32x2_t<4, LAYOUT, FLAGS, TAILS>(P, u, n, obs, oc, ot, st, L);
  }
}

// Two-pixel launchers of the built-in layouts (zl_fwd_f32x2_dirbe.cu, zl_fwd_f32x2_planck.cu);
// they return cudaErrorNotSupported for a flag set they are not compiled for.  tails: skip the
// bands' zero tails (coherent inputs).
cudaError_t launch_fwd_f32x2_dirbe(const KParamsF32& P, uint32_t flags, bool tails, const double* u, int64_t n,
                                   const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L);
cudaError_t launch_fwd_f32x2_planck(const KParamsF32& P, uint32_t flags, bool tails, const double* u, int64_t n,
                                    const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L);

}  // namespace zl
