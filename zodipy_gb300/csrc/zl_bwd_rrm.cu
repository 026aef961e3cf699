// Adjoint of the Rowan-Robinson & May (RRM) model: gradient of a per-pixel loss with respect to
// every parameter of the reference's rrm-experimental dictionary.
//
// The RRM integrand (zodipy/brightness.py:59-83) is, per component c and spectral set s,
//   out[s, c, i] = hs_c(i) sum_k w_k B_s(T_c(R_k)) n_c(X_k - X_0,c) cal_s
// with T_c = T_0,c R^-delta_c (R: distance from the Sun) and the densities of
// zodipy/number_density.py:184-404 (fan, comet, narrow and broad bands, interstellar
// dust, and the Kelsall ring and feature times an amplitude A).  One launch per component
// recomputes its line of sight (its own LOS range) node by node and accumulates, per pixel,
//   dL/dp = sum_s g[s,c] hs cal_s sum_k w_k B_s n_c d ln n_c / dp
// for the component's geometry and own parameters, the T_0 / delta derivatives through the
// blackbody table's segment slope, and the calibration's (linear) derivative.
//
// Masks: the fan (R <= R_outer), the comet and the bands (R_inner <= R <= R_outer) and the
// narrow band's latitude cut |beta| < beta_nb are step functions of the parameters; the
// quadrature's nodes do not move with them (the LOS cutoffs are fixed radii,
// zodipy/line_of_sight.py:28-49), so the derivative of the quadrature with respect to a mask
// edge is zero almost everywhere, and only the smooth dependences are differentiated (R_outer
// of the bands' power law (R / R_outer)^-gamma, beta_nb of exp(G (|beta| - beta_nb))).
//
// Determinism as the Kelsall adjoint: fixed 128-pixel tiles, a fixed shuffle tree per tile,
// tile partials summed in a fixed order by rrm_reduce_kernel.
#include <cstring>

#include "zl_bwd_f32.cuh"

namespace zl {

// Per-component partial row: slots 0-4 x_0, y_0, z_0, i, Omega; 5 .. 5 + own - 1 the type's own
// parameters; then T_0, delta; the calibrations of the spectral sets in the last ZL_MAX_SPEC slots.
constexpr int kRrmSlots = 20;
constexpr int kRrmCal = kRrmSlots - ZL_MAX_SPEC;
constexpr float kRad2Deg = 57.29577951308232f;

// Host-derived constants of the RRM derivatives, per component.
//   q: fan         gamma, Z_0, Q, P, 1/Z_0
//      comet       gamma, Z_0, P, amp, 1/Z_0
//      narrow band gamma, A, G, beta_nb [deg], R_outer
//      broad band  gamma, A, beta_bb [deg], sigma_bb [deg], R_outer
//      interstellar amp
//      ring        n_0, R, sigma_r, sigma_z, A
//      feature     n_0, R, sigma_r, sigma_z, A, theta [rad], sigma_theta [rad]
//   r2: squared mask radii (R_inner^2, R_outer^2); 0 / +inf where the type has none
struct KGradRrm {
  float dni[ZL_MAX_COMPS][3], dnO[ZL_MAX_COMPS][2];
  float q[ZL_MAX_COMPS][8];
  float r2in[ZL_MAX_COMPS], r2out[ZL_MAX_COMPS];
  float T0[ZL_MAX_COMPS], neg_delta[ZL_MAX_COMPS];
  float cal[ZL_MAX_SPEC];
  int32_t n_own[ZL_MAX_COMPS];
};

// Density of component c (type TYPE) at Xc = X - X_0 with |Xc| = Rc, height Z, and its
// log-derivatives: GR = d ln n / d Rc (Z fixed), GZ = d ln n / d Z (Rc fixed), d[j] = d ln n /
// d (own parameter j), and for the feature the angle dth (the caller forms the X_0 terms).
struct RrmTerms {
  float n, GR, GZ, d[7], dth;
};

template <int TYPE>
__device__ __forceinline__ RrmTerms rrm_terms(const float* q, float r2in, float r2out, float Rc2, float Rc, float rcinv,
                                              float Z, float dth) {
  RrmTerms t;
  t.n = 0.f;
  t.GR = t.GZ = t.dth = 0.f;
#pragma unroll
  for (int j = 0; j < 7; ++j) t.d[j] = 0.f;
  if (TYPE == ZL_INTERSTELLAR) {  // number_density.py:259-264: n = amp
    t.n = q[0];
    t.d[0] = 1.f / q[0];
    return t;
  }
  if (TYPE == ZL_RING_RRM || TYPE == ZL_FEATURE_RRM) {  // A x the Kelsall ring / feature (:345-403)
    const float dR = Rc - q[1];
    const float isr2 = 1.f / (q[2] * q[2]);
    float arg = dR * dR * isr2 + fabsf(Z) / q[3];
    if (TYPE == ZL_FEATURE_RRM) arg = fmaf(dth * dth, 1.f / (q[6] * q[6]), arg);
    t.n = q[0] * q[4] * __expf(-arg);
    t.GR = -2.f * dR * isr2;
    t.GZ = Z != 0.f ? -copysignf(1.f / q[3], Z) : 0.f;
    t.d[0] = 1.f / q[0];                                // n_0
    t.d[1] = 2.f * dR * isr2;                           // R
    t.d[2] = 2.f * dR * dR * isr2 / q[2];               // sigma_r
    t.d[3] = fabsf(Z) / (q[3] * q[3]);                  // sigma_z
    t.d[TYPE == ZL_RING_RRM ? 4 : 6] = 1.f / q[4];      // A (last of the ring's, last of the feature's)
    if (TYPE == ZL_FEATURE_RRM) {
      const float ist2 = 1.f / (q[6] * q[6]);
      t.d[4] = 2.f * dth * ist2 * kDeg;                  // theta [deg]: d(-dth^2/st^2)/dtheta
      t.d[5] = 2.f * dth * dth * ist2 / q[6] * kDeg;     // sigma_theta [deg]
      t.dth = -2.f * dth * ist2;                         // d ln n / d dth (for the X_0 terms)
    }
    return t;
  }
  // fan, comet, narrow and broad band: masks, latitude beta = asin(Z / Rc)
  if (Rc2 > r2out || Rc2 < r2in) return t;
  const float s = fminf(fmaxf(Z * rcinv, -1.f), 1.f);
  const float beta = asinf(s);
  const float cb = sqrtf(fmaxf(1.f - s * s, 0.f));
  // d beta / d Z and d beta / d Rc at fixed Rc, Z; cos(beta) floored at 1e-6 so that a node
  // on the axis (|Z| = Rc, where the derivative has no finite value) gives large but finite terms
  const float icb = 1.f / fmaxf(cb, 1e-6f);
  const float dbZ = rcinv * icb;
  const float dbR = -s * rcinv * icb;
  const float lnR = __logf(Rc);
  if (TYPE == ZL_FAN || TYPE == ZL_COMET) {  // number_density.py:184-256
    const float gamma = q[0], Z0 = q[1];
    const float aZ = fabsf(Z), ab = fabsf(beta);
    const bool in = aZ < Z0;
    const float eps = in ? 2.f - aZ * q[4] : 1.f;
    const float lab = ab > 0.f ? __logf(ab) : 0.f;
    const float be = ab > 0.f ? __expf(eps * lab) : 0.f;  // |beta|^eps
    float sn, cs;
    __sincosf(be, &sn, &cs);
    const float P = TYPE == ZL_FAN ? q[3] : q[2];
    float lnf = -P * sn;
    // d/d beta of -P sin(|beta|^eps): -P cos(|beta|^eps) eps |beta|^(eps-1) sign(beta)
    float Gb = ab > 0.f ? -P * cs * eps * be / ab * (beta < 0.f ? -1.f : 1.f) : 0.f;
    // d/d eps of -P sin(|beta|^eps): -P cos(|beta|^eps) |beta|^eps ln|beta|
    const float Ge = -P * cs * be * lab;
    if (TYPE == ZL_FAN) {
      const float Q = q[2];
      lnf += Q * __logf(fmaxf(cb, 1e-30f));
      Gb += -Q * s * icb;  // d/d beta of Q ln cos beta = -Q tan beta
    }
    const float amp = TYPE == ZL_FAN ? 1.f : q[3];
    t.n = amp * __expf(-gamma * lnR + lnf);
    t.GR = -gamma * rcinv + Gb * dbR;
    t.GZ = Gb * dbZ + (in && Z != 0.f ? Ge * -copysignf(q[4], Z) : 0.f);  // d eps / d Z = -sign(Z) / Z_0
    t.d[0] = -lnR;                                        // gamma
    t.d[1] = in ? Ge * aZ * q[4] * q[4] : 0.f;           // Z_0: d eps / d Z_0 = |Z| / Z_0^2
    if (TYPE == ZL_FAN) {
      t.d[2] = __logf(fmaxf(cb, 1e-30f));                // Q
      t.d[3] = -sn;                                       // P
    } else {
      t.d[2] = -sn;                                       // P
      t.d[3] = 1.f / q[3];                                // amp
    }
    return t;
  }
  const float gamma = q[0], A = q[1], Rout = q[4];
  const float bd = beta * kRad2Deg;
  const float radial = __expf(-gamma * (lnR - __logf(Rout)));  // (R / R_outer)^-gamma
  if (TYPE == ZL_NARROW_BAND) {  // number_density.py:267-304
    const float G = q[2], bnb = q[3];
    const float abd = fabsf(bd);
    if (!(abd < bnb)) return t;
    t.n = A * radial * __expf(G * (abd - bnb));
    const float Gb = G * kRad2Deg * (bd < 0.f ? -1.f : 1.f);  // d/d beta of G |beta_deg|
    t.GR = -gamma * rcinv + Gb * dbR;
    t.GZ = Gb * dbZ;
    t.d[0] = -(lnR - __logf(Rout));  // gamma
    t.d[1] = 1.f / A;                // A
    t.d[2] = abd - bnb;              // G
    t.d[4] = gamma / Rout;           // R_outer (the power law; the mask edge adds nothing)
    t.d[5] = -G;                     // beta_nb
    return t;
  }
  // broad band, number_density.py:307-342
  const float bbb = q[2], sbb = q[3];
  const float a = (bd - bbb) / sbb, b = (bd + bbb) / sbb;
  const float e1 = __expf(-0.5f * a * a), e2 = __expf(-0.5f * b * b);
  const float f = e1 + e2;
  t.n = A * radial * f;
  // 1/f where f is a normal float32 (e1 and e2 are both below f, so each ratio stays bounded);
  // where both Gaussians have underflowed the density and its derivatives are zero
  const float inf = f > 1e-30f ? 1.f / f : 0.f;
  const float Gb = -(a * e1 + b * e2) / sbb * inf * kRad2Deg;  // d ln f / d beta [rad]
  t.GR = -gamma * rcinv + Gb * dbR;
  t.GZ = Gb * dbZ;
  t.d[0] = -(lnR - __logf(Rout));            // gamma
  t.d[1] = 1.f / A;                          // A
  t.d[3] = gamma / Rout;                     // R_outer
  t.d[4] = (a * e1 - b * e2) / sbb * inf;    // beta_bb [deg]
  t.d[5] = (a * a * e1 + b * b * e2) / sbb * inf;  // sigma_bb [deg]
  return t;
}

// Own parameters of an RRM component type (the reference's dataclass fields after the geometry).
__host__ __device__ constexpr int rrm_own(int type) {
  return type == ZL_FAN ? 5 : type == ZL_INTERSTELLAR ? 1 : type == ZL_RING_RRM ? 5 : type == ZL_FEATURE_RRM ? 7 : 6;
}

template <int TYPE, int NSPEC>
__global__ void __launch_bounds__(kTile) bwd_rrm_kernel(const __grid_constant__ KParamsF32 P,
                                                        const __grid_constant__ KGradRrm A, int c,
                                                        const double* __restrict__ u, int64_t n_pix,
                                                        const ObsArgs OA, const double* __restrict__ g_comps,
                                                        const double* __restrict__ g_total,
                                                        double* __restrict__ partials, int64_t n_tiles) {
  constexpr int NOWN = rrm_own(TYPE);
  constexpr int ST0 = 5 + NOWN, SDL = ST0 + 1, SCAL = kRrmCal;
  static_assert(SDL < SCAL, "partial row too short");
  __shared__ float4 tab_sm[NSPEC * ZL_MAX_TEMPS];
  __shared__ float red_sm[kTile / 32][kRrmSlots];
  const int nT = P.n_temps;
  for (int t = threadIdx.x; t < nT * NSPEC; t += blockDim.x) tab_sm[t] = P.table[t / nT][t % nT];
  __syncthreads();
  const KCompF32& C = P.comp[c];
  const int r = C.range;
  const int nc = P.n_comps;
  const float* q = A.q[c];

  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t i = tile * kTile + threadIdx.x;
    float acc[kRrmSlots];
#pragma unroll
    for (int j = 0; j < kRrmSlots; ++j) acc[j] = 0.f;
    if (i < n_pix) {
      // ---- per-pixel set-up: the component's LOS range, frame, upstream gradient ----
      const ff ux = ff_split(u[i]), uy = ff_split(u[n_pix + i]), uz = ff_split(u[2 * n_pix + i]);
      const PixObs O = pixel_observer(OA, i, n_pix);
      const ff ox = ff_split(O.ox), oy = ff_split(O.oy), oz = ff_split(O.oz);
      const ff b = ff_scale(ff_add(ff_mul_nr(ox, ux), ff_mul_nr(oy, uy)), 2.0f);
      const ff r2 = ff_add(ff_add(ff_mul(ox, ox), ff_mul(oy, oy)), ff_mul(oz, oz));
      const ff st = ((O.outside >> (2 * r)) & 1u) ? ff{(float)kEps, 0.f}
                                                  : sphere_distance_ff(b, r2, ff{P.cut_in_hi[r], P.cut_in_lo[r]});
      const ff sp = ((O.outside >> (2 * r + 1)) & 1u) ? ff{(float)kEps, 0.f}
                                                      : sphere_distance_ff(b, r2, ff{P.cut_out_hi[r], P.cut_out_lo[r]});
      const ff hs = ff_scale(ff_add(sp, ff_neg(st)), 0.5f), md = ff_scale(ff_add(sp, st), 0.5f);
      const float uxf = ux.hi, uyf = uy.hi, uzf = uz.hi, oxf = ox.hi, oyf = oy.hi, ozf = oz.hi;
      const float dxc = oxf - C.ox, dyc = oyf - C.oy, dzc = ozf - C.oz;
      const float un = uxf * C.nx + uyf * C.ny + uzf * C.nz;
      const float on = dxc * C.nx + dyc * C.ny + dzc * C.nz;
      const float hsf = hs.hi + hs.lo;
      float gup0[NSPEC], gup[NSPEC];  // upstream gradient times (stop - start)/2, and times the calibration
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) {
        gup0[s] = d2f_bits(g_comps ? g_comps[((int64_t)s * nc + c) * n_pix + i] : g_total[(int64_t)s * n_pix + i]) * hsf;
        gup[s] = gup0[s] * A.cal[s];
      }
      // the feature's frame: longitude relative to Earth's minus theta (number_density.py:167-173)
      float rux = 0.f, ruy = 0.f, rox = 0.f, roy = 0.f, eqx = 0.f, eqy = 0.f;
      if (TYPE == ZL_FEATURE_RRM) {
        const float ex = (float)O.ex - C.ox, ey = (float)O.ey - C.oy;
        const float phi = atan2f(ey, ex) + q[5];
        float sphi, cphi;
        sincosf(phi, &sphi, &cphi);
        rux = cphi * uxf + sphi * uyf;
        ruy = cphi * uyf - sphi * uxf;
        rox = cphi * dxc + sphi * dyc;
        roy = cphi * dyc - sphi * dxc;
        const float e2 = ex * ex + ey * ey;
        eqx = ey / e2;   // d atan2(E - X_0) / d x_0
        eqy = -ex / e2;  // d atan2(E - X_0) / d y_0
      }
      float S1 = 0.f, S2 = 0.f, S3 = 0.f, S4 = 0.f, fthx = 0.f, fthy = 0.f;

#pragma unroll 1
      for (int k = 0; k < P.n_nodes; ++k) {
        const ff xk = {P.gl_x_hi[k], P.gl_x_lo[k]};
        const float wk = P.gl_w[k];
        const float Rl = lin_ff(hs, xk, md);
        const float X0 = fmaf(Rl, uxf, oxf), X1 = fmaf(Rl, uyf, oyf), X2 = fmaf(Rl, uzf, ozf);
        const float Rh2 = fmaf(X0, X0, fmaf(X1, X1, X2 * X2));
        const float lg2Rh = 0.5f * lg2_ftz(Rh2);
        const float Tn = ex2_ftz(A.neg_delta[c] * lg2Rh);  // R^-delta
        const float T = A.T0[c] * Tn;                     // blackbody.py:16-30
        float Bv[NSPEC], E = 0.f, Qd = 0.f;
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) {
          const float2 bd = bb_lookup_d(tab_sm + s * nT, T, P.t_min, P.t_max, P.inv_dt, nT);
          Bv[s] = bd.x;
          E = fmaf(gup[s], bd.x, E);
          Qd = fmaf(gup[s], bd.y, Qd);
        }
        const float Xc0 = X0 - C.ox, Xc1 = X1 - C.oy, Xc2 = X2 - C.oz;
        const float Rc2 = fmaf(Xc0, Xc0, fmaf(Xc1, Xc1, Xc2 * Xc2));
        const float rcinv = rsqrt_ftz(Rc2);
        const float Rc = Rc2 * rcinv;
        const float Z = fmaf(Rl, un, on);
        float dth = 0.f;
        if (TYPE == ZL_FEATURE_RRM) dth = atan2_poly(fmaf(Rl, ruy, roy), fmaf(Rl, rux, rox));
        const RrmTerms t = rrm_terms<TYPE>(q, A.r2in[c], A.r2out[c], Rc2, Rc, rcinv, Z, dth);
        if (t.n == 0.f) continue;
        const float wn = wk * t.n;
        const float coef = wn * E;
        const float cG = coef * t.GR * rcinv, cZ = coef * t.GZ;
        S1 = fmaf(cG, Rl, S1);
        S2 += cG;
        S3 += cZ;
        S4 = fmaf(cZ, Rl, S4);
        if (TYPE == ZL_FEATURE_RRM) {
          const float rr = 1.f / (Xc0 * Xc0 + Xc1 * Xc1);
          fthx = fmaf(coef * t.dth, Xc1 * rr - eqx, fthx);
          fthy = fmaf(coef * t.dth, -Xc0 * rr - eqy, fthy);
        }
#pragma unroll
        for (int j = 0; j < NOWN; ++j) acc[5 + j] = fmaf(coef, t.d[j], acc[5 + j]);
        const float wq = wn * Qd;
        acc[ST0] = fmaf(wq, Tn, acc[ST0]);                  // dT/dT_0 = R^-delta
        acc[SDL] = fmaf(-wq * T, lg2Rh * kLn2, acc[SDL]);   // dT/d delta = -T ln R
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) acc[SCAL + s] = fmaf(wn * gup0[s], Bv[s], acc[SCAL + s]);
      }
      // geometry: d/dX_0 = -(sum coef g_R (X - X_0)/R) - n sum coef g_Z (+ the feature's
      // longitude terms); d/di, d/dOmega = sum coef g_Z (X - X_0) . dn (as the Kelsall adjoint)
      acc[0] = -fmaf(uxf, S1, dxc * S2) - C.nx * S3 + fthx;
      acc[1] = -fmaf(uyf, S1, dyc * S2) - C.ny * S3 + fthy;
      acc[2] = -fmaf(uzf, S1, dzc * S2) - C.nz * S3;
      const float ui = uxf * A.dni[c][0] + uyf * A.dni[c][1] + uzf * A.dni[c][2];
      const float di = dxc * A.dni[c][0] + dyc * A.dni[c][1] + dzc * A.dni[c][2];
      const float uO = uxf * A.dnO[c][0] + uyf * A.dnO[c][1];
      const float dO = dxc * A.dnO[c][0] + dyc * A.dnO[c][1];
      acc[3] = fmaf(ui, S4, di * S3);
      acc[4] = fmaf(uO, S4, dO * S3);
    }
    // tile reduction: a fixed shuffle tree per slot, then the warps in order
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kRrmSlots; ++j) {
      float v = acc[j];
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
      if (lane == 0) red_sm[warp][j] = v;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kRrmSlots; j += blockDim.x) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < kTile / 32; ++w) s += (double)red_sm[w][j];
      partials[tile * kRrmSlots + j] = s;
    }
    __syncthreads();
  }
}

// Map of the gradient vector onto the partial rows: entry j sums slot slot[j] of component
// comp[j] over the tiles, or (comp[j] < 0) slot[j] of every component in order (a calibration).
struct RrmMap {
  int32_t comp[160], slot[160];
};

__global__ void __launch_bounds__(256) rrm_reduce_kernel(const double* __restrict__ partials, int64_t n_tiles,
                                                         int n_comps, const __grid_constant__ RrmMap M,
                                                         double* __restrict__ out) {
  __shared__ double sm[256];
  const int j = blockIdx.x;
  const int c0 = M.comp[j] < 0 ? 0 : M.comp[j], c1 = M.comp[j] < 0 ? n_comps : M.comp[j] + 1;
  double total = 0.0;
  for (int c = c0; c < c1; ++c) {  // components in order, each a fixed-order sum over its tiles
    const double* rows = partials + (size_t)c * n_tiles * kRrmSlots;
    double s = 0.0;
    for (int64_t t = threadIdx.x; t < n_tiles; t += 256) s += rows[t * kRrmSlots + M.slot[j]];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w >= 1; w >>= 1) {
      if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
      __syncthreads();
    }
    total += sm[0];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = total;
}

template <int TYPE>
static void launch_rrm_type(const KParamsF32& P, const KGradRrm& A, int c, const double* u, int64_t n,
                            const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                            int64_t n_tiles, cudaStream_t st, int64_t grid) {
  switch (P.n_spec) {
    case 1: bwd_rrm_kernel<TYPE, 1><<<(unsigned)grid, kTile, 0, st>>>(P, A, c, u, n, obs, g_comps, g_total, partials, n_tiles); break;
    case 2: bwd_rrm_kernel<TYPE, 2><<<(unsigned)grid, kTile, 0, st>>>(P, A, c, u, n, obs, g_comps, g_total, partials, n_tiles); break;
    case 3: bwd_rrm_kernel<TYPE, 3><<<(unsigned)grid, kTile, 0, st>>>(P, A, c, u, n, obs, g_comps, g_total, partials, n_tiles); break;
    default: bwd_rrm_kernel<TYPE, 4><<<(unsigned)grid, kTile, 0, st>>>(P, A, c, u, n, obs, g_comps, g_total, partials, n_tiles); break;
  }
}

// Number of gradient entries of an RRM model: per component 5 + its own, then T_0 and delta of
// every component, then one calibration per spectral set.
int rrm_grad_count(const ZlModel& m) {
  int n = 0;
  for (int c = 0; c < m.n_comps; ++c) n += 5 + rrm_own(m.comp[c].type);
  return n + 2 * m.n_comps + m.n_spec;
}

// One launch per component into partials[c][tile][kRrmSlots], then the fixed-order reduction.
cudaError_t launch_bwd_rrm(const ZlModel& m, const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs,
                           const double* g_comps, const double* g_total, double* partials, int64_t n_tiles,
                           double* grad_out, cudaStream_t st, int bps, int num_sms) {
  KGradRrm A;
  memset(&A, 0, sizeof(A));
  const double deg = M_PI / 180.0;
  for (int c = 0; c < m.n_comps; ++c) {
    const ZlComponent& C = m.comp[c];
    A.dni[c][0] = (float)(C.sin_Omega * C.cos_i * deg);
    A.dni[c][1] = (float)(-C.cos_Omega * C.cos_i * deg);
    A.dni[c][2] = (float)(-C.sin_i * deg);
    A.dnO[c][0] = (float)(C.cos_Omega * C.sin_i * deg);
    A.dnO[c][1] = (float)(C.sin_Omega * C.sin_i * deg);
    A.T0[c] = (float)m.comp_T_0[c];
    A.neg_delta[c] = (float)(-m.comp_delta[c]);
    A.n_own[c] = rrm_own(C.type);
    A.r2in[c] = 0.f;
    A.r2out[c] = INFINITY;
    const double* p = C.p;
    switch (C.type) {
      case ZL_FAN:
        A.q[c][0] = (float)p[0], A.q[c][1] = (float)p[1], A.q[c][2] = (float)p[2], A.q[c][3] = (float)p[3];
        A.q[c][4] = (float)(1.0 / p[1]);
        A.r2out[c] = (float)(p[4] * p[4]);
        break;
      case ZL_COMET:
        A.q[c][0] = (float)p[0], A.q[c][1] = (float)p[1], A.q[c][2] = (float)p[2], A.q[c][3] = (float)p[3];
        A.q[c][4] = (float)(1.0 / p[1]);
        A.r2in[c] = (float)(p[4] * p[4]);
        A.r2out[c] = (float)(p[5] * p[5]);
        break;
      case ZL_NARROW_BAND:
        A.q[c][0] = (float)p[0], A.q[c][1] = (float)p[1], A.q[c][2] = (float)p[2], A.q[c][3] = (float)p[5];
        A.q[c][4] = (float)p[4];
        A.r2in[c] = (float)(p[3] * p[3]);
        A.r2out[c] = (float)(p[4] * p[4]);
        break;
      case ZL_BROAD_BAND:
        A.q[c][0] = (float)p[0], A.q[c][1] = (float)p[1], A.q[c][2] = (float)p[4], A.q[c][3] = (float)p[5];
        A.q[c][4] = (float)p[3];
        A.r2in[c] = (float)(p[2] * p[2]);
        A.r2out[c] = (float)(p[3] * p[3]);
        break;
      case ZL_INTERSTELLAR:
        A.q[c][0] = (float)p[0];
        break;
      case ZL_RING_RRM:
        A.q[c][0] = (float)C.n_0, A.q[c][1] = (float)p[0], A.q[c][2] = (float)p[1], A.q[c][3] = (float)p[2];
        A.q[c][4] = (float)p[3];
        break;
      case ZL_FEATURE_RRM:
        A.q[c][0] = (float)C.n_0, A.q[c][1] = (float)p[0], A.q[c][2] = (float)p[1], A.q[c][3] = (float)p[2];
        A.q[c][4] = (float)p[5], A.q[c][5] = (float)p[3], A.q[c][6] = (float)p[4];
        break;
    }
  }
  for (int s = 0; s < m.n_spec; ++s) A.cal[s] = (float)m.spec[s].calibration;

  int64_t grid = (int64_t)num_sms * bps;
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  for (int c = 0; c < m.n_comps; ++c) {
    double* part = partials + (size_t)c * n_tiles * kRrmSlots;
    switch (m.comp[c].type) {
      case ZL_FAN: launch_rrm_type<ZL_FAN>(P, A, c, u, n, obs, g_comps, g_total, part, n_tiles, st, grid); break;
      case ZL_COMET: launch_rrm_type<ZL_COMET>(P, A, c, u, n, obs, g_comps, g_total, part, n_tiles, st, grid); break;
      case ZL_NARROW_BAND:
        launch_rrm_type<ZL_NARROW_BAND>(P, A, c, u, n, obs, g_comps, g_total, part, n_tiles, st, grid);
        break;
      case ZL_BROAD_BAND:
        launch_rrm_type<ZL_BROAD_BAND>(P, A, c, u, n, obs, g_comps, g_total, part, n_tiles, st, grid);
        break;
      case ZL_INTERSTELLAR:
        launch_rrm_type<ZL_INTERSTELLAR>(P, A, c, u, n, obs, g_comps, g_total, part, n_tiles, st, grid);
        break;
      case ZL_RING_RRM:
        launch_rrm_type<ZL_RING_RRM>(P, A, c, u, n, obs, g_comps, g_total, part, n_tiles, st, grid);
        break;
      case ZL_FEATURE_RRM:
        launch_rrm_type<ZL_FEATURE_RRM>(P, A, c, u, n, obs, g_comps, g_total, part, n_tiles, st, grid);
        break;
      default: return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // gradient layout -> (component, slot)
  RrmMap M;
  int j = 0;
  for (int c = 0; c < m.n_comps; ++c)
    for (int s = 0; s < 5 + rrm_own(m.comp[c].type); ++s, ++j) M.comp[j] = c, M.slot[j] = s;
  for (int c = 0; c < m.n_comps; ++c, ++j) M.comp[j] = c, M.slot[j] = 5 + rrm_own(m.comp[c].type);      // T_0
  for (int c = 0; c < m.n_comps; ++c, ++j) M.comp[j] = c, M.slot[j] = 5 + rrm_own(m.comp[c].type) + 1;  // delta
  for (int s = 0; s < m.n_spec; ++s, ++j) M.comp[j] = -1, M.slot[j] = kRrmCal + s;                     // calibration
  rrm_reduce_kernel<<<j, 256, 0, st>>>(partials, n_tiles, m.n_comps, M, grad_out);
  return cudaGetLastError();
}

}  // namespace zl
