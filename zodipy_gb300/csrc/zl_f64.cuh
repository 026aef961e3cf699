// Plain float64 line-of-sight arithmetic: ZodiPy's integral evaluated in float64
// throughout, every expression in the order the reference writes it.  The device
// functions here serve the float64 forward kernels (one thread per pixel,
// zl_fwd_f64.cu; one warp per pixel, zl_fwd_f64_warp.cu) and the density grid.
//
// Reference mapping:
//   sphere intersection .......... zodipy/line_of_sight.py:64-85
//   LOS range per component ...... zodipy/line_of_sight.py:88-105
//   quadrature (sequential sum) .. zodipy/line_of_sight.py:55-61
//   integrand .................... zodipy/brightness.py:21-56
//   T(R), blackbody lookup ....... zodipy/blackbody.py:16-30, numpy.interp
//   densities .................... zodipy/number_density.py:47-181 (Kelsall), :184-404 (RRM)
//   RRM integrand ................ zodipy/brightness.py:59-83
//   scattering ................... zodipy/scattering.py:11-59
//   total = sum over components .. zodipy/model.py:203
#pragma once

#include "zl_common.cuh"

namespace zl {

// numpy.interp(x, xp, fp) with default left/right (clamp), uniform xp.
__device__ __forceinline__ double np_interp(double x, const double* xp, const double* fp, const double* slope,
                                            int n, double x0, double inv_dx) {
  if (isnan(x)) return x;
  if (x < xp[0]) return fp[0];
  if (x > xp[n - 1]) return fp[n - 1];
  if (x == xp[n - 1]) return fp[n - 1];
  int j = (int)((x - x0) * inv_dx);
  j = j < 0 ? 0 : (j > n - 2 ? n - 2 : j);
  while (j > 0 && x < xp[j]) --j;  // xp is uniform: at most one step each way
  while (j < n - 2 && x >= xp[j + 1]) ++j;
  if (x == xp[j]) return fp[j];
  double r = slope[j] * (x - xp[j]) + fp[j];
  if (isnan(r)) {
    r = slope[j] * (x - xp[j + 1]) + fp[j + 1];
    if (isnan(r) && fp[j] == fp[j + 1]) r = fp[j];
  }
  return r;
}

// numpy.maximum: nan-propagating.
__device__ __forceinline__ double np_maximum(double a, double b) {
  if (isnan(a) || isnan(b)) return a + b;
  return a > b ? a : b;
}

// Python float % (numpy.remainder): result takes the sign of the divisor.
__device__ __forceinline__ double np_remainder(double a, double b) {
  double m = fmod(a, b);
  if (m != 0.0) {
    if ((b < 0.0) != (m < 0.0)) m += b;
  } else {
    m = copysign(0.0, b);
  }
  return m;
}

// Distance along the ray to the sphere |X| = cutoff (line_of_sight.py:74-85),
// given b (which, like the reference, omits z_obs * u_z) and r_obs.
// Where b == 0 the reference's expression is 0 * inf = nan; the same root is
// then taken as -0.5 (b + copysign(sqrt(D), b)), which is finite.
__device__ __forceinline__ double sphere_distance(double b, double r_obs, double cutoff) {
  double c = r_obs * r_obs - cutoff * cutoff;
  double sq = sqrt(b * b - 4.0 * c);
  double q = (b == 0.0) ? -0.5 * copysign(sq, b) : -0.5 * b * (1.0 + sq / fabs(b));
  return np_maximum(q, c / q);
}

// Number density of one component at heliocentric X (zodipy/number_density.py:47-404), every
// expression in the reference's order; (ex, ey) is Earth's heliocentric x, y (features only).
// The RRM densities are zero outside their radial mask, as the reference's filtered assignment
// leaves them (a nan distance fails the mask too).
__device__ __forceinline__ double density_f64(const ZlComponent& C, double X0, double X1, double X2, double ex,
                                              double ey) {
  // number_density.py: X - X_0, its norm, and the height above the symmetry plane
  const double Xc0 = X0 - C.offset[0], Xc1 = X1 - C.offset[1], Xc2 = X2 - C.offset[2];
  const double Rc = sqrt(Xc0 * Xc0 + Xc1 * Xc1 + Xc2 * Xc2);
  const double Zc = Xc0 * C.sin_Omega * C.sin_i - Xc1 * C.cos_Omega * C.sin_i + Xc2 * C.cos_i;
  if (C.type == ZL_CLOUD) {  // number_density.py:60-73
    const double zeta = fabs(Zc / Rc);
    const double mu = C.p[3];
    const double g = zeta < mu ? zeta * zeta / (2.0 * mu) : zeta - (mu / 2.0);
    return C.n_0 * pow(Rc, -C.p[0]) * exp(-C.p[1] * pow(g, C.p[2]));
  }
  if (C.type == ZL_BAND) {  // number_density.py:99-110
    const double zeta = fabs(Zc / Rc);
    const double zz = zeta / C.p[0];
    const double t1 = 3.0 * C.n_0 / Rc;
    const double t2 = exp(-pow(zz, 6.0));
    const double t3 = 1.0 + pow(zz, C.p[2]) / C.p[1];
    const double t4 = 1.0 - exp(-pow(Rc / C.p[3], 20.0));
    return t1 * t2 * t3 * t4;
  }
  if (C.type == ZL_RING || C.type == ZL_RING_RRM) {  // number_density.py:136-139; RRM :345-370
    const double d = Rc - C.p[0];
    const double t1 = -(d * d) / (C.p[1] * C.p[1]);
    const double t2 = fabs(Zc) / C.p[2];
    const double n = C.n_0 * exp(t1 - t2);
    return C.type == ZL_RING ? n : C.p[3] * n;
  }
  if (C.type == ZL_FEATURE || C.type == ZL_FEATURE_RRM) {  // number_density.py:167-181; RRM :373-403
    const double te = atan2(ey - C.offset[1], ex - C.offset[0]);
    double dth = (atan2(Xc1, Xc0) - te) - C.p[3];
    dth = np_remainder(dth + kPi, 2.0 * kPi) - kPi;
    const double d = Rc - C.p[0];
    double e = d * d / (C.p[1] * C.p[1]);
    e += fabs(Zc) / C.p[2];
    e += dth * dth / (C.p[4] * C.p[4]);
    const double n = C.n_0 * exp(-e);
    return C.type == ZL_FEATURE ? n : C.p[5] * n;
  }
  if (C.type == ZL_INTERSTELLAR) return C.p[0];  // number_density.py:259-264
  if (C.type == ZL_FAN) {  // number_density.py:184-218; p = gamma, Z_0, Q, P, R_outer
    if (!(Rc <= C.p[4])) return 0.0;
    const double beta = asin(Zc / Rc);
    const double Zabs = fabs(Zc);
    const double eps = Zabs < C.p[1] ? 2.0 - (Zabs / C.p[1]) : 1.0;
    const double f = pow(cos(beta), C.p[2]) * exp(-C.p[3] * sin(pow(fabs(beta), eps)));
    return pow(Rc, -C.p[0]) * f;
  }
  if (C.type == ZL_COMET) {  // number_density.py:221-256; p = gamma, Z_0, P, amp, R_inner, R_outer
    if (!(Rc >= C.p[4] && Rc <= C.p[5])) return 0.0;
    const double beta = asin(Zc / Rc);
    const double Zabs = fabs(Zc);
    const double eps = Zabs < C.p[1] ? 2.0 - (Zabs / C.p[1]) : 1.0;
    const double f = exp(-C.p[2] * sin(pow(fabs(beta), eps)));
    return C.p[3] * pow(Rc, -C.p[0]) * f;
  }
  if (C.type == ZL_NARROW_BAND) {  // number_density.py:267-304; p = gamma, A, G, R_inner, R_outer, beta_nb
    if (!(Rc >= C.p[3] && Rc <= C.p[4])) return 0.0;
    const double beta_abs = fabs(asin(Zc / Rc) * (180.0 / kPi));  // numpy.rad2deg
    const double f = beta_abs < C.p[5] ? exp(C.p[2] * (beta_abs - C.p[5])) : 0.0;
    return C.p[1] * pow(Rc / C.p[4], -C.p[0]) * f;
  }
  // broad band, number_density.py:307-342; p = gamma, A, R_inner, R_outer, beta_bb, sigma_bb
  if (!(Rc >= C.p[2] && Rc <= C.p[3])) return 0.0;
  const double beta = asin(Zc / Rc) * (180.0 / kPi);
  const double a = (beta - C.p[4]) / C.p[5], b = (beta + C.p[4]) / C.p[5];
  const double f = exp(-0.5 * (a * a)) + exp(-0.5 * (b * b));
  return C.p[1] * pow(Rc / C.p[3], -C.p[0]) * f;
}

// The blackbody table in shared memory as numpy.interp reads it: abscissae, values, slopes.
struct F64Table {
  const double* xp;  // [nT]
  const double* fp;  // [NSPEC][nT]
  const double* sl;  // [NSPEC][nT]
  int nT;
  double x0, inv_dx;
};

template <int NSPEC>
__device__ __forceinline__ F64Table stage_table_f64(const KParamsF64& P, double* sm) {
  const int nT = P.m.n_temps;
  double* xp = sm;
  double* fp = sm + nT;
  double* sl = sm + nT * (1 + NSPEC);
  for (int t = threadIdx.x; t < nT; t += blockDim.x) {
    xp[t] = P.m.temps[t];
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      fp[s * nT + t] = P.m.spec[s].bb[t];
      sl[s * nT + t] = P.slope[s][t];
    }
  }
  __syncthreads();
  return F64Table{xp, fp, sl, nT, P.m.temps[0], (double)(nT - 1) / (P.m.temps[nT - 1] - P.m.temps[0])};
}

// A pixel's line of sight: direction, observer, and the [start, stop] of every range
// (line_of_sight.py:70-105).
struct PixF64 {
  double ux, uy, uz;
  PixObs O;
  double start[ZL_MAX_RANGES], stop[ZL_MAX_RANGES];
};

__device__ __forceinline__ void pixel_setup_f64(const KParamsF64& P, const double* __restrict__ u, int64_t n_pix,
                                                const ObsArgs& OA, int64_t i, PixF64& X) {
  X.ux = u[i];
  X.uy = u[n_pix + i];
  X.uz = u[2 * n_pix + i];
  X.O = pixel_observer(OA, i, n_pix);
  const double ox = X.O.ox, oy = X.O.oy, oz = X.O.oz;
  const uint32_t outside = X.O.outside;
  // line_of_sight.py:70-85
  const double r_obs = sqrt(ox * ox + oy * oy + oz * oz);
  const double lon = atan2(X.uy, X.ux);
  const double lat = asin(X.uz);
  const double cos_lat = cos(lat);
  const double b = 2.0 * (ox * cos_lat * cos(lon) + oy * cos_lat * sin(lon));
#pragma unroll
  for (int r = 0; r < ZL_MAX_RANGES; ++r) {
    X.start[r] = X.stop[r] = 0.0;
    if (r < P.m.n_ranges) {
      X.start[r] = (outside >> (2 * r)) & 1u ? kEps : sphere_distance(b, r_obs, P.m.cutoff[r][0]);
      X.stop[r] = (outside >> (2 * r + 1)) & 1u ? kEps : sphere_distance(b, r_obs, P.m.cutoff[r][1]);
    }
  }
}

// Quadrature node (xk, wk) of every component of one line of sight, added to acc[c][s]
// (brightness.py:21-83, every expression in the reference's order).
// SMEM: X lives in shared memory (read the component's range by index) rather than in
// registers (select it with compile-time indices).
template <int NSPEC, bool SMEM>
__device__ __forceinline__ void node_f64(const KParamsF64& P, const F64Table& T, const PixF64& X, double xk, double wk,
                                         double (&acc)[ZL_MAX_COMPS][NSPEC]) {
  const int nc = P.m.n_comps;
  double R_los = 0.0, Xl0 = 0.0, Xl1 = 0.0, Xl2 = 0.0, X0 = 0.0, X1 = 0.0, X2 = 0.0, R = 0.0, theta = 0.0;
  double hs_len = 0.0;
  double bb[NSPEC];
#pragma unroll
  for (int s = 0; s < NSPEC; ++s) bb[s] = 0.0;
#pragma unroll
  for (int c = 0; c < ZL_MAX_COMPS; ++c) {
    if (c >= nc) break;
    const ZlComponent& C = P.m.comp[c];
    const int r = C.range;
    double st = 0.0, sp = 0.0;
    if (SMEM) {
      st = X.start[r];
      sp = X.stop[r];
    } else {
#pragma unroll
      for (int rr = 0; rr < ZL_MAX_RANGES; ++rr)
        if (rr == r) {
          st = X.start[rr];
          sp = X.stop[rr];
        }
    }
    if (P.first_in_range[c]) {
      // brightness.py:27-33
      R_los = 0.5 * (sp - st) * xk + 0.5 * (sp + st);
      Xl0 = R_los * X.ux;
      Xl1 = R_los * X.uy;
      Xl2 = R_los * X.uz;
      X0 = Xl0 + X.O.ox;
      X1 = Xl1 + X.O.oy;
      X2 = Xl2 + X.O.oz;
      R = sqrt(X0 * X0 + X1 * X1 + X2 * X2);
      const double Tk = P.range_T0[r] * pow(R, -P.range_delta[r]);
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) bb[s] = np_interp(Tk, T.xp, T.fp + s * T.nT, T.sl + s * T.nT, T.nT, T.x0, T.inv_dx);
      if (P.range_scat[r]) {  // scattering.py:26-31
        double ct = (Xl0 * X0 + Xl1 * X1 + Xl2 * X2) / (R_los * R);
        ct = ct < -1.0 ? -1.0 : (ct > 1.0 ? 1.0 : ct);
        theta = acos(-ct);
      }
      hs_len = sp - st;
    }
    const double dens = density_f64(C, X0, X1, X2, X.O.ex, X.O.ey);
    if (P.m.family == ZL_RRM) {  // brightness.py:80-83
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) acc[c][s] += bb[s] * dens * P.m.spec[s].calibration * 0.5 * hs_len * wk;
      continue;
    }
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      const double A = P.m.spec[s].albedo[c];
      double em = (1.0 - A) * (P.m.spec[s].emissivity[c] * bb[s]);
      if (A != 0.0) {
        const double flux = P.m.spec[s].solar_irradiance / (R * R);
        const ZlSpectrum& S = P.m.spec[s];
        const double phase = P.phase_norm[s] * (S.C1 + S.C2 * theta + exp(S.C3 * theta));
        em += A * flux * phase;
      }
      acc[c][s] += em * dens * 0.5 * hs_len * wk;
    }
  }
}

template <int NSPEC>
__device__ __forceinline__ void store_f64(const KParamsF64& P, int64_t n_pix, int64_t col,
                                          const double (&acc)[ZL_MAX_COMPS][NSPEC], double* __restrict__ out_comps,
                                          double* __restrict__ out_total) {
  const int nc = P.m.n_comps;
#pragma unroll
  for (int s = 0; s < NSPEC; ++s) {
    double tot = 0.0;
#pragma unroll
    for (int c = 0; c < ZL_MAX_COMPS; ++c) {
      if (c >= nc) break;
      if (out_comps) out_comps[((int64_t)s * nc + c) * n_pix + col] = acc[c][s];
      tot = (c == 0) ? acc[c][s] : tot + acc[c][s];
    }
    if (out_total) out_total[(int64_t)s * n_pix + col] = tot;
  }
}

}  // namespace zl
