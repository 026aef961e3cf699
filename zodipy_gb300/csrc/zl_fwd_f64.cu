// Plain float64 forward kernel: ZodiPy's line-of-sight integral evaluated in
// float64 throughout, one thread per pixel, every expression in the order the
// reference writes it.  It is the on-GPU oracle for the fast kernels and
// matches the reference's numpy result to ~1e-15 relative (transcendental
// functions differ from numpy's by a few ulp).
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

template <int NSPEC>
__global__ void __launch_bounds__(128) fwd_f64_kernel(const __grid_constant__ KParamsF64 P,
                                                      const double* __restrict__ u, int64_t n_pix,
                                                      const ObsArgs OA,
                                                      double* __restrict__ out_comps, double* __restrict__ out_total,
                                                      const Sched SC) {
  extern __shared__ double sm[];
  const int nT = P.m.n_temps;
  double* xp = sm;                  // [nT]
  double* fp = sm + nT;             // [NSPEC][nT]
  double* sl = sm + nT * (1 + NSPEC);  // [NSPEC][nT]
  for (int t = threadIdx.x; t < nT; t += blockDim.x) {
    xp[t] = P.m.temps[t];
#pragma unroll
    for (int s = 0; s < NSPEC; ++s) {
      fp[s * nT + t] = P.m.spec[s].bb[t];
      sl[s * nT + t] = P.slope[s][t];
    }
  }
  __syncthreads();
  const double x0 = P.m.temps[0];
  const double inv_dx = (double)(nT - 1) / (P.m.temps[nT - 1] - P.m.temps[0]);
  const int nc = P.m.n_comps;
  const int nr = P.m.n_ranges;

  ZL_SCHED_LOOP(kSchedAny, SC, n_pix, i) {
    const double ux = u[i], uy = u[n_pix + i], uz = u[2 * n_pix + i];
    const PixObs O = pixel_observer(OA, i, n_pix);
    const double ox = O.ox, oy = O.oy, oz = O.oz;
    const uint32_t outside = O.outside;

    // line_of_sight.py:70-85
    const double r_obs = sqrt(ox * ox + oy * oy + oz * oz);
    const double lon = atan2(uy, ux);
    const double lat = asin(uz);
    const double cos_lat = cos(lat);
    const double b = 2.0 * (ox * cos_lat * cos(lon) + oy * cos_lat * sin(lon));
    double start[ZL_MAX_RANGES], stop[ZL_MAX_RANGES];
#pragma unroll
    for (int r = 0; r < ZL_MAX_RANGES; ++r) {
      if (r < nr) {
        start[r] = (outside >> (2 * r)) & 1u ? kEps : sphere_distance(b, r_obs, P.m.cutoff[r][0]);
        stop[r] = (outside >> (2 * r + 1)) & 1u ? kEps : sphere_distance(b, r_obs, P.m.cutoff[r][1]);
      }
    }

    double acc[ZL_MAX_COMPS][NSPEC];
#pragma unroll
    for (int c = 0; c < ZL_MAX_COMPS; ++c)
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) acc[c][s] = 0.0;

    for (int k = 0; k < P.m.n_nodes; ++k) {
      const double xk = P.m.gl_x[k];
      const double wk = P.m.gl_w[k];
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
#pragma unroll
        for (int rr = 0; rr < ZL_MAX_RANGES; ++rr)
          if (rr == r) {
            st = start[rr];
            sp = stop[rr];
          }
        if (P.first_in_range[c]) {
          // brightness.py:27-33
          R_los = 0.5 * (sp - st) * xk + 0.5 * (sp + st);
          Xl0 = R_los * ux;
          Xl1 = R_los * uy;
          Xl2 = R_los * uz;
          X0 = Xl0 + ox;
          X1 = Xl1 + oy;
          X2 = Xl2 + oz;
          R = sqrt(X0 * X0 + X1 * X1 + X2 * X2);
          const double T = P.range_T0[r] * pow(R, -P.range_delta[r]);
#pragma unroll
          for (int s = 0; s < NSPEC; ++s) bb[s] = np_interp(T, xp, fp + s * nT, sl + s * nT, nT, x0, inv_dx);
          if (P.range_scat[r]) {  // scattering.py:26-31
            double ct = (Xl0 * X0 + Xl1 * X1 + Xl2 * X2) / (R_los * R);
            ct = ct < -1.0 ? -1.0 : (ct > 1.0 ? 1.0 : ct);
            theta = acos(-ct);
          }
          hs_len = sp - st;
        }
        const double dens = density_f64(C, X0, X1, X2, O.ex, O.ey);
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

    const int64_t col = out_col(SC, i);
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
  sched_finish<kSchedAny>(SC);
}

template <int NSPEC>
static cudaError_t launch_f64_t(const KParamsF64& P, const double* u, int64_t n, const ObsArgs& obs,
                                double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  const size_t smem = sizeof(double) * P.m.n_temps * (1 + 2 * NSPEC);
  fwd_f64_kernel<NSPEC><<<(unsigned)fwd_grid(L, n), L.tpb, smem, st>>>(P, u, n, obs, oc, ot, L.sched);
  return cudaGetLastError();
}

// Densities on a Cartesian mesh (zodipy/number_density.py:482-536): point (iy, ix, iz) of
// numpy.meshgrid(x, y, z) (default 'xy' indexing) is (x[ix], y[iy], z[iz]); out is
// [n_comps][ny][nx][nz].
__global__ void __launch_bounds__(256) density_grid_kernel(const __grid_constant__ ZlModel M,
                                                           const double* __restrict__ x, int nx,
                                                           const double* __restrict__ y, int ny,
                                                           const double* __restrict__ z, int nz, double ex, double ey,
                                                           double* __restrict__ out) {
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int iz = (int)(t % nz);
    const int ix = (int)((t / nz) % nx);
    const int iy = (int)(t / ((int64_t)nz * nx));
    const double X0 = x[ix], X1 = y[iy], X2 = z[iz];
    for (int c = 0; c < M.n_comps; ++c) out[(int64_t)c * n + t] = density_f64(M.comp[c], X0, X1, X2, ex, ey);
  }
}

cudaError_t launch_density_grid(const ZlModel& M, const double* x, int nx, const double* y, int ny, const double* z,
                                int nz, double ex, double ey, double* out, cudaStream_t st, int num_sms) {
  const int64_t n = (int64_t)nx * ny * nz;
  int64_t grid = (n + 255) / 256;
  if (grid > (int64_t)num_sms * 16) grid = (int64_t)num_sms * 16;
  if (grid < 1) grid = 1;
  density_grid_kernel<<<(unsigned)grid, 256, 0, st>>>(M, x, nx, y, ny, z, nz, ex, ey, out);
  return cudaGetLastError();
}

cudaError_t launch_fwd_f64(const KParamsF64& P, const double* u, int64_t n, const ObsArgs& obs,
                           double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  switch (P.m.n_spec) {
    case 1: return launch_f64_t<1>(P, u, n, obs, oc, ot, st, L);
    case 2: return launch_f64_t<2>(P, u, n, obs, oc, ot, st, L);
    case 3: return launch_f64_t<3>(P, u, n, obs, oc, ot, st, L);
    default: return launch_f64_t<4>(P, u, n, obs, oc, ot, st, L);
  }
}

}  // namespace zl
