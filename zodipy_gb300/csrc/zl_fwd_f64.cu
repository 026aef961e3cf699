// float64 forward kernel, one thread per pixel: nodes in the reference's order (a
// sequential sum, line_of_sight.py:55-61), the on-GPU oracle for the fast kernels; it
// matches the reference's numpy result to ~1e-15 relative (transcendental functions
// differ from numpy's by a few ulp).  Also the densities on a mesh (grid_number_density).
#include "zl_f64.cuh"

namespace zl {

// One thread per pixel, nodes in order (the reference's summation order).
template <int NSPEC>
__global__ void __launch_bounds__(128) fwd_f64_kernel(const __grid_constant__ KParamsF64 P,
                                                      const double* __restrict__ u, int64_t n_pix,
                                                      const ObsArgs OA,
                                                      double* __restrict__ out_comps, double* __restrict__ out_total,
                                                      const Sched SC) {
  extern __shared__ double sm[];
  const F64Table T = stage_table_f64<NSPEC>(P, sm);
  ZL_SCHED_LOOP(kSchedAny, SC, n_pix, i) {
    PixF64 X;
    pixel_setup_f64(P, u, n_pix, OA, i, X);
    double acc[ZL_MAX_COMPS][NSPEC];
#pragma unroll
    for (int c = 0; c < ZL_MAX_COMPS; ++c)
#pragma unroll
      for (int s = 0; s < NSPEC; ++s) acc[c][s] = 0.0;
    for (int k = 0; k < P.m.n_nodes; ++k) node_f64<NSPEC, false>(P, T, X, P.m.gl_x[k], P.m.gl_w[k], acc);
    store_f64<NSPEC>(P, n_pix, out_col(SC, i), acc, out_comps, out_total);
  }
  sched_finish<kSchedAny>(SC);
}

template <int NSPEC>
static cudaError_t launch_f64_t(const KParamsF64& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                double* ot, cudaStream_t st, const LaunchArgs& L) {
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

cudaError_t launch_fwd_f64_warp(const KParamsF64& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                double* ot, cudaStream_t st, const LaunchArgs& L);

cudaError_t launch_fwd_f64(const KParamsF64& P, bool warp, const double* u, int64_t n, const ObsArgs& obs,
                           double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  if (warp) return launch_fwd_f64_warp(P, u, n, obs, oc, ot, st, L);
  switch (P.m.n_spec) {
    case 1: return launch_f64_t<1>(P, u, n, obs, oc, ot, st, L);
    case 2: return launch_f64_t<2>(P, u, n, obs, oc, ot, st, L);
    case 3: return launch_f64_t<3>(P, u, n, obs, oc, ot, st, L);
    default: return launch_f64_t<4>(P, u, n, obs, oc, ot, st, L);
  }
}

}  // namespace zl
