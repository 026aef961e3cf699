// Launches of the component-paired DIRBE adjoint kernels (zl_bwd_dirbe.cuh).
#include "zl_bwd_dirbe.cuh"

namespace zl {

template <int NSPEC, bool SCAT>
static cudaError_t launch_cp_groups(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                    const ObsArgs& obs, const double* g_comps, const double* g_total,
                                    double* partials, int64_t n_tiles, cudaStream_t st, int64_t grid) {
  constexpr int NG = GradLay<kLayoutDirbe, NSPEC>::NG;
  bwd_dirbe_cb_kernel<NSPEC, SCAT>
      <<<(unsigned)grid, kTile, 0, st>>>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  bwd_dirbe_rf_kernel<NSPEC, SCAT><<<(unsigned)grid, kTile, 0, st>>>(P, A, u, n, obs, g_comps, g_total,
                                                                     partials + (size_t)n_tiles * NG, n_tiles);
  return cudaGetLastError();
}

template <int NSPEC>
static cudaError_t launch_cp_nspec(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                   const ObsArgs& obs, const double* g_comps, const double* g_total,
                                   double* partials, int64_t n_tiles, cudaStream_t st, int64_t grid) {
  if (P.has_scat) return launch_cp_groups<NSPEC, true>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  return launch_cp_groups<NSPEC, false>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
}

// The DIRBE layout's two component groups ({cloud, bands}, {ring, feature}) for a
// model with the built-in flags; partials as launch_bwd_f32.
#ifdef ZL_CP_NSPEC34
// three or four spectral sets (this file compiled a second time, in parallel)
cudaError_t launch_bwd_dirbe_cp34(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                  const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                  int64_t n_tiles, cudaStream_t st, int64_t grid) {
  if (P.n_spec == 3) return launch_cp_nspec<3>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  return launch_cp_nspec<4>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
}
#else
cudaError_t launch_bwd_dirbe_cp34(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                  const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                  int64_t n_tiles, cudaStream_t st, int64_t grid);

cudaError_t launch_bwd_dirbe_cp(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                int64_t n_tiles, cudaStream_t st, int64_t grid) {
  switch (P.n_spec) {
    case 1: return launch_cp_nspec<1>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
    case 2: return launch_cp_nspec<2>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
    default: return launch_bwd_dirbe_cp34(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  }
}
#endif

}  // namespace zl
