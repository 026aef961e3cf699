// Scalar DIRBE-layout adjoint kernels (run-time flags) for three or four spectral sets; one
// and two are in zl_bwd_f32_dirbe.cu.
#include "zl_bwd_f32.cuh"

namespace zl {

cudaError_t launch_bwd_f32_dirbe34(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                   const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                   int64_t n_tiles, cudaStream_t st, int64_t grid) {
  if (P.n_spec == 3)
    return launch_groups<kLayoutDirbe, 3, kFlagsRuntime>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  return launch_groups<kLayoutDirbe, 4, kFlagsRuntime>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
}

}  // namespace zl
