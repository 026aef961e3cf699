// Adjoint kernels of the Planck component layout (cloud | 3 bands).
#include "zl_bwd_f32.cuh"

namespace zl {

cudaError_t launch_bwd_f32_planck(const KParamsF32& P, const KGradAux& A, uint32_t flags, const double* u, int64_t n,
                                 const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                 int64_t n_tiles, cudaStream_t st, int64_t grid) {
  if ((flags & kBwdFlagsMask) == (kFlagsKelsall & kBwdFlagsMask))
    return launch_bwd_nspec<kLayoutPlanck, kFlagsKelsall & kBwdFlagsMask>(P, A, u, n, obs, g_comps, g_total, partials,
                                                                 n_tiles, st, grid);
  return launch_bwd_nspec<kLayoutPlanck, kFlagsRuntime>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
}

}  // namespace zl
