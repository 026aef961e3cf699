// Adjoint kernels of the DIRBE component layout (cloud | 3 bands | ring | feature).
// Models with the built-in flags take the component-paired kernels
// (zl_bwd_dirbe_cp.cu); the scalar kernel reads the flags at run time and serves
// every other DIRBE-layout model, and any model when the caller asks for the
// one-pixel kernels (ZL_KERNEL_ONE_PIXEL, for comparing the two).
#include "zl_bwd_f32.cuh"

namespace zl {

cudaError_t launch_bwd_dirbe_cp(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                int64_t n_tiles, cudaStream_t st, int64_t grid);

// three or four spectral sets: zl_bwd_f32_dirbe34.cu (compiled in parallel with this file)
cudaError_t launch_bwd_f32_dirbe34(const KParamsF32& P, const KGradAux& A, const double* u, int64_t n,
                                   const ObsArgs& obs, const double* g_comps, const double* g_total, double* partials,
                                   int64_t n_tiles, cudaStream_t st, int64_t grid);

cudaError_t launch_bwd_f32_dirbe(const KParamsF32& P, const KGradAux& A, uint32_t flags, bool unpaired, const double* u,
                                 int64_t n, const ObsArgs& obs, const double* g_comps, const double* g_total,
                                 double* partials, int64_t n_tiles, cudaStream_t st, int64_t grid) {
  if (!unpaired && (flags & kBwdFlagsMask) == (kFlagsKelsall & kBwdFlagsMask))
    return launch_bwd_dirbe_cp(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  switch (P.n_spec) {
    case 1: return launch_groups<kLayoutDirbe, 1, kFlagsRuntime>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
    case 2: return launch_groups<kLayoutDirbe, 2, kFlagsRuntime>(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
    default: return launch_bwd_f32_dirbe34(P, A, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  }
}

}  // namespace zl
