// Float32 forward kernels of the generic component layout (any Kelsall or RRM model).
#include "zl_fwd_f32.cuh"

namespace zl {

cudaError_t launch_fwd_f32_generic(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                   double* ot, cudaStream_t st, const LaunchArgs& L) {
  return launch_f32_flags<kLayoutGeneric, kFlagsRuntime>(P, u, n, obs, oc, ot, st, L);
}

}  // namespace zl
