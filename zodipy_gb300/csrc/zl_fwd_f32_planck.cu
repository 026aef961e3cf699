// Float32 forward kernels of the Planck component layout (cloud | 3 bands).
#include "zl_fwd_f32.cuh"

namespace zl {

cudaError_t launch_fwd_f32_planck(const KParamsF32& P, uint32_t flags, const double* u, int64_t n, const ObsArgs& obs,
                                  double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  if (flags == kFlagsKelsall)
    return launch_f32_flags<kLayoutPlanck, kFlagsKelsall>(P, u, n, obs, oc, ot, st, L);
  return launch_f32_flags<kLayoutPlanck, kFlagsRuntime>(P, u, n, obs, oc, ot, st, L);
}

}  // namespace zl
