// Two-pixel float32 forward kernels of the Planck component layout (cloud | 3 bands).
#include "zl_fwd_f32x2.cuh"

namespace zl {

cudaError_t launch_fwd_f32x2_planck(const KParamsF32& P, uint32_t flags, bool tails, const double* u, int64_t n,
                                    const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  if (flags == kFlagsKelsall)
    return tails ? launch_f32x2_flags<kLayoutPlanck, kFlagsKelsall, true>(P, u, n, obs, oc, ot, st, L)
                 : launch_f32x2_flags<kLayoutPlanck, kFlagsKelsall, false>(P, u, n, obs, oc, ot, st, L);
  return cudaErrorNotSupported;
}

}  // namespace zl
