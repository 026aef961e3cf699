// Two-pixel float32 forward kernels of the Planck component layout (cloud | 3 bands).
#include "zl_fwd_f32x2.cuh"

namespace zl {

cudaError_t launch_fwd_f32x2_planck(const KParamsF32& P, uint32_t flags, const double* u, int64_t n,
                                    const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, int tpb, int bps,
                                    int num_sms) {
  if (flags == kFlagsKelsall)
    return launch_f32x2_flags<kLayoutPlanck, kFlagsKelsall>(P, u, n, obs, oc, ot, st, tpb, bps, num_sms);
  return cudaErrorNotSupported;
}

}  // namespace zl
