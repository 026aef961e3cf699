// One-pixel float32 forward kernels of the registry's RRM arrangement (Lay<kLayoutRRM>): the
// component types and LOS ranges compiled in, the parameters read at run time.
#include "zl_fwd_f32.cuh"

namespace zl {

cudaError_t launch_fwd_f32_rrm(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                               double* ot, cudaStream_t st, const LaunchArgs& L) {
  return launch_f32_flags<kLayoutRRM, kFlagsRuntime>(P, u, n, obs, oc, ot, st, L);
}

}  // namespace zl
