// Float32 forward kernels of the DIRBE component layout (cloud | 3 bands | ring | feature).
#include "zl_fwd_f32.cuh"

namespace zl {

cudaError_t launch_fwd_f32_dirbe(const KParamsF32& P, uint32_t flags, bool plain_geometry, const double* u, int64_t n,
                                 const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  if (plain_geometry && P.n_spec == 1)
    return launch_f32_t<1, kLayoutDirbe, false, kFlagsRuntime>(P, u, n, obs, oc, ot, st, L);
  if (flags == kFlagsKelsall)
    return launch_f32_flags<kLayoutDirbe, kFlagsKelsall>(P, u, n, obs, oc, ot, st, L);
  if (flags == (kFlagsKelsall | 2u))
    return launch_f32_flags<kLayoutDirbe, kFlagsKelsall | 2u>(P, u, n, obs, oc, ot, st, L);
  return launch_f32_flags<kLayoutDirbe, kFlagsRuntime>(P, u, n, obs, oc, ot, st, L);
}

}  // namespace zl
