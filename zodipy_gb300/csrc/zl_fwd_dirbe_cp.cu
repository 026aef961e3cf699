// Component-paired float32 forward kernels of the DIRBE layout (zl_fwd_dirbe.cuh).
#include "zl_fwd_dirbe.cuh"

namespace zl {

template <uint32_t FLAGS>
static cudaError_t launch_cp_flags(const KParamsF32& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                   double* ot, cudaStream_t st, const LaunchArgs& L) {
  switch (P.n_spec) {
    case 1: return launch_dirbe_cp_t<1, FLAGS>(P, u, n, obs, oc, ot, st, L);
    case 2: return launch_dirbe_cp_t<2, FLAGS>(P, u, n, obs, oc, ot, st, L);
    case 3: return launch_dirbe_cp_t<3, FLAGS>(P, u, n, obs, oc, ot, st, L);
    default: return launch_dirbe_cp_t<4, FLAGS>(P, u, n, obs, oc, ot, st, L);
  }
}

cudaError_t launch_fwd_dirbe_cp(const KParamsF32& P, uint32_t flags, const double* u, int64_t n, const ObsArgs& obs,
                                double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  if (flags == kFlagsKelsall) return launch_cp_flags<kFlagsKelsall>(P, u, n, obs, oc, ot, st, L);
  if (flags == (kFlagsKelsall | 2u))
    return launch_cp_flags<kFlagsKelsall | 2u>(P, u, n, obs, oc, ot, st, L);
  return cudaErrorNotSupported;
}

}  // namespace zl
