// Two-pixel float32 forward kernels of the DIRBE component layout (cloud | 3 bands | ring | feature),
// without scattering; the scattering flag set is compiled in zl_fwd_f32x2_dirbe_scat.cu.
#include "zl_fwd_f32x2.cuh"

namespace zl {

cudaError_t launch_fwd_f32x2_dirbe_scat(const KParamsF32& P, bool tails, const double* u, int64_t n,
                                        const ObsArgs& obs, double* oc, double* ot, cudaStream_t st,
                                        const LaunchArgs& L);

cudaError_t launch_fwd_f32x2_dirbe(const KParamsF32& P, uint32_t flags, bool tails, const double* u, int64_t n,
                                   const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  if (flags == kFlagsKelsall)
    return tails ? launch_f32x2_flags<kLayoutDirbe, kFlagsKelsall, true>(P, u, n, obs, oc, ot, st, L)
                 : launch_f32x2_flags<kLayoutDirbe, kFlagsKelsall, false>(P, u, n, obs, oc, ot, st, L);
  if (flags == (kFlagsKelsall | 2u)) return launch_fwd_f32x2_dirbe_scat(P, tails, u, n, obs, oc, ot, st, L);
  return cudaErrorNotSupported;
}

}  // namespace zl
