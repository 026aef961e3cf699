// Two-pixel float32 forward kernels of the DIRBE component layout with scattering (its own
// translation unit so that the two flag sets compile in parallel).
#include "zl_fwd_f32x2.cuh"

namespace zl {

cudaError_t launch_fwd_f32x2_dirbe_scat(const KParamsF32& P, bool tails, const double* u, int64_t n,
                                        const ObsArgs& obs, double* oc, double* ot, cudaStream_t st,
                                        const LaunchArgs& L) {
  return tails ? launch_f32x2_flags<kLayoutDirbe, kFlagsKelsall | 2u, true>(P, u, n, obs, oc, ot, st, L)
               : launch_f32x2_flags<kLayoutDirbe, kFlagsKelsall | 2u, false>(P, u, n, obs, oc, ot, st, L);
}

}  // namespace zl
