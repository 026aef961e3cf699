// Float32 forward pass: choice of the compiled kernel for a model (the kernel itself is in
// zl_fwd_f32.cuh; its instantiations are spread over one translation unit per layout so that
// they compile in parallel).
#include "zl_fwd_f32.cuh"

namespace zl {

// Compile-time flag set of a model for the layout kernels (see KFlags), or kFlagsRuntime when
// the model's pattern is not one the layouts are compiled for.
uint32_t f32_flags(const KParamsF32& P, int layout) {
  if (layout == 0) return kFlagsRuntime;
  uint32_t f = P.has_scat ? 2u : 0u;
  for (int c = 0; c < P.n_comps; ++c) {
    const KCompF32& K = P.comp[c];
    if (!K.zero_offset) f |= 1u << (8 + c);
    if (K.type == ZL_BAND) {
      if (K.c[5] != 0.f) f |= 1u << (16 + c);
      if (K.share_t4 >= 0) {
        if (K.share_t4 != 1) return kFlagsRuntime;  // the layouts' first band is component 1
        f |= 1u << (24 + c);
      }
    }
  }
  return f;
}

// layout: 1 = DIRBE-like, 2 = Planck-like, 0 = generic; plain_geometry selects the
// all-float32 variant of the DIRBE layout (kept for the precision/speed study).
cudaError_t launch_fwd_f32(const KParamsF32& P, int layout, bool plain_geometry, const double* u, int64_t n,
                           const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, int tpb, int bps,
                           int num_sms) {
  const uint32_t flags = f32_flags(P, layout);
  if (layout == 1) return launch_fwd_f32_dirbe(P, flags, plain_geometry, u, n, obs, oc, ot, st, tpb, bps, num_sms);
  if (layout == 2) return launch_fwd_f32_planck(P, flags, u, n, obs, oc, ot, st, tpb, bps, num_sms);
  return launch_fwd_f32_generic(P, u, n, obs, oc, ot, st, tpb, bps, num_sms);
}

}  // namespace zl
