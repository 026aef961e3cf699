// Float32 forward pass: choice of the compiled kernel for a model (the kernel itself is in
// zl_fwd_f32.cuh; its instantiations are spread over one translation unit per layout so that
// they compile in parallel).
#include "zl_fwd_dirbe.cuh"

namespace zl {

// Compile-time flag set of a model for the layout kernels (see KFlags), or kFlagsRuntime when
// the model's pattern is not one the layouts are compiled for.
uint32_t f32_flags(const KParamsF32& P, int layout) {
  if (layout == 0 || layout == 3) return kFlagsRuntime;
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

// kernel (ZL_KERNEL_* of the C ABI): AUTO takes the fastest measured kernel of the layout --
// the component-paired kernel for the DIRBE layout, the two-pixel kernel for the Planck layout
// (measured on GB300 at nside 512: Planck layout 0.79 ms two-pixel vs 0.91 ms one-pixel; the
// two-pixel DIRBE kernel needs 168 registers and loses, 2.01 vs 1.88 ms); ONE_PIXEL the
// one-pixel kernel with components in order; TWO_PIXEL the two-pixel kernel for either
// built-in layout; PLAIN_GEOMETRY the all-float32-geometry variant of the DIRBE layout (kept
// for the precision study).  tails: band tails in the two-pixel kernel (coherent inputs).
// Models outside the compiled flag sets run the one-pixel kernel with run-time flags.
cudaError_t launch_fwd_f32(const KParamsF32& P, int layout, int kernel, bool tails, const double* u, int64_t n,
                           const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, const LaunchArgs& L) {
  const uint32_t flags = f32_flags(P, layout);
  const bool plain_geometry = kernel == ZL_KERNEL_PLAIN_GEOMETRY;
  if ((kernel == ZL_KERNEL_AUTO || kernel == ZL_KERNEL_TWO_PIXEL) && flags != kFlagsRuntime) {
    cudaError_t e = cudaErrorNotSupported;
    if (layout == 1)
      e = kernel == ZL_KERNEL_TWO_PIXEL ? launch_fwd_f32x2_dirbe(P, flags, tails, u, n, obs, oc, ot, st, L)
                                        : launch_fwd_dirbe_cp(P, flags, u, n, obs, oc, ot, st, L);
    if (layout == 2) e = launch_fwd_f32x2_planck(P, flags, tails, u, n, obs, oc, ot, st, L);
    if (e != cudaErrorNotSupported) return e;
  }
  if (layout == 1) return launch_fwd_f32_dirbe(P, flags, plain_geometry, u, n, obs, oc, ot, st, L);
  if (layout == 2) return launch_fwd_f32_planck(P, flags, u, n, obs, oc, ot, st, L);
  if (layout == 3 && !plain_geometry) return launch_fwd_f32_rrm(P, u, n, obs, oc, ot, st, L);
  return launch_fwd_f32_generic(P, u, n, obs, oc, ot, st, L);
}

}  // namespace zl
