// Float32 forward pass: choice of the compiled kernel for a model (the kernel itself is in
// zl_fwd_f32.cuh; its instantiations are spread over one translation unit per layout so that
// they compile in parallel).
#include "zl_fwd_dirbe.cuh"

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

int g_two_pixel_dirbe = 0;

// layout: 1 = DIRBE-like, 2 = Planck-like, 0 = generic; plain_geometry selects the
// all-float32 variant of the DIRBE layout (kept for the precision/speed study); one_pixel
// keeps the one-pixel kernel where the two-pixel one (zl_fwd_f32x2.cuh) would run.
cudaError_t launch_fwd_f32(const KParamsF32& P, int layout, bool plain_geometry, bool one_pixel, const double* u,
                           int64_t n, const ObsArgs& obs, double* oc, double* ot, cudaStream_t st, int tpb, int bps,
                           int num_sms) {
  const uint32_t flags = f32_flags(P, layout);
  // The two-pixel kernel wins where its doubled per-pixel state still leaves enough warps:
  // measured on GB300 at nside 512, Planck layout 0.79 vs 0.91 ms; for the DIRBE layout it
  // needs 168 registers and loses (2.01 vs 1.88 ms), so that layout keeps the one-pixel
  // kernel unless asked (two_pixel_dirbe, a testing hook).
  // The DIRBE layout runs the component-paired kernel (zl_fwd_dirbe.cuh): ring/feature and
  // band 1/2 in packed lanes, one pixel per thread.
  if (!one_pixel && !plain_geometry && flags != kFlagsRuntime) {
    cudaError_t e = cudaErrorNotSupported;
    if (layout == 1)
      e = g_two_pixel_dirbe ? launch_fwd_f32x2_dirbe(P, flags, u, n, obs, oc, ot, st, tpb, bps, num_sms)
                            : launch_fwd_dirbe_cp(P, flags, u, n, obs, oc, ot, st, tpb, bps, num_sms);
    if (layout == 2) e = launch_fwd_f32x2_planck(P, flags, u, n, obs, oc, ot, st, tpb, bps, num_sms);
    if (e != cudaErrorNotSupported) return e;
  }
  if (layout == 1) return launch_fwd_f32_dirbe(P, flags, plain_geometry, u, n, obs, oc, ot, st, tpb, bps, num_sms);
  if (layout == 2) return launch_fwd_f32_planck(P, flags, u, n, obs, oc, ot, st, tpb, bps, num_sms);
  return launch_fwd_f32_generic(P, u, n, obs, oc, ot, st, tpb, bps, num_sms);
}

}  // namespace zl
