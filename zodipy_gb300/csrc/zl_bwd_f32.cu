// Adjoint: launch selection, the fixed-order reduction of the tile partials and the
// gradient layout (the kernel itself is in zl_bwd_f32.cuh, instantiated per layout in
// zl_bwd_f32_dirbe.cu and zl_bwd_f32_planck.cu).
#include "zl_bwd_f32.cuh"

namespace zl {

// Sum partial rows column by column in a fixed order: thread t adds rows
// t, t + 256, ...; then a fixed tree.
__global__ void __launch_bounds__(256) reduce_tiles_kernel(const double* __restrict__ partials, int64_t n_rows,
                                                            int ng, double* __restrict__ out) {
  __shared__ double sm[256];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int64_t t = threadIdx.x; t < n_rows; t += 256) s += partials[t * ng + j];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w >= 1; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = sm[0];
}

// Gradient vector length for a layout (1 = DIRBE, 2 = Planck) and n_spec; -1 otherwise.
int grad_count_layout(int layout, int n_spec) {
  if (layout == 1) return GradLay<kLayoutDirbe, 1>::NCP + 2 + n_spec * GradLay<kLayoutDirbe, 1>::PER_SPEC;
  if (layout == 2) return GradLay<kLayoutPlanck, 1>::NCP + 2 + n_spec * GradLay<kLayoutPlanck, 1>::PER_SPEC;
  return -1;
}

// Component groups per layout: DIRBE = {cloud, bands} + {ring, feature}; Planck = one group.
int bwd_groups(int layout) { return layout == 1 ? 2 : 1; }

// partials: [bwd_groups(layout)][n_tiles][grad_count_layout(layout, n_spec)]
// unpaired: the one-pixel kernel with components in order even where the component-paired
// kernels would run (for comparing the two)
cudaError_t launch_bwd_f32(const KParamsF32& P, const KGradAux& A, int layout, bool unpaired, const double* u,
                           int64_t n, const ObsArgs& obs, const double* g_comps, const double* g_total,
                           double* partials, int64_t n_tiles, cudaStream_t st, int bps, int num_sms) {
  int64_t grid = (int64_t)num_sms * bps;
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  const uint32_t flags = f32_flags(P, layout);
  if (layout == 1)
    return launch_bwd_f32_dirbe(P, A, flags, unpaired, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
  return launch_bwd_f32_planck(P, A, flags, u, n, obs, g_comps, g_total, partials, n_tiles, st, grid);
}

cudaError_t launch_reduce_tiles(const double* partials, int64_t n_rows, int ng, double* out, cudaStream_t st) {
  reduce_tiles_kernel<<<ng, 256, 0, st>>>(partials, n_rows, ng, out);
  return cudaGetLastError();
}

}  // namespace zl
