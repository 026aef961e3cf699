// float64 forward kernel, one warp per pixel (ZL_KERNEL_WARP_PER_PIXEL).
#include "zl_f64.cuh"

namespace zl {

// One warp per pixel, the quadrature nodes across its lanes (node k on lane k mod 32) and a
// butterfly of warp shuffles adding the lanes' partial sums.  A warp takes 32 pixels at a
// time: lane j sets up pixel j (the per-pixel geometry, evaluated once, not by every lane)
// into shared memory, then the warp integrates the 32 pixels one after another, every lane
// reading pixel j's set-up from the same shared-memory words.  The sum over nodes is
// associated differently from the reference's sequential sum (lanes' partial sums, then the
// tree), so the result differs from the one-thread-per-pixel kernel's in the last bits.  No
// work queue (the grid strides over groups of 32 pixels); out_index applies.
template <int NSPEC>
__global__ void __launch_bounds__(128) fwd_f64_warp_kernel(const __grid_constant__ KParamsF64 P,
                                                           const double* __restrict__ u, int64_t n_pix,
                                                           const ObsArgs OA, double* __restrict__ out_comps,
                                                           double* __restrict__ out_total, const Sched SC) {
  extern __shared__ double sm[];
  const F64Table T = stage_table_f64<NSPEC>(P, sm);
  // then one PixF64 per thread (the table's size in doubles keeps 8-byte alignment)
  PixF64* pix = reinterpret_cast<PixF64*>(sm + P.m.n_temps * (1 + 2 * NSPEC)) + (threadIdx.x & ~31);
  const int lane = threadIdx.x & 31;
  const int nc = P.m.n_comps;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;  // pixels per pass of the grid
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n_pix; base += stride) {
    const int64_t ip = base + lane;
    __syncwarp();  // the previous group's reads of pix are done
    if (ip < n_pix) pixel_setup_f64(P, u, n_pix, OA, ip, pix[lane]);
    __syncwarp();
    const int np = n_pix - base < 32 ? (int)(n_pix - base) : 32;
    for (int j = 0; j < np; ++j) {
      const PixF64& X = pix[j];
      double acc[ZL_MAX_COMPS][NSPEC];
#pragma unroll
      for (int c = 0; c < ZL_MAX_COMPS; ++c)
#pragma unroll
        for (int s = 0; s < NSPEC; ++s) acc[c][s] = 0.0;
      for (int k = lane; k < P.m.n_nodes; k += 32) node_f64<NSPEC, true>(P, T, X, P.m.gl_x[k], P.m.gl_w[k], acc);
#pragma unroll
      for (int c = 0; c < ZL_MAX_COMPS; ++c) {
        if (c >= nc) break;
#pragma unroll
        for (int s = 0; s < NSPEC; ++s)
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) acc[c][s] += __shfl_xor_sync(0xffffffffu, acc[c][s], off);
      }
      if (lane == 0) store_f64<NSPEC>(P, n_pix, out_col(SC, base + j), acc, out_comps, out_total);
    }
  }
}

template <int NSPEC>
static cudaError_t launch_f64_warp_t(const KParamsF64& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                     double* ot, cudaStream_t st, const LaunchArgs& L) {
  // a block takes tpb pixels per pass, as the thread-per-pixel kernel does: the same grid;
  // shared memory: the blackbody table, then one pixel set-up per thread
  const size_t smem = sizeof(double) * P.m.n_temps * (1 + 2 * NSPEC) + sizeof(PixF64) * L.tpb;
  fwd_f64_warp_kernel<NSPEC><<<(unsigned)fwd_grid(L, n), L.tpb, smem, st>>>(P, u, n, obs, oc, ot, L.sched);
  return cudaGetLastError();
}

cudaError_t launch_fwd_f64_warp(const KParamsF64& P, const double* u, int64_t n, const ObsArgs& obs, double* oc,
                                double* ot, cudaStream_t st, const LaunchArgs& L) {
  switch (P.m.n_spec) {
    case 1: return launch_f64_warp_t<1>(P, u, n, obs, oc, ot, st, L);
    case 2: return launch_f64_warp_t<2>(P, u, n, obs, oc, ot, st, L);
    case 3: return launch_f64_warp_t<3>(P, u, n, obs, oc, ot, st, L);
    default: return launch_f64_warp_t<4>(P, u, n, obs, oc, ot, st, L);
  }
}

}  // namespace zl
