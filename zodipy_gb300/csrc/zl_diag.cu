// Pipe-throughput probes used as roofline denominators.
//
// The line-of-sight kernels are bound by the MUFU (XU) pipe and the FP32 FMA
// pipe, neither of which has a vendor-measured peak in the benchmark inputs, so
// the benchmark measures both with these kernels on the same GPU and clock:
//  - which = 0: ex2.approx.ftz.f32 (one MUFU op each), 8 independent chains per thread
//  - which = 1: fma.rn.f32 (one FFMA each), 8 independent chains per thread
//  - which = 2: packed fma.rn.f32x2 (two FMAs each), 8 independent float2 chains per thread;
//    counted in FMAs, so it shows whether a packed instruction doubles the FP32 rate
// Every result feeds a store guarded by an impossible condition so the chains
// are not removed.
#include <cuda_runtime.h>

#include "../../include/zodigb.h"
#include "zl_common.cuh"

namespace {

__global__ void __launch_bounds__(256) xu_probe(float* sink, int iters, float seed) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = seed * (float)(threadIdx.x + j) * 1e-9f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float r;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a[j]));
      a[j] = r * -1e-3f;
    }
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == 1234.5f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) fma_probe(float* sink, int iters, float seed) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = seed + (float)(threadIdx.x + j);
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == 1234.5f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) fma2_probe(float* sink, int iters, float seed) {
  float2 a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = make_float2(seed + (float)(threadIdx.x + j), seed - (float)j);
  const float2 m = make_float2(0.999999f, 0.999998f), c = make_float2(1e-7f, 2e-7f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = __ffma2_rn(a[j], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j].x + a[j].y;
  if (s == 1234.5f) sink[blockIdx.x] = s;
}

__global__ void atan2_eval(const float* __restrict__ y, const float* __restrict__ x, float* __restrict__ out,
                           int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = zl::atan2_poly(y[i], x[i]);
}

__global__ void d2f_eval(const double* __restrict__ d, float* __restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const zl::ff p = zl::ff_split(d[i]);
    out[3 * i] = p.hi;
    out[3 * i + 1] = p.lo;
    out[3 * i + 2] = zl::d2f_bits(d[i]);
  }
}

__global__ void f2d_eval(const float* __restrict__ f, double* __restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = zl::f2d_bits(f[i]);
}

}  // namespace

extern "C" ZL_API int zl_diag_f2d(const float* f_dev, double* out_dev, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (!f_dev || !out_dev))) return ZL_ERR_ARG;
  if (n == 0) return ZL_OK;
  const int64_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  f2d_eval<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(f_dev, out_dev, n);
  return cudaGetLastError() == cudaSuccess ? ZL_OK : ZL_ERR_CUDA;
}

extern "C" ZL_API int zl_diag_d2f(const double* d_dev, float* out_dev, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (!d_dev || !out_dev))) return ZL_ERR_ARG;
  if (n == 0) return ZL_OK;
  const int64_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  d2f_eval<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(d_dev, out_dev, n);
  return cudaGetLastError() == cudaSuccess ? ZL_OK : ZL_ERR_CUDA;
}

extern "C" ZL_API int zl_diag_atan2(const float* y_dev, const float* x_dev, float* out_dev, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (!y_dev || !x_dev || !out_dev))) return ZL_ERR_ARG;
  if (n == 0) return ZL_OK;
  const int64_t blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  atan2_eval<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(y_dev, x_dev, out_dev, n);
  return cudaGetLastError() == cudaSuccess ? ZL_OK : ZL_ERR_CUDA;
}

extern "C" ZL_API int zl_diag_pipe_probe(int32_t which, int32_t iters, float* sink_dev, int32_t sink_len,
                                         double* ops_per_launch, void* stream) {
  if (which < 0 || which > 2 || iters < 1 || !sink_dev || !ops_per_launch) return ZL_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ZL_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ZL_ERR_CUDA;
  const int blocks = nsm * 8;
  if (sink_len < blocks) return ZL_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (which == 0)
    xu_probe<<<blocks, 256, 0, st>>>(sink_dev, iters, 1.0f);
  else if (which == 1)
    fma_probe<<<blocks, 256, 0, st>>>(sink_dev, iters, 1.0f);
  else
    fma2_probe<<<blocks, 256, 0, st>>>(sink_dev, iters, 1.0f);
  if (cudaGetLastError() != cudaSuccess) return ZL_ERR_CUDA;
  *ops_per_launch = (double)blocks * 256.0 * 8.0 * (double)iters * (which == 2 ? 2.0 : 1.0);
  return ZL_OK;
}
