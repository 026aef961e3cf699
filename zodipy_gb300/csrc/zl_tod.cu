// Time-ordered input on the device: the pieces of zodipy/model.py:119-203 and
// zodipy/bodies.py:16-50 that run per sample.
//
//  - cutoff flags of a whole call: the OR over every sample's observer of the
//    rule of zodipy/line_of_sight.py:72-73 (one word, read by the forward and
//    adjoint kernels for every pixel);
//  - body positions at the sample times from the cubic spline through hourly
//    knots (bodies.py:16-35 builds scipy's CubicSpline; here the host builds
//    the same piecewise polynomial and the device evaluates it, in the order
//    of scipy.interpolate.PPoly: interval search, then the power sum from the
//    constant term up);
//  - the SEMB-L2 observer (bodies.py:38-50);
//  - sky directions from longitude/latitude rotated into the ecliptic frame
//    (the transform of model.py:244-251 for frames related by a fixed rotation).
#include <cmath>

#include "zl_common.cuh"

namespace zl {
int set_error(int code, const char* fmt, ...);
}

using namespace zl;

namespace {

constexpr int kTodThreads = 256;

int launch_grid(int64_t n, int cap_blocks) {
  int64_t g = (n + kTodThreads - 1) / kTodThreads;
  if (g > cap_blocks) g = cap_blocks;
  return (int)(g < 1 ? 1 : g);
}

int cuda_err(cudaError_t e, const char* what) {
  return set_error(ZL_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

struct Cutoffs {
  double r[ZL_MAX_RANGES][2];
  int32_t n;
};

// OR of the per-sample cutoff flags; warps combine with a ballot-free shuffle OR, one atomic per warp.
__global__ void __launch_bounds__(kTodThreads) tod_flags_kernel(const double* __restrict__ obs, int64_t n,
                                                                const Cutoffs C, uint32_t* __restrict__ flags) {
  uint32_t f = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = obs[i], y = obs[n + i], z = obs[2 * n + i];
    const double r = sqrt(x * x + y * y + z * z);
    for (int k = 0; k < C.n; ++k) {
      if (r > C.r[k][0]) f |= 1u << (2 * k);
      if (r > C.r[k][1]) f |= 1u << (2 * k + 1);
    }
  }
  for (int o = 16; o > 0; o >>= 1) f |= __shfl_xor_sync(0xffffffffu, f, o);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(flags, f);
}

// Interval of t among ascending breakpoints x[0..nk-1] as scipy's PPoly finds it:
// x[j] <= t < x[j+1]; the first interval below x[0], the last one at or above x[nk-1].
__device__ __forceinline__ int spline_interval(const double* __restrict__ x, int nk, double t) {
  if (t < x[0]) return 0;
  if (t >= x[nk - 1]) return nk - 2;
  int lo = 0, hi = nk - 2;  // invariant: x[lo] <= t < x[hi + 1]
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (x[mid] <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// c: [4][nk-1][3], highest power first (scipy's PPoly.c of a CubicSpline over axis -1 of a (3, nk) array).
__global__ void __launch_bounds__(kTodThreads) spline_eval_kernel(const double* __restrict__ x, int nk,
                                                                  const double* __restrict__ c,
                                                                  const double* __restrict__ t, int64_t n,
                                                                  double* __restrict__ out) {
  const int64_t seg = (int64_t)(nk - 1) * 3;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ti = t[i];
    if (isnan(ti)) {
      out[i] = out[n + i] = out[2 * n + i] = ti;
      continue;
    }
    const int j = spline_interval(x, nk, ti);
    const double s = ti - x[j];
    const double s2 = __dmul_rn(s, s), s3 = __dmul_rn(s2, s);
    for (int a = 0; a < 3; ++a) {
      const double* cj = c + (int64_t)j * 3 + a;
      double r = cj[3 * seg];
      r = __dadd_rn(r, __dmul_rn(cj[2 * seg], s));
      r = __dadd_rn(r, __dmul_rn(cj[seg], s2));
      r = __dadd_rn(r, __dmul_rn(cj[0], s3));
      out[a * n + i] = r;
    }
  }
}

// SEMB-L2 per sample: Earth's direction from the Sun, pushed out by d (bodies.py:38-50 for one instant).
__global__ void __launch_bounds__(kTodThreads) semb_l2_kernel(const double* __restrict__ e, int64_t n, double d,
                                                              double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = e[i], y = e[n + i], z = e[2 * n + i];
    const double r = sqrt(x * x + y * y + z * z);
    const double f = r + d;
    out[i] = x / r * f;
    out[n + i] = y / r * f;
    out[2 * n + i] = z / r * f;
  }
}

// Sum of squares of a[0..m) in a fixed order: each block strides its share, then a fixed shared-memory tree.
__global__ void __launch_bounds__(kTodThreads) sumsq_partials_kernel(const double* __restrict__ a, int64_t m,
                                                                     double* __restrict__ partials) {
  __shared__ double sm[kTodThreads];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(a[i], a[i], s);
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = kTodThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sm[0];
}

// SEMB-L2 for a sequence of times as the reference forms it: numpy.linalg.norm of the whole (3, n)
// position array (bodies.py:46) scales every sample, e / |E| * (|E| + d).
__global__ void __launch_bounds__(kTodThreads) semb_l2_whole_kernel(const double* __restrict__ e, int64_t n, double d,
                                                                    const double* __restrict__ partials, int np,
                                                                    double* __restrict__ out) {
  __shared__ double norm_sm;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < np; ++k) s += partials[k];
    norm_sm = sqrt(s);
  }
  __syncthreads();
  const double norm = norm_sm;
  const double f = norm + d;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = e[i] / norm * f;
}

struct Mat3 {
  double m[9];
};

__global__ void __launch_bounds__(kTodThreads) directions_kernel(const double* __restrict__ lon,
                                                                 const double* __restrict__ lat, int64_t n,
                                                                 const Mat3 M, double* __restrict__ u) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double sl, cl, sb, cb;
    sincos(lon[i], &sl, &cl);
    sincos(lat[i], &sb, &cb);
    const double v0 = cb * cl, v1 = cb * sl, v2 = sb;
    for (int a = 0; a < 3; ++a) u[a * n + i] = M.m[3 * a] * v0 + M.m[3 * a + 1] * v1 + M.m[3 * a + 2] * v2;
  }
}

int sm_blocks(int per_sm) {
  int dev = 0, nsm = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm * per_sm;
}

}  // namespace

namespace zl {
// Cutoff flags of a time-ordered call into *flags (zeroed first), on stream st.
cudaError_t launch_tod_flags(const ZlModel& m, const double* obs, int64_t n, uint32_t* flags, cudaStream_t st,
                             int num_sms) {
  cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess || n == 0) return e;
  Cutoffs C;
  C.n = m.n_ranges;
  for (int r = 0; r < m.n_ranges; ++r) {
    C.r[r][0] = m.cutoff[r][0];
    C.r[r][1] = m.cutoff[r][1];
  }
  tod_flags_kernel<<<launch_grid(n, num_sms * 4), kTodThreads, 0, st>>>(obs, n, C, flags);
  return cudaGetLastError();
}
}  // namespace zl

extern "C" ZL_API int zl_spline_eval(const double* knots, int32_t n_knots, const double* coef, const double* t,
                                     int64_t n, double* out, void* stream) {
  if (n < 0) return set_error(ZL_ERR_ARG, "n < 0");
  if (n_knots < 2) return set_error(ZL_ERR_ARG, "a spline needs at least 2 knots, got %d", n_knots);
  if (n == 0) return ZL_OK;
  if (!knots || !coef || !t || !out) return set_error(ZL_ERR_ARG, "NULL pointer argument");
  spline_eval_kernel<<<launch_grid(n, sm_blocks(8)), kTodThreads, 0, (cudaStream_t)stream>>>(knots, n_knots, coef, t,
                                                                                             n, out);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ZL_OK : cuda_err(e, "zl_spline_eval launch");
}

extern "C" ZL_API int zl_semb_l2(const double* earth, int64_t n, double l2_distance, int32_t whole_array_norm,
                                 double* scratch, int64_t scratch_len, double* out, void* stream) {
  if (n < 0) return set_error(ZL_ERR_ARG, "n < 0");
  if (n == 0) return ZL_OK;
  if (!earth || !out) return set_error(ZL_ERR_ARG, "NULL pointer argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (!whole_array_norm) {
    semb_l2_kernel<<<launch_grid(n, sm_blocks(8)), kTodThreads, 0, st>>>(earth, n, l2_distance, out);
  } else {
    if (!scratch || scratch_len < ZL_SEMB_L2_SCRATCH)
      return set_error(ZL_ERR_SPACE, "scratch of %lld doubles is smaller than the %d required", (long long)scratch_len,
                       ZL_SEMB_L2_SCRATCH);
    const int np = launch_grid(3 * n, ZL_SEMB_L2_SCRATCH);
    sumsq_partials_kernel<<<np, kTodThreads, 0, st>>>(earth, 3 * n, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(e, "zl_semb_l2 launch");
    semb_l2_whole_kernel<<<launch_grid(3 * n, sm_blocks(8)), kTodThreads, 0, st>>>(earth, n, l2_distance, scratch,
                                                                                   np, out);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ZL_OK : cuda_err(e, "zl_semb_l2 launch");
}

extern "C" ZL_API int zl_directions(const double* lon, const double* lat, int64_t n, const double* rotation,
                                    double* unit_vectors, void* stream) {
  if (n < 0) return set_error(ZL_ERR_ARG, "n < 0");
  if (n == 0) return ZL_OK;
  if (!lon || !lat || !unit_vectors) return set_error(ZL_ERR_ARG, "NULL pointer argument");
  Mat3 M;
  for (int k = 0; k < 9; ++k) M.m[k] = rotation ? rotation[k] : (k % 4 == 0 ? 1.0 : 0.0);
  directions_kernel<<<launch_grid(n, sm_blocks(8)), kTodThreads, 0, (cudaStream_t)stream>>>(lon, lat, n, M,
                                                                                            unit_vectors);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ZL_OK : cuda_err(e, "zl_directions launch");
}
