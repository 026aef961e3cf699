// zl_backward_static: the adjoint for callers that cannot allocate device memory.
//
// zl_backward needs a scratch buffer (the per-tile partial sums of the
// gradient) that its caller allocates.  Some callers cannot: a host framework
// that owns every byte of device memory through its own pool and forbids
// libraries from calling cudaMalloc, a real-time loop that must not allocate
// (an allocation may synchronise the device), or a thin foreign-function
// binding that has raw device pointers but no allocator.  This entry point
// takes the same inputs and outputs as zl_backward and uses a fixed scratch
// array compiled into the library instead.
//
// The array (kStaticScratchBytes = 32 MiB) is a file-scope __device__
// variable: every GPU that loads this library holds it until the process
// exits.  It bounds the problem size: the call is rejected with ZL_ERR_SPACE
// when zl_backward_workspace_bytes() exceeds it (a single-band DIRBE model
// fits 3.4 million pixels, e.g. a full HEALPix nside-512 map; a Planck model
// 9.9 million).  Nothing in the array needs clearing: every partial sum the
// reduction reads is written earlier in the same call.  All calls share the
// one array, so calls whose GPU work overlaps (different streams, or several
// host threads) race on it; serialise them.  The first call on each device
// looks up the array's device address with cudaGetSymbolAddress (once per
// device, with that device current); make that first call before any stream
// capture.  The looked-up address is cached per device for the life of the
// process; cudaDeviceReset() (or any destruction of the primary context) unloads
// the module that holds the array, so after a reset the cached address is stale
// and zl_backward_static must not be called again in that process.  The entry
// point itself calls no allocating CUDA or library routine.
#include <mutex>

#include "zl_common.cuh"

namespace zl {
int set_error(int code, const char* fmt, ...);
}

namespace {

constexpr size_t kStaticScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double zl_static_scratch[kStaticScratchBytes / sizeof(double)];

std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {nullptr};

}  // namespace

extern "C" ZL_API int zl_backward_static(const ZlModel* model, const double* u, int64_t n_pix,
                                         const ZlObserver* obs, int32_t n_obs, const double* g_comps,
                                         const double* g_total, double* grad_out, void* stream) {
  size_t need = 0;
  int rc = zl_backward_workspace_bytes(model, n_pix, &need);
  if (rc) return rc;
  if (need > kStaticScratchBytes)
    return zl::set_error(ZL_ERR_SPACE,
                         "zl_backward_static: %lld pixels need %zu bytes of scratch, more than the %zu bytes "
                         "built into the library; use zl_backward with a caller-allocated workspace",
                         (long long)n_pix, need, kStaticScratchBytes);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return zl::set_error(ZL_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return zl::set_error(ZL_ERR_CUDA, "device %d out of range", dev);
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, zl_static_scratch);
      if (e != cudaSuccess)
        return zl::set_error(ZL_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
      g_scratch_addr[dev] = p;
    }
    scratch = g_scratch_addr[dev];
  }
  return zl_backward(model, u, n_pix, obs, n_obs, g_comps, g_total, grad_out, scratch, kStaticScratchBytes, stream);
}
