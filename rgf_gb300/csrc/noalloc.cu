// Allocation-free residual norm.
//
// Some callers must not allocate device memory: a framework whose caching
// allocator has reserved nearly all of the GPU, a serving loop that keeps
// every cudaMalloc/cudaFree out of its steady state because cudaFree waits
// for the whole device, or an embedding that hands in pre-placed device
// buffers and forbids hidden allocations.  rgf_residual_norm_noalloc serves
// them: the caller passes device inputs and a device output, and the only
// scratch (the product A x, one double per row) lives in the fixed array
// below, which the module holds on every GPU that loads this library until
// the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/rgf.h"
#include "rgf_internal.h"

namespace {

constexpr size_t kNoAllocMaxN = RGF_NOALLOC_MAX_N;
constexpr int kMaxDevices = 64;

// Scratch for A x; every call shares it and it keeps the last call's values.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxN];

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  Host code may
// not pass &g_noalloc_scratch to a kernel (that is a host-side stand-in), so
// the address is looked up once per device, with that device current.
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return RGF_ECUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return RGF_ENOTSUP;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return RGF_ECUDA;
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return RGF_OK;
}

}  // namespace

extern "C" int rgf_residual_norm_noalloc(size_t n, const size_t* d_ia, const size_t* d_ja,
                                         const double* d_a, const double* d_x,
                                         const double* d_b, double* d_out, void* stream) {
  if (!d_ia || !d_ja || !d_a || !d_x || !d_b || !d_out) return RGF_EINVAL;
  if (n == 0 || n > kNoAllocMaxN) return RGF_EINVAL;
  double* scratch = nullptr;
  const int st = scratch_for_current_device(&scratch);
  if (st) return st;
  // launch_residual zeroes the first n scratch entries before accumulating.
  rgf::launch_residual((long long)n, d_ia, d_ja, d_a, d_x, d_b, scratch, d_out,
                       static_cast<cudaStream_t>(stream));
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RGF_OK : RGF_ECUDA;
}
