// Allocation-free residual norm.
//
// Some callers must not allocate device memory: a framework whose caching
// allocator has reserved nearly all of the GPU, a serving loop that keeps
// every cudaMalloc/cudaFree out of its steady state because cudaFree waits
// for the whole device, or an embedding that hands in pre-placed device
// buffers and forbids hidden allocations.  rgf_residual_norm_noalloc serves
// them: the caller passes device inputs and a device output, and the only
// scratch (the product A x, one double per row, plus an error flag) lives in
// the fixed array below, which the module holds on every GPU that loads this
// library until the process exits.  With lazy module loading (the CUDA
// default) the module, and with it the array, is loaded on a device by the
// first call there.
#include <cuda_runtime.h>

#include "../../include/rgf.h"
#include "rgf_internal.h"

namespace {

constexpr size_t kNoAllocMaxN = RGF_NOALLOC_MAX_N;
// doubles after the A x scratch: room for the bad-index flag (one int)
constexpr size_t kFlagSlots = 32;

// Scratch for A x, then the flag; every call shares it and it keeps the last
// call's values (both parts are cleared at the start of each call).
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxN + kFlagSlots];

// Device address of the scratch array in the current context.  Host code may
// not pass &g_noalloc_scratch to a kernel (that is a host-side stand-in), so
// the address is looked up on every call, with the caller's device current;
// the lookup allocates nothing and also follows a context that was reset and
// created again.
int scratch_for_current_device(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? RGF_ENOMEM : RGF_ECUDA;
  }
  *out = static_cast<double*>(p);
  return RGF_OK;
}

}  // namespace

extern "C" int rgf_residual_norm_noalloc(size_t n, const size_t* d_ia, const size_t* d_ja,
                                         const double* d_a, const double* d_x,
                                         const double* d_b, double* d_out, void* stream) {
  if (!d_ia || !d_ja || !d_a || !d_x || !d_b || !d_out) return RGF_EINVAL;
  if (n == 0 || n > kNoAllocMaxN) return RGF_EINVAL;
  // An error the caller left pending is the caller's: report it without
  // clearing it instead of launching on a context that may be broken.
  if (cudaPeekAtLastError() != cudaSuccess) return RGF_ECUDA;
  double* scratch = nullptr;
  const int st = scratch_for_current_device(&scratch);
  if (st) return st;
  int* bad = reinterpret_cast<int*>(scratch + kNoAllocMaxN);
  // zeroes scratch[0, n) and the flag, then accumulates A x and the norms;
  // rows outside [c, n) in column c are skipped and make d_out NaN
  const cudaError_t e = rgf::launch_residual((long long)n, d_ia, d_ja, d_a, d_x, d_b, scratch,
                                             d_out, bad, static_cast<cudaStream_t>(stream));
  if (e == cudaErrorMemoryAllocation) return RGF_ENOMEM;
  return e == cudaSuccess ? RGF_OK : RGF_ECUDA;
}
