// Split-precision (Ozaki-scheme) GEMM engine: FP64 operands are cut into
// bf16 slices, slice products run on the tcgen05 tensor cores with FP32
// accumulation in tensor memory, and the exact partial sums are combined in
// 64-bit integer fixed point before one conversion back to FP64.
#pragma once

#include "rgf_internal.h"

namespace rgf {

class SplitEngine {
 public:
  // Returns nullptr and sets *status on failure.
  static SplitEngine* create(int slices, int* status);
  ~SplitEngine();
  // Smallest inner dimension routed to the split path.
  int min_k() const { return min_k_; }
  // Issue D = alpha op(A) op(B) + beta C; returns the kernels launched.
  long long gemm(const GemmDesc& g, cudaStream_t s);

 private:
  SplitEngine() = default;
  int slices_ = 0;
  int min_k_ = 1 << 30;
};

}  // namespace rgf
