// Split-precision (Ozaki-scheme) GEMM engine: FP64 operands are cut into
// bf16 digit slices, slice products run on the tcgen05 tensor cores with FP32
// accumulation in tensor memory, and the exact partial sums are combined in
// 64-bit integer fixed point before one conversion back to FP64.
#pragma once

#include <cuda.h>

#include <cstddef>
#include <map>
#include <tuple>

#include "rgf_internal.h"

namespace rgf {

class SplitEngine {
 public:
  // Returns nullptr and sets *status when the device or driver cannot run it.
  static SplitEngine* create(int slices, int* status);
  ~SplitEngine();
  // Size the slice workspace for operands of up to max_rows rows and max_k
  // terms (allocates once, outside any graph capture).
  // batch_hint: largest batch the caller issues (sizes the workspace so that
  // batched problems run in few chunks; capped at 1 GiB).
  // The split-K workspace is cleared on stream s (before its first use there).
  int prepare(int max_rows, int max_k, int batch_hint, cudaStream_t s);
  // True when g can run on the tensor cores (k >= min_k and within the
  // prepared sizes; batched problems run in chunks that fit the workspace).
  bool supports(const GemmDesc& g) const;
  int slices() const { return slices_; }
  // Largest split-K degree (1 = none); a tuning knob.
  void set_splitk_max(int k) { splitk_max_ = k > 0 ? k : 16; }
  // MMA streams per output tile and K term at S slices (each one N=256 MMA
  // of one A digit against two B digits, or N=128 against one)
  static int slots(int S);
  // Estimated device time of gemm(g, ..., slices), in seconds.
  double estimate_seconds(const GemmDesc& g, int slices = 0) const;
  int min_k() const { return min_k_; }
  // Issue D = alpha op(A) op(B) + beta C on stream s; returns kernels launched
  // and, in *tensor_flops (if given), the bf16 slice-product flops it runs.
  // slices > 0 overrides the engine's slice count (up to 8) for this call.
  long long gemm(const GemmDesc& g, cudaStream_t s, DevStatus* st,
                 double* tensor_flops = nullptr, int slices = 0);
  // Zero the split-K workspace and counters (they clear themselves after
  // every launch that completes; a launch that gave up on a wait may leave
  // them dirty).
  int reset_splitk(cudaStream_t s);

 private:
  SplitEngine() = default;
  int ensure_ws(size_t bytes);
  bool map_for(CUtensorMap* out, void* base, int S, int Rp, int Kp);
  std::map<std::tuple<void*, int, int, int>, CUtensorMap> maps_;
  int ensure_splitk(long long tiles, cudaStream_t s);
  int reserve(int max_rows, int max_k, int batch_hint);
  int slices_ = 0;
  int min_k_ = 1 << 30;
  int max_rows_ = 0, max_k_ = 0;
  void* ws_ = nullptr;
  size_t ws_bytes_ = 0;
  int num_sms_ = 148;
  int splitk_max_ = 16;
  // split K: int64 partial sums (128 x 128 per tile) and arrival counters
  long long* wsk_ = nullptr;
  int* cnt_ = nullptr;
  long long wsk_tiles_ = 0;
};

}  // namespace rgf
