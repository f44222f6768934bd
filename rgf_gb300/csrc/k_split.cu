// Split-precision GEMM engine (not available in this build yet).
#include "../../include/rgf.h"
#include "rgf_split.h"

namespace rgf {

SplitEngine* SplitEngine::create(int slices, int* status) {
  (void)slices;
  *status = RGF_ENOTSUP;
  return nullptr;
}

SplitEngine::~SplitEngine() = default;

long long SplitEngine::gemm(const GemmDesc& g, cudaStream_t s) {
  launch_gemm_fp64(g, s);
  return 1;
}

}  // namespace rgf
