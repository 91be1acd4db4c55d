// mm_tc.cu -- float32 matmult as split-bf16 products on the tcgen05 tensor
// cores (placeholder until the kernel lands: reports unsupported).
#include "args.cuh"

namespace pg {
bool matmult_tc_supported(const MMArgs &) { return false; }
pdlgb300_error launch_matmult_tc(int, const MMArgs &, cudaStream_t) {
  return pgh::err(PDLGB300_EFATAL, "tensor-core matmult not built");
}
}  // namespace pg
