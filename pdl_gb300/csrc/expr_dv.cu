// expr_dv.cu -- the fused expression reductions for D leaves
// (16-byte vector loads).
#include "expr.cuh"

namespace pg {
template pdlgb300_error launch_expr_typed<PDLGB300_D, true>(int, const ExprArgs &, const RedArgs &, int,
                                                       int, cudaStream_t);
}  // namespace pg
