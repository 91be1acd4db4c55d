// expr_l.cu -- the fused expression reductions for L leaves
// (strided or broadcast rows).
#include "expr.cuh"

namespace pg {
template pdlgb300_error launch_expr_typed<PDLGB300_L, false>(int, const ExprArgs &, const RedArgs &, int,
                                                       int, cudaStream_t);
}  // namespace pg
