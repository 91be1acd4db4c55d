// expr_ll.cu -- the fused expression reductions for LL leaves
// (strided or broadcast rows).
#include "expr.cuh"

namespace pg {
template pdlgb300_error launch_expr_typed<PDLGB300_LL, false>(int, const ExprArgs &, const RedArgs &, int,
                                                       int, cudaStream_t);
}  // namespace pg
