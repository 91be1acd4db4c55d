// expr_f.cu -- the fused expression reductions for F leaves
// (strided or broadcast rows).
#include "expr.cuh"

namespace pg {
template pdlgb300_error launch_expr_typed<PDLGB300_F, false>(int, const ExprArgs &, const RedArgs &, int,
                                                       int, cudaStream_t);
}  // namespace pg
