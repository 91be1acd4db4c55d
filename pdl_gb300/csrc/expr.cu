// expr.cu -- which expression reductions are fused, and the launch by
// type (the kernels are in expr.cuh, instantiated by expr_<type>.cu).
#include "args.cuh"

namespace pg {

template <int DT, bool VL>
pdlgb300_error launch_expr_typed(int op, const ExprArgs &g, const RedArgs &ra, int grid, int block,
                                 cudaStream_t s);

bool expr_fusable(int op, int dt) {
  const bool t_ok = dt == PDLGB300_L || dt == PDLGB300_LL || dt == PDLGB300_F || dt == PDLGB300_D;
  if (!t_ok) return false;
  const bool is_int = dt == PDLGB300_L || dt == PDLGB300_LL;
  switch (op) {
    case R_SUM: case R_DSUM: case R_AVG: case R_DAVG: case R_MIN: case R_MAX:
    case R_MIN_IND: case R_MAX_IND: case R_AND: case R_OR: case R_XOR: case R_ZC:
      return true;
    case R_PROD: case R_BAND: case R_BOR: case R_BXOR:
      return is_int;
    default:
      return false;
  }
}

size_t expr_acc_size(int op, int dt, int comp) {
  if (red_is_logic(op)) return red_acc_size_logic(op, dt);
  return red_acc_size(op, dt, comp);
}

pdlgb300_error launch_expr_reduce(int op, int dt, const ExprArgs &g, const RedArgs &ra, int grid,
                                  int block, cudaStream_t s) {
  switch (dt) {
    case PDLGB300_L:
      return g.vec ? launch_expr_typed<PDLGB300_L, true>(op, g, ra, grid, block, s)
                   : launch_expr_typed<PDLGB300_L, false>(op, g, ra, grid, block, s);
    case PDLGB300_LL:
      return g.vec ? launch_expr_typed<PDLGB300_LL, true>(op, g, ra, grid, block, s)
                   : launch_expr_typed<PDLGB300_LL, false>(op, g, ra, grid, block, s);
    case PDLGB300_F:
      return g.vec ? launch_expr_typed<PDLGB300_F, true>(op, g, ra, grid, block, s)
                   : launch_expr_typed<PDLGB300_F, false>(op, g, ra, grid, block, s);
    case PDLGB300_D:
      return g.vec ? launch_expr_typed<PDLGB300_D, true>(op, g, ra, grid, block, s)
                   : launch_expr_typed<PDLGB300_D, false>(op, g, ra, grid, block, s);
    default: break;
  }
  return pgh::err(PDLGB300_EUSERERROR, "expression reduction: type %d is not fusable", dt);
}

}  // namespace pg
