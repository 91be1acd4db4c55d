// red_logic.cu -- andover, orover, xorover, zcover, bandover, borover,
// bxorover, firstnonzeroover instantiations (lib/PDL/Ufunc.pd:143-187).
#include "reduce.cuh"

namespace pg {

template <int DT>
static pdlgb300_error logic_family(int op, RedArgs a, const RedLaunch &lc, cudaStream_t s) {
  using T = typename TT<DT>::T;
  constexpr bool INT = std::is_integral_v<T>;
  switch (op) {
    case R_AND: return launch_red_typed<OpLogic<T, 0>, T, T>(a, lc, s);
    case R_OR: return launch_red_typed<OpLogic<T, 1>, T, T>(a, lc, s);
    case R_XOR: return launch_red_typed<OpLogic<T, 2>, T, T>(a, lc, s);
    case R_ZC: return launch_red_typed<OpLogic<T, 3>, T, T>(a, lc, s);
    case R_FIRSTNZ: return launch_red_typed<OpFirstNZ<T>, T, T>(a, lc, s);
    case R_BAND: if constexpr (INT) return launch_red_typed<OpLogic<T, 4>, T, T>(a, lc, s); break;
    case R_BOR: if constexpr (INT) return launch_red_typed<OpLogic<T, 5>, T, T>(a, lc, s); break;
    case R_BXOR: if constexpr (INT) return launch_red_typed<OpLogic<T, 6>, T, T>(a, lc, s); break;
  }
  return pgh::err(PDLGB300_EUSERERROR, "reduction %d: unsupported type %d", op, DT);
}

pdlgb300_error launch_red_logic(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                                cudaStream_t s) {
  PG_DISPATCH(in_dt, return logic_family<DT>(op, args, lc, s));
  return pgh::err(PDLGB300_EUSERERROR, "reduction: unsupported type %d", in_dt);
}

int red_occ_logic(int op, int in_dt, bool bad, int block) {
  int r = 1;
  PG_DISPATCH(in_dt, {
    using T = typename TT<DT>::T;
    if (op == R_FIRSTNZ) r = red_occ_typed<OpFirstNZ<T>, T, T>(bad, block);
    else r = red_occ_typed<OpLogic<T, 1>, T, T>(bad, block);
  });
  return r;
}

size_t red_acc_size_logic(int op, int in_dt) {
  size_t r = 0;
  PG_DISPATCH(in_dt, {
    using T = typename TT<DT>::T;
    if (op == R_FIRSTNZ) r = acc_size<OpFirstNZ<T>>();
    else if (op >= R_BAND && op <= R_BXOR) r = acc_size<OpLogic<T, 4>>();
    else r = acc_size<OpLogic<T, 0>>();
  });
  return r;
}

}  // namespace pg
