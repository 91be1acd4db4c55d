// red_minmax.cu -- minimum, maximum, minimum_ind, maximum_ind instantiations.
#include "reduce.cuh"

namespace pg {

template <int DT>
static pdlgb300_error mm_family(int op, RedArgs a, const RedLaunch &lc, cudaStream_t s) {
  using T = typename TT<DT>::T;
  switch (op) {
    case R_MIN: return launch_red_typed<OpMM<T, false, false>, T, T>(a, lc, s);
    case R_MAX: return launch_red_typed<OpMM<T, true, false>, T, T>(a, lc, s);
    case R_MIN_IND: return launch_red_typed<OpMM<T, false, true>, T, int64_t>(a, lc, s);
    case R_MAX_IND: return launch_red_typed<OpMM<T, true, true>, T, int64_t>(a, lc, s);
  }
  return pgh::err(PDLGB300_EFATAL, "minmax family: bad op %d", op);
}

pdlgb300_error launch_red_minmax(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                                 cudaStream_t s) {
  PG_DISPATCH(in_dt, return mm_family<DT>(op, args, lc, s));
  return pgh::err(PDLGB300_EUSERERROR, "reduction: unsupported type %d", in_dt);
}

int red_occ_minmax(int op, int in_dt, bool bad, int block) {
  int r = 1;
  PG_DISPATCH(in_dt, {
    using T = typename TT<DT>::T;
    switch (op) {
      case R_MIN: r = red_occ_typed<OpMM<T, false, false>, T, T>(bad, block); break;
      case R_MAX: r = red_occ_typed<OpMM<T, true, false>, T, T>(bad, block); break;
      case R_MIN_IND: r = red_occ_typed<OpMM<T, false, true>, T, int64_t>(bad, block); break;
      case R_MAX_IND: r = red_occ_typed<OpMM<T, true, true>, T, int64_t>(bad, block); break;
    }
  });
  return r;
}

// Size of one split-mode partial accumulator.
size_t red_acc_size(int op, int in_dt, int comp) {
  size_t r = 0;
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    switch (op) {
      case R_SUM: r = comp ? acc_size<OpSum<In, OutP, true>>() : acc_size<OpSum<In, OutP, false>>(); break;
      case R_DSUM: r = acc_size<OpSum<In, double, false>>(); break;
      case R_AVG: r = comp ? acc_size<OpAvg<In, OutP, true>>() : acc_size<OpAvg<In, OutP, false>>(); break;
      case R_DAVG: r = acc_size<OpAvg<In, double, false>>(); break;
      case R_PROD: r = acc_size<OpProd<In, OutP>>(); break;
      case R_DPROD: r = acc_size<OpProd<In, double>>(); break;
      default: r = acc_size<OpMM<In, false, false>>(); break;
    }
  });
  return r;
}

}  // namespace pg
