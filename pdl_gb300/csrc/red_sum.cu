// red_sum.cu -- sumover, dsumover, average, daverage instantiations.
#include "reduce.cuh"

namespace pg {

template <int DT>
static pdlgb300_error sum_family(int op, RedArgs a, const RedLaunch &lc, cudaStream_t s) {
  using In = typename TT<DT>::T;
  using OutP = typename TT<intplus(DT)>::T;
  constexpr bool F32 = std::is_same_v<OutP, float>;
  switch (op) {
    case R_SUM:
      if constexpr (F32)
        if (a.f32_comp) return launch_red_typed<OpSum<In, OutP, true>, In, OutP>(a, lc, s);
      return launch_red_typed<OpSum<In, OutP, false>, In, OutP>(a, lc, s);
    case R_DSUM:
      return launch_red_typed<OpSum<In, double, false>, In, double>(a, lc, s);
    case R_AVG:
      if constexpr (F32)
        if (a.f32_comp) return launch_red_typed<OpAvg<In, OutP, true>, In, OutP>(a, lc, s);
      return launch_red_typed<OpAvg<In, OutP, false>, In, OutP>(a, lc, s);
    case R_DAVG:
      return launch_red_typed<OpAvg<In, double, false>, In, double>(a, lc, s);
  }
  return pgh::err(PDLGB300_EFATAL, "sum family: bad op %d", op);
}

pdlgb300_error launch_red_sum(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                              cudaStream_t s) {
  PG_DISPATCH(in_dt, return sum_family<DT>(op, args, lc, s));
  return pgh::err(PDLGB300_EUSERERROR, "reduction: unsupported type %d", in_dt);
}

int red_occ_sum(int op, int in_dt, int comp, bool bad, int block) {
  int r = 1;
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    constexpr bool F32 = std::is_same_v<OutP, float>;
    switch (op) {
      case R_SUM:
        if constexpr (F32)
          if (comp) { r = red_occ_typed<OpSum<In, OutP, true>, In, OutP>(bad, block); break; }
        r = red_occ_typed<OpSum<In, OutP, false>, In, OutP>(bad, block);
        break;
      case R_DSUM: r = red_occ_typed<OpSum<In, double, false>, In, double>(bad, block); break;
      case R_AVG:
        if constexpr (F32)
          if (comp) { r = red_occ_typed<OpAvg<In, OutP, true>, In, OutP>(bad, block); break; }
        r = red_occ_typed<OpAvg<In, OutP, false>, In, OutP>(bad, block);
        break;
      case R_DAVG: r = red_occ_typed<OpAvg<In, double, false>, In, double>(bad, block); break;
    }
  });
  return r;
}

}  // namespace pg
