// red_prod.cu -- prodover, dprodover instantiations.
#include "reduce.cuh"

namespace pg {

template <int DT>
static pdlgb300_error prod_family(int op, RedArgs a, const RedLaunch &lc, cudaStream_t s) {
  using In = typename TT<DT>::T;
  using OutP = typename TT<intplus(DT)>::T;
  if (op == R_PROD) return launch_red_typed<OpProd<In, OutP>, In, OutP>(a, lc, s);
  return launch_red_typed<OpProd<In, double>, In, double>(a, lc, s);
}

pdlgb300_error launch_red_prod(int op, int in_dt, RedArgs args, const RedLaunch &lc,
                               cudaStream_t s) {
  PG_DISPATCH(in_dt, return prod_family<DT>(op, args, lc, s));
  return pgh::err(PDLGB300_EUSERERROR, "reduction: unsupported type %d", in_dt);
}

int red_occ_prod(int op, int in_dt, bool bad, int block) {
  int r = 1;
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    if (op == R_PROD) r = red_occ_typed<OpProd<In, OutP>, In, OutP>(bad, block);
    else r = red_occ_typed<OpProd<In, double>, In, double>(bad, block);
  });
  return r;
}

}  // namespace pg
