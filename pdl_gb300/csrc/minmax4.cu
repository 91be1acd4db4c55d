// minmax4.cu -- minmaximum (lib/PDL/Ufunc.pd:563-613): a(n); [o]cmin();
// [o]cmax(); indx [o]cmin_ind(); indx [o]cmax_ind().  Bad and NaN elements
// are skipped; the first remaining element starts both extremes and later
// ones replace them only when strictly smaller / larger, so ties keep the
// first index.  A row with nothing left sets all four outputs BAD and their
// bad state, with or without bad-value mode.
//
// One warp per row, lanes striding along n (coalesced for contiguous rows);
// each lane sees its elements in increasing index order, and the shuffle
// merge breaks ties by index.
#include "args.cuh"

namespace pg {
namespace {

template <class T> struct MM4 {
  T vmin, vmax;
  int64_t imin, imax;  // imin < 0: nothing yet
};

template <class T> __device__ __forceinline__ void mm4_merge(MM4<T> &a, const MM4<T> &b) {
  if (b.imin < 0) return;
  if (a.imin < 0) {
    a = b;
    return;
  }
  if (b.vmin < a.vmin || (b.vmin == a.vmin && b.imin < a.imin)) {
    a.vmin = b.vmin;
    a.imin = b.imin;
  }
  if (b.vmax > a.vmax || (b.vmax == a.vmax && b.imax < a.imax)) {
    a.vmax = b.vmax;
    a.imax = b.imax;
  }
}

template <class T, bool BAD>
__global__ void __launch_bounds__(256) k_minmaximum(const MM4Args g) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < g.rows;
       row += nw) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    MM4<T> acc{(T)0, (T)0, -1, -1};
    for (int64_t i = lane; i < g.n; i += 32) {
      const T v = a[i * g.inc_n];
      if (BAD && bv.is(v)) continue;
      if (isnan_any(v)) continue;
      if (acc.imin < 0) {
        acc = MM4<T>{v, v, i, i};
      } else {
        if (v < acc.vmin) {
          acc.vmin = v;
          acc.imin = i;
        }
        if (v > acc.vmax) {
          acc.vmax = v;
          acc.imax = i;
        }
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      MM4<T> o = shfl_down_any(acc, d);
      mm4_merge(acc, o);
    }
    if (lane == 0) {
      T *cmin = reinterpret_cast<T *>(g.out[0]) + offs[1];
      T *cmax = reinterpret_cast<T *>(g.out[1]) + offs[2];
      int64_t *imin = reinterpret_cast<int64_t *>(g.out[2]) + offs[3];
      int64_t *imax = reinterpret_cast<int64_t *>(g.out[3]) + offs[4];
      if (acc.imin < 0) {
        *cmin = from_bits<T>(g.obad[0]);
        *cmax = from_bits<T>(g.obad[1]);
        *imin = (int64_t)g.obad[2];
        *imax = (int64_t)g.obad[3];
        *g.setbad = 1;
      } else {
        *cmin = acc.vmin;
        *cmax = acc.vmax;
        *imin = acc.imin;
        *imax = acc.imax;
      }
    }
  }
}

template <class T> pdlgb300_error mm4_typed(const MM4Args &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.rows == 0) return e;
  const int64_t grid = std::min<int64_t>((g.rows + 7) / 8, (int64_t)1 << 30);
  if (g.bad) k_minmaximum<T, true><<<(int)grid, 256, 0, s>>>(g);
  else k_minmaximum<T, false><<<(int)grid, 256, 0, s>>>(g);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_minmaximum")) return e;
  pgh::record_kernel("k_minmaximum", grid, 256);
  return e;
}

}  // namespace

pdlgb300_error launch_minmaximum(int dt, const MM4Args &g, cudaStream_t s) {
  PG_DISPATCH(dt, return mm4_typed<typename TT<DT>::T>(g, s));
  return pgh::err(PDLGB300_EUSERERROR, "minmaximum: unsupported type %d", dt);
}

}  // namespace pg
