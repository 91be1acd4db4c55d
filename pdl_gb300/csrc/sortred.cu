// sortred.cu -- the sort-based functions of PDL::Ufunc over dim 0
// (lib/PDL/Ufunc.pd:744-1115): qsort, qsorti, medover, oddmedover, pctover,
// oddpctover, modeover.
//
// The reference sorts with its own quicksort (lib/PDL/Core/pdl.h.PL:618-640
// for values, Ufunc.pd:745-767 for indices: the middle element as pivot,
// the two scans, swap, then the ranges [a,j] and [i,b]).  Its results are
// not those of every sort: the order of equal keys in qsorti, the placement
// of NaN, and which of -0 and +0 comes first all follow from the steps it
// takes.  So wherever the result could depend on the sort, a row runs the
// same steps here, one thread over a private copy of the row: the results
// are the reference's in every case.  Everywhere else a faster sort gives
// the same array: rows up to 8192 sort in shared memory (a warp or a block
// per row), longer rows of the value functions by a device-wide merge sort.  The two ranges after a partition are
// disjoint, so sorting the smaller one first (an explicit stack, at most
// 64 entries) and continuing with the larger one gives the same array.
// Scans are bounded by their range (they cannot leave it: the pivot and the
// elements swapped behind the scans stop them); a violation sets an error
// bit and ends the row.
#include <limits>

#include "args.cuh"

namespace pg {
namespace {

constexpr int QS_STACK = 64;

template <class T>
__device__ bool qs_values(T *xx, int64_t a, int64_t b) {
  int64_t st[2 * QS_STACK];
  int sp = 0;
  for (;;) {
    while (a < b) {
      int64_t i = a, j = b;
      const T median = xx[(i + j) / 2];
      do {
        while (xx[i] < median) {
          if (++i > b) return false;
        }
        while (median < xx[j]) {
          if (--j < a) return false;
        }
        if (i <= j) {
          const T t = xx[i];
          xx[i] = xx[j];
          xx[j] = t;
          i++;
          j--;
        }
      } while (i <= j);
      // [a, j] and [i, b]: push the larger, continue with the smaller
      int64_t la = a, lb = j, ra = i, rb = b;
      if (j - a > b - i) {
        la = i; lb = b; ra = a; rb = j;
      }
      if (ra < rb) {
        if (sp >= QS_STACK) return false;
        st[2 * sp] = ra;
        st[2 * sp + 1] = rb;
        sp++;
      }
      a = la;
      b = lb;
    }
    if (sp == 0) return true;
    sp--;
    a = st[2 * sp];
    b = st[2 * sp + 1];
  }
}

template <class T, class I>
__device__ bool qs_indices(const T *xx, I *ix, int64_t a, int64_t b) {
  int64_t st[2 * QS_STACK];
  int sp = 0;
  for (;;) {
    while (a < b) {
      int64_t i = a, j = b;
      const T median = xx[ix[(i + j) / 2]];
      do {
        while (xx[ix[i]] < median) {
          if (++i > b) return false;
        }
        while (median < xx[ix[j]]) {
          if (--j < a) return false;
        }
        if (i <= j) {
          const I t = ix[i];
          ix[i] = ix[j];
          ix[j] = t;
          i++;
          j--;
        }
      } while (i <= j);
      int64_t la = a, lb = j, ra = i, rb = b;
      if (j - a > b - i) {
        la = i; lb = b; ra = a; rb = j;
      }
      if (ra < rb) {
        if (sp >= QS_STACK) return false;
        st[2 * sp] = ra;
        st[2 * sp + 1] = rb;
        sp++;
      }
      a = la;
      b = lb;
    }
    if (sp == 0) return true;
    sp--;
    a = st[2 * sp];
    b = st[2 * sp + 1];
  }
}

// 0.5 * (x + y) in the reference's C: the sum in the promoted type
// (integers wrap), the product in double, then back to T.
template <class T> __device__ __forceinline__ T half_sum(T x, T y) {
  if constexpr (std::is_floating_point_v<T>) {
    return (T)(0.5 * (double)(x + y));
  } else {
    using P = decltype(x + y);
    using U = std::make_unsigned_t<P>;
    const P s = (P)(U)((U)(P)x + (U)(P)y);
    return (T)(0.5 * (double)s);
  }
}

// The outputs of a row from its sorted good values tmp[0, nn): qsort
// writes all n (lanes `lane` of G in parallel), the others one value
// (lane 0).
template <class T, int K>
__device__ __forceinline__ void finish_values(const SortArgs &g, const T *tmp, int64_t nn,
                                              const int64_t *offs, T *out, T obad, int lane,
                                              int G) {
  if constexpr (K == SR_QSORT) {
    for (int64_t t = lane; t < g.n; t += G) out[t * g.inc_b] = t < nn ? tmp[t] : obad;
    return;
  }
  if (lane != 0) return;
  if constexpr (K == SR_MODE) {
    int64_t i = 0, most = 0;
    T curmode = 0, curval = 0;
    for (int64_t t = 0; t < nn; t++) {
      if (t == 0 || curval != tmp[t]) {
        curval = tmp[t];
        i = 0;
      } else if (++i > most) {
        most = i;
        curmode = curval;
      }
    }
    *out = curmode;
    return;
  }
  if (nn == 0) {
    *out = obad;  // a row with no good element (bad-value mode only)
    return;
  }
  const int64_t last = nn - 1;
  if constexpr (K == SR_MED) {
    const int64_t n1 = last / 2;
    *out = last % 2 == 0 ? tmp[n1] : half_sum<T>(tmp[n1], tmp[n1 + 1]);
  } else if constexpr (K == SR_ODDMED) {
    *out = tmp[last / 2];
  } else if constexpr (K == SR_PCT) {
    const T p = *(reinterpret_cast<const T *>(g.p) + offs[1]);
    // the reference's mixed-type arithmetic, step by step
    const double np = last * p;
    const double lo0 = 0 > np ? 0 : np, lo1 = 0 > np + 1 ? 0 : np + 1;
    const int64_t n1 = (int64_t)(last < lo0 ? (double)last : lo0);
    const int64_t n2 = (int64_t)(last < lo1 ? (double)last : lo1);
    double pp1 = 0, pp2 = 0;
    if (last != 0) {
      pp1 = (double)n1 / (double)last;
      pp2 = (double)n2 / (double)last;
    }
    T r;
    if (np <= 0.0) r = tmp[0];
    else if (np >= last) r = tmp[last];
    else if (tmp[n2] == tmp[n1]) r = tmp[n1];
    else if (p == pp1) r = tmp[n1];
    else if (p == pp2) r = tmp[n2];
    else  // no contraction into a fused multiply-add, as in the reference's C
      r = (T)__dadd_rn(__dmul_rn(np - (double)n1, (double)(tmp[n2] - tmp[n1])),
                       (double)tmp[n1]);
    *out = r;
  } else {  // SR_ODDPCT
    const T p = *(reinterpret_cast<const T *>(g.p) + offs[1]);
    const auto q = (last + 1) * p;
    const auto m = last < q ? (decltype(q))last : q;
    const int64_t np = (int64_t)(0 > m ? (decltype(q))0 : m);
    *out = tmp[np];
  }
}

// Short rows (n <= SF_MAX): one warp per row over shared memory.  Where
// the result cannot depend on how the row is sorted -- the good values
// hold no NaN and not both -0 and +0 (for qsorti also no two equal
// values) -- the warp sorts with a bitonic network (ties broken by
// position, a total order); any other row is sorted by lane 0 with the
// reference's quicksort (qs_values / qs_indices) over the same copy.
// The bad indices of qsorti are final when found: from the end backwards.
constexpr int SF_MAX = 512, SF_WARPS = 4;

template <class T> __device__ __forceinline__ bool sf_unsafe_float(T v, bool &neg0, bool &pos0) {
  if constexpr (std::is_floating_point_v<T>) {
    if (v != v) return true;
    if (v == (T)0) {
      if (signbit(v)) neg0 = true;
      else pos0 = true;
    }
  }
  return false;
}

template <class T, int K, bool BAD>
__global__ void __launch_bounds__(SF_WARPS * 32) k_sortred_warp(const SortArgs g) {
  constexpr bool IND = K == SR_QSORTI;
  __shared__ T s_val[SF_WARPS][SF_MAX];
  __shared__ int32_t s_ix[SF_WARPS][SF_MAX];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T *const v = s_val[w];
  int32_t *const ix = s_ix[w];
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  const T obad = from_bits<T>(g.obad);
  const int n = (int)g.n;
  const unsigned lt = (1u << lane) - 1u;
  for (int64_t row = (int64_t)blockIdx.x * SF_WARPS + w; row < g.rows;
       row += (int64_t)gridDim.x * SF_WARPS) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    // good values compacted in order (qsorti: the row as is, good
    // positions compacted in ix, bad positions straight to the output)
    int nn = 0, nbad = 0;
    bool unsafe = false, neg0 = false, pos0 = false;
    for (int base = 0; base < n; base += 32) {
      const int t = base + lane;
      T x = (T)0;
      bool good = false;
      if (t < n) {
        x = a[(int64_t)t * g.inc_a];
        good = !(K != SR_MODE && BAD && bv.is(x));
      }
      const unsigned gm = __ballot_sync(0xffffffffu, good);
      const unsigned bm = __ballot_sync(0xffffffffu, t < n && !good);
      if (good) {
        const int pos = nn + __popc(gm & lt);
        if constexpr (IND) ix[pos] = t;
        else v[pos] = x;
        unsafe |= sf_unsafe_float<T>(x, neg0, pos0);
      }
      if constexpr (IND) {
        if (t < n) v[t] = x;
        if (t < n && !good)
          reinterpret_cast<int64_t *>(g.b)[offs[g.out_pdl] +
                                           (int64_t)(n - 1 - (nbad + __popc(bm & lt))) * g.inc_b] = t;
      }
      nn += __popc(gm);
      nbad += __popc(bm);
    }
    unsafe = __any_sync(0xffffffffu, unsafe) ||
             (__any_sync(0xffffffffu, neg0) && __any_sync(0xffffffffu, pos0));
    __syncwarp();
    // bitonic sort of positions [0, P): (key, position) in lexicographic
    // order, positions >= nn after everything
    int P = 1;
    while (P < nn) P <<= 1;
    if (!unsafe && nn > 1) {
      if constexpr (!IND) {
        for (int i = nn + lane; i < P; i += 32) v[i] = (T)0;
        for (int i = lane; i < P; i += 32) ix[i] = i;  // tie-break by position
      }
      for (int i = nn + lane; i < P; i += 32) {
        if constexpr (IND) ix[i] = -1;
      }
      __syncwarp();
      for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int i = lane; i < P; i += 32) {
            const int l = i ^ j;
            if (l > i) {
              bool greater;  // element i after element l
              if constexpr (IND) {
                const int32_t pi = ix[i], pl = ix[l];
                if (pi < 0) greater = pl >= 0;
                else if (pl < 0) greater = false;
                else greater = v[pl] < v[pi] || (v[pl] == v[pi] && pl < pi);
              } else {
                const int32_t pi = ix[i], pl = ix[l];
                const bool si = pi >= nn, sl = pl >= nn;
                if (si || sl) greater = si && (!sl || pl < pi);
                else greater = v[l] < v[i] || (v[l] == v[i] && pl < pi);
              }
              if (greater == ((i & k) == 0)) {
                if constexpr (!IND) {
                  const T tv = v[i];
                  v[i] = v[l];
                  v[l] = tv;
                }
                const int32_t tp = ix[i];
                ix[i] = ix[l];
                ix[l] = tp;
              }
            }
          }
          __syncwarp();
        }
      }
      if constexpr (IND) {
        // equal values: the reference's order of their indices is its own
        bool tie = false;
        for (int i = lane; i + 1 < nn; i += 32) tie |= v[ix[i]] == v[ix[i + 1]];
        if (__any_sync(0xffffffffu, tie)) {
          unsafe = true;
          // the good positions in order again
          int m = 0;
          for (int base = 0; base < n; base += 32) {
            const int t = base + lane;
            const bool good = t < n && !(BAD && bv.is(v[t]));
            const unsigned gm = __ballot_sync(0xffffffffu, good);
            if (good) ix[m + __popc(gm & lt)] = t;
            m += __popc(gm);
          }
          __syncwarp();
        }
      }
    }
    if (unsafe && nn > 1 && lane == 0) {
      bool ok;
      if constexpr (IND) ok = qs_indices<T, int32_t>(v, ix, 0, nn - 1);
      else ok = qs_values<T>(v, 0, nn - 1);
      if (!ok) atomicOr(g.err, 1);
    }
    __syncwarp();
    if constexpr (IND) {
      int64_t *out = reinterpret_cast<int64_t *>(g.b) + offs[g.out_pdl];
      for (int i = lane; i < nn; i += 32) out[(int64_t)i * g.inc_b] = ix[i];
    } else {
      T *out = reinterpret_cast<T *>(g.b) + offs[g.out_pdl];
      finish_values<T, K>(g, v, nn, offs, out, obad, lane, 32);
    }
    __syncwarp();
  }
}

// Longer rows (SF_MAX < n <= SB_MAX): one block per row over dynamic
// shared memory, the warp kernel's steps at block scale: good values
// compacted in order (block-wide, from per-warp ballots), the bitonic
// network where the result cannot depend on the sort, else the reference's
// quicksort by thread 0 over the same copy.
constexpr int SB_MAX = 8192, SB_THREADS = 256;

template <class T, int K, bool BAD>
__global__ void __launch_bounds__(SB_THREADS) k_sortred_block(const SortArgs g) {
  constexpr bool IND = K == SR_QSORTI;
  extern __shared__ __align__(16) unsigned char sb_smem[];
  const int n = (int)g.n;
  int Pmax = 1;
  while (Pmax < n) Pmax <<= 1;
  T *const v = reinterpret_cast<T *>(sb_smem);
  int32_t *const ix = reinterpret_cast<int32_t *>(sb_smem + (size_t)Pmax * sizeof(T));
  __shared__ int s_cnt[SB_THREADS / 32], s_fl;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  const T obad = from_bits<T>(g.obad);
  // block-wide counts of the warps before this one, and the totals
  auto scan2 = [&](unsigned gm, unsigned bm, int &gb, int &bb, int &gt, int &bt) {
    if (lane == 0) s_cnt[w] = (__popc(gm) << 16) | __popc(bm);
    __syncthreads();
    gb = bb = gt = bt = 0;
    for (int k = 0; k < SB_THREADS / 32; k++) {
      const int c = s_cnt[k];
      if (k < w) {
        gb += c >> 16;
        bb += c & 0xFFFF;
      }
      gt += c >> 16;
      bt += c & 0xFFFF;
    }
    __syncthreads();  // s_cnt is reused by the next call
  };
  for (int64_t row = blockIdx.x; row < g.rows; row += gridDim.x) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    if (tid == 0) s_fl = 0;
    int nn = 0, nbad = 0;
    bool unsafe = false, neg0 = false, pos0 = false;
    for (int base = 0; base < n; base += SB_THREADS) {
      const int t = base + tid;
      T x = (T)0;
      bool good = false;
      if (t < n) {
        x = a[(int64_t)t * g.inc_a];
        good = !(K != SR_MODE && BAD && bv.is(x));
      }
      const unsigned gm = __ballot_sync(0xffffffffu, good);
      const unsigned bm = __ballot_sync(0xffffffffu, t < n && !good);
      int gb, bb, gt, bt;
      scan2(gm, bm, gb, bb, gt, bt);
      if (good) {
        const int pos = nn + gb + __popc(gm & lt);
        if constexpr (IND) ix[pos] = t;
        else v[pos] = x;
        unsafe |= sf_unsafe_float<T>(x, neg0, pos0);
      }
      if constexpr (IND) {
        if (t < n) v[t] = x;
        if (t < n && !good)
          reinterpret_cast<int64_t *>(g.b)[offs[g.out_pdl] +
                                           (int64_t)(n - 1 - (nbad + bb + __popc(bm & lt))) * g.inc_b] = t;
      }
      nn += gt;
      nbad += bt;
    }
    if (unsafe) atomicOr(&s_fl, 1);
    if (neg0) atomicOr(&s_fl, 2);
    if (pos0) atomicOr(&s_fl, 4);
    __syncthreads();
    unsafe = (s_fl & 1) || (s_fl & 6) == 6;
    int P = 1;
    while (P < nn) P <<= 1;
    if (!unsafe && nn > 1) {
      if constexpr (!IND) {
        for (int i = nn + tid; i < P; i += SB_THREADS) v[i] = (T)0;
        for (int i = tid; i < P; i += SB_THREADS) ix[i] = i;  // tie-break by position
      } else {
        for (int i = nn + tid; i < P; i += SB_THREADS) ix[i] = -1;
      }
      __syncthreads();
      for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int i = tid; i < P; i += SB_THREADS) {
            const int l = i ^ j;
            if (l > i) {
              bool greater;  // element i after element l
              const int32_t pi = ix[i], pl = ix[l];
              if constexpr (IND) {
                if (pi < 0) greater = pl >= 0;
                else if (pl < 0) greater = false;
                else greater = v[pl] < v[pi] || (v[pl] == v[pi] && pl < pi);
              } else {
                const bool si = pi >= nn, sl = pl >= nn;
                if (si || sl) greater = si && (!sl || pl < pi);
                else greater = v[l] < v[i] || (v[l] == v[i] && pl < pi);
              }
              if (greater == ((i & k) == 0)) {
                if constexpr (!IND) {
                  const T tv = v[i];
                  v[i] = v[l];
                  v[l] = tv;
                }
                ix[i] = pl;
                ix[l] = pi;
              }
            }
          }
          __syncthreads();
        }
      }
      if constexpr (IND) {
        // equal values: the reference's order of their indices is its own
        bool tie = false;
        for (int i = tid; i + 1 < nn; i += SB_THREADS) tie |= v[ix[i]] == v[ix[i + 1]];
        if (tie) atomicOr(&s_fl, 8);
        __syncthreads();
        if (s_fl & 8) {
          unsafe = true;
          int m = 0;  // the good positions in order again
          for (int base = 0; base < n; base += SB_THREADS) {
            const int t = base + tid;
            const bool good = t < n && !(BAD && bv.is(v[t]));
            const unsigned gm = __ballot_sync(0xffffffffu, good);
            int gb, bb, gt, bt;
            scan2(gm, 0u, gb, bb, gt, bt);
            if (good) ix[m + gb + __popc(gm & lt)] = t;
            m += gt;
          }
        }
      }
    }
    __syncthreads();
    if (unsafe && nn > 1 && tid == 0) {
      bool ok;
      if constexpr (IND) ok = qs_indices<T, int32_t>(v, ix, 0, nn - 1);
      else ok = qs_values<T>(v, 0, nn - 1);
      if (!ok) atomicOr(g.err, 1);
    }
    __syncthreads();
    if constexpr (IND) {
      int64_t *out = reinterpret_cast<int64_t *>(g.b) + offs[g.out_pdl];
      for (int i = tid; i < nn; i += SB_THREADS) out[(int64_t)i * g.inc_b] = ix[i];
    } else {
      T *out = reinterpret_cast<T *>(g.b) + offs[g.out_pdl];
      finish_values<T, K>(g, v, nn, offs, out, obad, tid, SB_THREADS);
    }
    __syncthreads();
  }
}

// Rows longer than SB_MAX, value functions (all but qsorti, whose order of
// equal keys is the quicksort's own): a device-wide merge sort.  Where the
// row's good values hold no NaN and not both -0 and +0, equal values are
// equal bits and the sorted row is the same whatever sorts it.
// * k_lsort_tile: each block takes a tile of LS_TILE elements of a row,
//   puts a top value (above every good value) in place of bad elements and
//   past the row's end, sorts the tile with a bitonic network in shared
//   memory, and counts the row's good values and notes NaN and zero signs.
// * k_lsort_merge: merge passes, runs of w -> 2w, each thread 8 outputs
//   found by a merge-path search (equal values: the first run's first).
// * k_lsort_finish: the outputs from the sorted good prefix; a row with
//   NaN or both zeros is sorted again by one thread with the reference's
//   quicksort (qs_values) over its good elements in their order.
constexpr int LS_TILE = 4096, LS_THREADS = 512, LS_PER = 8, LS_MT = 256, LS_FT = 256;

template <class T> __device__ __forceinline__ T ls_top() {
  if constexpr (std::is_floating_point_v<T>) return (T)INFINITY;
  else return std::numeric_limits<T>::max();
}
constexpr int LS_NAN = 1, LS_NEG0 = 2, LS_POS0 = 4;

template <class T, int K, bool BAD>
__global__ void __launch_bounds__(LS_THREADS) k_lsort_tile(const SortArgs g, int64_t np, T *buf,
                                                           unsigned long long *cnt, int *flags) {
  __shared__ T sv[LS_TILE];
  __shared__ int s_good, s_fl;
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  const int64_t tiles = np / LS_TILE;
  const int tid = threadIdx.x;
  for (int64_t bt = blockIdx.x; bt < g.rows * tiles; bt += gridDim.x) {
    const int64_t row = bt / tiles, t0 = (bt - row * tiles) * LS_TILE;
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    if (tid == 0) {
      s_good = 0;
      s_fl = 0;
    }
    __syncthreads();
    int good = 0, fl = 0;
    for (int i = tid; i < LS_TILE; i += LS_THREADS) {
      const int64_t idx = t0 + i;
      T v = ls_top<T>();
      if (idx < g.n) {
        const T x = a[idx * g.inc_a];
        if (!(K != SR_MODE && BAD && bv.is(x))) {
          v = x;
          good++;
          if constexpr (std::is_floating_point_v<T>) {
            if (x != x) fl |= LS_NAN;
            else if (x == (T)0) fl |= signbit(x) ? LS_NEG0 : LS_POS0;
          }
        }
      }
      sv[i] = v;
    }
    if (good) atomicAdd(&s_good, good);
    if (fl) atomicOr(&s_fl, fl);
    __syncthreads();
    // bitonic network, ascending (with NaN the order is not used)
    for (int k = 2; k <= LS_TILE; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
        for (int q = 0; q < LS_TILE / (2 * LS_THREADS); q++) {
          const int pi = q * LS_THREADS + tid;              // pair index
          const int i = ((pi & ~(j - 1)) << 1) | (pi & (j - 1)), ixj = i + j;  // j: a power of 2
          const bool up = (i & k) == 0;
          const T x = sv[i], y = sv[ixj];
          if ((y < x) == up) {
            sv[i] = y;
            sv[ixj] = x;
          }
        }
        __syncthreads();
      }
    }
    T *o = buf + row * np + t0;
    for (int i = tid; i < LS_TILE; i += LS_THREADS) o[i] = sv[i];
    if (tid == 0) {
      if (s_good) atomicAdd(&cnt[row], (unsigned long long)s_good);
      if (s_fl) atomicOr(&flags[row], s_fl);
    }
    __syncthreads();
  }
}

template <class T> struct LsLess {
  __device__ bool operator()(const T &a, const T &b) const { return a < b; }
};

template <class T, class Less>
__global__ void __launch_bounds__(LS_MT) k_lsort_merge(const T *in, T *out, int64_t np, int64_t w,
                                                       int64_t rows) {
  const Less less;
  const int64_t per_row = np / LS_PER;
  for (int64_t q = (int64_t)blockIdx.x * LS_MT + threadIdx.x; q < rows * per_row;
       q += (int64_t)gridDim.x * LS_MT) {
    const int64_t row = q / per_row, o = (q - row * per_row) * LS_PER;
    const T *r = in + row * np;
    const int64_t p0 = o / (2 * w) * (2 * w);
    const int64_t a1 = p0 + w < np ? p0 + w : np, b1 = p0 + 2 * w < np ? p0 + 2 * w : np;
    const T *A = r + p0, *B = r + a1;
    const int64_t na = a1 - p0, nb = b1 - a1, d = o - p0;
    int64_t lo = d - nb > 0 ? d - nb : 0, hi = d < na ? d : na;
    while (lo < hi) {  // A elements among the first d outputs
      const int64_t mid = (lo + hi) >> 1;
      if (!less(B[d - 1 - mid], A[mid])) lo = mid + 1;
      else hi = mid;
    }
    int64_t i = lo, j = d - lo;
    T *dst = out + row * np + o;
#pragma unroll
    for (int e = 0; e < LS_PER; e++) {
      const bool takeA = j >= nb || (i < na && !less(B[j], A[i]));
      dst[e] = takeA ? A[i++] : B[j++];
    }
  }
}

template <class T, int K, bool BAD>
__global__ void __launch_bounds__(LS_FT) k_lsort_finish(const SortArgs g, const T *sorted,
                                                        T *spare, int64_t np,
                                                        const unsigned long long *cnt,
                                                        const int *flags, int64_t chunks) {
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  const T obad = from_bits<T>(g.obad);
  for (int64_t bc = blockIdx.x; bc < g.rows * chunks; bc += gridDim.x) {
    const int64_t row = bc / chunks, ch = bc - row * chunks;
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    T *out = reinterpret_cast<T *>(g.b) + offs[g.out_pdl];
    const int fl = flags[row];
    const bool unsafe = (fl & LS_NAN) || ((fl & LS_NEG0) && (fl & LS_POS0));
    if (unsafe) {
      if (ch == 0 && threadIdx.x == 0) {
        const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
        T *tmp = spare + row * np;
        int64_t nn = 0;
        for (int64_t t = 0; t < g.n; t++) {
          const T v = a[t * g.inc_a];
          if (K != SR_MODE && BAD && bv.is(v)) continue;
          tmp[nn++] = v;
        }
        if (nn > 0 && !qs_values<T>(tmp, 0, nn - 1)) atomicOr(g.err, 1);
        finish_values<T, K>(g, tmp, nn, offs, out, obad, 0, 1);
      }
      continue;
    }
    const int64_t nn = (int64_t)cnt[row];
    const T *v = sorted + row * np;
    if constexpr (K == SR_QSORT) {
      const int64_t lo = ch * (int64_t)LS_TILE, hi = lo + LS_TILE < g.n ? lo + LS_TILE : g.n;
      for (int64_t t = lo + threadIdx.x; t < hi; t += LS_FT) out[t * g.inc_b] = t < nn ? v[t] : obad;
    } else if (ch == 0) {
      finish_values<T, K>(g, v, nn, offs, out, obad, threadIdx.x, LS_FT);
    }
  }
}

// qsorti of rows longer than SB_MAX: (value, index) pairs.  Bad elements
// and the padding past the row's end carry LS_PAD in the index and sort
// after every good pair, by index.  Where the good values hold no NaN, not
// both zeros and no two equal values, the quicksort's order of indices is
// the sorted one; the bad indices follow in the order the reference leaves
// them (filled from the row's end backwards).  Other rows: the reference's
// quicksort on one thread, as before.
constexpr int64_t LS_PAD = (int64_t)1 << 62;
constexpr int LSI_TILE = 2048;  // pairs per tile: 32 KiB of shared memory

template <class T> struct alignas(16) LsPair {
  T v;
  int64_t i;
};
template <class T> struct LsPairLess {
  __device__ bool operator()(const LsPair<T> &a, const LsPair<T> &b) const {
    const bool pa = (a.i & LS_PAD) != 0, pb = (b.i & LS_PAD) != 0;
    if (pa != pb) return pb;
    if (!pa) {
      if (a.v < b.v) return true;
      if (b.v < a.v) return false;
    }
    return a.i < b.i;
  }
};

template <class T, bool BAD>
__global__ void __launch_bounds__(LS_THREADS) k_lsorti_tile(const SortArgs g, int64_t np,
                                                            LsPair<T> *buf,
                                                            unsigned long long *cnt, int *flags) {
  __shared__ LsPair<T> sv[LSI_TILE];
  __shared__ int s_good, s_fl;
  const LsPairLess<T> less;
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  const int64_t tiles = np / LSI_TILE;
  const int tid = threadIdx.x;
  for (int64_t bt = blockIdx.x; bt < g.rows * tiles; bt += gridDim.x) {
    const int64_t row = bt / tiles, t0 = (bt - row * tiles) * LSI_TILE;
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    if (tid == 0) {
      s_good = 0;
      s_fl = 0;
    }
    __syncthreads();
    int good = 0, fl = 0;
    for (int i = tid; i < LSI_TILE; i += LS_THREADS) {
      const int64_t idx = t0 + i;
      LsPair<T> p{(T)0, idx | LS_PAD};
      if (idx < g.n) {
        const T x = a[idx * g.inc_a];
        p.v = x;
        if (!(BAD && bv.is(x))) {
          p.i = idx;
          good++;
          if constexpr (std::is_floating_point_v<T>) {
            if (x != x) fl |= LS_NAN;
            else if (x == (T)0) fl |= signbit(x) ? LS_NEG0 : LS_POS0;
          }
        }
      }
      sv[i] = p;
    }
    if (good) atomicAdd(&s_good, good);
    if (fl) atomicOr(&s_fl, fl);
    __syncthreads();
    for (int k = 2; k <= LSI_TILE; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
        for (int q = 0; q < LSI_TILE / (2 * LS_THREADS); q++) {
          const int pi = q * LS_THREADS + tid;
          const int i = ((pi & ~(j - 1)) << 1) | (pi & (j - 1)), ixj = i + j;
          const bool up = (i & k) == 0;
          const LsPair<T> x = sv[i], y = sv[ixj];
          if (less(y, x) == up) {
            sv[i] = y;
            sv[ixj] = x;
          }
        }
        __syncthreads();
      }
    }
    LsPair<T> *o = buf + row * np + t0;
    for (int i = tid; i < LSI_TILE; i += LS_THREADS) o[i] = sv[i];
    if (tid == 0) {
      if (s_good) atomicAdd(&cnt[row], (unsigned long long)s_good);
      if (s_fl) atomicOr(&flags[row], s_fl);
    }
    __syncthreads();
  }
}

template <class T, bool BAD>
__global__ void __launch_bounds__(LS_FT) k_lsorti_finish(const SortArgs g, const LsPair<T> *sorted,
                                                         LsPair<T> *spare, int64_t np,
                                                         const unsigned long long *cnt,
                                                         const int *flags) {
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  for (int64_t row = blockIdx.x; row < g.rows; row += gridDim.x) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    int64_t *out = reinterpret_cast<int64_t *>(g.b) + offs[g.out_pdl];
    const int fl = flags[row];
    const int64_t nn = (int64_t)cnt[row];
    const LsPair<T> *p = sorted + row * np;
    bool unsafe = (fl & LS_NAN) || ((fl & LS_NEG0) && (fl & LS_POS0));
    if (!unsafe) {  // equal good values: the quicksort's order of their indices is its own
      int tie = 0;
      for (int64_t k = threadIdx.x; k + 1 < nn; k += LS_FT)
        if (!(p[k].v < p[k + 1].v)) tie = 1;
      unsafe = __syncthreads_or(tie) != 0;
    }
    if (unsafe) {
      if (threadIdx.x == 0) {
        const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
        T *tmp = reinterpret_cast<T *>(spare + row * np);
        int64_t *ix = reinterpret_cast<int64_t *>(spare + row * np) + g.n;
        int64_t m = 0, nb = g.n - 1;
        for (int64_t t = 0; t < g.n; t++) {
          const T v = a[t * g.inc_a];
          tmp[t] = v;
          if (BAD && bv.is(v)) ix[nb--] = t;
          else ix[m++] = t;
        }
        if (m > 0 && !qs_indices<T, int64_t>(tmp, ix, 0, m - 1)) atomicOr(g.err, 1);
        for (int64_t t = 0; t < g.n; t++) out[t * g.inc_b] = ix[t];
      }
    } else {
      const int64_t nbad = g.n - nn;
      for (int64_t t = threadIdx.x; t < g.n; t += LS_FT)
        out[t * g.inc_b] = t < nn ? p[t].i : (p[nn + (nbad - 1 - (t - nn))].i & ~LS_PAD);
    }
    __syncthreads();
  }
}

int64_t lsorti_np(int64_t n) { return (n + LSI_TILE - 1) / LSI_TILE * LSI_TILE; }

template <class T>
pdlgb300_error go_lsorti(const SortArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const int nsm = pgh::num_sms();
  const int64_t np = lsorti_np(g.n), tiles = np / LSI_TILE;
  using E = LsPair<T>;
  E *b0 = reinterpret_cast<E *>(g.scratch);
  E *b1 = b0 + g.rows * np;
  unsigned long long *cnt = reinterpret_cast<unsigned long long *>(b1 + g.rows * np);
  int *flags = reinterpret_cast<int *>(cnt + g.rows);
  if (!pgh::cuda_check(cudaMemsetAsync(cnt, 0, (size_t)g.rows * (sizeof *cnt + sizeof *flags), s),
                       &e, "lsorti counters"))
    return e;
  const int64_t gt = std::max<int64_t>(1, std::min<int64_t>(g.rows * tiles, (int64_t)nsm * 16));
  if (g.bad) k_lsorti_tile<T, true><<<(int)gt, LS_THREADS, 0, s>>>(g, np, b0, cnt, flags);
  else k_lsorti_tile<T, false><<<(int)gt, LS_THREADS, 0, s>>>(g, np, b0, cnt, flags);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_lsorti_tile")) return e;
  pgh::record_kernel("k_lsorti_tile", gt, LS_THREADS);
  E *cur = b0, *nxt = b1;
  const int64_t gm = std::max<int64_t>(
      1, std::min<int64_t>((g.rows * (np / LS_PER) + LS_MT - 1) / LS_MT, (int64_t)nsm * 32));
  for (int64_t w = LSI_TILE; w < np; w *= 2) {
    k_lsort_merge<E, LsPairLess<T>><<<(int)gm, LS_MT, 0, s>>>(cur, nxt, np, w, g.rows);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_lsort_merge")) return e;
    pgh::record_kernel("k_lsort_merge", gm, LS_MT);
    std::swap(cur, nxt);
  }
  const int64_t gf = std::max<int64_t>(1, std::min<int64_t>(g.rows, (int64_t)nsm * 16));
  if (g.bad) k_lsorti_finish<T, true><<<(int)gf, LS_FT, 0, s>>>(g, cur, nxt, np, cnt, flags);
  else k_lsorti_finish<T, false><<<(int)gf, LS_FT, 0, s>>>(g, cur, nxt, np, cnt, flags);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_lsorti_finish")) return e;
  pgh::record_kernel("k_lsorti_finish", gf, LS_FT);
  return e;
}

// scratch of the long-row merge sort: two buffers of rows x np values,
// then the rows' good counts and flags
int64_t lsort_np(int64_t n) { return (n + LS_TILE - 1) / LS_TILE * LS_TILE; }

template <class T, int K>
pdlgb300_error go_lsort(const SortArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const int nsm = pgh::num_sms();
  const int64_t np = lsort_np(g.n), tiles = np / LS_TILE;
  T *b0 = reinterpret_cast<T *>(g.scratch);
  T *b1 = b0 + g.rows * np;
  unsigned long long *cnt = reinterpret_cast<unsigned long long *>(b1 + g.rows * np);
  int *flags = reinterpret_cast<int *>(cnt + g.rows);
  if (!pgh::cuda_check(cudaMemsetAsync(cnt, 0, (size_t)g.rows * (sizeof *cnt + sizeof *flags), s),
                       &e, "lsort counters"))
    return e;
  const int64_t gt = std::max<int64_t>(1, std::min<int64_t>(g.rows * tiles, (int64_t)nsm * 16));
  if (g.bad) k_lsort_tile<T, K, true><<<(int)gt, LS_THREADS, 0, s>>>(g, np, b0, cnt, flags);
  else k_lsort_tile<T, K, false><<<(int)gt, LS_THREADS, 0, s>>>(g, np, b0, cnt, flags);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_lsort_tile")) return e;
  pgh::record_kernel("k_lsort_tile", gt, LS_THREADS);
  T *cur = b0, *nxt = b1;
  const int64_t gm = std::max<int64_t>(
      1, std::min<int64_t>((g.rows * (np / LS_PER) + LS_MT - 1) / LS_MT, (int64_t)nsm * 32));
  for (int64_t w = LS_TILE; w < np; w *= 2) {
    k_lsort_merge<T, LsLess<T>><<<(int)gm, LS_MT, 0, s>>>(cur, nxt, np, w, g.rows);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_lsort_merge")) return e;
    pgh::record_kernel("k_lsort_merge", gm, LS_MT);
    std::swap(cur, nxt);
  }
  const int64_t chunks = K == SR_QSORT ? tiles : 1;
  const int64_t gf = std::max<int64_t>(1, std::min<int64_t>(g.rows * chunks, (int64_t)nsm * 16));
  if (g.bad) k_lsort_finish<T, K, true><<<(int)gf, LS_FT, 0, s>>>(g, cur, nxt, np, cnt, flags, chunks);
  else k_lsort_finish<T, K, false><<<(int)gf, LS_FT, 0, s>>>(g, cur, nxt, np, cnt, flags, chunks);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_lsort_finish")) return e;
  pgh::record_kernel("k_lsort_finish", gf, LS_FT);
  return e;
}

// dynamic shared memory of k_sortred_block for rows of n values of tsize bytes
size_t sortred_block_smem(int64_t n, int tsize) {
  int64_t P = 1;
  while (P < n) P <<= 1;
  return (size_t)P * (tsize + 4);
}

template <class T, int K>
pdlgb300_error go_sort(const SortArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const int nsm = pgh::num_sms();
  if (g.n <= SF_MAX) {
    const int64_t grid =
        std::max<int64_t>(1, std::min<int64_t>((g.rows + SF_WARPS - 1) / SF_WARPS, (int64_t)nsm * 32));
    if (g.bad) k_sortred_warp<T, K, true><<<(int)grid, SF_WARPS * 32, 0, s>>>(g);
    else k_sortred_warp<T, K, false><<<(int)grid, SF_WARPS * 32, 0, s>>>(g);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_sortred_warp")) return e;
    pgh::record_kernel("k_sortred_warp", grid, SF_WARPS * 32);
    return e;
  }
  if (g.n <= SB_MAX) {
    const size_t smem = sortred_block_smem(g.n, (int)sizeof(T));
    auto kern = g.bad ? k_sortred_block<T, K, true> : k_sortred_block<T, K, false>;
    // (the kernel's own static shared words count against the default 48 KB too)
    if (smem + 1024 > 48 * 1024 &&
        !pgh::cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem), &e, "k_sortred_block smem"))
      return e;
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(g.rows, (int64_t)nsm * 8));
    kern<<<(int)grid, SB_THREADS, smem, s>>>(g);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_sortred_block")) return e;
    pgh::record_kernel("k_sortred_block", grid, SB_THREADS);
    return e;
  }
  if (!g.scratch) return pgh::err(PDLGB300_EFATAL, "sort: no scratch for long rows");
  if constexpr (K == SR_QSORTI) return go_lsorti<T>(g, s);
  else return go_lsort<T, K>(g, s);
}

template <int DT>
pdlgb300_error sort_family(int k, const SortArgs &g, cudaStream_t s) {
  using T = typename TT<DT>::T;
  switch (k) {
    case SR_QSORT: return go_sort<T, SR_QSORT>(g, s);
    case SR_QSORTI: return go_sort<T, SR_QSORTI>(g, s);
    case SR_MED: return go_sort<T, SR_MED>(g, s);
    case SR_ODDMED: return go_sort<T, SR_ODDMED>(g, s);
    case SR_PCT: return go_sort<T, SR_PCT>(g, s);
    case SR_ODDPCT: return go_sort<T, SR_ODDPCT>(g, s);
    case SR_MODE:
      if constexpr (std::is_integral_v<T>) return go_sort<T, SR_MODE>(g, s);
      break;
  }
  return pgh::err(PDLGB300_EUSERERROR, "sort-based function %d: unsupported type %d", k, DT);
}

}  // namespace

size_t sortred_long_scratch(int kind, int64_t rows, int64_t n, int tsize) {
  const size_t buf = kind == SR_QSORTI ? (size_t)2 * rows * lsorti_np(n) * 16
                                       : (size_t)2 * rows * lsort_np(n) * tsize;
  return buf + (size_t)rows * (sizeof(unsigned long long) + sizeof(int));
}

pdlgb300_error launch_sortred(int k, int dt, const SortArgs &g, cudaStream_t s) {
  PG_DISPATCH(dt, return sort_family<DT>(k, g, s));
  return pgh::err(PDLGB300_EUSERERROR, "sort-based function: unsupported type %d", dt);
}

}  // namespace pg
