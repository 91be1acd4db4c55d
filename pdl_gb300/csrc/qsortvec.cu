// qsortvec.cu -- PDL::Ufunc's vector sorts (lib/PDL/Ufunc.pd:1115-1231):
// qsortvec (a(n,m) -> [o]b(n,m): the m vectors of length n in lexicographic
// order) and qsortveci (a(n,m) -> indx [o]indx(m): their positions in that
// order).  Vectors with a bad component go to the end, the first of them
// last (the `nb--` compaction); the good ones are sorted by the reference's
// vector quicksort (Ufunc.pd:788-812: middle vector as pivot, tracked by
// position as swaps move it; pdl_cmpvec compares component by component
// with < and >).
//
// A sorted list of vectors is the same whatever sort made it when no two
// good vectors compare equal and no component is NaN (the comparison is
// then a strict total order); where two compare equal (or a NaN makes the
// comparison no order at all), which of them comes first, and qsortveci's
// indices, follow from the quicksort's steps.  So a block sorts each
// broadcast row in shared memory with a bitonic network, checks the sorted
// neighbours, and a row with a tie or a NaN is sorted again by one thread
// with the reference's steps from the original order.  Rows too large for
// shared memory run those steps one thread per row over device scratch.
// Every scan is bounded by its range; a violation (never expected: the
// pivot stops the scans) sets an error bit and ends the row.
#include "args.cuh"

namespace pg {
namespace {

constexpr int QV_THREADS = 256, QV_STACK = 64;

}  // namespace

// Bytes of shared memory the block kernel needs for m vectors of n values
// of tsize bytes: the vectors, the order ix[m] and the network's keys sx[P]
// (P the power of two >= m).  The host decides between the kernels with it.
size_t qsortvec_smem_bytes(int64_t n, int64_t m, int tsize) {
  int64_t P = 1;
  while (P < m) P <<= 1;
  return ((size_t)(n * m * tsize + 15) & ~(size_t)15) + (size_t)((m + 3) & ~(int64_t)3) * 4 +
         (size_t)P * 4;
}

namespace {

// pdl_cmpvec: -1, 0, 1 as the first differing component compares
template <class T> __device__ __forceinline__ int cmpvec(const T *a, const T *b, int64_t n) {
  for (int64_t k = 0; k < n; k++) {
    if (a[k] < b[k]) return -1;
    if (a[k] > b[k]) return 1;
  }
  return 0;
}

// The reference's vector quicksort on positions ix[a..b] of vectors xx
// (PDL_QSORTVEC with INDEXTERM ix[...]); the smaller range first through an
// explicit stack, the larger continued: the two ranges are disjoint, so the
// result is the recursion's.
template <class T, class I>
__device__ bool qs_vec(const T *xx, I *ix, int64_t n, int64_t a, int64_t b) {
  int64_t st[2 * QV_STACK];
  int sp = 0;
  for (;;) {
    while (a < b) {
      int64_t i = a, j = b, med = (i + j) / 2;
      do {
        while (cmpvec(xx + n * ix[i], xx + n * ix[med], n) < 0) {
          if (++i > b) return false;
        }
        while (cmpvec(xx + n * ix[j], xx + n * ix[med], n) > 0) {
          if (--j < a) return false;
        }
        if (i <= j) {
          const I t = ix[i];
          ix[i] = ix[j];
          ix[j] = t;
          if (med == i) med = j;
          else if (med == j) med = i;
          i++;
          j--;
        }
      } while (i <= j);
      int64_t la = a, lb = j, ra = i, rb = b;
      if (j - a > b - i) {
        la = i; lb = b; ra = a; rb = j;
      }
      if (ra < rb) {
        if (sp >= QV_STACK) return false;
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

template <class T> __device__ __forceinline__ bool has_nan(T v) {
  if constexpr (std::is_floating_point_v<T>) return v != v;
  else return false;
}

template <class T, bool BAD>
__device__ __forceinline__ bool vec_bad(const T *v, int64_t n, const Bad<T> &bv) {
  if constexpr (BAD) {
    for (int64_t k = 0; k < n; k++)
      if (bv.is(v[k])) return true;
  }
  return false;
}

// The outputs of one row from the vectors xx (n x m, vector-contiguous)
// and the order ix[0, m).
template <class T, bool IND, bool BAD, class I>
__device__ __forceinline__ void write_row(const VecSortArgs &g, const T *xx, const I *ix,
                                          const int64_t *offs, const Bad<T> &bv, T obad,
                                          int64_t t0, int64_t dt) {
  const int64_t N = g.n, M = g.m;
  if constexpr (IND) {
    int64_t *out = reinterpret_cast<int64_t *>(g.b) + offs[1];
    for (int64_t m = t0; m < M; m += dt) out[m * g.inc_bm] = (int64_t)ix[m];
  } else {
    T *out = reinterpret_cast<T *>(g.b) + offs[1];
    for (int64_t e = t0; e < N * M; e += dt) {
      const int64_t m = e / N, k = e - m * N;
      T v = xx[(int64_t)ix[m] * N + k];
      if (BAD && bv.is(v)) v = obad;
      out[k * g.inc_bn + m * g.inc_bm] = v;
    }
  }
}

// One block per broadcast row; dynamic shared memory: the vectors
// (m x n values), the compacted order ix[m] and the network's keys sx[P].
template <class T, bool IND, bool BAD>
__global__ void __launch_bounds__(QV_THREADS) k_qsortvec_block(const VecSortArgs g) {
  extern __shared__ __align__(16) unsigned char qv_smem[];
  const int64_t N = g.n, M = g.m;
  T *xx = reinterpret_cast<T *>(qv_smem);
  int32_t *ix = reinterpret_cast<int32_t *>(qv_smem + ((N * M * sizeof(T) + 15) & ~(int64_t)15));
  int32_t *sx = ix + ((M + 3) & ~(int64_t)3);
  __shared__ int s_cnt[QV_THREADS / 32], s_flag;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  const T obad = from_bits<T>(g.obad);
  for (int64_t row = blockIdx.x; row < g.rows; row += gridDim.x) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    for (int64_t e = tid; e < N * M; e += QV_THREADS) {
      const int64_t m = e / N, k = e - m * N;
      xx[e] = a[k * g.inc_an + m * g.inc_am];
    }
    if (tid == 0) s_flag = 0;
    __syncthreads();
    // compaction in order: good vectors from the front, vectors with a bad
    // component from the back (the first of them last)
    int nn = 0, nbad = 0;
    bool nan = false;
    for (int64_t base = 0; base < M; base += QV_THREADS) {
      const int64_t m = base + tid;
      bool good = false, bad = false;
      if (m < M) {
        const T *v = xx + m * N;
        bad = vec_bad<T, BAD>(v, N, bv);
        good = !bad;
        if (good)
          for (int64_t k = 0; k < N; k++) nan |= has_nan(v[k]);
      }
      const unsigned gm = __ballot_sync(0xffffffffu, good), bm = __ballot_sync(0xffffffffu, bad);
      if (lane == 0) s_cnt[w] = (__popc(gm) << 16) | __popc(bm);
      __syncthreads();
      int gb = 0, bb = 0, gt = 0, bt = 0;
      for (int k = 0; k < QV_THREADS / 32; k++) {
        const int c = s_cnt[k];
        if (k < w) {
          gb += c >> 16;
          bb += c & 0xFFFF;
        }
        gt += c >> 16;
        bt += c & 0xFFFF;
      }
      const unsigned lt = (1u << lane) - 1u;
      if (good) ix[nn + gb + __popc(gm & lt)] = (int32_t)m;
      if (bad) ix[M - 1 - (nbad + bb + __popc(bm & lt))] = (int32_t)m;
      nn += gt;
      nbad += bt;
      __syncthreads();
    }
    if (nan) s_flag = 1;
    __syncthreads();
    bool unsafe = s_flag != 0;
    if (!unsafe && nn > 1) {
      int p2 = 1;
      while (p2 < nn) p2 <<= 1;
      for (int i = tid; i < p2; i += QV_THREADS) sx[i] = i < nn ? ix[i] : -1;
      __syncthreads();
      for (int k = 2; k <= p2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int i = tid; i < p2; i += QV_THREADS) {
            const int l = i ^ j;
            if (l > i) {
              const int32_t pi = sx[i], pl = sx[l];
              bool greater;  // element i after element l
              if (pi < 0) greater = pl >= 0;
              else if (pl < 0) greater = false;
              else {
                const int c = cmpvec(xx + (int64_t)pi * N, xx + (int64_t)pl * N, N);
                greater = c > 0 || (c == 0 && pi > pl);
              }
              if (greater == ((i & k) == 0)) {
                sx[i] = pl;
                sx[l] = pi;
              }
            }
          }
          __syncthreads();
        }
      }
      bool tie = false;
      for (int i = tid; i + 1 < nn; i += QV_THREADS)
        tie |= cmpvec(xx + (int64_t)sx[i] * N, xx + (int64_t)sx[i + 1] * N, N) == 0;
      if (tie) s_flag = 1;
      __syncthreads();
      unsafe = s_flag != 0;
      if (!unsafe)
        for (int i = tid; i < nn; i += QV_THREADS) ix[i] = sx[i];
    }
    if (unsafe && nn > 1 && tid == 0) {
      if (!qs_vec<T, int32_t>(xx, ix, N, 0, nn - 1)) atomicOr(g.err, 1);
    }
    __syncthreads();
    write_row<T, IND, BAD, int32_t>(g, xx, ix, offs, bv, obad, tid, QV_THREADS);
    __syncthreads();
  }
}

// Rows beyond shared memory: one thread per row, the reference's steps over
// the row's vectors copied into device scratch.
template <class T, bool IND, bool BAD>
__global__ void __launch_bounds__(128) k_qsortvec_thread(const VecSortArgs g) {
  const int64_t N = g.n, M = g.m;
  const Bad<T> bv{from_bits<T>(g.abad), (bool)g.abad_isnan};
  const T obad = from_bits<T>(g.obad);
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < g.rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    T *xx = reinterpret_cast<T *>(g.scratch) + row * N * M;
    int64_t *ix = g.iscratch + row * M;
    int64_t nn = 0, nb = M - 1;
    for (int64_t m = 0; m < M; m++) {
      bool bad = false;
      for (int64_t k = 0; k < N; k++) {
        const T v = a[k * g.inc_an + m * g.inc_am];
        xx[m * N + k] = v;
        bad |= BAD && bv.is(v);
      }
      ix[bad ? nb-- : nn++] = m;
    }
    if (nn > 1 && !qs_vec<T, int64_t>(xx, ix, N, 0, nn - 1)) atomicOr(g.err, 1);
    write_row<T, IND, BAD, int64_t>(g, xx, ix, offs, bv, obad, 0, 1);
  }
}

template <class T, bool IND, bool BAD>
pdlgb300_error go(const VecSortArgs &g, size_t smem_limit, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const int nsm = pgh::num_sms();
  const size_t smem = qsortvec_smem_bytes(g.n, g.m, (int)sizeof(T));
  if (g.m < (1 << 30) && smem <= smem_limit) {
    auto kern = k_qsortvec_block<T, IND, BAD>;
    // (the kernel's own static shared words count against the default 48 KB too)
    if (smem + 1024 > 48 * 1024 &&
        !pgh::cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem), &e, "qsortvec smem"))
      return e;
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(g.rows, (int64_t)nsm * 8));
    kern<<<(int)grid, QV_THREADS, smem, s>>>(g);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_qsortvec_block")) return e;
    pgh::record_kernel("k_qsortvec_block", grid, QV_THREADS);
    return e;
  }
  if (!g.scratch) return pgh::err(PDLGB300_EFATAL, "qsortvec: no scratch for long rows");
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>((g.rows + 127) / 128, (int64_t)nsm * 16));
  k_qsortvec_thread<T, IND, BAD><<<(int)grid, 128, 0, s>>>(g);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_qsortvec_thread")) return e;
  pgh::record_kernel("k_qsortvec_thread", grid, 128);
  return e;
}

template <int DT>
pdlgb300_error typed(bool ind, const VecSortArgs &g, size_t smem_limit, cudaStream_t s) {
  using T = typename TT<DT>::T;
  if (ind) return g.bad ? go<T, true, true>(g, smem_limit, s) : go<T, true, false>(g, smem_limit, s);
  return g.bad ? go<T, false, true>(g, smem_limit, s) : go<T, false, false>(g, smem_limit, s);
}

}  // namespace

pdlgb300_error launch_qsortvec(bool ind, int dt, const VecSortArgs &g, size_t smem_limit,
                               cudaStream_t s) {
  PG_DISPATCH(dt, return typed<DT>(ind, g, smem_limit, s));
  return pgh::err(PDLGB300_EUSERERROR, "qsortvec: unsupported type %d", dt);
}

}  // namespace pg
