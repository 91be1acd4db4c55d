// expr.cuh -- a deferred elementwise expression of PDL::Ops binary ops
// (lib/PDL/Ops.pd:104-153, 288-307) over up to four broadcast leaves,
// reduced over dim 0 by one of the PDL::Ufunc reductions
// (lib/PDL/Ufunc.pd:94-187, 413-500) in one pass: the intermediates are
// never written to memory.
//
// Every element of every intermediate is computed as the unfused ops
// compute it: all leaves and intermediates have one type T (the host fuses
// nothing else), each op rounds or wraps in T, and the bad-value rule of
// each op is applied in turn -- an operand is bad when its ndarray has the
// bad flag and its value equals its badvalue; a node's bad flag is the OR
// of its operands' flags and its badvalue is T's default, exactly as a
// materialised intermediate would have them.
//
// The program is uniform across the launch, so the per-node switches and
// operand selections are uniform branches and selects on registers.  One
// group of threads per output row (a warp for rows up to 32 KiB of T, a
// block otherwise); few long rows split over several blocks whose partial
// accumulators the row reduction's combine kernel merges.
#pragma once
#include "biop.cuh"
#include "reduce.cuh"

namespace pg {
namespace {

constexpr int NV = EXPR_MAXL + EXPR_MAXN;

// v[i] for a runtime i below `lim` (a chain of selects on registers).
template <class T, int LIM>
__device__ __forceinline__ T pick(const T (&v)[NV], int i) {
  T r = v[0];
#pragma unroll
  for (int c = 1; c < LIM; c++)
    if (i == c) r = v[c];
  return r;
}
template <int LIM>
__device__ __forceinline__ bool pickb(const bool (&v)[NV], int i) {
  bool r = v[0];
#pragma unroll
  for (int c = 1; c < LIM; c++)
    if (i == c) r = v[c];
  return r;
}

template <class T>
__device__ __forceinline__ T apply_code(int op, T a, T b) {
  switch (op) {
    case B_PLUS: return biop_apply<T, B_PLUS>(a, b);
    case B_MULT: return biop_apply<T, B_MULT>(a, b);
    case B_MINUS: return biop_apply<T, B_MINUS>(a, b);
    case B_DIVIDE: return biop_apply<T, B_DIVIDE>(a, b);
    case B_GT: return biop_apply<T, B_GT>(a, b);
    case B_LT: return biop_apply<T, B_LT>(a, b);
    case B_LE: return biop_apply<T, B_LE>(a, b);
    case B_GE: return biop_apply<T, B_GE>(a, b);
    case B_EQ: return biop_apply<T, B_EQ>(a, b);
    case B_NE: return biop_apply<T, B_NE>(a, b);
    default: break;
  }
  if constexpr (std::is_integral_v<T>) {
    switch (op) {
      case B_SHL: return biop_apply<T, B_SHL>(a, b);
      case B_SHR: return biop_apply<T, B_SHR>(a, b);
      case B_OR2: return biop_apply<T, B_OR2>(a, b);
      case B_AND2: return biop_apply<T, B_AND2>(a, b);
      case B_XOR: return biop_apply<T, B_XOR>(a, b);
      default: break;
    }
  }
  return a;  // not reached: the host validates the program
}

// Node K and the nodes after it (K is a template argument so that the
// operand selections stay on registers).
template <class T, bool BAD, int K>
__device__ __forceinline__ void node_step(const ExprArgs &g, T (&v)[NV], bool (&b)[NV],
                                          const Bad<T> &tb, T &last, bool &lastbad) {
  if constexpr (K < EXPR_MAXN) {
    if (K >= g.nnode) return;
    const ExprNode nd = g.node[K];
    const T x = pick<T, EXPR_MAXL + K>(v, nd.a), y = pick<T, EXPR_MAXL + K>(v, nd.b);
    T r;
    if constexpr (BAD) {
      const bool bx = pickb<EXPR_MAXL + K>(b, nd.a), by = pickb<EXPR_MAXL + K>(b, nd.b);
      r = (bx || by) ? tb.val : apply_code<T>(nd.op, x, y);
      lastbad = b[EXPR_MAXL + K] = g.nflag[K] && tb.is(r);
    } else {
      r = apply_code<T>(nd.op, x, y);
    }
    last = v[EXPR_MAXL + K] = r;
    node_step<T, BAD, K + 1>(g, v, b, tb, last, lastbad);
  }
}

// Element t of the expression; returns false when it is bad.  Node slots
// are written before any later node can select them, so they need no
// initial value; the last node evaluated is the result.
template <class T, bool BAD>
__device__ __forceinline__ bool expr_eval(const ExprArgs &g, const T (&leaf)[EXPR_MAXL],
                                          const bool (&leafbad)[EXPR_MAXL], T &out) {
  T v[NV];
  bool b[NV];
#pragma unroll
  for (int l = 0; l < EXPR_MAXL; l++) {
    v[l] = leaf[l];
    b[l] = BAD && leafbad[l];
  }
  const Bad<T> tb{from_bits<T>(g.tbad), (bool)g.tbad_isnan};
  bool lastbad = false;
  node_step<T, BAD, 0>(g, v, b, tb, out, lastbad);
  return !(BAD && lastbad);
}

template <class T, bool BAD>
__device__ __forceinline__ void load_leaves(const ExprArgs &g, const T *const (&p)[EXPR_MAXL],
                                            int64_t t, T (&leaf)[EXPR_MAXL],
                                            bool (&leafbad)[EXPR_MAXL]) {
#pragma unroll
  for (int l = 0; l < EXPR_MAXL; l++) {
    leaf[l] = (T)0;
    leafbad[l] = false;
    if (l < g.nleaf) {
      leaf[l] = p[l][t * g.inc_n[l]];
      if constexpr (BAD)
        leafbad[l] = g.lflag[l] && Bad<T>{from_bits<T>(g.lbad[l]), (bool)g.lbad_isnan[l]}.is(leaf[l]);
    }
  }
}

template <class Op, class T, class Out, bool BAD>
__global__ void __launch_bounds__(256) k_expr_rows(const ExprArgs g) {
  using Acc = typename Op::Acc;
  using AC = AccCnt<Acc>;
  const int G = g.group;
  const int lane = G <= 32 ? (threadIdx.x & 31) : threadIdx.x;
  const int gpb = G <= 32 ? (blockDim.x >> 5) : 1;
  const int gid = G <= 32 ? (threadIdx.x >> 5) : 0;
  const Out obad = from_bits<Out>(g.obad);
  const int64_t nunits = g.rows * g.nsplit;
  for (int64_t u = (int64_t)blockIdx.x * gpb + gid; u < nunits; u += (int64_t)gridDim.x * gpb) {
    const int64_t row = u / g.nsplit;
    const int split = (int)(u - row * g.nsplit);
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *p[EXPR_MAXL];
#pragma unroll
    for (int l = 0; l < EXPR_MAXL; l++)
      p[l] = reinterpret_cast<const T *>(g.leaf[l]) + (l < g.nleaf ? offs[l] : 0);
    int64_t lo = 0, hi = g.n;
    if (g.nsplit > 1) {
      int64_t chunk = (g.n + g.nsplit - 1) / g.nsplit;
      chunk = (chunk + 31) & ~(int64_t)31;
      lo = split * chunk;
      hi = lo + chunk < g.n ? lo + chunk : g.n;
      if (lo > hi) lo = hi;
    }
    AC ac{Op::init(), 0};
    for (int64_t t = lo + lane; t < hi; t += G) {
      T leaf[EXPR_MAXL];
      bool lb[EXPR_MAXL];
      load_leaves<T, BAD>(g, p, t, leaf, lb);
      T v;
      if (expr_eval<T, BAD>(g, leaf, lb, v)) {
        Op::add(ac.acc, v, t);
        ac.cnt++;
      }
    }
    ac = group_reduce<Op>(ac, G);
    if (lane == 0) {
      if (g.nsplit > 1) {
        reinterpret_cast<Acc *>(g.partials)[u] = ac.acc;
        g.pcounts[u] = ac.cnt;
      } else {
        Out r = Op::fin(ac.acc, ac.cnt, BAD, obad, g.setbad);
        *(reinterpret_cast<Out *>(g.out) + offs[EXPR_MAXL]) = r;
      }
    }
  }
}

// Rows whose leaves are each contiguous along dim 0 (16-byte aligned at
// every row start) or constant along it.  Each thread streams its own
// 16-byte vectors of the contiguous leaves through a private ring of
// EXPR_STAGES slots in shared memory with cp.async (EXPR_STAGES-1 vectors
// per leaf in flight per thread, no registers held for them); the constant
// leaves are read once per row.  Only the thread that copied a slot reads
// it, so the ring needs no barrier: cp.async.wait_group orders each
// thread's own copies.
constexpr int EXPR_STAGES = 4;

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <class Op, class T, class Out, bool BAD>
__global__ void __launch_bounds__(256, 3) k_expr_rows_vec(const ExprArgs g) {
  using Acc = typename Op::Acc;
  using AC = AccCnt<Acc>;
  constexpr int VEC = 16 / sizeof(T);
  constexpr int P = EXPR_STAGES;
  using V = VecT<T, VEC>;
  extern __shared__ __align__(16) unsigned char xs_raw[];
  const int G = g.group;
  const int lane = G <= 32 ? (threadIdx.x & 31) : threadIdx.x;
  const int gpb = G <= 32 ? (blockDim.x >> 5) : 1;
  const int gid = G <= 32 ? (threadIdx.x >> 5) : 0;
  const Out obad = from_bits<Out>(g.obad);
  const int nl = g.nleaf;
  // slot (stage, leaf) of this thread: [stage][leaf][thread], 16 bytes each
  const uint32_t ring = (uint32_t)__cvta_generic_to_shared(xs_raw) + threadIdx.x * 16u;
  const uint32_t sstride = blockDim.x * 16u;
  const V *ringp = reinterpret_cast<const V *>(xs_raw) + threadIdx.x;
  const int64_t nunits = g.rows * g.nsplit;
  for (int64_t u = (int64_t)blockIdx.x * gpb + gid; u < nunits; u += (int64_t)gridDim.x * gpb) {
    const int64_t row = u / g.nsplit;
    const int split = (int)(u - row * g.nsplit);
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *p[EXPR_MAXL];
    T cst[EXPR_MAXL];
    bool cbad[EXPR_MAXL];
#pragma unroll
    for (int l = 0; l < EXPR_MAXL; l++) {
      p[l] = reinterpret_cast<const T *>(g.leaf[l]) + (l < nl ? offs[l] : 0);
      cst[l] = (T)0;
      cbad[l] = false;
      if (l < nl && g.inc_n[l] == 0) {
        cst[l] = p[l][0];
        if constexpr (BAD)
          cbad[l] = g.lflag[l] && Bad<T>{from_bits<T>(g.lbad[l]), (bool)g.lbad_isnan[l]}.is(cst[l]);
      }
    }
    int64_t lo = 0, hi = g.n;
    if (g.nsplit > 1) {
      int64_t chunk = (g.n + g.nsplit - 1) / g.nsplit;
      chunk = (chunk + 31) & ~(int64_t)31;
      lo = split * chunk;
      hi = lo + chunk < g.n ? lo + chunk : g.n;
      if (lo > hi) lo = hi;
    }
    // two accumulators (even and odd elements of a vector): two independent
    // dependency chains per thread
    AC ac{Op::init(), 0}, ac2{Op::init(), 0};
    auto one = [&](const T (&leaf)[EXPR_MAXL], int64_t t, AC &a) {
      bool lb[EXPR_MAXL];
#pragma unroll
      for (int l = 0; l < EXPR_MAXL; l++) {
        lb[l] = false;
        if constexpr (BAD) {
          if (l < nl)
            lb[l] = g.inc_n[l] == 0 ? cbad[l]
                                    : g.lflag[l] && Bad<T>{from_bits<T>(g.lbad[l]),
                                                           (bool)g.lbad_isnan[l]}.is(leaf[l]);
        }
      }
      T v;
      if (expr_eval<T, BAD>(g, leaf, lb, v)) {
        Op::add(a.acc, v, t);
        a.cnt++;
      }
    };
    // lo is a multiple of 32 elements, so every vector below is aligned
    const int64_t nvec = (hi - lo) / VEC;
    auto issue = [&](int64_t q, int st) {
      if (q < nvec) {
#pragma unroll
        for (int l = 0; l < EXPR_MAXL; l++)
          if (l < nl && g.inc_n[l] != 0)
            cp_async16(ring + (uint32_t)(st * nl + l) * sstride, p[l] + lo + q * VEC);
      }
      cp_commit();
    };
#pragma unroll
    for (int s = 0; s < P - 1; s++) issue(lane + s * (int64_t)G, s);
    int st = 0;
    for (int64_t q = lane; q < nvec; q += G) {
      cp_wait<P - 2>();  // this iteration's copies have landed
      V w[EXPR_MAXL];
#pragma unroll
      for (int l = 0; l < EXPR_MAXL; l++)
        if (l < nl && g.inc_n[l] != 0) w[l] = ringp[(st * nl + l) * (int)blockDim.x];
      // refill the slot read one iteration ago
      issue(q + (P - 1) * (int64_t)G, st == 0 ? P - 1 : st - 1);
#pragma unroll
      for (int e = 0; e < VEC; e++) {
        T leaf[EXPR_MAXL];
#pragma unroll
        for (int l = 0; l < EXPR_MAXL; l++) leaf[l] = g.inc_n[l] != 0 ? w[l].e[e] : cst[l];
        one(leaf, lo + q * VEC + e, (e & 1) ? ac2 : ac);
      }
      st = st == P - 1 ? 0 : st + 1;
    }
    cp_wait<0>();
    for (int64_t t = lo + nvec * VEC + lane; t < hi; t += G) {
      T leaf[EXPR_MAXL];
#pragma unroll
      for (int l = 0; l < EXPR_MAXL; l++) leaf[l] = g.inc_n[l] != 0 ? p[l][t] : cst[l];
      one(leaf, t, ac);
    }
    merge_ac<Op>(ac, ac2);
    ac = group_reduce<Op>(ac, G);
    if (lane == 0) {
      if (g.nsplit > 1) {
        reinterpret_cast<Acc *>(g.partials)[u] = ac.acc;
        g.pcounts[u] = ac.cnt;
      } else {
        Out r = Op::fin(ac.acc, ac.cnt, BAD, obad, g.setbad);
        *(reinterpret_cast<Out *>(g.out) + offs[EXPR_MAXL]) = r;
      }
    }
  }
}

template <class Op, class T, class Out, bool VL>
pdlgb300_error go(const ExprArgs &g, const RedArgs &ra, int grid, int block, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const char *nm = VL ? "k_expr_rows_vec" : "k_expr_rows";
  if constexpr (VL) {
    const int smem = EXPR_STAGES * g.nleaf * block * 16;
    auto k = g.bad ? k_expr_rows_vec<Op, T, Out, true> : k_expr_rows_vec<Op, T, Out, false>;
    // the default limit (48 KiB) includes the static shared memory
    if (smem > 32 * 1024 &&
        !pgh::cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                         &e, nm))
      return e;
    k<<<grid, block, smem, s>>>(g);
  } else {
    if (g.bad) k_expr_rows<Op, T, Out, true><<<grid, block, 0, s>>>(g);
    else k_expr_rows<Op, T, Out, false><<<grid, block, 0, s>>>(g);
  }
  if (!pgh::cuda_check(cudaGetLastError(), &e, nm)) return e;
  pgh::record_kernel(nm, grid, block);
  if (g.nsplit > 1) {
    const int gc = (int)std::min<int64_t>((g.rows + 3) / 4, 65535);
    if (g.bad) k_red_combine<Op, T, Out, true><<<gc, 128, 0, s>>>(ra);
    else k_red_combine<Op, T, Out, false><<<gc, 128, 0, s>>>(ra);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_red_combine")) return e;
    pgh::record_kernel("k_red_combine", gc, 128);
  }
  return e;
}

template <int DT, bool VL>
pdlgb300_error expr_family(int op, const ExprArgs &g, const RedArgs &ra, int grid, int block,
                           cudaStream_t s) {
  using T = typename TT<DT>::T;
  using OutP = typename TT<intplus(DT)>::T;
  constexpr bool F32 = std::is_same_v<OutP, float>;
  constexpr bool INT = std::is_integral_v<T>;
  switch (op) {
    case R_SUM:
      if constexpr (F32)
        if (g.f32_comp) return go<OpSum<T, OutP, true>, T, OutP, VL>(g, ra, grid, block, s);
      return go<OpSum<T, OutP, false>, T, OutP, VL>(g, ra, grid, block, s);
    case R_DSUM: return go<OpSum<T, double, false>, T, double, VL>(g, ra, grid, block, s);
    case R_AVG:
      if constexpr (F32)
        if (g.f32_comp) return go<OpAvg<T, OutP, true>, T, OutP, VL>(g, ra, grid, block, s);
      return go<OpAvg<T, OutP, false>, T, OutP, VL>(g, ra, grid, block, s);
    case R_DAVG: return go<OpAvg<T, double, false>, T, double, VL>(g, ra, grid, block, s);
    case R_PROD:
      if constexpr (INT) return go<OpProd<T, OutP>, T, OutP, VL>(g, ra, grid, block, s);
      break;
    case R_MIN: return go<OpMM<T, false, false>, T, T, VL>(g, ra, grid, block, s);
    case R_MAX: return go<OpMM<T, true, false>, T, T, VL>(g, ra, grid, block, s);
    case R_MIN_IND: return go<OpMM<T, false, true>, T, int64_t, VL>(g, ra, grid, block, s);
    case R_MAX_IND: return go<OpMM<T, true, true>, T, int64_t, VL>(g, ra, grid, block, s);
    case R_AND: return go<OpLogic<T, 0>, T, T, VL>(g, ra, grid, block, s);
    case R_OR: return go<OpLogic<T, 1>, T, T, VL>(g, ra, grid, block, s);
    case R_XOR: return go<OpLogic<T, 2>, T, T, VL>(g, ra, grid, block, s);
    case R_ZC: return go<OpLogic<T, 3>, T, T, VL>(g, ra, grid, block, s);
    case R_BAND:
      if constexpr (INT) return go<OpLogic<T, 4>, T, T, VL>(g, ra, grid, block, s);
      break;
    case R_BOR:
      if constexpr (INT) return go<OpLogic<T, 5>, T, T, VL>(g, ra, grid, block, s);
      break;
    case R_BXOR:
      if constexpr (INT) return go<OpLogic<T, 6>, T, T, VL>(g, ra, grid, block, s);
      break;
    default: break;
  }
  return pgh::err(PDLGB300_EUSERERROR, "expression reduction %d: not fusable for type %d", op, DT);
}

}  // namespace

// One instantiation per type and kernel variant, each in its own
// translation unit (expr_<type>[v].cu), so that they compile in parallel.
template <int DT, bool VL>
pdlgb300_error launch_expr_typed(int op, const ExprArgs &g, const RedArgs &ra, int grid, int block,
                                 cudaStream_t s) {
  return expr_family<DT, VL>(op, g, ra, grid, block, s);
}

}  // namespace pg
