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
// every row start) or constant along it: the program runs a 16-byte vector
// at a time.  Each thread owns one column of shared memory slots (16 bytes
// each): a ring of EXPR_STAGES slots per contiguous leaf that cp.async
// fills ahead of use (EXPR_STAGES-1 vectors per leaf in flight), one slot
// per constant leaf (its value broadcast, written once per row) and one per
// node.  A node's operands are slot addresses (plain arithmetic on the
// operand index) and its op is dispatched once per vector, so the per-
// element work is the op itself.  In bad-value mode a 32-bit mask per slot
// holds the elements' bad flags.  Only the thread that wrote a slot reads
// it: no barriers; cp.async.wait_group orders each thread's own copies.
constexpr int EXPR_STAGES = 4;

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <class T, int VEC>
__device__ __forceinline__ void apply_vec(int op, const VecT<T, VEC> &x, const VecT<T, VEC> &y,
                                          VecT<T, VEC> &r) {
#define PG_EXPR_CASE(C)                                             \
  case C:                                                           \
    _Pragma("unroll") for (int e = 0; e < VEC; e++)                 \
        r.e[e] = biop_apply<T, C>(x.e[e], y.e[e]);                  \
    return;
  switch (op) {
    PG_EXPR_CASE(B_PLUS)
    PG_EXPR_CASE(B_MULT)
    PG_EXPR_CASE(B_MINUS)
    PG_EXPR_CASE(B_DIVIDE)
    PG_EXPR_CASE(B_GT)
    PG_EXPR_CASE(B_LT)
    PG_EXPR_CASE(B_LE)
    PG_EXPR_CASE(B_GE)
    PG_EXPR_CASE(B_EQ)
    PG_EXPR_CASE(B_NE)
    default: break;
  }
  if constexpr (std::is_integral_v<T>) {
    switch (op) {
      PG_EXPR_CASE(B_SHL)
      PG_EXPR_CASE(B_SHR)
      PG_EXPR_CASE(B_OR2)
      PG_EXPR_CASE(B_AND2)
      PG_EXPR_CASE(B_XOR)
      default: break;
    }
  }
#undef PG_EXPR_CASE
  r = x;  // not reached: the host validates the program
}

// Shared memory bytes of the vector kernel for a block of `block` threads.
inline int expr_vec_smem(int nleaf, int nnode, int block, bool bad) {
  const int slots = EXPR_STAGES * nleaf + nleaf + nnode;
  return slots * block * 16 + (bad ? (nleaf + nnode) * block * 4 : 0);
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
  const int nl = g.nleaf, nn = g.nnode, bd = blockDim.x;
  // this thread's column: slot i at col[i * bd]
  V *const col = reinterpret_cast<V *>(xs_raw) + threadIdx.x;
  V *const ring = col;                          // [stage][leaf]
  V *const cslot = col + P * nl * bd;           // [leaf]
  V *const nslot = cslot + nl * bd;             // [node]
  uint32_t *const mcol = reinterpret_cast<uint32_t *>(
      reinterpret_cast<V *>(xs_raw) + (P * nl + nl + nn) * bd) + threadIdx.x;  // [leaf], [node]
  const uint32_t ring_sh = (uint32_t)__cvta_generic_to_shared(ring);
  const Bad<T> tb{from_bits<T>(g.tbad), (bool)g.tbad_isnan};
  const int64_t nunits = g.rows * g.nsplit;
  for (int64_t u = (int64_t)blockIdx.x * gpb + gid; u < nunits; u += (int64_t)gridDim.x * gpb) {
    const int64_t row = u / g.nsplit;
    const int split = (int)(u - row * g.nsplit);
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *p[EXPR_MAXL];
#pragma unroll
    for (int l = 0; l < EXPR_MAXL; l++) {
      p[l] = reinterpret_cast<const T *>(g.leaf[l]) + (l < nl ? offs[l] : 0);
      if (l < nl && g.inc_n[l] == 0) {
        const T c = p[l][0];
        V cv;
#pragma unroll
        for (int e = 0; e < VEC; e++) cv.e[e] = c;
        cslot[l * bd] = cv;
        if constexpr (BAD) {
          const bool cb =
              g.lflag[l] && Bad<T>{from_bits<T>(g.lbad[l]), (bool)g.lbad_isnan[l]}.is(c);
          mcol[l * bd] = cb ? (1u << VEC) - 1 : 0u;
        }
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
    AC ac{Op::init(), 0}, ac2{Op::init(), 0};
    // lo is a multiple of 32 elements, so every vector below is aligned
    const int64_t nvec = (hi - lo) / VEC;
    auto issue = [&](int64_t q, int st) {
      if (q < nvec) {
#pragma unroll
        for (int l = 0; l < EXPR_MAXL; l++)
          if (l < nl && g.inc_n[l] != 0)
            cp_async16(ring_sh + (uint32_t)((st * nl + l) * bd) * 16u, p[l] + lo + q * VEC);
      }
      cp_commit();
    };
#pragma unroll
    for (int s = 0; s < P - 1; s++) issue(lane + s * (int64_t)G, s);
    int st = 0;
    for (int64_t q = lane; q < nvec; q += G) {
      cp_wait<P - 2>();  // this iteration's copies have landed
      V *const stage = ring + st * nl * bd;
      if constexpr (BAD) {
        for (int l = 0; l < nl; l++) {
          if (g.inc_n[l] == 0) continue;
          const V w = stage[l * bd];
          const Bad<T> lb{from_bits<T>(g.lbad[l]), (bool)g.lbad_isnan[l]};
          uint32_t m = 0;
#pragma unroll
          for (int e = 0; e < VEC; e++) m |= (g.lflag[l] && lb.is(w.e[e])) ? 1u << e : 0u;
          mcol[l * bd] = m;
        }
      }
      V last;
      uint32_t lastm = 0;
      // programs of one or two nodes without bad values: the node results
      // stay in registers (node 0's operands are leaves, node 1's leaves or
      // node 0)
      bool done = false;
      if constexpr (!BAD) {
        if (nn <= 2) {
          auto leaf_at = [&](int i) -> const V & {
            return g.inc_n[i] != 0 ? stage[i * bd] : cslot[i * bd];
          };
          const ExprNode n0 = g.node[0];
          apply_vec<T, VEC>(n0.op, leaf_at(n0.a), leaf_at(n0.b), last);
          if (nn == 2) {
            const ExprNode n1 = g.node[1];
            const V r0 = last;
            const V x = n1.a < EXPR_MAXL ? leaf_at(n1.a) : r0;
            const V y = n1.b < EXPR_MAXL ? leaf_at(n1.b) : r0;
            apply_vec<T, VEC>(n1.op, x, y, last);
          }
          done = true;
        }
      }
      for (int k = 0; k < nn && !done; k++) {
        const ExprNode nd = g.node[k];
        // operand i: leaf i (ring slot of this stage, or its constant
        // slot) or node i - EXPR_MAXL
        auto at = [&](int i) -> const V & {
          return i < EXPR_MAXL ? (g.inc_n[i] != 0 ? stage[i * bd] : cslot[i * bd])
                               : nslot[(i - EXPR_MAXL) * bd];
        };
        const V x = at(nd.a), y = at(nd.b);
        V r;
        apply_vec<T, VEC>(nd.op, x, y, r);
        if constexpr (BAD) {
          auto mk = [&](int i) -> uint32_t {
            return i < EXPR_MAXL ? mcol[i * bd] : mcol[(nl + i - EXPR_MAXL) * bd];
          };
          const uint32_t mb = mk(nd.a) | mk(nd.b);
          uint32_t mr = 0;
#pragma unroll
          for (int e = 0; e < VEC; e++) {
            if (mb >> e & 1u) r.e[e] = tb.val;
            mr |= (g.nflag[k] && tb.is(r.e[e])) ? 1u << e : 0u;
          }
          mcol[(nl + k) * bd] = mr;
          lastm = mr;
        }
        nslot[k * bd] = r;
        last = r;
      }
      // refill the slot read one iteration ago
      issue(q + (P - 1) * (int64_t)G, st == 0 ? P - 1 : st - 1);
      const int64_t t0 = lo + q * VEC;
#pragma unroll
      for (int e = 0; e < VEC; e++) {
        if (BAD && (lastm >> e & 1u)) continue;
        AC &a = (e & 1) ? ac2 : ac;
        Op::add(a.acc, last.e[e], t0 + e);
        a.cnt++;
      }
      st = st == P - 1 ? 0 : st + 1;
    }
    cp_wait<0>();
    // the ragged end: element by element through the register evaluator
    for (int64_t t = lo + nvec * VEC + lane; t < hi; t += G) {
      T leaf[EXPR_MAXL];
      bool lb[EXPR_MAXL];
#pragma unroll
      for (int l = 0; l < EXPR_MAXL; l++) {
        leaf[l] = (T)0;
        lb[l] = false;
        if (l < nl) {
          leaf[l] = g.inc_n[l] != 0 ? p[l][t] : p[l][0];
          if constexpr (BAD)
            lb[l] = g.lflag[l] && Bad<T>{from_bits<T>(g.lbad[l]), (bool)g.lbad_isnan[l]}.is(leaf[l]);
        }
      }
      T v;
      if (expr_eval<T, BAD>(g, leaf, lb, v)) {
        Op::add(ac.acc, v, t);
        ac.cnt++;
      }
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
    const int smem = expr_vec_smem(g.nleaf, g.nnode, block, g.bad);
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
