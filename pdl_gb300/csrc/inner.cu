// inner.cu -- PDL::Primitive inner (lib/PDL/Primitive.pd:48-76):
// c = sum_n a(n)*b(n).  The reference rounds each product in the generic
// type (C promotion for 8/16-bit ints, wrap for wider ints) and accumulates
// in complex long double.  Here: integer products accumulate exactly in
// 64/128-bit integers; float32 products (exact in double) accumulate in
// double; float64 products (__dmul_rn) accumulate in F64Sum blocks, which
// keeps the FP64 pipe for the products only.  Any bad pair makes c bad and
// sets the output's badflag (:56-59).
#include "args.cuh"
#include "f64sum.cuh"

namespace pg {
namespace {

template <class T> struct InnerAcc {
  using P = std::conditional_t<(sizeof(T) <= 2), int32_t, T>;  // product type
  using A = std::conditional_t<std::is_floating_point_v<T>,
                               std::conditional_t<std::is_same_v<T, float>, double, F64Sum>,
                               std::conditional_t<(sizeof(T) <= 4), int64_t, __int128>>;
  __device__ static A zero() {
    A a;
    memset(&a, 0, sizeof a);
    return a;
  }
  __device__ static P prod(T x, T y) {
    if constexpr (std::is_floating_point_v<T>) return rn_mul(x, y);
    else if constexpr (sizeof(T) <= 2) return wmul<int32_t>((int32_t)x, (int32_t)y);  // int promotion, wraps
    else return wmul<T>(x, y);
  }
  __device__ static void add(A &a, P p) {
    if constexpr (std::is_same_v<A, F64Sum>) a.add_fp64(p);
    else if constexpr (std::is_same_v<A, double>) a = __dadd_rn(a, (double)p);
    else a += (A)p;
  }
  template <int B> __device__ static void add_block(A &a, const P *p) {
    if constexpr (std::is_same_v<A, F64Sum>) a.template add_block<B>(p);
    else {
#pragma unroll
      for (int i = 0; i < B; i++) add(a, p[i]);
    }
  }
  __device__ static void merge(A &a, const A &b) {
    if constexpr (std::is_same_v<A, F64Sum>) a.merge(b);
    else if constexpr (std::is_same_v<A, double>) a = __dadd_rn(a, b);
    else a += b;
  }
  __device__ static T value(const A &a) {
    if constexpr (std::is_same_v<A, F64Sum>) return (T)a.value();
    else if constexpr (std::is_same_v<A, double>) return (T)a;
    else return (T)a;
  }
};

template <class T> struct alignas(16) V16 {
  T e[16 / sizeof(T)];
};

// The products of a block; float64 ones alternate between the FP64 pipe and
// the integer pipe (dmul_rn_split), which together keep up with HBM.
template <class T, class IA, int U, int VEC, int... J>
__device__ __forceinline__ void block_products(const V16<T> (&xa)[U], const V16<T> (&xb)[U],
                                               typename IA::P *p,
                                               std::integer_sequence<int, J...>) {
  if constexpr (std::is_same_v<T, double>)
    ((p[J] = dmul_rn_split<J>(xa[J / VEC].e[J % VEC], xb[J / VEC].e[J % VEC])), ...);
  else
    ((p[J] = IA::prod(xa[J / VEC].e[J % VEC], xb[J / VEC].e[J % VEC])), ...);
}

// Each thread streams its own 16-byte vectors of a and b through a ring of
// INNER_ST stages in shared memory (cp.async), INNER_U vectors of each per
// stage: two stages stay in flight while the third is multiplied and
// summed, without holding registers (the float64 products need them).  The
// order of the products and sums is that of plain loads.
constexpr int INNER_ST = 3, INNER_U = 4;
constexpr int INNER_SLOT_B = INNER_ST * INNER_U * 2 * 16;  // ring bytes per thread

template <class T, bool BAD>
__global__ void __launch_bounds__(256) k_inner_rows(const InnerArgs g) {
  using IA = InnerAcc<T>;
  using A = typename IA::A;
  using P = typename IA::P;
  constexpr int VEC = 16 / sizeof(T);
  constexpr int U = INNER_U;
  Bad<T> ba{from_bits<T>(g.abad), (bool)g.abad_isnan};
  Bad<T> bb{from_bits<T>(g.bbad), (bool)g.bbad_isnan};
  const T cbad = from_bits<T>(g.cbad);
  const int G = g.group;
  const int lane = G <= 32 ? (threadIdx.x & 31) : threadIdx.x;
  const int gpb = G <= 32 ? (blockDim.x >> 5) : 1;
  const int gid = G <= 32 ? (threadIdx.x >> 5) : 0;
  __shared__ A s_acc[32];
  __shared__ int s_bad[32];
  extern __shared__ __align__(16) unsigned char inner_ring[];
  // this thread's slots: [stage][operand][u], 16 bytes each, blockDim apart
  const uint32_t ring0 = (uint32_t)__cvta_generic_to_shared(inner_ring) + threadIdx.x * 16u;
  auto slot = [&](int st, int op, int u) {
    return ring0 + (uint32_t)(((st * 2 + op) * U + u) * blockDim.x) * 16u;
  };
  for (int64_t row = (int64_t)blockIdx.x * gpb + gid; row < g.rows;
       row += (int64_t)gridDim.x * gpb) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    const T *b = reinterpret_cast<const T *>(g.b) + offs[1];
    A acc = IA::zero();
    int anybad = 0;
    bool vec = g.inc_a == 1 && g.inc_b == 1 && ((uintptr_t)a % 16 == 0) &&
               ((uintptr_t)b % 16 == 0);
    int64_t nv = vec ? g.n / VEC : 0;
    const V16<T> *av = reinterpret_cast<const V16<T> *>(a);
    const V16<T> *bv = reinterpret_cast<const V16<T> *>(b);
    const int64_t step = (int64_t)G * U;
    auto issue = [&](int64_t k, int st) {
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int64_t kk = k + (int64_t)u * G;
        if (kk < nv) {
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(slot(st, 0, u)),
                       "l"(av + kk)
                       : "memory");
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(slot(st, 1, u)),
                       "l"(bv + kk)
                       : "memory");
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
#pragma unroll
    for (int st = 0; st < INNER_ST - 1; st++) issue(lane + st * step, st);
    int st = 0;
    for (int64_t k = lane; k < nv; k += step) {
      asm volatile("cp.async.wait_group %0;" ::"n"(INNER_ST - 2) : "memory");
      V16<T> xa[U], xb[U];
      const bool full = k + (int64_t)(U - 1) * G < nv;
#pragma unroll
      for (int u = 0; u < U; u++) {
        float4 fa, fb;
        asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];"
                     : "=f"(fa.x), "=f"(fa.y), "=f"(fa.z), "=f"(fa.w)
                     : "r"(slot(st, 0, u)));
        asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];"
                     : "=f"(fb.x), "=f"(fb.y), "=f"(fb.z), "=f"(fb.w)
                     : "r"(slot(st, 1, u)));
        memcpy(&xa[u], &fa, 16);
        memcpy(&xb[u], &fb, 16);
      }
      // the stage read one iteration ago takes the next copies
      issue(k + (INNER_ST - 1) * step, st == 0 ? INNER_ST - 1 : st - 1);
      if (full && !BAD) {
        P p[U * VEC];
        block_products<T, IA, U, VEC>(xa, xb, p, std::make_integer_sequence<int, U * VEC>{});
        IA::template add_block<U * VEC>(acc, p);
      } else {
#pragma unroll
        for (int u = 0; u < U; u++) {
          int64_t kk = k + (int64_t)u * G;
          if (full || kk < nv) {
#pragma unroll
            for (int e = 0; e < VEC; e++) {
              T x = xa[u].e[e], y = xb[u].e[e];
              if (BAD && (ba.is(x) || bb.is(y))) anybad = 1;
              else IA::add(acc, IA::prod(x, y));
            }
          }
        }
      }
      st = st == INNER_ST - 1 ? 0 : st + 1;
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    for (int64_t t = nv * VEC + lane; t < g.n; t += G) {
      T x = a[t * g.inc_a], y = b[t * g.inc_b];
      if (BAD && (ba.is(x) || bb.is(y))) anybad = 1;
      else IA::add(acc, IA::prod(x, y));
    }
    // group reduction
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      A o = shfl_down_any(acc, d);
      IA::merge(acc, o);
      anybad |= __shfl_down_sync(0xffffffffu, anybad, d);
    }
    if (G > 32) {
      int w = threadIdx.x >> 5, l = threadIdx.x & 31;
      __syncthreads();
      if (l == 0) { s_acc[w] = acc; s_bad[w] = anybad; }
      __syncthreads();
      if (w == 0) {
        int nw = blockDim.x >> 5;
        acc = l < nw ? s_acc[l] : IA::zero();
        anybad = l < nw ? s_bad[l] : 0;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
          A o = shfl_down_any(acc, d);
          IA::merge(acc, o);
          anybad |= __shfl_down_sync(0xffffffffu, anybad, d);
        }
      }
    }
    if (lane == 0) {
      T *c = reinterpret_cast<T *>(g.c) + offs[2];
      if (BAD && anybad) {
        *c = cbad;
        *g.setbad = 1;
      } else {
        *c = IA::value(acc);
      }
    }
  }
}

template <class T, bool BAD>
__global__ void k_inner_thread(const InnerArgs g) {
  using IA = InnerAcc<T>;
  Bad<T> ba{from_bits<T>(g.abad), (bool)g.abad_isnan};
  Bad<T> bb{from_bits<T>(g.bbad), (bool)g.bbad_isnan};
  const T cbad = from_bits<T>(g.cbad);
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < g.rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    const T *b = reinterpret_cast<const T *>(g.b) + offs[1];
    auto acc = IA::zero();
    bool bad = false;
    for (int64_t i = 0; i < g.n; i++) {
      T x = a[i * g.inc_a], y = b[i * g.inc_b];
      if (BAD && (ba.is(x) || bb.is(y))) { bad = true; break; }
      IA::add(acc, IA::prod(x, y));
    }
    T *c = reinterpret_cast<T *>(g.c) + offs[2];
    if (bad) { *c = cbad; *g.setbad = 1; }
    else *c = IA::value(acc);
  }
}

template <class T>
pdlgb300_error inner_typed(const InnerArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.rows == 0) return e;
  const int nsm = pgh::num_sms();
  if (g.group == 0) {
    int64_t grid = std::min<int64_t>((g.rows + 127) / 128, (int64_t)nsm * 32);
    if (g.bad) k_inner_thread<T, true><<<(int)grid, 128, 0, s>>>(g);
    else k_inner_thread<T, false><<<(int)grid, 128, 0, s>>>(g);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_inner_thread")) return e;
    pgh::record_kernel("k_inner_thread", grid, 128);
    return e;
  }
  // a warp per row: blocks of 4 warps, so that four blocks' rings (48 KiB
  // each) and registers fit on an SM
  int block = g.group <= 32 ? 128 : g.group;
  int gpb = g.group <= 32 ? block / 32 : 1;
  int64_t grid = std::min<int64_t>((g.rows + gpb - 1) / gpb, (int64_t)1 << 30);
  const size_t smem = (size_t)block * INNER_SLOT_B;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_inner_rows<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         256 * INNER_SLOT_B);
    cudaFuncSetAttribute(k_inner_rows<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         256 * INNER_SLOT_B);
    attr = true;
  }
  if (g.bad) k_inner_rows<T, true><<<(int)grid, block, smem, s>>>(g);
  else k_inner_rows<T, false><<<(int)grid, block, smem, s>>>(g);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_inner_rows")) return e;
  pgh::record_kernel("k_inner_rows", grid, block);
  return e;
}

}  // namespace

pdlgb300_error launch_inner(int dt, const InnerArgs &g, cudaStream_t s) {
  PG_DISPATCH(dt, return inner_typed<typename TT<DT>::T>(g, s));
  return pgh::err(PDLGB300_EUSERERROR, "inner: unsupported type %d", dt);
}

}  // namespace pg
