// reduce.cuh -- the PDL::Ufunc reductions over dim 0 (a(n) -> b()) as
// GB300 kernels.  Semantics per op follow lib/PDL/Ufunc.pd:
//   sumover/dsumover :94-118, prodover/dprodover :91-118 (leftzero),
//   average/daverage :413-444, minimum/maximum :446-475,
//   minimum_ind/maximum_ind :477-500.
// Rows (one output each) are the collapsed broadcast dims; the reduced dim
// n is walked by a group of threads (contiguous n: 16-byte vector loads) or
// by one thread (strided n, the reference's own sequential order).
#pragma once
#include "args.cuh"
#include "f64sum.cuh"

namespace pg {


// ---------------------------------------------------------------- accums

// Float-float (compensated) float32 accumulator: TwoSum per element.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ void ff_add(FF &a, float x) {
  float s = __fadd_rn(a.hi, x);
  float bp = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, e);
}
__device__ __forceinline__ void ff_merge(FF &a, const FF &b) {
  float s = __fadd_rn(a.hi, b.hi);
  float bp = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  float h = __fadd_rn(s, e);
  a.lo = __fsub_rn(e, __fsub_rn(h, s));
  a.hi = h;
}

// Sum of In into Out.  Integers wrap in Out's width (order-free, so exact);
// float32 is compensated or plain; float64 uses F64Sum (exact-within-block
// integer alignment plus FP64 adds, no less accurate than FP64).
template <class In, class Out, bool COMP> struct SumAcc {
  using Acc = std::conditional_t<
      std::is_integral_v<Out>, uns_t<Out>,
      std::conditional_t<std::is_same_v<Out, float>,
                         std::conditional_t<COMP, FF, float>,
                         std::conditional_t<std::is_same_v<In, double>, F64Sum, double>>>;
  __device__ static Acc init() {
    Acc a;
    memset(&a, 0, sizeof a);
    return a;
  }
  __device__ static void add(Acc &a, In v) {
    if constexpr (std::is_integral_v<Out>) {
      a += (Acc)(Out)v;
    } else if constexpr (std::is_same_v<Acc, FF>) {
      ff_add(a, (float)v);
    } else if constexpr (std::is_same_v<Acc, F64Sum>) {
      a.add_fp64(v);
    } else {
      a = rn_add(a, (Acc)v);
    }
  }
  __device__ static void merge(Acc &a, const Acc &b) {
    if constexpr (std::is_integral_v<Out>) a += b;
    else if constexpr (std::is_same_v<Acc, FF>) ff_merge(a, b);
    else if constexpr (std::is_same_v<Acc, F64Sum>) a.merge(b);
    else a = rn_add(a, b);
  }
  __device__ static Out value(const Acc &a) {
    if constexpr (std::is_integral_v<Out>) return (Out)a;
    else if constexpr (std::is_same_v<Acc, FF>) return __fadd_rn(a.hi, a.lo);
    else if constexpr (std::is_same_v<Acc, F64Sum>) return a.value();
    else return (Out)a;
  }
};

// --------------------------------------------------------------------- ops
// Each op: Acc, init, add(acc, v, idx), merge(a, b) (a holds lower indices),
// finalize(acc, cnt, bad, badval, &setbad) -> Out, kCount (needs good count).

template <class In, class Out, bool COMP> struct OpSum {
  using S = SumAcc<In, Out, COMP>;
  using Acc = typename S::Acc;
  static constexpr bool kZero = false, kLeftZero = false;
  static constexpr bool kCount = false, kVec = true, kNeutral = true;
  __device__ static In neutral() { return (In)0; }
  static constexpr bool kBlock = std::is_same_v<Acc, F64Sum>;
  static constexpr int kU = kBlock ? 8 : 0;
  template <int VEC, int U>
  __device__ static void add_block(Acc &a, const In *v, int64_t, int64_t) {
    if constexpr (kBlock) a.template add_block<VEC * U>(v);
  }
  __device__ static Acc init() { return S::init(); }
  __device__ static void add(Acc &a, In v, int64_t) { S::add(a, v); }
  template <int VEC> __device__ static void add_vec(Acc &a, const In *v, int64_t) {
    if constexpr (std::is_same_v<Acc, F64Sum> && VEC == 2) a.add_block2(v);
    else {
#pragma unroll
      for (int e = 0; e < VEC; e++) S::add(a, v[e]);
    }
  }
  __device__ static void merge(Acc &a, const Acc &b) { S::merge(a, b); }
  __device__ static Out fin(const Acc &a, int64_t cnt, bool bad, Out badval, int *) {
    if (bad && cnt == 0) return badval;
    return S::value(a);
  }
};

// x == 0 on the integer pipe (the float64 compare would use the FP64 pipe)
template <class T> __device__ __forceinline__ bool is_zero_bits(T x) {
  if constexpr (sizeof(T) == 8) return zero_bits64((uint64_t)__double_as_longlong((double)x));
  else return ((uint32_t)__float_as_uint((float)x) << 1) == 0;
}

// Products.  The reference stops at the first element that makes the
// running product zero (Ufunc.pd:107, `if (tmp == 0) break`).  Integer
// products are unchanged by that (0 times anything wraps to 0); floating
// ones would differ where inf or NaN follow a zero, so their accumulator
// also carries the index of the first good exact zero, and rows that have
// one are recomputed over [0, z] (k_prod_fix).  The sequential thread kernel
// breaks exactly as the reference does.
template <class Out> struct ProdZ {
  Out p;
  int64_t z;  // first good element equal to 0, or INT64_MAX
};
template <class In, class Out> struct OpProd {
  static constexpr bool kZero = std::is_floating_point_v<Out>;
  using Acc = std::conditional_t<std::is_integral_v<Out>, uns_t<Out>, ProdZ<Out>>;
  static constexpr bool kCount = false, kVec = true, kBlock = false, kNeutral = true;
  static constexpr bool kLeftZero = true;
  __device__ static In neutral() { return (In)1; }
  static constexpr int kU = 0;
  template <int VEC, int U>
  __device__ static void add_block(Acc &, const In *, int64_t, int64_t) {}
  __device__ static Acc init() {
    if constexpr (kZero) return Acc{(Out)1, INT64_MAX};
    else return (Acc)1;
  }
  __device__ static void add(Acc &a, In v, int64_t i) {
    if constexpr (kZero) {
      const Out x = (Out)v;
      a.p = rn_mul(a.p, x);
      if (is_zero_bits(x) && i < a.z) a.z = i;
    } else {
      a = (Acc)wmul<Out>((Out)a, (Out)v);
    }
  }
  template <int VEC> __device__ static void add_vec(Acc &a, const In *v, int64_t i) {
#pragma unroll
    for (int e = 0; e < VEC; e++) add(a, v[e], i + e);
  }
  __device__ static void merge(Acc &a, const Acc &b) {
    if constexpr (kZero) {
      a.p = rn_mul(a.p, b.p);
      if (b.z < a.z) a.z = b.z;
    } else {
      a = (Acc)wmul<Out>((Out)a, (Out)b);
    }
  }
  // the running product is zero: the reference's loop stops here
  __device__ static bool left_zero(const Acc &a) {
    if constexpr (kZero) return a.p == (Out)0;
    else return a == 0;
  }
  __device__ static Out fin(const Acc &a, int64_t cnt, bool bad, Out badval, int *) {
    if (bad && cnt == 0) return badval;
    if constexpr (kZero) return a.p;
    else return (Out)a;
  }
};

template <class In, class Out, bool COMP> struct OpAvg {
  using S = SumAcc<In, Out, COMP>;
  using Acc = typename S::Acc;
  static constexpr bool kZero = false, kLeftZero = false;
  static constexpr bool kCount = true, kVec = true, kNeutral = true;
  __device__ static In neutral() { return (In)0; }
  static constexpr bool kBlock = std::is_same_v<Acc, F64Sum>;
  static constexpr int kU = kBlock ? 8 : 0;
  template <int VEC, int U>
  __device__ static void add_block(Acc &a, const In *v, int64_t, int64_t) {
    if constexpr (kBlock) a.template add_block<VEC * U>(v);
  }
  __device__ static Acc init() { return S::init(); }
  __device__ static void add(Acc &a, In v, int64_t) { S::add(a, v); }
  template <int VEC> __device__ static void add_vec(Acc &a, const In *v, int64_t) {
    if constexpr (std::is_same_v<Acc, F64Sum> && VEC == 2) a.add_block2(v);
    else {
#pragma unroll
      for (int e = 0; e < VEC; e++) S::add(a, v[e]);
    }
  }
  __device__ static void merge(Acc &a, const Acc &b) { S::merge(a, b); }
  __device__ static Out fin(const Acc &a, int64_t cnt, bool bad, Out badval, int *) {
    if (cnt == 0) {
      if (bad) return badval;
      if constexpr (std::is_floating_point_v<Out>) return (Out)NAN; else return (Out)0;
    }
    Out tmp = S::value(a);
    // `tmp / cnt` with cnt a PDL_Indx: C's usual arithmetic conversions.
    if constexpr (std::is_floating_point_v<Out>) {
      return tmp / (Out)cnt;
    } else if constexpr (std::is_same_v<Out, uint64_t>) {
      return tmp / (uint64_t)cnt;
    } else {
      return (Out)((int64_t)tmp / cnt);
    }
  }
};

// minimum/maximum(+_ind): the sequential rule "replace when first, when
// a OP cur, or when cur is NaN" equals the total order: non-NaN beats NaN;
// among non-NaN the smaller (larger) value, ties to the lower index; among
// NaNs the higher index.  That order is associative, so any split works.
template <class T> struct MMAcc {
  int64_t idx;  // -1: empty
  T v;
};
template <class T, bool MAX, bool IND> struct OpMM {
  using Acc = MMAcc<T>;
  static constexpr bool kZero = false, kLeftZero = false;
  using Out = std::conditional_t<IND, int64_t, T>;
  static constexpr bool kCount = false, kVec = true, kBlock = false, kNeutral = false;
  __device__ static T neutral() { return (T)0; }
  static constexpr int kU = 8;
  template <int VEC, int U>
  __device__ static void add_block(Acc &, const T *, int64_t, int64_t) {}
  __device__ static Acc init() { return Acc{-1, (T)0}; }
  __device__ static bool better(T x, int64_t ix, T y, int64_t iy) {
    // does (x, ix) replace (y, iy)?  (ix > iy in sequential order)
    bool xn = isnan_any(x), yn = isnan_any(y);
    if (yn) return !xn || ix > iy;
    if (xn) return false;
    if constexpr (MAX) return x > y || (x == y && ix < iy);
    else return x < y || (x == y && ix < iy);
  }
  __device__ static void add(Acc &a, T v, int64_t i) {
    if (a.idx < 0 || better(v, i, a.v, a.idx)) { a.v = v; a.idx = i; }
  }
  template <int VEC> __device__ static void add_vec(Acc &a, const T *v, int64_t i) {
#pragma unroll
    for (int e = 0; e < VEC; e++) add(a, v[e], i + e);
  }
  __device__ static void merge(Acc &a, const Acc &b) {
    if (b.idx < 0) return;
    if (a.idx < 0 || better(b.v, b.idx, a.v, a.idx)) a = b;
  }
  __device__ static Out fin(const Acc &a, int64_t, bool, Out badval, int *setbad) {
    if (a.idx < 0) {
      *setbad = 1;  // $SETBAD(c()); $PDLSTATESETBAD(c) even without bad mode
      return badval;
    }
    if constexpr (IND) return a.idx; else return a.v;
  }
};

// Logical and bitwise reductions (lib/PDL/Ufunc.pd:143-187), all order free:
// K 0 andover (tmp &= a != 0), 1 orover, 2 xorover, 3 zcover (tmp &= a == 0),
// 4 bandover (tmp &= a), 5 borover, 6 bxorover.  The reference stops early
// once the result cannot change (its leftzero); that changes no result.
// A bad element is replaced by the op's neutral element; no good element
// in bad-value mode gives BAD.
template <class T, int K> struct OpLogic {
  static constexpr bool kBits = K >= 4 && std::is_integral_v<T>;
  // bit ops work on the unsigned image, widened to 4 bytes for the shuffles
  // (the low bits, which is all the result keeps, are the same)
  using Acc = std::conditional_t<kBits && (sizeof(T) >= 4), uns_t<T>, uint32_t>;
  static constexpr bool kCount = false, kVec = true, kBlock = false, kNeutral = true;
  static constexpr bool kZero = false, kLeftZero = false;
  static constexpr int kU = 0;
  __device__ static T neutral() {
    if constexpr (K == 0) return (T)1;  // a != 0 leaves "and" as it is
    else if constexpr (K == 4 && kBits) return (T)(~(uns_t<T>)0);
    else return (T)0;
  }
  template <int VEC, int U>
  __device__ static void add_block(Acc &, const T *, int64_t, int64_t) {}
  __device__ static Acc init() {
    if constexpr (K == 0 || K == 3) return 1;
    else if constexpr (K == 4) return (Acc)(~(Acc)0);
    else return 0;
  }
  __device__ static void add(Acc &a, T v, int64_t) {
    if constexpr (K == 0) a &= (Acc)(v != (T)0);
    else if constexpr (K == 1) a |= (Acc)(v != (T)0);
    else if constexpr (K == 2) a ^= (Acc)(v != (T)0);
    else if constexpr (K == 3) a &= (Acc)(v == (T)0);
    else if constexpr (K == 4) a &= (Acc)v;
    else if constexpr (K == 5) a |= (Acc)v;
    else a ^= (Acc)v;
  }
  template <int VEC> __device__ static void add_vec(Acc &a, const T *v, int64_t i) {
#pragma unroll
    for (int e = 0; e < VEC; e++) add(a, v[e], i + e);
  }
  __device__ static void merge(Acc &a, const Acc &b) {
    if constexpr (K == 0 || K == 3 || K == 4) a &= b;
    else if constexpr (K == 1 || K == 5) a |= b;
    else a ^= b;
  }
  __device__ static T fin(const Acc &a, int64_t cnt, bool bad, T badval, int *) {
    if (bad && cnt == 0) return badval;
    return (T)a;
  }
};

// firstnonzeroover (lib/PDL/Ufunc.pd:144-145): `tmp = a` until tmp is
// nonzero, so the first nonzero good element, else the last good element
// (a zero, with its sign), else 0 (n == 0) or BAD (all bad).
template <class T> struct OpFirstNZ {
  struct Acc {
    int64_t nz;    // index of the first nonzero seen, INT64_MAX: none
    int64_t last;  // index of the last good element seen, -1: none
    T nzv, lastv;
  };
  static constexpr bool kCount = false, kVec = true, kBlock = false, kNeutral = false;
  static constexpr bool kZero = false, kLeftZero = false;
  static constexpr int kU = 8;
  __device__ static T neutral() { return (T)0; }
  template <int VEC, int U>
  __device__ static void add_block(Acc &, const T *, int64_t, int64_t) {}
  __device__ static Acc init() { return Acc{INT64_MAX, -1, (T)0, (T)0}; }
  __device__ static void add(Acc &a, T v, int64_t i) {
    if (v != (T)0 && i < a.nz) {  // NaN is nonzero, as in C
      a.nz = i;
      a.nzv = v;
    }
    if (i > a.last) {
      a.last = i;
      a.lastv = v;
    }
  }
  template <int VEC> __device__ static void add_vec(Acc &a, const T *v, int64_t i) {
#pragma unroll
    for (int e = 0; e < VEC; e++) add(a, v[e], i + e);
  }
  __device__ static void merge(Acc &a, const Acc &b) {
    if (b.nz < a.nz) {
      a.nz = b.nz;
      a.nzv = b.nzv;
    }
    if (b.last > a.last) {
      a.last = b.last;
      a.lastv = b.lastv;
    }
  }
  __device__ static T fin(const Acc &a, int64_t, bool bad, T badval, int *) {
    if (a.last < 0) return bad ? badval : (T)0;
    return a.nz != INT64_MAX ? a.nzv : a.lastv;
  }
};

// float64 minimum/maximum(+_ind) on the integer pipe.  GB300 retires about
// 2 FP64 instructions per clock per SM, so FP64 compares cannot keep up
// with HBM; instead each double maps to an ordered int64 key (sign-magnitude
// to two's complement: monotonic, -0 == +0) and a 16-element block is
// settled by an integer tournament in index order (branch-free; a filter
// on the high word alone, with a per-element branch, measured slower).
// Blocks holding an inf or NaN take the exact per-element rule.  In key
// space (maximum negates the key) NaN is the worst key; equal keys go to
// the lower index, except NaN against NaN, which goes to the higher index.
__device__ __forceinline__ int64_t dkey(uint64_t b) {
  const int64_t mag = (int64_t)and_b64(b, 0x7FFFFFFFFFFFFFFFull);
  const int64_t s = (int64_t)b >> 63;
  return (mag ^ s) - s;
}
constexpr int64_t KEY_NAN = 0x7FFFFFFFFFFFFFFFll;

template <bool MAX, bool IND> struct OpMM<double, MAX, IND> {
  static constexpr bool kZero = false, kLeftZero = false;
  struct Acc {
    int64_t key;
    int64_t idx;  // -1: empty
    uint64_t bits;
  };
  using Out = std::conditional_t<IND, int64_t, double>;
  static constexpr bool kCount = false, kVec = true, kBlock = true, kNeutral = false;
  __device__ static double neutral() { return 0.0; }
  static constexpr int kU = 8;
  __device__ static int64_t key_of(uint64_t b) {
    if (and_b64(b, 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return KEY_NAN;
    int64_t k = dkey(b);
    return MAX ? -k : k;
  }
  __device__ static bool better(int64_t k, int64_t i, int64_t k2, int64_t i2) {
    return k < k2 || (k == k2 && (k == KEY_NAN ? i > i2 : i < i2));
  }
  __device__ static Acc init() { return Acc{KEY_NAN, -1, 0}; }
  __device__ static void add(Acc &a, double v, int64_t i) {
    uint64_t b = (uint64_t)__double_as_longlong(v);
    int64_t k = key_of(b);
    if (a.idx < 0 || better(k, i, a.key, a.idx)) a = Acc{k, i, b};
  }
  template <int VEC> __device__ static void add_vec(Acc &a, const double *v, int64_t i) {
#pragma unroll
    for (int e = 0; e < VEC; e++) add(a, v[e], i + e);
  }
  template <int VEC, int U>
  __device__ static void add_block(Acc &a, const double *v, int64_t base, int64_t ustride) {
    constexpr int B = VEC * U;
    const uint64_t *bits = reinterpret_cast<const uint64_t *>(v);
    int64_t k[B];
    uint64_t w[B];
    int p[B];
    uint32_t special = 0;
#pragma unroll
    for (int j = 0; j < B; j++) {
      const uint32_t hi = hi_b32(bits[j]);
      special |= (~hi & 0x7FF00000u) == 0;  // exponent all ones: inf or NaN
      int64_t kk = dkey(bits[j]);
      k[j] = MAX ? -kk : kk;
      w[j] = bits[j];
      p[j] = j;
    }
    if (special) {
#pragma unroll
      for (int j = 0; j < B; j++)
        add(a, v[j], base + (j / VEC) * ustride + (j % VEC));
      return;
    }
    // The block's smallest key in 32-bit halves (64-bit integer min and
    // compare go to GB300's narrow FP64 pipe): the least high word, then the
    // least low word among the keys with that high word, then the first
    // index holding both (ties go to the lower index).
    int32_t mh = (int32_t)(k[0] >> 32);
#pragma unroll
    for (int j = 1; j < B; j++) mh = min(mh, (int32_t)(k[j] >> 32));
    uint32_t ml = 0xFFFFFFFFu;
#pragma unroll
    for (int j = 0; j < B; j++)
      ml = min(ml, (int32_t)(k[j] >> 32) == mh ? (uint32_t)k[j] : 0xFFFFFFFFu);
    int pj = 0;
    uint64_t wb = 0;
#pragma unroll
    for (int j = B - 1; j >= 0; j--) {
      const bool hit = (int32_t)(k[j] >> 32) == mh && (uint32_t)k[j] == ml;
      pj = hit ? j : pj;
      if constexpr (!IND) wb = hit ? w[j] : wb;
    }
    (void)p;
    const int64_t bk = (int64_t)(((uint64_t)(uint32_t)mh << 32) | ml);
    const bool take = a.idx < 0 || (int32_t)(a.key >> 32) > mh ||
                      ((int32_t)(a.key >> 32) == mh && (uint32_t)a.key > ml);
    if (take) {
      a.key = bk;
      a.idx = base + (pj / VEC) * ustride + (pj % VEC);
      a.bits = IND ? 0 : wb;
    }
  }
  __device__ static void merge(Acc &a, const Acc &b) {
    if (b.idx < 0) return;
    if (a.idx < 0 || better(b.key, b.idx, a.key, a.idx)) a = b;
  }
  __device__ static Out fin(const Acc &a, int64_t, bool, Out badval, int *setbad) {
    if (a.idx < 0) {
      *setbad = 1;
      return badval;
    }
    if constexpr (IND) return a.idx;
    else return __longlong_as_double((long long)a.bits);
  }
};

// ------------------------------------------------------------- reductions

template <class Acc> struct AccCnt {
  Acc acc;
  int64_t cnt;
};

template <class Op>
__device__ __forceinline__ void merge_ac(AccCnt<typename Op::Acc> &x,
                                         const AccCnt<typename Op::Acc> &y) {
  Op::merge(x.acc, y.acc);
  x.cnt += y.cnt;
}

// Reduce across the G threads of a group; G is 32 (a warp; several rows per
// block) or blockDim.x (one row per block).  Result valid in lane 0.
template <class Op>
__device__ __forceinline__ AccCnt<typename Op::Acc> group_reduce(
    AccCnt<typename Op::Acc> v, int G) {
  using AC = AccCnt<typename Op::Acc>;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    AC o;
    o.acc = shfl_down_any(v.acc, d);
    o.cnt = __shfl_down_sync(0xffffffffu, v.cnt, d);
    merge_ac<Op>(v, o);
  }
  if (G <= 32) return v;
  __shared__ AC sm[32];
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    v = l < nw ? sm[l] : AC{Op::init(), 0};
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      AC o;
      o.acc = shfl_down_any(v.acc, d);
      o.cnt = __shfl_down_sync(0xffffffffu, v.cnt, d);
      merge_ac<Op>(v, o);
    }
  }
  return v;
}

template <class In, int VEC> struct alignas(16) VecT {
  In e[VEC];
};

// 16-byte streaming load (read once: evict-first).
template <class V> __device__ __forceinline__ V ldv(const V *p) {
  static_assert(sizeof(V) == 16, "16-byte vectors");
  float4 f = __ldcs(reinterpret_cast<const float4 *>(p));
  V v;
  memcpy(&v, &f, 16);
  return v;
}

// Accumulate elements [lo, hi) of a contiguous row, G threads, lane `lane`.
// Ops with a neutral element (sums, products) add it in place of a bad
// value, so the inner loop has no branches; the good count is the range
// size (added by lane 0) minus each lane's bad count.
template <class Op, class In, int BM>
__device__ __forceinline__ void row_accumulate(const In *row, int64_t lo, int64_t hi,
                                               int lane, int G, In bad,
                                               AccCnt<typename Op::Acc> &ac) {
  constexpr int VEC = 16 / sizeof(In);
  constexpr int U = Op::kU ? Op::kU : 16;  // 16-byte vectors in flight per thread
  uint32_t nb = 0;
  auto take = [&](In v, int64_t idx, uint32_t &cnt) {
    if constexpr (BM == 0) {
      Op::add(ac.acc, v, idx);
    } else {
      const bool b = is_bad<In, BM>(v, bad);
      cnt += b;
      if constexpr (Op::kNeutral) Op::add(ac.acc, b ? Op::neutral() : v, idx);
      else if (!b) Op::add(ac.acc, v, idx);
    }
  };
  // scalar head up to a 16-byte boundary
  int64_t mis = ((uintptr_t)(row + lo) & 15) / sizeof(In);
  int64_t head = mis ? (VEC - mis) : 0;
  if (head > hi - lo) head = hi - lo;
  if (lane < head) take(row[lo + lane], lo + lane, nb);
  const int64_t i = lo + head;
  const VecT<In, VEC> *vp = reinterpret_cast<const VecT<In, VEC> *>(row + i);
  const int64_t nv = (hi - i) / VEC;
  const int64_t per = (int64_t)G * U;
  int64_t nbad = 0;
  int64_t k = lane;
  // full iterations: all U vectors in range, no per-vector checks
  for (; k + (int64_t)(U - 1) * G < nv; k += per) {
    VecT<In, VEC> buf[U];
#pragma unroll
    for (int u = 0; u < U; u++) buf[u] = ldv(vp + k + (int64_t)u * G);
    if constexpr (BM == 0 && Op::kBlock) {
      Op::template add_block<VEC, U>(ac.acc, reinterpret_cast<const In *>(buf), i + k * VEC,
                                     (int64_t)G * VEC);
    } else {
      uint32_t nbi = 0;
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int64_t base = i + (k + (int64_t)u * G) * VEC;
        if constexpr (BM == 0) {
          Op::template add_vec<VEC>(ac.acc, buf[u].e, base);
        } else {
#pragma unroll
          for (int e = 0; e < VEC; e++) take(buf[u].e[e], base + e, nbi);
        }
      }
      nbad += nbi;
    }
  }
  // the last, partial iteration
  if (k < nv) {
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t kk = k + (int64_t)u * G;
      if (kk < nv) {
        VecT<In, VEC> v = ldv(vp + kk);
        const int64_t base = i + kk * VEC;
        if constexpr (BM == 0) {
          Op::template add_vec<VEC>(ac.acc, v.e, base);
        } else {
#pragma unroll
          for (int e = 0; e < VEC; e++) take(v.e[e], base + e, nb);
        }
      }
    }
  }
  // scalar tail
  for (int64_t t = i + nv * VEC + lane; t < hi; t += G) take(row[t], t, nb);
  ac.cnt += (lane == 0 ? hi - lo : 0) - nbad - (int64_t)nb;
}

// Accumulate elements [lo, hi) of a strided row (scalar loads).
template <class Op, class In, bool BAD>
__device__ __forceinline__ void row_accumulate_strided(const In *row, int64_t inc,
                                                       int64_t lo, int64_t hi, int lane,
                                                       int G, const Bad<In> &bv,
                                                       AccCnt<typename Op::Acc> &ac) {
  for (int64_t t = lo + lane; t < hi; t += G) {
    In v = row[t * inc];
    if (!(BAD && bv.is(v))) {
      Op::add(ac.acc, v, t);
      ac.cnt++;
    }
  }
}

// A value written by another block in this launch: read through L2.
template <class T> __device__ __forceinline__ T ldcg_any(const T *p) {
  static_assert(sizeof(T) % 4 == 0, "4-byte words");
  unsigned w[sizeof(T) / 4];
#pragma unroll
  for (int i = 0; i < (int)(sizeof(T) / 4); i++) w[i] = __ldcg(reinterpret_cast<const unsigned *>(p) + i);
  T v;
  memcpy(&v, w, sizeof(T));
  return v;
}

template <class Out> __device__ __forceinline__ void store_out(char *p, Out v) {
  *reinterpret_cast<Out *>(p) = v;
}

// Group-per-row kernel.  Contiguous n.  nsplit > 1: each block does one
// chunk of one row and writes its partial accumulator.
template <class Op, class In, class Out, bool BAD>
__global__ void __launch_bounds__(512) k_red_rows(const RedArgs args) {
  using Acc = typename Op::Acc;
  using AC = AccCnt<Acc>;
  const int G = args.group;
  const int lane = G <= 32 ? (threadIdx.x & 31) : threadIdx.x;
  const int gpb = G <= 32 ? (blockDim.x >> 5) : 1;  // groups per block
  const int gid = G <= 32 ? (threadIdx.x >> 5) : 0;
  Bad<In> bv{from_bits<In>(args.abad_bits), (bool)args.abad_isnan};
  Out obad = from_bits<Out>(args.bbad_bits);
  const int64_t nunits = args.rows * args.nsplit;
  for (int64_t u = (int64_t)blockIdx.x * gpb + gid; u < nunits;
       u += (int64_t)gridDim.x * gpb) {
    int64_t row = u / args.nsplit;
    int split = (int)(u - row * args.nsplit);
    int64_t offs[MAXP];
    loop_offsets(args.L, row, offs);
    const In *a = reinterpret_cast<const In *>(args.a) + offs[0];
    int64_t lo = 0, hi = args.n;
    if (args.nsplit > 1) {
      int64_t chunk = (args.n + args.nsplit - 1) / args.nsplit;
      chunk = (chunk + 31) & ~(int64_t)31;
      lo = split * chunk;
      hi = lo + chunk < args.n ? lo + chunk : args.n;
      if (lo > hi) lo = hi;
    }
    AC ac{Op::init(), 0};
    if (args.inc_n == 1) {
      if constexpr (!BAD) {
        row_accumulate<Op, In, 0>(a, lo, hi, lane, G, bv.val, ac);
      } else if constexpr (std::is_floating_point_v<In>) {
        if (bv.isnan_) row_accumulate<Op, In, 2>(a, lo, hi, lane, G, bv.val, ac);
        else row_accumulate<Op, In, 1>(a, lo, hi, lane, G, bv.val, ac);
      } else {
        row_accumulate<Op, In, 1>(a, lo, hi, lane, G, bv.val, ac);
      }
    } else
      row_accumulate_strided<Op, In, BAD>(a, args.inc_n, lo, hi, lane, G, bv, ac);
    ac = group_reduce<Op>(ac, G);
    bool last = false;
    if (lane == 0) {
      if (args.nsplit > 1) {
        reinterpret_cast<Acc *>(args.partials)[u] = ac.acc;
        args.pcounts[u] = ac.cnt;
        if (args.split_ctr) {
          __threadfence();
          last = atomicAdd(&args.split_ctr[row], 1) == args.nsplit - 1;
        }
      } else {
        int64_t cnt = (BAD || Op::kCount || args.inc_n != 1) ? ac.cnt : args.n;
        Out r = Op::fin(ac.acc, cnt, BAD, obad, args.setbad);
        store_out<Out>(args.b + offs[1] * (int64_t)sizeof(Out), r);
        if constexpr (Op::kZero) args.zidx[row] = ac.acc.z;
      }
    }
    if (args.nsplit > 1 && args.split_ctr) {
      // the row's last split to arrive merges the row's partials (a group
      // is the whole block whenever rows are split)
      __shared__ int s_last;
      if (lane == 0) s_last = last;
      __syncthreads();
      if (s_last) {
        __threadfence();
        const Acc *p = reinterpret_cast<const Acc *>(args.partials) + row * args.nsplit;
        const int64_t *pc = args.pcounts + row * args.nsplit;
        AC m{Op::init(), 0};
        for (int sp = lane; sp < args.nsplit; sp += G) {
          AC o{ldcg_any(p + sp), (int64_t)__ldcg((const long long *)(pc + sp))};
          merge_ac<Op>(m, o);
        }
        m = group_reduce<Op>(m, G);
        if (lane == 0) {
          const int64_t cnt = (BAD || Op::kCount || args.inc_n != 1) ? m.cnt : args.n;
          Out r = Op::fin(m.acc, cnt, BAD, obad, args.setbad);
          store_out<Out>(args.b + offs[1] * (int64_t)sizeof(Out), r);
          if constexpr (Op::kZero) args.zidx[row] = m.acc.z;
          args.split_ctr[row] = 0;  // ready for the next launch
        }
      }
    }
  }
}

// Combine the per-split partials of each row: one warp per row, each lane
// merging every 32nd split, then a shuffle tree (min/max ties are settled by
// index inside merge, so the order of the merges does not matter for them).
template <class Op, class In, class Out, bool BAD>
__global__ void k_red_combine(const RedArgs args) {
  using Acc = typename Op::Acc;
  using AC = AccCnt<Acc>;
  Out obad = from_bits<Out>(args.bbad_bits);
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       row < args.rows; row += nw) {
    const Acc *p = reinterpret_cast<const Acc *>(args.partials) + row * args.nsplit;
    const int64_t *pc = args.pcounts + row * args.nsplit;
    AC ac{Op::init(), 0};
    for (int s = lane; s < args.nsplit; s += 32) {
      AC o{p[s], pc[s]};
      merge_ac<Op>(ac, o);
    }
    ac = group_reduce<Op>(ac, 32);
    if (lane == 0) {
      int64_t offs[MAXP];
      loop_offsets(args.L, row, offs);
      const int64_t cnt = (BAD || Op::kCount || args.inc_n != 1) ? ac.cnt : args.n;
      Out r = Op::fin(ac.acc, cnt, BAD, obad, args.setbad);
      store_out<Out>(args.b + offs[1] * (int64_t)sizeof(Out), r);
      if constexpr (Op::kZero) args.zidx[row] = ac.acc.z;
    }
  }
}

// Floating products of rows holding a good exact zero at z: the product of
// elements [0, z], which is what the reference's loop leaves when it stops
// at that zero (one warp per row; rows without a zero return at once).
template <class Op, class In, class Out, bool BAD>
__global__ void k_prod_fix(const RedArgs args) {
  if constexpr (Op::kZero) {
    using AC = AccCnt<typename Op::Acc>;
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    const Bad<In> bv{from_bits<In>(args.abad_bits), (bool)args.abad_isnan};
    const Out obad = from_bits<Out>(args.bbad_bits);
    for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
         row < args.rows; row += nw) {
      const int64_t z = args.zidx[row];
      if (z >= args.n) continue;
      int64_t offs[MAXP];
      loop_offsets(args.L, row, offs);
      const In *a = reinterpret_cast<const In *>(args.a) + offs[0];
      AC ac{Op::init(), 0};
      if (args.inc_n == 1) {
        if constexpr (!BAD) {
          row_accumulate<Op, In, 0>(a, 0, z + 1, lane, 32, bv.val, ac);
        } else if constexpr (std::is_floating_point_v<In>) {
          if (bv.isnan_) row_accumulate<Op, In, 2>(a, 0, z + 1, lane, 32, bv.val, ac);
          else row_accumulate<Op, In, 1>(a, 0, z + 1, lane, 32, bv.val, ac);
        } else {
          row_accumulate<Op, In, 1>(a, 0, z + 1, lane, 32, bv.val, ac);
        }
      } else {
        row_accumulate_strided<Op, In, BAD>(a, args.inc_n, 0, z + 1, lane, 32, bv, ac);
      }
      ac = group_reduce<Op>(ac, 32);
      if (lane == 0) {
        Out r = Op::fin(ac.acc, ac.cnt, BAD, obad, args.setbad);
        store_out<Out>(args.b + offs[1] * (int64_t)sizeof(Out), r);
      }
    }
  }
}

// Thread-per-row kernel: any increments, the reference's sequential order
// along n.  Adjacent threads take adjacent rows (coalesced when the
// innermost broadcast dim is contiguous).
template <class Op, class In, class Out, bool BAD>
__global__ void k_red_thread(const RedArgs args) {
  Bad<In> bv{from_bits<In>(args.abad_bits), (bool)args.abad_isnan};
  Out obad = from_bits<Out>(args.bbad_bits);
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < args.rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    int64_t offs[MAXP];
    loop_offsets(args.L, row, offs);
    const In *a = reinterpret_cast<const In *>(args.a) + offs[0];
    AccCnt<typename Op::Acc> ac{Op::init(), 0};
    for (int64_t i = 0; i < args.n; i++) {
      In v = a[i * args.inc_n];
      if (BAD && bv.is(v)) continue;
      Op::add(ac.acc, v, i);
      ac.cnt++;
      if constexpr (Op::kLeftZero)
        if (Op::left_zero(ac.acc)) break;
    }
    Out r = Op::fin(ac.acc, ac.cnt, BAD, obad, args.setbad);
    store_out<Out>(args.b + offs[1] * (int64_t)sizeof(Out), r);
  }
}

template <class Op, class In, class Out>
pdlgb300_error launch_red_typed(RedArgs args, const RedLaunch &lc, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  auto launched = [&](const char *nm, int64_t grid, int block) {
    if (!pgh::cuda_check(cudaGetLastError(), &e, nm)) return false;
    pgh::record_kernel(nm, grid, block);
    return true;
  };
  if (lc.kind == 1) {
    if (args.bad) k_red_thread<Op, In, Out, true><<<lc.grid, lc.block, 0, s>>>(args);
    else k_red_thread<Op, In, Out, false><<<lc.grid, lc.block, 0, s>>>(args);
    launched("k_red_thread", lc.grid, lc.block);
    return e;
  }
  if (args.bad) k_red_rows<Op, In, Out, true><<<lc.grid, lc.block, 0, s>>>(args);
  else k_red_rows<Op, In, Out, false><<<lc.grid, lc.block, 0, s>>>(args);
  if (!launched("k_red_rows", lc.grid, lc.block)) return e;
  if (args.nsplit > 1 && !args.split_ctr) {
    const int g = (int)std::min<int64_t>((args.rows + 3) / 4, 65535);
    if (args.bad) k_red_combine<Op, In, Out, true><<<g, 128, 0, s>>>(args);
    else k_red_combine<Op, In, Out, false><<<g, 128, 0, s>>>(args);
    if (!launched("k_red_combine", g, 128)) return e;
  }
  if constexpr (Op::kZero) {
    const int g = (int)std::min<int64_t>((args.rows + 7) / 8, 65535);
    if (args.bad) k_prod_fix<Op, In, Out, true><<<g, 256, 0, s>>>(args);
    else k_prod_fix<Op, In, Out, false><<<g, 256, 0, s>>>(args);
    launched("k_prod_fix", g, 256);
  }
  return e;
}

template <class Op> size_t acc_size() { return sizeof(typename Op::Acc); }

// Resident blocks per SM of the row kernel for this op (for sizing splits).
template <class Op, class In, class Out>
int red_occ_typed(bool bad, int block) {
  int occ = 0;
  if (bad) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_red_rows<Op, In, Out, true>, block, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_red_rows<Op, In, Out, false>, block, 0);
  return occ > 0 ? occ : 1;
}

}  // namespace pg
