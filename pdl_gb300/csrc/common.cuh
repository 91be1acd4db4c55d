// common.cuh -- types, type dispatch, launch plans and device helpers shared
// by the kernels of libpdlgb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>
#include <type_traits>
#include <utility>

#include "../../include/pdlgb300.h"

namespace pg {

constexpr int MAXP = 5;                       // max ndarrays of one op (minmaximum: 5)
constexpr int MAXB = PDLGB300_MAXDIMS + 2;    // max broadcast dims
constexpr int NSM_GB300 = 152;

// ------------------------------------------------------------------ types

template <int DT> struct TT;
#define PG_TT(E, CT, ISF, ISU, SYM)                                   \
  template <> struct TT<E> {                                          \
    using T = CT;                                                     \
    static constexpr bool is_float = ISF, is_unsigned = ISU;          \
  };
PG_TT(PDLGB300_SB, int8_t, false, false, A)
PG_TT(PDLGB300_B, uint8_t, false, true, B)
PG_TT(PDLGB300_S, int16_t, false, false, S)
PG_TT(PDLGB300_US, uint16_t, false, true, U)
PG_TT(PDLGB300_L, int32_t, false, false, L)
PG_TT(PDLGB300_UL, uint32_t, false, true, K)
PG_TT(PDLGB300_IND, int64_t, false, false, N)
PG_TT(PDLGB300_ULL, uint64_t, false, true, P)
PG_TT(PDLGB300_LL, int64_t, false, false, Q)
PG_TT(PDLGB300_F, float, true, false, F)
PG_TT(PDLGB300_D, double, true, false, D)
#undef PG_TT

// Dispatch a runtime datatype to a template lambda body with DT bound.
#define PG_DISPATCH(dt, ...)                                              \
  switch (dt) {                                                            \
    case PDLGB300_SB: { constexpr int DT = PDLGB300_SB; __VA_ARGS__; } break;     \
    case PDLGB300_B: { constexpr int DT = PDLGB300_B; __VA_ARGS__; } break;       \
    case PDLGB300_S: { constexpr int DT = PDLGB300_S; __VA_ARGS__; } break;       \
    case PDLGB300_US: { constexpr int DT = PDLGB300_US; __VA_ARGS__; } break;     \
    case PDLGB300_L: { constexpr int DT = PDLGB300_L; __VA_ARGS__; } break;       \
    case PDLGB300_UL: { constexpr int DT = PDLGB300_UL; __VA_ARGS__; } break;     \
    case PDLGB300_IND: { constexpr int DT = PDLGB300_IND; __VA_ARGS__; } break;   \
    case PDLGB300_ULL: { constexpr int DT = PDLGB300_ULL; __VA_ARGS__; } break;   \
    case PDLGB300_LL: { constexpr int DT = PDLGB300_LL; __VA_ARGS__; } break;     \
    case PDLGB300_F: { constexpr int DT = PDLGB300_F; __VA_ARGS__; } break;       \
    case PDLGB300_D: { constexpr int DT = PDLGB300_D; __VA_ARGS__; } break;       \
    default: break;                                                        \
  }

// make_unsigned for integers, the type itself otherwise (safe inside
// std::conditional_t, which names both branches).
template <class T, bool = std::is_integral_v<T>> struct UnsOr { using type = T; };
template <class T> struct UnsOr<T, true> { using type = std::make_unsigned_t<T>; };
template <class T> using uns_t = typename UnsOr<T>::type;

// "int+" output type: max(long, T) in PDL's type order.
constexpr int intplus(int dt) { return dt < PDLGB300_L ? PDLGB300_L : dt; }

// Wrapping integer arithmetic without UB: compute in the unsigned type.
template <class T> __host__ __device__ __forceinline__ T wadd(T a, T b) {
  if constexpr (std::is_integral_v<T>) {
    using U = std::make_unsigned_t<T>;
    return (T)(U)((U)a + (U)b);
  } else {
    return a + b;
  }
}
template <class T> __host__ __device__ __forceinline__ T wmul(T a, T b) {
  if constexpr (std::is_integral_v<T>) {
    // C promotes narrow types to int before multiplying; the result is
    // truncated on store.  Doing it in the wide unsigned type gives the
    // same low bits.
    using W = std::conditional_t<(sizeof(T) <= 4), uint32_t, uint64_t>;
    return (T)(W)((W)(std::make_unsigned_t<T>)a * (W)(std::make_unsigned_t<T>)b);
  } else {
    return a * b;
  }
}

// IEEE binary64 product, round to nearest even, on the integer pipe: GB300
// multiplies doubles at a small fraction of its integer rate, which bounds
// streaming float64 products below HBM speed.  Normal operands with a
// normal (or overflowing) result take the 53 x 53-bit significand product
// and round it here; zeros, subnormals, inf, NaN and results near the
// underflow range go to the hardware multiply.  Same bits as __dmul_rn.
__device__ __forceinline__ double dmul_rn_int(double a, double b) {
  const uint64_t ua = (uint64_t)__double_as_longlong(a), ub = (uint64_t)__double_as_longlong(b);
  const uint32_t ea = (uint32_t)(ua >> 52) & 0x7FFu, eb = (uint32_t)(ub >> 52) & 0x7FFu;
  const int e = (int)(ea + eb) - 1023;  // exponent field when the significand product is < 2
  if (ea - 1u >= 2046u || eb - 1u >= 2046u || e < 1 || e > 2045) return __dmul_rn(a, b);
  constexpr uint64_t H = 1ull << 52;
  const uint64_t ma = (ua & (H - 1)) | H, mb = (ub & (H - 1)) | H;
  const uint64_t hi = __umul64hi(ma, mb), lo = ma * mb;  // product in [2^104, 2^106)
  const bool top = (hi >> 41) != 0;                       // product >= 2^105
  const uint64_t m = top ? ((hi << 11) | (lo >> 53)) : ((hi << 12) | (lo >> 52));
  const uint64_t rem = lo & (top ? (2 * H - 1) : (H - 1));
  const uint64_t half = top ? H : (H >> 1);
  const uint64_t up = (rem > half || (rem == half && (m & 1))) ? 1u : 0u;
  // m carries the hidden bit: (field - 1) << 52 plus m, and a rounding carry
  // out of the significand moves into the exponent (to inf past the range)
  const uint64_t mag = ((uint64_t)(e - 1 + (top ? 1 : 0)) << 52) + m + up;
  return __longlong_as_double((long long)(((ua ^ ub) & (1ull << 63)) | mag));
}

// Products of a block spread over both pipes: even positions on the FP64
// pipe, odd ones on the integer pipe (the same bits either way).
template <int J> __device__ __forceinline__ double dmul_rn_split(double a, double b) {
  if constexpr (J & 1) return dmul_rn_int(a, b);
  else return __dmul_rn(a, b);
}

// Exact IEEE ops with no FMA contraction (PDL's C code rounds every
// product and sum).
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return dmul_rn_int(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
template <class T> __device__ __forceinline__ T op_mul(T a, T b) {
  if constexpr (std::is_floating_point_v<T>) return rn_mul(a, b); else return wmul(a, b);
}
template <class T> __device__ __forceinline__ T op_add(T a, T b) {
  if constexpr (std::is_floating_point_v<T>) return rn_add(a, b); else return wadd(a, b);
}

// Bit operations on the raw bits of a double, opaque to the compiler: a
// mask of the sign bit or a shifted zero test on bits that came from a
// double is otherwise rewritten into fabs / an FP64 compare, which run on
// GB300's narrow FP64 pipe.
__device__ __forceinline__ uint64_t and_b64(uint64_t a, uint64_t m) {
  uint64_t r;
  asm("and.b64 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(m));
  return r;
}
__device__ __forceinline__ uint32_t hi_b32(uint64_t a) {
  uint32_t lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(a));
  return hi;
}
__device__ __forceinline__ bool zero_bits64(uint64_t a) {  // +0 or -0
  uint32_t lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(a));
  return ((hi << 1) | lo) == 0;
}

// PDL_ISBAD2: NaN badvalue => isnan, else equality.
template <class T> struct Bad {
  T val;
  bool isnan_;
  __device__ __forceinline__ bool is(T v) const {
    if constexpr (std::is_floating_point_v<T>) {
      return isnan_ ? (v != v) : (v == val);
    } else {
      return v == val;
    }
  }
};

template <class T> __host__ __device__ inline bool isnan_any(T v) {
  if constexpr (std::is_floating_point_v<T>) return v != v; else return false;
}

// Bad-value test with the mode fixed at compile time: BM 0 = no bad values,
// 1 = the badvalue compares equal, 2 = the badvalue is NaN.
template <class In, int BM> __device__ __forceinline__ bool is_bad(In v, In bad) {
  if constexpr (BM == 0) return false;
  else if constexpr (BM == 2) return isnan_any(v);
  else return v == bad;
}

// ------------------------------------------------------------ loop plans

// A broadcast loop after collapsing: nd dims (innermost first) with sizes
// and per-ndarray element increments.  Offsets are in elements.
struct Loop {
  int nd;
  int np;
  int64_t total;
  int64_t size[MAXB];
  int64_t inc[MAXP][MAXB];
};

// Element offsets of each ndarray for flat broadcast index r.
__device__ __forceinline__ void loop_offsets(const Loop &L, int64_t r, int64_t *offs) {
#pragma unroll
  for (int p = 0; p < MAXP; p++) offs[p] = 0;
  if (L.nd == 1) {
#pragma unroll
    for (int p = 0; p < MAXP; p++) offs[p] = r * L.inc[p][0];
    return;
  }
  for (int k = 0; k < L.nd; k++) {
    int64_t s = L.size[k];
    int64_t q = r / s, i = r - q * s;
    r = q;
#pragma unroll
    for (int p = 0; p < MAXP; p++) offs[p] += i * L.inc[p][k];
  }
}

// ------------------------------------------------------- warp utilities

template <class T> __device__ __forceinline__ T shfl_down_any(T v, int d) {
  static_assert(sizeof(T) % 4 == 0, "shuffle of 4-byte words");
  constexpr int W = sizeof(T) / 4;
  union { T t; uint32_t w[W]; } u;
  u.t = v;
#pragma unroll
  for (int i = 0; i < W; i++) u.w[i] = __shfl_down_sync(0xffffffffu, u.w[i], d);
  return u.t;
}

}  // namespace pg

// ---------------------------------------------------------- host helpers
namespace pgh {
void set_error(pdlgb300_error *e, int kind, const char *fmt, ...);
pdlgb300_error ok();
pdlgb300_error err(int kind, const char *fmt, ...);
cudaStream_t stream();
bool cuda_check(cudaError_t e, pdlgb300_error *out, const char *what);
void record_kernel(const char *name, int64_t grid, int64_t block);
int num_sms();
}  // namespace pgh
