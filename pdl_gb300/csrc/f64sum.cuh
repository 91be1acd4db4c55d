// f64sum.cuh -- float64 summation without one FP64 add per element.
//
// GB300 retires about 1.6 FP64 adds per clock per SM, while streaming
// float64 from HBM at 6.8 TB/s delivers about 2.7 elements per clock per SM,
// so a plain FP64 accumulation loop runs at ~40% of HBM bandwidth.  F64Sum
// therefore sums blocks of 16 doubles in 64-bit integer fixed point aligned
// to the block's largest exponent (integer pipe only: exponent extract,
// 64-bit funnel shifts, sign fold, add), then converts the block sum with one
// cvt.rn.f64.s64 and folds it in with one FP64 add.
//
// Accuracy: an element loses only the bits below 2^-58 of the block's
// largest magnitude (truncation), the block sum is rounded once to double,
// and one FP64 add per block follows: no worse than the reference's
// sequential FP64 loop, which rounds after every element.  Blocks holding an
// inf/NaN, numbers within 2^64 of the subnormal range, or numbers within a
// factor 32 of overflow take the exact per-element FP64 path, so special
// values propagate exactly as IEEE addition does.
#pragma once
#include <stdint.h>

namespace pg {

__device__ __forceinline__ uint64_t shr64_clamped(uint64_t x, uint32_t s) {
  // PTX shr clamps shift amounts above 64 (result 0 for .b64).
  uint64_t r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(s));
  return r;
}

struct F64Sum {
  double s;

  __device__ __forceinline__ void add_fp64(double v) { s = __dadd_rn(s, v); }
  __device__ __forceinline__ void merge(const F64Sum &o) { s = __dadd_rn(s, o.s); }
  __device__ __forceinline__ double value() const { return s; }

  // Sum B doubles (B <= 16) given as raw bits.
  template <int B>
  __device__ __forceinline__ void add_block_bits(const uint64_t *bits) {
    static_assert(B <= 16, "block of at most 16 keeps the int64 sum exact");
    uint32_t e[B];
    uint32_t E = 0;
#pragma unroll
    for (int i = 0; i < B; i++) {
      e[i] = (uint32_t)(bits[i] >> 52) & 0x7FFu;
      E = max(E, e[i]);
    }
    if (E < 65u || E > 2040u) {  // subnormal neighbourhood / inf / NaN / huge
#pragma unroll
      for (int i = 0; i < B; i++) s = __dadd_rn(s, __longlong_as_double((long long)bits[i]));
      return;
    }
    // x = mantissa (implicit bit forced; elements with e == 0 are zeros or
    // subnormals, shifted out entirely because E >= 65) with its top bit at
    // bit 63, shifted right by (E - e) + 5: every term is below 2^59.
    long long S = 0;
    const uint32_t E5 = E + 5u;
#pragma unroll
    for (int i = 0; i < B; i++) {
      uint64_t m = (bits[i] << 11) | 0x8000000000000000ull;
      uint64_t f = shr64_clamped(m, E5 - e[i]);
      long long sm = (long long)bits[i] >> 63;  // 0 or -1
      S += ((long long)f ^ sm) - sm;
    }
    // block value = S * 2^(E - 1081)
    double d = __ll2double_rn(S);
    if (S != 0) d = __longlong_as_double(__double_as_longlong(d) + ((long long)((int)E - 1081) << 52));
    s = __dadd_rn(s, d);
  }

  template <int B>
  __device__ __forceinline__ void add_block(const double *v) {
    add_block_bits<B>(reinterpret_cast<const uint64_t *>(v));
  }
  __device__ __forceinline__ void add_block2(const double *v) {
    s = __dadd_rn(s, v[0]);
    s = __dadd_rn(s, v[1]);
  }
};

}  // namespace pg
