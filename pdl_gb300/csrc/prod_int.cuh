// prod_int.cuh -- a float64 multiply on the integer pipe for the normal
// range (used by prod_seq.cu; host-compilable so that it can be checked
// against the CPU's IEEE multiply).
#pragma once
#include <cstdint>

namespace pg {

// One float64 product on the integer pipe, for operands and result in the
// normal range: A is a significand with its leading bit at bit 63 (11 zero
// bits below), b the operand's in the same form, e and be the unbiased
// exponents.  The 128-bit product's leading 53 bits rounded to nearest
// even, the exponent carried beside: the bits of the IEEE product.  On a
// dependent chain this is about a dozen integer operations per step, where
// GB300's FP64 multiply has a much longer latency.
__host__ __device__ __forceinline__ void nmul(uint64_t &A, int &e, uint64_t b, int be) {
#ifdef __CUDA_ARCH__
  const uint64_t hi = __umul64hi(A, b);
#else
  const uint64_t hi = (uint64_t)(((unsigned __int128)A * b) >> 64);
#endif
  const uint64_t lo = A * b;
  // the product of two significands in [1, 2) lies in [1, 4): bit 127 of
  // the 128-bit product says which; sh: the bits below the 53 kept
  const uint32_t top = (uint32_t)(hi >> 63);
  const uint32_t sh = 10 + top;
  uint64_t mant = hi >> sh;
  const uint64_t guard = (hi >> (sh - 1)) & 1u;
  const uint64_t sticky = ((hi & ((1ull << (sh - 1)) - 1)) | lo) != 0;
  mant += guard & (sticky | (mant & 1u));
  const uint32_t ovf = (uint32_t)(mant >> 53);  // rounded up to 2^53
  mant >>= ovf;
  e += be + (int)top + (int)ovf;
  A = mant << 11;
}

}  // namespace pg
