// Host check of pg::nmul (pdl_gb300/csrc/prod_int.cuh) against the CPU's
// IEEE double multiply: random normal operands of every exponent, operands
// near rounding ties (significands with long runs of ones or zeros), and
// 64-step chains kept inside the normal range.  Prints the number of
// mismatches; exit status 1 on any.
#include <cmath>
#include <cstdio>
#include <cstring>
#include "../../pdl_gb300/csrc/prod_int.cuh"

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t next() {  // xorshift64*
  s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
  return s * 2685821657736338717ull;
}
static double bits2d(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t d2bits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }

static double normal_of(int e, uint64_t frac, int sign) {
  return bits2d(((uint64_t)sign << 63) | ((uint64_t)(e + 1023) << 52) | (frac & ((1ull << 52) - 1)));
}
static uint64_t frac_kind(int k) {
  uint64_t r = next();
  switch (k % 5) {
    case 0: return r;
    case 1: return r | 0xFFFFFFF000000ull;            // long run of ones
    case 2: return r & 0xFFF0000000000ull;            // long run of zeros
    case 3: return (1ull << 52) - 1 - (r & 0xFF);     // near 2 - ulp
    default: return r & 0xFF;                          // near 1
  }
}
// (A, e, sign) -> double, as prod_seq.cu encodes it
static double encode(uint64_t A, int e, uint32_t sg) {
  return bits2d(((uint64_t)sg << 63) | ((uint64_t)(e + 1023) << 52) | ((A >> 11) & ((1ull << 52) - 1)));
}

int main(int argc, char **argv) {
  long n = argc > 1 ? atol(argv[1]) : 4000000;
  long bad = 0;
  for (long i = 0; i < n; i++) {
    const int ea = (int)(next() % 2000) - 1000, eb = (int)(next() % 40) - 20 - (ea > 0 ? ea / 2 : 0);
    const double a = normal_of(ea, frac_kind((int)i), (int)(next() & 1));
    const double b = normal_of(eb, frac_kind((int)(i / 5)), (int)(next() & 1));
    const double p = a * b;
    if (!std::isnormal(p)) continue;
    uint64_t A = (d2bits(a) << 11) | (1ull << 63);
    int e = ea;
    pg::nmul(A, e, (d2bits(b) << 11) | (1ull << 63), eb);
    const uint32_t sg = (uint32_t)((d2bits(a) ^ d2bits(b)) >> 63);
    if (d2bits(encode(A, e, sg)) != d2bits(p)) {
      if (bad < 5) fprintf(stderr, "single: %a * %a = %a, got %a\n", a, b, p, encode(A, e, sg));
      bad++;
    }
  }
  // chains of 64 in the normal range, as the kernel runs them
  for (long c = 0; c < n / 64; c++) {
    double t = normal_of((int)(next() % 200) - 100, next(), 0);
    uint64_t A = (d2bits(t) << 11) | (1ull << 63);
    int e = (int)((d2bits(t) >> 52) & 0x7FF) - 1023;
    uint32_t sg = 0;
    for (int j = 0; j < 64; j++) {
      const double x = normal_of((int)(next() % 7) - 3, frac_kind(j + (int)c), (int)(next() & 1));
      t = t * x;
      sg ^= (uint32_t)(d2bits(x) >> 63);
      pg::nmul(A, e, (d2bits(x) << 11) | (1ull << 63), (int)((d2bits(x) >> 52) & 0x7FF) - 1023);
    }
    if (std::isnormal(t) && d2bits(encode(A, e, sg)) != d2bits(t)) {
      if (bad < 5) fprintf(stderr, "chain %ld: %a, got %a\n", c, t, encode(A, e, sg));
      bad++;
    }
  }
  printf("%ld\n", bad);
  return bad ? 1 : 0;
}
