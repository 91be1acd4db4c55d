// prod_seq.cu -- floating prodover / dprodover with the reference's exact
// early exit (lib/PDL/Ufunc.pd:88-118: `tmp *= a; if (tmp == 0) break;`).
//
// A floating running product that underflows to zero stops the reference's
// loop there; its sign is the product's sign at that point, and elements
// after it (an inf, a NaN) are never seen.  Where a product stays within the
// normal range from start to end, any order of multiplication gives the
// product within (n+2) ulps and no overflow or underflow; where it does not,
// only the reference's own order gives its result.  So:
//
//  1. Sequential prefix.  Each warp takes 32 rows, one per lane, and runs
//     the reference's loop over the first S elements of its row exactly
//     (same order, one rounding per product, the break).  The warp stages
//     64-element chunks of its 32 rows in shared memory with cp.async, two
//     chunks in flight, so the lanes' dependent multiply chains do not wait
//     on scattered loads.  Rows that end or stop inside
//     the prefix are done: uniform[-1,1) data, for one, underflows after
//     about 750 elements.
//  2. Suffix check.  For each row that goes on, the warp reads the rest of
//     the row together: the product of the remaining good elements, their
//     count, the first exact zero, any inf/NaN/subnormal, and bounds on the
//     log2 magnitude every partial product can reach (sums of per-element
//     lower bounds e + f and upper bounds e + f + 0.0861 of log2|x|, x =
//     2^e (1 + f)).  If the prefix's product is normal and every partial
//     product is bounded inside the normal range (with a margin), the
//     result is prefix * suffix (or, with a zero at z, prefix * the product
//     over [S, z], a signed zero); otherwise the row continues as in 3.
//  3. Sequential continuation.  Rows whose products may leave the normal
//     range run the reference's loop on from the prefix, one lane each.
//
// The float64 products use the FP64 pipe (__dmul_rn): the dependent chain
// is latency-bound and the hardware multiply has the shortest latency.
#include "reduce.cuh"

namespace pg {
namespace {

constexpr int PS_CH = 64;  // elements per staged chunk of a row (a multiple of 32)

template <class Out> struct LogLim;
template <> struct LogLim<float> {
  static constexpr float lo = -126.0f + 4.0f, hi = 127.0f - 4.0f;
};
template <> struct LogLim<double> {
  static constexpr float lo = -1022.0f + 4.0f, hi = 1023.0f - 4.0f;
};

// x normal and nonzero: bounds of log2|x| from its exponent and the top
// mantissa bits (log2(1 + f) lies in [f, f + 0.0861] for f in [0, 1)).
template <class Out> __device__ __forceinline__ bool normal_nz(Out x) {
  if constexpr (sizeof(Out) == 8) {
    const uint32_t e = (hi_b32((uint64_t)__double_as_longlong(x)) >> 20) & 0x7FFu;
    return e != 0 && e != 0x7FF;
  } else {
    const uint32_t e = (__float_as_uint(x) >> 23) & 0xFFu;
    return e != 0 && e != 0xFF;
  }
}
template <class Out> __device__ __forceinline__ float log2_lo(Out x) {
  if constexpr (sizeof(Out) == 8) {
    const uint32_t h = hi_b32((uint64_t)__double_as_longlong(x));
    const int e = (int)((h >> 20) & 0x7FF) - 1023;
    const float f = __uint_as_float(0x3F800000u | ((h & 0xFFFFF) << 3)) - 1.0f;
    return (float)e + f;
  } else {
    const uint32_t b = __float_as_uint(x);
    const int e = (int)((b >> 23) & 0xFF) - 127;
    const float f = __uint_as_float(0x3F800000u | (b & 0x7FFFFF)) - 1.0f;
    return (float)e + f;
  }
}
constexpr float LOG2_SLACK = 0.0861f;

template <class Out> __device__ __forceinline__ Out mul_rn(Out a, Out b) {
  if constexpr (sizeof(Out) == 8) return __dmul_rn(a, b);
  else return __fmul_rn(a, b);
}

template <class In, bool BAD> __device__ __forceinline__ bool bad_el(In v, const Bad<In> &bv) {
  if constexpr (BAD) return bv.is(v);
  else return false;
}

// The suffix summary of one row, reduced over a warp.
template <class Out> struct Suffix {
  Out q;        // product of the good elements (any order)
  int64_t cnt;  // good elements
  int64_t z;    // first good exact zero, or INT64_MAX
  float lo, hi; // sums of min(0, lower bound) and max(0, upper bound) of log2|x|
  int special;  // an inf, NaN or subnormal good element
};

template <class In, class Out, bool BAD>
__device__ void suffix_scan(const In *a, int64_t inc, int64_t from, int64_t to, int lane,
                            const Bad<In> &bv, Suffix<Out> &s, bool to_zero_only) {
  s.q = (Out)1;
  s.cnt = 0;
  s.z = INT64_MAX;
  s.lo = 0.0f;
  s.hi = 0.0f;
  s.special = 0;
#pragma unroll 4
  for (int64_t i = from + lane; i < to; i += 32) {
    const In v = a[i * inc];
    if (bad_el<In, BAD>(v, bv)) continue;
    const Out x = (Out)v;
    s.q = mul_rn(s.q, x);
    s.cnt++;
    if (is_zero_bits(x)) {
      if (i < s.z) s.z = i;
    } else if (!normal_nz(x)) {
      s.special = 1;
    } else if (!to_zero_only) {
      const float l = log2_lo(x);
      s.lo += fminf(l, 0.0f);
      s.hi += fmaxf(l + LOG2_SLACK, 0.0f);
    }
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    s.q = mul_rn(s.q, __shfl_xor_sync(0xffffffffu, s.q, d));
    s.cnt += __shfl_xor_sync(0xffffffffu, s.cnt, d);
    const int64_t oz = __shfl_xor_sync(0xffffffffu, s.z, d);
    s.z = oz < s.z ? oz : s.z;
    s.lo += __shfl_xor_sync(0xffffffffu, s.lo, d);
    s.hi += __shfl_xor_sync(0xffffffffu, s.hi, d);
    s.special |= __shfl_xor_sync(0xffffffffu, s.special, d);
  }
}

template <class In, class Out, bool BAD>
__global__ void __launch_bounds__(32) k_prod_seq(const RedArgs args, int64_t S) {
  // two chunks of PS_CH elements of the warp's 32 rows in flight:
  // [stage][element][row], a row's elements down one column
  __shared__ __align__(16) In tile[2][PS_CH][33];
  const int lane = threadIdx.x;
  const int64_t row0 = (int64_t)blockIdx.x * 32;
  const int64_t row = row0 + lane;
  const bool have = row < args.rows;
  const Bad<In> bv{from_bits<In>(args.abad_bits), (bool)args.abad_isnan};
  const Out obad = from_bits<Out>(args.bbad_bits);
  int64_t offs[MAXP];
  loop_offsets(args.L, have ? row : row0, offs);
  const In *a = reinterpret_cast<const In *>(args.a) + offs[0];
  const int64_t inc = args.inc_n;
  const int64_t n = args.n;
  const int64_t pend = S < n ? S : n;

  Out tmp = (Out)1;
  int64_t cnt = 0;
  bool live = have;  // still multiplying
  // -------------------------------------------- 1. sequential prefix
  // lane j copies elements i0 + j, i0 + 32 + j, ... of every live row
  // straight into shared memory (cp.async: nothing held in registers while
  // in flight); elements past the prefix are zero-filled and never used
  auto fetch = [&](int st, int64_t i0, unsigned rows_live) {
#pragma unroll 4
    for (int r = 0; r < 32; r++) {
      const In *ar = reinterpret_cast<const In *>(
          __shfl_sync(0xffffffffu, (unsigned long long)a, r));
#pragma unroll
      for (int h = 0; h < PS_CH / 32; h++) {
        const int e = h * 32 + lane;
        const int64_t i = i0 + e;
        const bool in = ((rows_live >> r) & 1u) && i < pend;
        if constexpr (sizeof(In) >= 4) {
          const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tile[st][e][r]);
          const In *src = in ? ar + i * inc : ar;
          asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(dst), "l"(src),
                       "n"(sizeof(In)), "r"(in ? (int)sizeof(In) : 0)
                       : "memory");
        } else {
          // (1- and 2-byte types: cp.async copies 4, 8 or 16 bytes)
          tile[st][e][r] = in ? ar[i * inc] : (In)0;
        }
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  unsigned live_mask = __ballot_sync(0xffffffffu, live);
  if (pend > 0 && live_mask) {
    fetch(0, 0, live_mask);
    if (PS_CH < pend) fetch(1, PS_CH, live_mask);
  }
  int st = 0;
  for (int64_t i0 = 0; i0 < pend && live_mask; i0 += PS_CH, st ^= 1) {
    // this chunk's group has landed (the next one may still be in flight)
    if (i0 + PS_CH < pend) asm volatile("cp.async.wait_group 1;" ::: "memory");
    else asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncwarp();
    const int m = (int)(pend - i0 < PS_CH ? pend - i0 : PS_CH);
    if (live) {
      // The chunk's products alone (a bad element multiplies by 1): the
      // dependent chain is one multiply per element.  A product that reaches
      // zero stops the reference's loop; later products of a zero are zero
      // or NaN, so only a chunk that ends zero or NaN is run again from its
      // start, element by element, to stop at the first zero.
      const Out start = tmp;
      auto elem = [&](int j) {
        const In v = tile[st][j][lane];
        Out x = (Out)v;
        if constexpr (BAD) {
          const bool b = bad_el<In, BAD>(v, bv);
          x = b ? (Out)1 : x;
          cnt += b ? 0 : 1;
        }
        return x;
      };
      if (m == PS_CH) {
#pragma unroll
        for (int j = 0; j < PS_CH; j++) tmp = mul_rn(tmp, elem(j));
      } else {
        for (int j = 0; j < m; j++) tmp = mul_rn(tmp, elem(j));
      }
      if constexpr (!BAD) cnt += m;
      if (is_zero_bits(tmp) || tmp != tmp) {
        tmp = start;
        for (int j = 0; j < m; j++) {
          const In v = tile[st][j][lane];
          if (bad_el<In, BAD>(v, bv)) continue;
          tmp = mul_rn(tmp, (Out)v);
          if (is_zero_bits(tmp)) {
            live = false;
            break;
          }
        }
      }
    }
    live_mask = __ballot_sync(0xffffffffu, live);
    __syncwarp();  // every lane is done with this stage before it is refilled
    if (i0 + 2 * PS_CH < pend && live_mask) fetch(st, i0 + 2 * PS_CH, live_mask);
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // -------------------------------------------- 2. suffix check
  bool seq = false;
  unsigned cont = __ballot_sync(0xffffffffu, live && n > pend);
  while (cont) {
    const int r = __ffs(cont) - 1;
    cont &= cont - 1;
    const In *ar = reinterpret_cast<const In *>(__shfl_sync(0xffffffffu, (unsigned long long)a, r));
    const Out pr = __shfl_sync(0xffffffffu, tmp, r);
    Suffix<Out> s;
    suffix_scan<In, Out, BAD>(ar, inc, pend, n, lane, bv, s, false);
    // every partial product, of the reference's order (prefix first) and
    // of the warp's (the suffix alone), stays inside the normal range
    const float p_lo = log2_lo(pr);
    const bool safe = normal_nz(pr) && !s.special && p_lo + s.lo >= LogLim<Out>::lo &&
                      p_lo + LOG2_SLACK + s.hi <= LogLim<Out>::hi && s.lo >= LogLim<Out>::lo &&
                      s.hi <= LogLim<Out>::hi;
    Out res = mul_rn(pr, s.q);
    if (safe && s.z != INT64_MAX) {
      // stops at the zero: the product up to and including it
      Suffix<Out> t;
      suffix_scan<In, Out, BAD>(ar, inc, pend, s.z + 1, lane, bv, t, true);
      res = mul_rn(pr, t.q);
    }
    if (lane == r) {
      cnt += s.cnt;
      if (safe) {
        tmp = res;
        live = false;
      } else {
        seq = true;
      }
    }
  }
  // -------------------------------------------- 3. sequential continuation
  if (seq) {
    for (int64_t i = pend; i < n; i++) {
      const In v = a[i * inc];
      if (bad_el<In, BAD>(v, bv)) continue;
      tmp = mul_rn(tmp, (Out)v);
      if (is_zero_bits(tmp)) break;
    }
  }
  if (have) {
    // (the count only decides "any good element" in bad mode)
    const Out r = (BAD && cnt == 0) ? obad : tmp;
    *reinterpret_cast<Out *>(args.b + offs[1] * (int64_t)sizeof(Out)) = r;
  }
}

template <class In, class Out>
pdlgb300_error launch_typed(const RedArgs &a, int64_t S, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const int64_t g = (a.rows + 31) / 32;
  if (a.bad) k_prod_seq<In, Out, true><<<(unsigned)g, 32, 0, s>>>(a, S);
  else k_prod_seq<In, Out, false><<<(unsigned)g, 32, 0, s>>>(a, S);
  if (pgh::cuda_check(cudaGetLastError(), &e, "k_prod_seq")) pgh::record_kernel("k_prod_seq", g, 32);
  return e;
}

}  // namespace

// Floating prodover (float/double input) and dprodover (any input):
// the reference's sequential product with its early exit.
pdlgb300_error launch_prod_seq(int op, int in_dt, const RedArgs &a, int64_t S, cudaStream_t s) {
  if (a.rows == 0) return pgh::ok();
  if (a.rows > (int64_t)0x7FFFFFFF * 32)
    return pgh::err(PDLGB300_EUSERERROR, "prodover: too many rows");
  if (op == R_PROD) {
    if (in_dt == PDLGB300_F) return launch_typed<float, float>(a, S, s);
    if (in_dt == PDLGB300_D) return launch_typed<double, double>(a, S, s);
    return pgh::err(PDLGB300_EFATAL, "prod_seq: integer prodover has no early exit to keep");
  }
  PG_DISPATCH(in_dt, return launch_typed<typename TT<DT>::T, double>(a, S, s));
  return pgh::err(PDLGB300_EUSERERROR, "reduction: unsupported type %d", in_dt);
}

}  // namespace pg
