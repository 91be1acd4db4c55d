// scan.cu -- cumusumover / dcumusumover (lib/PDL/Ufunc.pd:120-140):
// b(n) = inclusive running sum of a(n); a bad element gives a bad output
// and leaves the running sum unchanged.
//
// Contiguous rows run warp-synchronously, one warp per row (k_scan_warp);
// long rows with few rows are cut into chunks whose totals are summed
// first.  Strided rows: one thread per row in the reference's order.
#include "args.cuh"
#include "f64sum.cuh"

namespace pg {

namespace {

struct FF2 {
  float hi, lo;
};
__device__ __forceinline__ FF2 ff2_add1(FF2 a, float x) {
  float s = __fadd_rn(a.hi, x);
  float bp = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
  return FF2{s, __fadd_rn(a.lo, e)};
}
__device__ __forceinline__ FF2 ff2_add(FF2 a, FF2 b) {
  float s = __fadd_rn(a.hi, b.hi);
  float bp = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  float h = __fadd_rn(s, e);
  return FF2{h, __fsub_rn(e, __fsub_rn(h, s))};
}

// Running-sum arithmetic in Out's type.
template <class In, class Out, bool COMP> struct ScanT {
  using Acc = std::conditional_t<std::is_integral_v<Out>, uns_t<Out>,
                                 std::conditional_t<std::is_same_v<Out, float> && COMP, FF2, Out>>;
  __device__ static Acc zero() {
    Acc a;
    memset(&a, 0, sizeof a);
    return a;
  }
  __device__ static Acc add1(Acc a, In v) {
    if constexpr (std::is_integral_v<Out>) return a + (Acc)(Out)v;
    else if constexpr (std::is_same_v<Acc, FF2>) return ff2_add1(a, (float)v);
    else return rn_add(a, (Out)v);
  }
  __device__ static Acc add(Acc a, Acc b) {
    if constexpr (std::is_integral_v<Out>) return a + b;
    else if constexpr (std::is_same_v<Acc, FF2>) return ff2_add(a, b);
    else return rn_add(a, b);
  }
  __device__ static Out value(Acc a) {
    if constexpr (std::is_integral_v<Out>) return (Out)a;
    else if constexpr (std::is_same_v<Acc, FF2>) return __fadd_rn(a.hi, a.lo);
    else return a;
  }
};

template <class T> __device__ __forceinline__ T shfl_up_any(T v, int d) {
  constexpr int W = (sizeof(T) + 3) / 4;
  union { T t; uint32_t w[W]; } u;
  u.t = v;
#pragma unroll
  for (int i = 0; i < W; i++) u.w[i] = __shfl_up_sync(0xffffffffu, u.w[i], d);
  return u.t;
}

template <class T> __device__ __forceinline__ T shfl_any(T v, int src) {
  constexpr int W = (sizeof(T) + 3) / 4;
  union { T t; uint32_t w[W]; } u;
  u.t = v;
#pragma unroll
  for (int i = 0; i < W; i++) u.w[i] = __shfl_sync(0xffffffffu, u.w[i], src);
  return u.t;
}
template <class T> __device__ __forceinline__ T shfl_down_any2(T v, int d) {
  constexpr int W = (sizeof(T) + 3) / 4;
  union { T t; uint32_t w[W]; } u;
  u.t = v;
#pragma unroll
  for (int i = 0; i < W; i++) u.w[i] = __shfl_down_sync(0xffffffffu, u.w[i], d);
  return u.t;
}

constexpr int SB = 256, SI = 8, STILE = SB * SI;

// Contiguous rows: one warp per row (or per chunk of a long row), warp-
// synchronous only -- no shared memory, no block barriers.  Each step a lane
// takes 32 contiguous bytes (two 16-byte vectors; 16 bytes for 1-2 byte
// types), totals them, the warp scans the lane totals with shuffles, and
// each lane writes its running sums with 16-byte stores; the next step's
// vectors are loaded before the current step is scanned.  The carry stays
// in registers.  Long rows with few rows are cut into chunks: chunk totals
// first (mode 1), then each chunk scanned from the sum of its row's earlier
// chunk totals, which its warp adds up itself (mode 2).
template <class In, class Out, bool BAD, bool COMP>
__global__ void __launch_bounds__(256) k_scan_warp(const ScanArgs g) {
  using S = ScanT<In, Out, COMP>;
  using Acc = typename S::Acc;
  constexpr int VEC = 16 / sizeof(In);
  constexpr int PER = sizeof(In) >= 4 ? 2 * VEC : VEC;  // elements per lane per step
  constexpr int STEP = 32 * PER;
  Bad<In> bv{from_bits<In>(g.abad), (bool)g.abad_isnan};
  const Out obad = from_bits<Out>(g.bbad);
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t units = g.rows * g.nchunk;
  for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < units;
       u += nwarps) {
    const int64_t row = u / g.nchunk;
    const int chunk = (int)(u - row * g.nchunk);
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const In *a = reinterpret_cast<const In *>(g.a) + offs[0];
    Out *b = reinterpret_cast<Out *>(g.b) + offs[1];
    int64_t lo = (int64_t)chunk * g.chunk;
    int64_t hi = lo + g.chunk < g.n ? lo + g.chunk : g.n;
    if (g.nchunk == 1) { lo = 0; hi = g.n; }
    const bool va = ((uintptr_t)(a + lo) % 16) == 0;
    const bool vb = ((uintptr_t)(b + lo) % 16) == 0 && ((PER * sizeof(Out)) % 16) == 0;
    Acc carry = S::zero();
    if (g.mode == 2 && chunk > 0) {
      const Acc *p = reinterpret_cast<const Acc *>(g.partials) + row * g.nchunk;
      Acc sacc = S::zero();
      for (int c = lane; c < chunk; c += 32) sacc = S::add(sacc, p[c]);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) sacc = S::add(sacc, shfl_down_any2(sacc, d));
      carry = shfl_any(sacc, 0);
    }
    auto load = [&](In (&v)[PER], int64_t s0) {
      const int64_t base = s0 + (int64_t)lane * PER;
      if (va && base + PER <= hi) {
#pragma unroll
        for (int q = 0; q < PER * (int)sizeof(In) / 16; q++) {
          float4 f = __ldcs(reinterpret_cast<const float4 *>(a + base) + q);
          memcpy(reinterpret_cast<char *>(v) + 16 * q, &f, 16);
        }
      } else {
#pragma unroll
        for (int j = 0; j < PER; j++) v[j] = base + j < hi ? a[base + j] : (In)0;
      }
    };
    In cur[PER], nxt[PER];
    if (lo < hi) load(cur, lo);
    Acc lanesum = S::zero();  // mode 1: totals only
    for (int64_t s0 = lo; s0 < hi; s0 += STEP) {
      if (s0 + STEP < hi) load(nxt, s0 + STEP);
      const int64_t base = s0 + (int64_t)lane * PER;
      bool good[PER];
#pragma unroll
      for (int j = 0; j < PER; j++) good[j] = base + j < hi && !(BAD && bv.is(cur[j]));
      Acc tot = S::zero();
      if constexpr (std::is_same_v<Out, double> && std::is_same_v<In, double> && !BAD) {
        F64Sum fs{0.0};
        double w[PER];
#pragma unroll
        for (int j = 0; j < PER; j++) w[j] = good[j] ? cur[j] : 0.0;
        fs.add_block<PER>(w);
        tot = fs.s;
      } else {
#pragma unroll
        for (int j = 0; j < PER; j++)
          if (good[j]) tot = S::add1(tot, cur[j]);
      }
      if (g.mode == 1) {
        lanesum = S::add(lanesum, tot);
      } else {
        Acc inc = tot;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          Acc o = shfl_up_any(inc, d);
          if (lane >= d) inc = S::add(o, inc);
        }
        Acc excl = shfl_up_any(inc, 1);
        if (lane == 0) excl = S::zero();
        const Acc wtot = shfl_any(inc, 31);
        Acc run = S::add(carry, excl);
        Out o[PER];
#pragma unroll
        for (int j = 0; j < PER; j++) {
          if (good[j]) {
            run = S::add1(run, cur[j]);
            o[j] = S::value(run);
          } else {
            o[j] = obad;
          }
        }
        if (vb && base + PER <= hi) {
#pragma unroll
          for (int q = 0; q < PER * (int)sizeof(Out) / 16; q++) {
            float4 f;
            memcpy(&f, reinterpret_cast<const char *>(o) + 16 * q, 16);
            __stcs(reinterpret_cast<float4 *>(b + base) + q, f);
          }
        } else {
#pragma unroll
          for (int j = 0; j < PER; j++)
            if (base + j < hi) b[base + j] = o[j];
        }
        carry = S::add(carry, wtot);
      }
#pragma unroll
      for (int j = 0; j < PER; j++) cur[j] = nxt[j];
    }
    if (g.mode == 1) {
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) lanesum = S::add(lanesum, shfl_down_any2(lanesum, d));
      if (lane == 0) reinterpret_cast<Acc *>(g.partials)[u] = lanesum;
    }
  }
}

// One thread per row, any increments, the reference's order.
template <class In, class Out, bool BAD, bool COMP>
__global__ void k_scan_thread(const ScanArgs g) {
  using S = ScanT<In, Out, COMP>;
  Bad<In> bv{from_bits<In>(g.abad), (bool)g.abad_isnan};
  const Out obad = from_bits<Out>(g.bbad);
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < g.rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const In *a = reinterpret_cast<const In *>(g.a) + offs[0];
    Out *b = reinterpret_cast<Out *>(g.b) + offs[1];
    auto run = S::zero();
    for (int64_t i = 0; i < g.n; i++) {
      In v = a[i * g.inc_a];
      if (BAD && bv.is(v)) {
        b[i * g.inc_b] = obad;
        continue;
      }
      run = S::add1(run, v);
      b[i * g.inc_b] = S::value(run);
    }
  }
}

template <class In, class Out, bool COMP>
pdlgb300_error scan_typed(ScanArgs g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.rows == 0) return e;
  const int nsm = pgh::num_sms();
  if (g.mode < 0) {  // thread kernel
    int64_t grid = std::min<int64_t>((g.rows + 127) / 128, (int64_t)nsm * 32);
    if (g.bad) k_scan_thread<In, Out, true, COMP><<<(int)grid, 128, 0, s>>>(g);
    else k_scan_thread<In, Out, false, COMP><<<(int)grid, 128, 0, s>>>(g);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_scan_thread")) return e;
    pgh::record_kernel("k_scan_thread", grid, 128);
    return e;
  }
  // contiguous rows: warp per row (per chunk for long rows)
  auto warp_kernel = [&](ScanArgs a) {
    const int64_t units = a.rows * a.nchunk;
    const int64_t grid = std::min<int64_t>((units + 7) / 8, (int64_t)nsm * 16);
    if (a.bad) k_scan_warp<In, Out, true, COMP><<<(int)grid, SB, 0, s>>>(a);
    else k_scan_warp<In, Out, false, COMP><<<(int)grid, SB, 0, s>>>(a);
    pgh::record_kernel("k_scan_warp", grid, SB);
    return cudaGetLastError();
  };
  if (g.nchunk <= 1) {
    g.mode = 0;
    g.nchunk = 1;
    if (!pgh::cuda_check(warp_kernel(g), &e, "k_scan_warp")) return e;
    return e;
  }
  ScanArgs a = g;
  a.mode = 1;
  if (!pgh::cuda_check(warp_kernel(a), &e, "k_scan_warp(totals)")) return e;
  a.mode = 2;
  if (!pgh::cuda_check(warp_kernel(a), &e, "k_scan_warp(scan)")) return e;
  return e;
}

}  // namespace

// dop: 0 cumusumover (int+), 1 dcumusumover (double)
pdlgb300_error launch_cumusum(int dop, int in_dt, ScanArgs g, cudaStream_t s) {
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    if (dop == 1) return scan_typed<In, double, false>(g, s);
    if constexpr (std::is_same_v<OutP, float>)
      if (g.f32_comp) return scan_typed<In, OutP, true>(g, s);
    return scan_typed<In, OutP, false>(g, s);
  });
  return pgh::err(PDLGB300_EUSERERROR, "cumusumover: unsupported type %d", in_dt);
}

size_t scan_acc_size(int dop, int in_dt, int comp) {
  size_t r = 0;
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    if (dop == 1) r = sizeof(typename ScanT<In, double, false>::Acc);
    else if (comp) r = sizeof(typename ScanT<In, OutP, true>::Acc);
    else r = sizeof(typename ScanT<In, OutP, false>::Acc);
  });
  return r;
}

}  // namespace pg
