// scan.cu -- cumusumover / dcumusumover (lib/PDL/Ufunc.pd:120-140):
// b(n) = inclusive running sum of a(n); a bad element gives a bad output
// and leaves the running sum unchanged.
//
// Contiguous rows: one block walks a row in tiles of 256 x 8 elements,
// staged through shared memory for coalesced loads and stores.  Each thread
// first totals its 8 elements (float64: one F64Sum block, integer pipe), the
// block scans the thread totals, then each thread re-walks its elements
// from its exclusive prefix with one add per element.  Long rows with few
// rows are cut into chunks: chunk totals, a per-row exclusive scan of the
// totals, then every chunk scanned from its carry (three passes, no
// inter-block waiting).  Strided rows: one thread per row in the
// reference's order.
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

constexpr int SB = 256, SI = 8, STILE = SB * SI;

template <class In, class Out, bool BAD, bool COMP>
__global__ void __launch_bounds__(SB) k_scan_rows(const ScanArgs g) {
  using S = ScanT<In, Out, COMP>;
  using Acc = typename S::Acc;
  __shared__ In s_in[STILE];
  __shared__ Out s_out[STILE];
  __shared__ Acc s_warp[SB / 32];
  __shared__ Acc s_carry;
  Bad<In> bv{from_bits<In>(g.abad), (bool)g.abad_isnan};
  const Out obad = from_bits<Out>(g.bbad);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t units = g.rows * g.nchunk;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    int64_t row = u / g.nchunk;
    int chunk = (int)(u - row * g.nchunk);
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const In *a = reinterpret_cast<const In *>(g.a) + offs[0];
    Out *b = reinterpret_cast<Out *>(g.b) + offs[1];
    int64_t lo = (int64_t)chunk * g.chunk;
    int64_t hi = lo + g.chunk < g.n ? lo + g.chunk : g.n;
    if (g.nchunk == 1) { lo = 0; hi = g.n; }
    Acc carry = S::zero();
    if (g.mode == 2) carry = reinterpret_cast<const Acc *>(g.partials)[u];
    for (int64_t t0 = lo; t0 < hi; t0 += STILE) {
      const int64_t cnt = hi - t0 < STILE ? hi - t0 : STILE;
      __syncthreads();
#pragma unroll
      for (int k = 0; k < SI; k++) {
        int j = tid + k * SB;
        if (j < cnt) s_in[j] = __ldcs(a + t0 + j);
      }
      __syncthreads();
      In v[SI];
      bool ok[SI];
#pragma unroll
      for (int j = 0; j < SI; j++) {
        int idx = tid * SI + j;
        v[j] = idx < cnt ? s_in[idx] : (In)0;
        ok[j] = idx < cnt && !(BAD && bv.is(v[j]));
      }
      // thread total
      Acc tot = S::zero();
      if constexpr (std::is_same_v<Out, double> && std::is_same_v<In, double> && !BAD) {
        F64Sum fs{0.0};
        double w[SI];
#pragma unroll
        for (int j = 0; j < SI; j++) w[j] = ok[j] ? v[j] : 0.0;
        fs.add_block<SI>(w);
        tot = fs.s;
      } else {
#pragma unroll
        for (int j = 0; j < SI; j++)
          if (ok[j]) tot = S::add1(tot, v[j]);
      }
      // block exclusive scan of thread totals
      Acc inc = tot;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        Acc o = shfl_up_any(inc, d);
        if (lane >= d) inc = S::add(o, inc);
      }
      if (lane == 31) s_warp[warp] = inc;
      __syncthreads();
      if (warp == 0) {
        Acc w = lane < SB / 32 ? s_warp[lane] : S::zero();
#pragma unroll
        for (int d = 1; d < SB / 32; d <<= 1) {
          Acc o = shfl_up_any(w, d);
          if (lane >= d) w = S::add(o, w);
        }
        if (lane < SB / 32) s_warp[lane] = w;  // inclusive warp prefixes
      }
      __syncthreads();
      Acc excl = shfl_up_any(inc, 1);
      if (lane == 0) excl = S::zero();
      if (warp > 0) excl = S::add(s_warp[warp - 1], excl);
      Acc blocktot = s_warp[SB / 32 - 1];
      if (g.mode != 1) {
        Acc run = S::add(carry, excl);
#pragma unroll
        for (int j = 0; j < SI; j++) {
          int idx = tid * SI + j;
          if (idx < cnt) {
            if (ok[j]) {
              run = S::add1(run, v[j]);
              s_out[idx] = S::value(run);
            } else {
              s_out[idx] = obad;
            }
          }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SI; k++) {
          int j = tid + k * SB;
          if (j < cnt) b[t0 + j] = s_out[j];
        }
      }
      carry = S::add(carry, blocktot);
    }
    if (g.mode == 1 && tid == 0) reinterpret_cast<Acc *>(g.partials)[u] = carry;
  }
}

// Per-row exclusive scan of chunk totals, in place.
template <class In, class Out, bool COMP>
__global__ void k_scan_carries(const ScanArgs g) {
  using S = ScanT<In, Out, COMP>;
  using Acc = typename S::Acc;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < g.rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    Acc *p = reinterpret_cast<Acc *>(g.partials) + row * g.nchunk;
    Acc run = S::zero();
    for (int c = 0; c < g.nchunk; c++) {
      Acc t = p[c];
      p[c] = run;
      run = S::add(run, t);
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
  auto rows_kernel = [&](ScanArgs a) {
    int64_t units = a.rows * a.nchunk;
    int64_t grid = std::min<int64_t>(units, (int64_t)nsm * 64);
    if (a.bad) k_scan_rows<In, Out, true, COMP><<<(int)grid, SB, 0, s>>>(a);
    else k_scan_rows<In, Out, false, COMP><<<(int)grid, SB, 0, s>>>(a);
    pgh::record_kernel("k_scan_rows", grid, SB);
    return cudaGetLastError();
  };
  if (g.nchunk <= 1) {
    g.mode = 0;
    g.nchunk = 1;
    if (!pgh::cuda_check(rows_kernel(g), &e, "k_scan_rows")) return e;
    return e;
  }
  ScanArgs a = g;
  a.mode = 1;
  if (!pgh::cuda_check(rows_kernel(a), &e, "k_scan_rows(totals)")) return e;
  int64_t grid = std::min<int64_t>((g.rows + 127) / 128, 4096);
  k_scan_carries<In, Out, COMP><<<(int)grid, 128, 0, s>>>(g);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_scan_carries")) return e;
  pgh::record_kernel("k_scan_carries", grid, 128);
  a.mode = 2;
  if (!pgh::cuda_check(rows_kernel(a), &e, "k_scan_rows(carry)")) return e;
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
