// scan.cu -- cumusumover / dcumusumover (lib/PDL/Ufunc.pd:120-140):
// b(n) = inclusive running sum of a(n); a bad element gives a bad output
// and leaves the running sum unchanged.
//
// Contiguous 16-byte aligned rows of 4- and 8-byte types: many rows of
// equally wide types run a block per row (k_scan_rowblk: the row's 32 KiB
// chunks in order, the carry in registers, the next load in flight); other
// rows the chained single-pass scan (k_scan_chain: a block per chunk of
// 64 KiB, or 32 KiB for 8-byte types, its carry found by decoupled
// look-back across the row's earlier chunks).  Other contiguous rows run
// warp-synchronously, one warp per row (k_scan_warp); long rows with few
// rows are cut into chunks whose totals are summed first.  Strided rows:
// one thread per row in the reference's order.
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

// Running arithmetic in Out's type.  M: 0 sum, 1 compensated float32 sum,
// 2 product (cumuprodover, lib/PDL/Ufunc.pd:120-140 with `*=`).  zero() is
// the identity; pad() the input value that changes nothing.
template <class In, class Out, int M> struct ScanT {
  static constexpr bool kProd = M == 2;
  using Acc = std::conditional_t<std::is_integral_v<Out>, uns_t<Out>,
                                 std::conditional_t<std::is_same_v<Out, float> && M == 1, FF2, Out>>;
  __device__ static Acc zero() {
    Acc a;
    if constexpr (kProd) {
      a = (Acc)1;
    } else {
      memset(&a, 0, sizeof a);
    }
    return a;
  }
  __device__ static In pad() { return kProd ? (In)1 : (In)0; }
  __device__ static Acc add1(Acc a, In v) {
    if constexpr (kProd) {
      if constexpr (std::is_integral_v<Out>) return (Acc)wmul<Out>((Out)a, (Out)v);
      else return rn_mul(a, (Out)v);
    } else if constexpr (std::is_integral_v<Out>) {
      return a + (Acc)(Out)v;
    } else if constexpr (std::is_same_v<Acc, FF2>) {
      return ff2_add1(a, (float)v);
    } else {
      return rn_add(a, (Out)v);
    }
  }
  __device__ static Acc add(Acc a, Acc b) {
    if constexpr (kProd) {
      if constexpr (std::is_integral_v<Out>) return (Acc)wmul<Out>((Out)a, (Out)b);
      else return rn_mul(a, b);
    } else if constexpr (std::is_integral_v<Out>) {
      return a + b;
    } else if constexpr (std::is_same_v<Acc, FF2>) {
      return ff2_add(a, b);
    } else {
      return rn_add(a, b);
    }
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
template <class In, class Out, bool BAD, int COMP>
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
      if constexpr (std::is_same_v<Out, double> && std::is_same_v<In, double> && !BAD && !S::kProd) {
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

// ----------------------------------------------------------- chained scan
// Contiguous, 16-byte aligned rows of 4- and 8-byte types: one block per
// chunk of a row (16384 elements of 4 bytes, 4096 of 8), each thread owning
// 128 contiguous bytes.  Loads are striped 16-byte cp.async copies into a
// shared-memory tile whose 16-byte slots are XOR-swizzled by lane, so both
// the striped copies and each thread's blocked reads are free of bank
// conflicts; outputs go back the same way and leave as coalesced 16-byte
// stores.  Inside the chunk: thread totals, a warp scan, a block scan.
// Across the chunks of a row the carry travels by decoupled look-back:
// each chunk publishes its total (A), then its inclusive prefix (P), in a
// slot tagged with a 64-bit unit id (no reset between launches); a chunk
// reads 32 predecessors per round (one per lane) and stops at the nearest P.
// Chunks are taken in blockIdx order, so a chunk only waits on chunks whose
// blocks were dispatched before it.  Every wait is bounded: on timeout the
// status word gets bit 4 and the chunk goes on with what it has.
// threads per chained-scan block: 512 for 4-byte equal-width types (half
// as many chunks to chain through look-back), 256 otherwise (shared memory)
template <class In, class Out> constexpr int chain_threads() {
  return (sizeof(In) == 4 && sizeof(Out) == 4) ? 512 : 256;
}
constexpr int LB_PER_LANE = 1;  // look-back slots read per lane per round

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
template <class A> __device__ __forceinline__ unsigned long long acc_to_u64(A a) {
  static_assert(sizeof(A) <= 8, "look-back values are at most 8 bytes");
  unsigned long long u = 0;
  memcpy(&u, &a, sizeof a);
  return u;
}
template <class A> __device__ __forceinline__ A u64_to_acc(unsigned long long u) {
  A a;
  memcpy(&a, &u, sizeof a);
  return a;
}

// state 1: aggregate only, 2: inclusive prefix
__device__ __forceinline__ void chain_publish(ChainSlot *sl, uint64_t gid, int state,
                                              unsigned long long v) {
  st_relaxed_u64(state == 2 ? &sl->incl : &sl->agg, v);
  st_release_u64(&sl->flag, (gid << 2) | (uint64_t)state);
}

// Look-back of chunk c > 0 of a row (warp 0): the sum of its predecessors'
// values up to the nearest inclusive prefix.  gid is the chunk's unit id.
template <class S, class Acc>
__device__ __forceinline__ Acc chain_lookback(const ScanArgs &g, ChainSlot *slots, uint64_t gid,
                                              int c, int lane) {
  Acc excl = S::zero();
  const uint64_t gid0 = gid - (uint64_t)c;  // the row's chunk 0
  int64_t pos = c - 1;                      // newest predecessor not yet added
  constexpr int WIN = 32 * LB_PER_LANE;
  while (true) {
    int st[LB_PER_LANE];
    unsigned long long val[LB_PER_LANE];
    int kp = 1 << 30;
#pragma unroll
    for (int qq = 0; qq < LB_PER_LANE; qq++) {
      const int k = lane * LB_PER_LANE + qq;
      const int64_t p = pos - k;
      st[qq] = 3;  // before the row's start: nothing to add, stop here
      val[qq] = 0;
      if (p >= 0) {
        const uint64_t gp = gid0 + (uint64_t)p;
        ChainSlot *sl = &slots[gp & g.status_mask];
        unsigned long long f = 0;
        int spins = 0;
        while (true) {
          f = ld_acquire_u64(&sl->flag);
          if ((f >> 2) == gp && (f & 3)) break;
          if (++spins > (1 << 21)) {
            atomicOr(g.err, 4);
            f = (gp << 2) | 3;
            break;
          }
          __nanosleep(32);
        }
        st[qq] = (int)(f & 3);
        if (st[qq] == 1) val[qq] = ld_relaxed_u64(&sl->agg);
        else if (st[qq] == 2) val[qq] = ld_relaxed_u64(&sl->incl);
      }
      if (st[qq] >= 2 && k < kp) kp = k;
    }
    __syncwarp();
    const int kmin = __reduce_min_sync(0xffffffffu, kp);
    Acc part = S::zero();
#pragma unroll
    for (int qq = LB_PER_LANE - 1; qq >= 0; qq--) {
      const int k = lane * LB_PER_LANE + qq;
      if (k <= kmin && st[qq] != 3) part = S::add(part, u64_to_acc<Acc>(val[qq]));
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) part = S::add(shfl_down_any2(part, d), part);
    part = shfl_any(part, 0);
    excl = S::add(part, excl);
    if (kmin < WIN) break;
    pos -= WIN;
  }
  return excl;
}

// Chunk geometry of the chained scans: CB threads, ITEMS = 128 / sizeof(In)
// items per thread, one warp's 32 x ITEMS items in a 4 KiB swizzled tile
// (a lane's 16-byte vector q sits in slot q ^ (lane & 7)).
template <class In, int CB> struct ChainGeom {
  static constexpr int ITEMS = 128 / sizeof(In);
  static constexpr int VEC = 16 / sizeof(In);
  static constexpr int NV = ITEMS / VEC;  // 8 input vectors per thread
  static constexpr int WSPAN = 32 * ITEMS;
  static constexpr int CH = (CB / 32) * WSPAN;
  static constexpr int WIN_B = 32 * NV * 16;
};

// Start the load of unit u's chunk into a warp's input tile at sin: full
// warp spans as 16-byte cp.async copies (not waited for here), the ragged
// end of a row as plain loads with the identity past the row's end.
template <class In, class Out, int COMP, int CB>
__device__ __forceinline__ void chain_load(const ScanArgs &g, int64_t u, uint32_t sin, int lane,
                                           int warp) {
  using S = ScanT<In, Out, COMP>;
  using GM = ChainGeom<In, CB>;
  constexpr int NV = GM::NV, VEC = GM::VEC, ITEMS = GM::ITEMS;
  const int64_t row = u / g.nchunk;
  const int c = (int)(u - row * g.nchunk);
  int64_t offs[MAXP];
  loop_offsets(g.L, row, offs);
  const In *a = reinterpret_cast<const In *>(g.a) + offs[0];
  const int64_t lo = (int64_t)c * GM::CH;
  const int64_t hi = lo + GM::CH < g.n ? lo + GM::CH : g.n;
  const int64_t wlo = lo + (int64_t)warp * GM::WSPAN;
  if (wlo + GM::WSPAN <= hi) {
#pragma unroll
    for (int r = 0; r < NV; r++) {
      const int gv = r * 32 + lane;
      const int own = gv / NV, q = gv % NV;
      const uint32_t dst = sin + (uint32_t)(own * NV * 16 + ((q ^ (own & 7)) * 16));
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst),
                   "l"(a + wlo + (int64_t)gv * VEC)
                   : "memory");
    }
  } else {
    const int64_t t0 = wlo + (int64_t)lane * ITEMS;
    const int64_t left = hi - t0;
    const int nvalid = left <= 0 ? 0 : (left >= ITEMS ? ITEMS : (int)left);
#pragma unroll
    for (int q = 0; q < NV; q++) {
      In x[VEC];
#pragma unroll
      for (int e = 0; e < VEC; e++) x[e] = q * VEC + e < nvalid ? a[t0 + q * VEC + e] : S::pad();
      float4 f;
      memcpy(&f, x, 16);
      const uint32_t dst = sin + (uint32_t)(lane * NV * 16 + ((q ^ (lane & 7)) * 16));
      asm volatile("st.shared.v4.f32 [%0], {%1,%2,%3,%4};" ::"r"(dst), "f"(f.x), "f"(f.y),
                   "f"(f.z), "f"(f.w)
                   : "memory");
    }
  }
}

// Scan unit u's chunk from the warp's loaded input tile at sin: thread
// totals, warp and block scans of the totals, the look-back across the
// row's earlier chunks (warp 0, while the other warps wait at the block
// barrier), the running sums written to the output tile at sout (the input
// tile itself when the types are equally wide), then 16-byte streaming
// stores.  Calls __syncthreads twice: every thread of the block runs it.
//
// LOOK false: the chunks of a row are scanned in order by one block, and the
// exclusive prefix is `carry` (warp 0's, advanced here by the chunk total).
template <class In, class Out, int BM, int COMP, int CB, bool LOOK = true>
__device__ __forceinline__ void chain_body(const ScanArgs &g, int64_t u, uint32_t sin,
                                           uint32_t sout, typename ScanT<In, Out, COMP>::Acc *s_w,
                                           int lane, int warp,
                                           typename ScanT<In, Out, COMP>::Acc &carry) {
  using S = ScanT<In, Out, COMP>;
  using Acc = typename S::Acc;
  using GM = ChainGeom<In, CB>;
  constexpr int ITEMS = GM::ITEMS, VEC = GM::VEC, NV = GM::NV;
  constexpr int VO = 16 / sizeof(Out);  // outputs per 16-byte vector
  constexpr int OV = ITEMS / VO;        // output vectors per thread
  static_assert(NV == 8 && (OV == 8 || OV == 16), "swizzle needs 8 or 16 slots per row");
  const int64_t row = u / g.nchunk;
  const int c = (int)(u - row * g.nchunk);
  const int64_t lo = (int64_t)c * GM::CH;
  const int64_t hi = lo + GM::CH < g.n ? lo + GM::CH : g.n;
  const int64_t wlo = lo + (int64_t)warp * GM::WSPAN;
  const bool fast = wlo + GM::WSPAN <= hi;
  const In bad = from_bits<In>(g.abad);
  auto slot_in = [&](int q) { return sin + (uint32_t)(lane * NV * 16 + ((q ^ (lane & 7)) * 16)); };
  auto ldin = [&](int q, In (&x)[VEC]) {
    float4 f;
    asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(f.x), "=f"(f.y), "=f"(f.z), "=f"(f.w)
                 : "r"(slot_in(q)));
    memcpy(x, &f, 16);
  };
  const int64_t t0 = wlo + (int64_t)lane * ITEMS;
  int nvalid = ITEMS;  // items of this thread inside the row (ragged end)
  if (!fast) {
    const int64_t left = hi - t0;
    nvalid = left <= 0 ? 0 : (left >= ITEMS ? ITEMS : (int)left);
  }
  // items past the row's end hold the identity and are never stored
  auto good = [&](In x) { return !is_bad<In, BM>(x, bad); };

  // thread total
  Acc tot = S::zero();
  if constexpr (std::is_same_v<In, double> && std::is_same_v<Out, double> && !S::kProd) {
    // float64: two exact 8-element blocks (integer alignment, one FP64 add each)
    F64Sum fs{0.0};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      double w[NV];
#pragma unroll
      for (int q = 0; q < NV / 2; q++) {
        In x[VEC];
        ldin(h * (NV / 2) + q, x);
#pragma unroll
        for (int e = 0; e < VEC; e++) w[q * VEC + e] = good(x[e]) ? x[e] : 0.0;
      }
      fs.add_block<NV>(w);
    }
    tot = fs.s;
  } else {
#pragma unroll
    for (int q = 0; q < NV; q++) {
      In x[VEC];
      ldin(q, x);
#pragma unroll
      for (int e = 0; e < VEC; e++)
        if (good(x[e])) tot = S::add1(tot, x[e]);
    }
  }
  // warp scan of the thread totals
  Acc inc = tot;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    Acc o = shfl_up_any(inc, d);
    if (lane >= d) inc = S::add(o, inc);
  }
  Acc lex = shfl_up_any(inc, 1);
  if (lane == 0) lex = S::zero();
  if (lane == 31) s_w[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    constexpr int NW = CB / 32;
    Acc wt = lane < NW ? s_w[lane] : S::zero();
#pragma unroll
    for (int d = 1; d < NW; d <<= 1) {
      Acc o = shfl_up_any(wt, d);
      if (lane >= d) wt = S::add(o, wt);
    }
    const Acc agg = shfl_any(wt, NW - 1);
    Acc wex = shfl_up_any(wt, 1);
    if (lane == 0) wex = S::zero();
    Acc excl = S::zero();
    if constexpr (!LOOK) {
      excl = carry;
      carry = S::add(carry, agg);
    } else if (g.nchunk > 1) {
      ChainSlot *slots = reinterpret_cast<ChainSlot *>(g.status);
      const uint64_t gid = g.gid_base + (uint64_t)u;
      if (c == 0) {
        if (lane == 0) chain_publish(&slots[gid & g.status_mask], gid, 2, acc_to_u64(agg));
      } else {
        if (lane == 0) chain_publish(&slots[gid & g.status_mask], gid, 1, acc_to_u64(agg));
        excl = chain_lookback<S, Acc>(g, slots, gid, c, lane);
        if (lane == 0)
          chain_publish(&slots[gid & g.status_mask], gid, 2, acc_to_u64(S::add(excl, agg)));
      }
    }
    if (lane < NW) s_w[lane] = S::add(excl, wex);
  }
  __syncthreads();
  Acc run = S::add(s_w[warp], lex);

  // running sums: read a vector, write its outputs (in place when as wide)
  const Out obad = from_bits<Out>(g.bbad);
#pragma unroll
  for (int q = 0; q < NV; q++) {
    In x[VEC];
    ldin(q, x);
    Out o[VEC];
#pragma unroll
    for (int e = 0; e < VEC; e++) {
      if (good(x[e])) {
        run = S::add1(run, x[e]);
        o[e] = S::value(run);
      } else {
        o[e] = obad;
      }
    }
#pragma unroll
    for (int h = 0; h < VEC / VO; h++) {  // 1 (equal width) or 2 output vectors
      const int pv = q * (VEC / VO) + h;
      float4 f;
      memcpy(&f, &o[h * VO], 16);
      const uint32_t dst = sout + (uint32_t)(lane * OV * 16 + ((pv ^ (lane & 7)) * 16));
      asm volatile("st.shared.v4.f32 [%0], {%1,%2,%3,%4};" ::"r"(dst), "f"(f.x), "f"(f.y),
                   "f"(f.z), "f"(f.w)
                   : "memory");
    }
  }
  __syncwarp();
  int64_t offs[MAXP];
  loop_offsets(g.L, row, offs);
  Out *b = reinterpret_cast<Out *>(g.b) + offs[1];
  if (fast) {
#pragma unroll
    for (int r = 0; r < OV; r++) {
      const int gv = r * 32 + lane;
      const int own = gv / OV, pv = gv % OV;
      const uint32_t src = sout + (uint32_t)(own * OV * 16 + ((pv ^ (own & 7)) * 16));
      float4 f;
      asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];"
                   : "=f"(f.x), "=f"(f.y), "=f"(f.z), "=f"(f.w)
                   : "r"(src));
      __stcs(reinterpret_cast<float4 *>(b + wlo + (int64_t)gv * VO), f);
    }
  } else {
    for (int j = 0; j < nvalid; j++) {
      const int pv = j / VO;
      const uint32_t src = sout + (uint32_t)(lane * OV * 16 + ((pv ^ (lane & 7)) * 16)) +
                           (uint32_t)((j % VO) * sizeof(Out));
      Out o;
      if constexpr (sizeof(Out) == 8) {
        unsigned long long w;
        asm volatile("ld.shared.u64 %0, [%1];" : "=l"(w) : "r"(src));
        memcpy(&o, &w, 8);
      } else {
        unsigned int w;
        asm volatile("ld.shared.u32 %0, [%1];" : "=r"(w) : "r"(src));
        memcpy(&o, &w, 4);
      }
      b[t0 + j] = o;
    }
  }
  __syncwarp();
}

// One block per chunk.  The chunk's input stays in the swizzled tile (read
// once for the thread totals, once for the running sums), so a thread holds
// no input registers across the block barriers and more blocks fit on an SM
// to cover the look-back latency.  Equal-width outputs overwrite their input
// slots; wider outputs (float32 -> float64) use a second, larger tile.
template <class In, class Out, int BM, int COMP>
__global__ void __launch_bounds__(chain_threads<In, Out>(), (sizeof(In) == 4 && sizeof(Out) == 4) ? 3 : 4)
    k_scan_chain(const ScanArgs g, int64_t u0) {
  constexpr int CB = chain_threads<In, Out>();
  using S = ScanT<In, Out, COMP>;
  using GM = ChainGeom<In, CB>;
  constexpr int OV = GM::ITEMS / (16 / sizeof(Out));
  constexpr int WOUT_B = OV == GM::NV ? 0 : 32 * OV * 16;  // separate output tile per warp
  extern __shared__ __align__(16) unsigned char sm_tile[];
  __shared__ typename S::Acc s_w[CB / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t sin = (uint32_t)__cvta_generic_to_shared(sm_tile) + (uint32_t)(warp * GM::WIN_B);
  const uint32_t sout = OV == GM::NV ? sin
                                     : (uint32_t)__cvta_generic_to_shared(sm_tile) +
                                           (uint32_t)((CB / 32) * GM::WIN_B + warp * WOUT_B);
  const int64_t u = u0 + blockIdx.x;
  chain_load<In, Out, COMP, CB>(g, u, sin, lane, warp);
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
  __syncwarp();
  typename S::Acc carry = S::zero();
  chain_body<In, Out, BM, COMP, CB>(g, u, sin, sout, s_w, lane, warp, carry);
}

// Many rows of equally wide types: one block per row walks the row's
// chunks in order, the carry in warp 0's registers (no look-back, no
// flags), the next chunk's load in flight while the current one is scanned.
// Blocks of 256 threads and two 32 KiB tiles: three blocks per SM, three
// independent rows in progress on each.
constexpr int ROWBLK_CB = 256;
template <class In> constexpr size_t rowblk_smem() { return (size_t)2 * ROWBLK_CB * 128; }

template <class In, class Out, int BM, int COMP>
__global__ void __launch_bounds__(ROWBLK_CB, 3) k_scan_rowblk(const ScanArgs g) {
  static_assert(sizeof(In) == sizeof(Out), "the tiles hold equal-width outputs in place");
  using S = ScanT<In, Out, COMP>;
  constexpr int CB = ROWBLK_CB;
  using GM = ChainGeom<In, CB>;
  constexpr uint32_t STAGE_B = (uint32_t)CB * 128;
  extern __shared__ __align__(16) unsigned char sm_tile[];
  __shared__ typename S::Acc s_w[CB / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(sm_tile) + (uint32_t)(warp * GM::WIN_B);
  for (int64_t row = blockIdx.x; row < g.rows; row += gridDim.x) {
    const int64_t u0 = row * g.nchunk;
    chain_load<In, Out, COMP, CB>(g, u0, base, lane, warp);
    asm volatile("cp.async.commit_group;" ::: "memory");
    typename S::Acc carry = S::zero();
    for (int c = 0; c < g.nchunk; c++) {
      const uint32_t t = base + (uint32_t)(c & 1) * STAGE_B;
      // the other tile held chunk c - 1, read and stored already
      if (c + 1 < g.nchunk)
        chain_load<In, Out, COMP, CB>(g, u0 + c + 1, base + (uint32_t)((c + 1) & 1) * STAGE_B,
                                      lane, warp);
      asm volatile("cp.async.commit_group;\ncp.async.wait_group 1;" ::: "memory");
      __syncwarp();
      chain_body<In, Out, BM, COMP, CB, false>(g, u0 + c, t, t, s_w, lane, warp, carry);
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// One thread per row, any increments, the reference's order.
template <class In, class Out, bool BAD, int COMP>
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

template <class In, class Out> constexpr bool chain_ok() {
  return (sizeof(In) == 4 || sizeof(In) == 8) &&
         (sizeof(Out) == sizeof(In) || sizeof(Out) == 2 * sizeof(In));
}

template <class In, class Out, int COMP>
pdlgb300_error scan_chain_typed(ScanArgs g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if constexpr (chain_ok<In, Out>()) {
    constexpr int ITEMS = 128 / sizeof(In);
    constexpr int CB = chain_threads<In, Out>();
    constexpr size_t smem = (size_t)CB * 128 + (sizeof(Out) == sizeof(In) ? 0 : (size_t)CB * ITEMS * sizeof(Out));
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_scan_chain<In, Out, 0, COMP>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      cudaFuncSetAttribute(k_scan_chain<In, Out, 1, COMP>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      cudaFuncSetAttribute(k_scan_chain<In, Out, 2, COMP>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      cudaFuncSetAttribute(k_scan_chain<In, Out, 0, COMP>,
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      cudaFuncSetAttribute(k_scan_chain<In, Out, 1, COMP>,
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      cudaFuncSetAttribute(k_scan_chain<In, Out, 2, COMP>,
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      attr = true;
    }
    const int64_t units = g.rows * g.nchunk;
    for (int64_t u0 = 0; u0 < units; u0 += (int64_t)1 << 30) {
      const int grid = (int)std::min<int64_t>(units - u0, (int64_t)1 << 30);
      if (!g.bad) k_scan_chain<In, Out, 0, COMP><<<grid, CB, smem, s>>>(g, u0);
      else if (g.abad_isnan) k_scan_chain<In, Out, 2, COMP><<<grid, CB, smem, s>>>(g, u0);
      else k_scan_chain<In, Out, 1, COMP><<<grid, CB, smem, s>>>(g, u0);
      if (!pgh::cuda_check(cudaGetLastError(), &e, "k_scan_chain")) return e;
      pgh::record_kernel("k_scan_chain", grid, CB);
    }
  } else {
    e = pgh::err(PDLGB300_EFATAL, "chained scan: unsupported type pair");
  }
  return e;
}

template <class In, class Out, int COMP>
pdlgb300_error scan_rowblk_typed(ScanArgs g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if constexpr (sizeof(In) == sizeof(Out) && chain_ok<In, Out>()) {
    constexpr size_t smem = rowblk_smem<In>();
    static bool attr = false;
    if (!attr) {
      for (void *k : {(void *)k_scan_rowblk<In, Out, 0, COMP>, (void *)k_scan_rowblk<In, Out, 1, COMP>,
                      (void *)k_scan_rowblk<In, Out, 2, COMP>}) {
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      }
      attr = true;
    }
    const int grid = (int)std::min<int64_t>(g.rows, (int64_t)1 << 30);
    if (!g.bad) k_scan_rowblk<In, Out, 0, COMP><<<grid, ROWBLK_CB, smem, s>>>(g);
    else if (g.abad_isnan) k_scan_rowblk<In, Out, 2, COMP><<<grid, ROWBLK_CB, smem, s>>>(g);
    else k_scan_rowblk<In, Out, 1, COMP><<<grid, ROWBLK_CB, smem, s>>>(g);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_scan_rowblk")) return e;
    pgh::record_kernel("k_scan_rowblk", grid, ROWBLK_CB);
  } else {
    e = pgh::err(PDLGB300_EFATAL, "row-block scan: unsupported type pair");
  }
  return e;
}

template <class In, class Out> constexpr int64_t chain_chunk() {
  if constexpr (chain_ok<In, Out>()) return (int64_t)chain_threads<In, Out>() * (128 / sizeof(In));
  return 0;
}

template <class In, class Out, int COMP>
pdlgb300_error scan_typed(ScanArgs g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.rows == 0) return e;
  if (g.mode == 4) return scan_rowblk_typed<In, Out, COMP>(g, s);
  if (g.status || g.mode == 3) return scan_chain_typed<In, Out, COMP>(g, s);
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

// dop: 0 cumusumover (int+), 1 dcumusumover (double), 2 cumuprodover
// (int+), 3 dcumuprodover (double)
pdlgb300_error launch_cumusum(int dop, int in_dt, ScanArgs g, cudaStream_t s) {
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    if (dop == 1) return scan_typed<In, double, 0>(g, s);
    if (dop == 2) return scan_typed<In, OutP, 2>(g, s);
    if (dop == 3) return scan_typed<In, double, 2>(g, s);
    if constexpr (std::is_same_v<OutP, float>)
      if (g.f32_comp) return scan_typed<In, OutP, 1>(g, s);
    return scan_typed<In, OutP, 0>(g, s);
  });
  return pgh::err(PDLGB300_EUSERERROR, "cumusumover: unsupported type %d", in_dt);
}

// elements per chunk of the row-block scan (0: not used for this op/type)
int64_t scan_rowblk_chunk(int dop, int in_dt) {
  int64_t r = 0;
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    if (dop == 1 || dop == 3) {
      if constexpr (sizeof(In) == sizeof(double) && chain_ok<In, double>())
        r = (int64_t)ROWBLK_CB * (128 / sizeof(In));
    } else if constexpr (sizeof(In) == sizeof(OutP) && chain_ok<In, OutP>()) {
      r = (int64_t)ROWBLK_CB * (128 / sizeof(In));
    }
  });
  return r;
}

int64_t scan_chain_chunk(int dop, int in_dt, int comp) {
  int64_t r = 0;
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    (void)comp;
    if (dop == 1 || dop == 3) r = chain_chunk<In, double>();
    else r = chain_chunk<In, OutP>();
  });
  return r;
}

size_t scan_acc_size(int dop, int in_dt, int comp) {
  size_t r = 0;
  PG_DISPATCH(in_dt, {
    using In = typename TT<DT>::T;
    using OutP = typename TT<intplus(DT)>::T;
    if (dop == 1) r = sizeof(typename ScanT<In, double, 0>::Acc);
    else if (dop == 2) r = sizeof(typename ScanT<In, OutP, 2>::Acc);
    else if (dop == 3) r = sizeof(typename ScanT<In, double, 2>::Acc);
    else if (comp) r = sizeof(typename ScanT<In, OutP, 1>::Acc);
    else r = sizeof(typename ScanT<In, OutP, 0>::Acc);
  });
  return r;
}

}  // namespace pg
