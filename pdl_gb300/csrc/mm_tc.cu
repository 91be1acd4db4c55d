// mm_tc.cu -- float32 matmult (lib/PDL/Primitive.pd:191-264) as split-bf16
// products on the tcgen05 tensor cores with FP32 accumulation in TMEM.
//
// Split: every float32 x becomes bf16 limbs x0 = rn(x), x1 = rn(x - x0),
// x2 = rn(x - x0 - x1) (each difference is exact in float32).  With three
// limbs the six products a0b0 + a0b1 + a1b0 + a0b2 + a1b1 + a2b0 leave out
// only terms below 2^-24 |a||b|, float32 territory; with two limbs the three
// products a0b0 + a0b1 + a1b0 leave ~2^-16.  The split kernel writes the
// limbs K-major (A: [limb][batch][h][t], B transposed: [limb][batch][w][t]),
// t padded to a multiple of 32 with zeros.
//
// GEMM: one CTA (10 warps) per 128 (h) x 256 (w) output tile.  Warp 8
// streams K-slabs of 32 through a 3-4 stage ring with TMA (64-byte swizzle);
// warp 9 issues tcgen05.mma (M=128, N=256, K=16, bf16 in, f32 accumulate)
// for every limb product of a slab into one of two 256-column TMEM buffers,
// starting the buffer fresh and adding the small limb products before the
// large a0*b0 ones.  The tensor core's float32 accumulation truncates, so
// long accumulation chains in TMEM drift toward zero (about 8e-6 normwise at
// K=1024); instead warps 0-7 drain each finished slab buffer (tcgen05.ld
// 32x32b, each warp its 32 lanes and half of the columns) into registers
// with round-to-nearest adds while the next slab runs in the other buffer,
// and finally store the tile.  Every mbarrier wait gives up after ~4 s of
// clock64 time, records an error the host reads back, and the CTA still
// frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "args.cuh"

namespace pg {
namespace {

constexpr int TC_M = 128, TC_N = 256, TC_BK = 32;
constexpr uint32_t A_TILE = TC_M * TC_BK * 2;  // 8 KiB
constexpr uint32_t B_TILE = TC_N * TC_BK * 2;  // 16 KiB
constexpr uint32_t TMEM_COLS = 512;  // two 256-column slab accumulators
constexpr long long WAIT_CYCLES = 8000000000LL;  // ~4 s at 2 GHz

// K-slabs accumulated in one TMEM buffer before the accumulator warps
// drain it into round-to-nearest registers (2: 64-deep chains, 24
// truncating accumulations for bf16x6; the drain runs half as often)
constexpr int SPB = 2;

template <int LIMBS> struct TcCfg {
  static constexpr int STAGES = LIMBS == 3 ? 3 : 4;
  static constexpr int NPROD = LIMBS == 3 ? 6 : 3;
  static constexpr uint32_t STAGE_BYTES = LIMBS * (A_TILE + B_TILE);
  static constexpr uint32_t SMEM = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
};

struct TcArgs {
  char *c;
  int64_t M, N, K, Kp;
  int64_t c_n, c_m;
  int64_t nA, nB;  // limb batches (1 when the operand is broadcast)
  Loop L;          // batch loop: pdl 2 = c
  int *err;
  int64_t tiles_n, tiles_m, batch;  // the output tiles: w, h, batch
};

__device__ __forceinline__ uint32_t su32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(phase)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and the error flag set) after WAIT_CYCLES.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t phase, int *err) {
  if (mbar_try(b, phase)) return true;
  const long long t0 = clock64();
  while (!mbar_try(b, phase)) {
    if (clock64() - t0 > WAIT_CYCLES) {
      atomicExch(err, 1);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(su32(dst)),
      "l"((uint64_t)map), "r"(su32(bar)), "r"(x), "r"(y)
      : "memory");
}
// Shared-memory matrix descriptor, K-major, 64-byte swizzle: rows of 64 B,
// 8-row groups 512 B apart (SBO), descriptor version 1, layout SWIZZLE_64B.
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused here)
  d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;            // version
  d |= (uint64_t)4 << 61;            // SWIZZLE_64B
  return d;
}
// Instruction descriptor: kind::f16, A/B bf16, D f32, both K-major.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                           ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          su32(bar))
      : "memory");
}

template <int LIMBS>
__global__ void __launch_bounds__(320, 1)
    k_mm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
            const TcArgs g) {
  using C = TcCfg<LIMBS>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(base + C::STAGES * C::STAGE_BYTES);
  uint64_t *empty = full + C::STAGES;
  uint64_t *accf = empty + C::STAGES;  // slab accumulated in TMEM buffer b
  uint64_t *acce = accf + 2;           // TMEM buffer b drained by the 8 accumulator warps
  uint32_t *tmem_slot = (uint32_t *)(acce + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     su32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 288) {
    for (int s = 0; s < C::STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 8);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // Persistent: this CTA computes tiles blockIdx.x, blockIdx.x + gridDim.x,
  // ... (w fastest, then h, then the batch: neighbouring CTAs share A
  // tiles in L2).  The stage ring and the two TMEM buffers carry on across
  // tiles, so the accumulator warps' stores of one tile overlap the MMAs of
  // the next, and the set-up is paid once per CTA.
  const int nk = (int)(g.Kp / TC_BK);
  const int npr = (nk + SPB - 1) / SPB;  // K-ranges (TMEM buffer uses) per tile
  const int64_t tiles = g.tiles_n * g.tiles_m * g.batch;
  auto coords = [&](int64_t t, int &z, int64_t &m0, int64_t &n0) {
    n0 = (t % g.tiles_n) * TC_N;
    m0 = ((t / g.tiles_n) % g.tiles_m) * TC_M;
    z = (int)(t / (g.tiles_n * g.tiles_m));
  };
  // limb products (a limb, b limb), smallest first: each range starts a fresh
  // accumulator, so only the last (a0 b0) products are added at full size
  constexpr int PA3[6] = {2, 1, 0, 1, 0, 0}, PB3[6] = {0, 1, 2, 0, 1, 0};
  constexpr int PA2[3] = {1, 0, 0}, PB2[3] = {0, 1, 0};
  bool ok = true;

  if (warp == 8) {
    if (lane == 0) {
      // -------------------------------------------------------- producer
      int64_t kg = 0;  // slabs loaded by this CTA so far
      for (int64_t t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        int z;
        int64_t m0, n0;
        coords(t, z, m0, n0);
        const int za = g.nA == 1 ? 0 : z, zb = g.nB == 1 ? 0 : z;
        for (int kb = 0; kb < nk && ok; kb++, kg++) {
          const int s = (int)(kg % C::STAGES);
          const int64_t use = kg / C::STAGES;
          if (use > 0) ok = mbar_wait(&empty[s], (uint32_t)((use - 1) & 1), g.err);
          if (!ok) break;
          uint8_t *st = base + s * C::STAGE_BYTES;
          mbar_expect_tx(&full[s], C::STAGE_BYTES);
#pragma unroll
          for (int l = 0; l < LIMBS; l++)
            tma_load_2d(st + l * A_TILE, &tmA, &full[s], kb * TC_BK,
                        (int)((l * g.nA + za) * g.M + m0));
#pragma unroll
          for (int l = 0; l < LIMBS; l++)
            tma_load_2d(st + LIMBS * A_TILE + l * B_TILE, &tmB, &full[s], kb * TC_BK,
                        (int)((l * g.nB + zb) * g.N + n0));
        }
      }
    }
  } else if (warp == 9) {
    if (lane == 0) {
      // ------------------------------------------------------------- MMA
      int64_t kg = 0, pbase = 0;  // slabs and K-ranges issued by this CTA so far
      for (int64_t t = blockIdx.x; t < tiles && ok; t += gridDim.x, pbase += npr) {
        for (int kb = 0; kb < nk && ok; kb++, kg++) {
          const int s = (int)(kg % C::STAGES);
          const int64_t use = kg / C::STAGES;
          const int64_t pr = pbase + kb / SPB, j = pr >> 1;
          const int b = (int)(pr & 1);
          const bool opens = kb % SPB == 0, closes = kb % SPB == SPB - 1 || kb == nk - 1;
          if (opens && j > 0) ok = mbar_wait(&acce[b], (uint32_t)((j - 1) & 1), g.err);
          if (ok) ok = mbar_wait(&full[s], (uint32_t)(use & 1), g.err);
          if (!ok) break;
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = su32(base + s * C::STAGE_BYTES);
          const uint32_t d = tmem + (uint32_t)(b * TC_N);
          int first = opens ? 1 : 0;
#pragma unroll
          for (int p = 0; p < C::NPROD; p++) {
#pragma unroll
            for (int ks = 0; ks < TC_BK / 16; ks++) {
              const int pa = LIMBS == 3 ? PA3[p] : PA2[p], pb = LIMBS == 3 ? PB3[p] : PB2[p];
              const uint64_t ad = sdesc_sw64(st + pa * A_TILE + ks * 32);
              const uint64_t bd = sdesc_sw64(st + LIMBS * A_TILE + pb * B_TILE + ks * 32);
              umma(d, ad, bd, first ? 0u : 1u);
              first = 0;
            }
          }
          umma_commit(&empty[s]);
          if (closes) umma_commit(&accf[b]);
        }
      }
    }
  } else {
    // ------------------------------------------- accumulators (warps 0-7)
    // warp w reads TMEM lanes 32*(w%4).. (its 32 rows) and columns
    // 128*(w/4).. (its half of the tile), adding each range with RN fp32,
    // then stores its part of the tile.
    const int q = warp & 3, half = warp >> 2;
    const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(half * 128);
    int64_t pbase = 0;
    for (int64_t t = blockIdx.x; t < tiles && ok; t += gridDim.x, pbase += npr) {
      int z;
      int64_t m0, n0;
      coords(t, z, m0, n0);
      float acc[128];
#pragma unroll
      for (int i = 0; i < 128; i++) acc[i] = 0.f;
      for (int r = 0; r < npr && ok; r++) {
        const int64_t pr = pbase + r;
        const int b = (int)(pr & 1);
        if (lane == 0) ok = mbar_wait(&accf[b], (uint32_t)((pr >> 1) & 1), g.err);
        ok = __shfl_sync(0xffffffffu, ok, 0);  // warp-uniform for tcgen05.ld
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int c = 0; c < 4; c++) {
          uint32_t rg[32];
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
              "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
              "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
              : "=r"(rg[0]), "=r"(rg[1]), "=r"(rg[2]), "=r"(rg[3]), "=r"(rg[4]), "=r"(rg[5]),
                "=r"(rg[6]), "=r"(rg[7]), "=r"(rg[8]), "=r"(rg[9]), "=r"(rg[10]), "=r"(rg[11]),
                "=r"(rg[12]), "=r"(rg[13]), "=r"(rg[14]), "=r"(rg[15]), "=r"(rg[16]), "=r"(rg[17]),
                "=r"(rg[18]), "=r"(rg[19]), "=r"(rg[20]), "=r"(rg[21]), "=r"(rg[22]), "=r"(rg[23]),
                "=r"(rg[24]), "=r"(rg[25]), "=r"(rg[26]), "=r"(rg[27]), "=r"(rg[28]), "=r"(rg[29]),
                "=r"(rg[30]), "=r"(rg[31])
              : "r"(tl + (uint32_t)(b * TC_N + c * 32)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int i = 0; i < 32; i++)
            acc[c * 32 + i] = __fadd_rn(acc[c * 32 + i], __uint_as_float(rg[i]));
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0)
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&acce[b])) : "memory");
      }
      if (!ok) break;
      int64_t offs[MAXP];
      loop_offsets(g.L, z, offs);
      float *C0 = reinterpret_cast<float *>(g.c) + offs[2];
      const int64_t m = m0 + q * 32 + lane;
      const int64_t nb = n0 + half * 128;
      const bool vec = g.c_n == 1 && ((uintptr_t)C0 % 16 == 0) && (g.c_m % 4 == 0);
      if (m < g.M) {
        float *row = C0 + m * g.c_m;
        if (vec && nb + 128 <= g.N) {
          float4 *p = reinterpret_cast<float4 *>(row + nb);
#pragma unroll
          for (int i = 0; i < 32; i++)
            p[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
        } else {
#pragma unroll
          for (int i = 0; i < 128; i++)
            if (nb + i < g.N) row[(nb + i) * g.c_n] = acc[i];
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 8)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
}

// ------------------------------------------------------------------ split

struct SplitArgs {
  const float *src;
  __nv_bfloat16 *dst;    // [LIMBS][nb][rows][Kp]
  int64_t rows, K, Kp, nb;
  int64_t s_row, s_k;    // element increments of a row / of k in src
  Loop L;                // batch loop (pdl index `p`)
  int p;
};

// The limbs of one float32: x0 = rn(x), x1 = rn(x - x0), x2 = rn(x - x0 - x1).
template <int LIMBS>
__device__ __forceinline__ void split1(float x, __nv_bfloat16 (&h)[3]) {
  h[0] = __float2bfloat16_rn(x);
  const float r1 = __fsub_rn(x, __bfloat162float(h[0]));
  h[1] = __float2bfloat16_rn(r1);
  h[2] = LIMBS == 3 ? __float2bfloat16_rn(__fsub_rn(r1, __bfloat162float(h[1])))
                    : __float2bfloat16_rn(0.f);
}

// Rows whose k is contiguous (s_k == 1): a thread splits 8 consecutive k of
// one row and writes 16 bytes per limb; k past K (the padding) is zero.
// Each thread takes two such items per round, both loads issued first.
template <int LIMBS>
__global__ void __launch_bounds__(256) k_split(const SplitArgs g) {
  const int64_t kc = g.Kp / 8, nrow = g.rows * g.nb, total = nrow * kc;
  const int64_t per_limb = g.nb * g.rows * g.Kp;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  auto load = [&](int64_t i, float (&x)[8]) {
    const int64_t rr = i / kc, k0 = (i - rr * kc) * 8;
    const int64_t z = rr / g.rows, r = rr - z * g.rows;
    int64_t offs[MAXP];
    loop_offsets(g.L, z, offs);
    const float *src = g.src + offs[g.p] + r * g.s_row;
    if (k0 + 8 <= g.K && ((uintptr_t)(src + k0) & 15) == 0) {
      const float4 u = __ldcs(reinterpret_cast<const float4 *>(src + k0));
      const float4 v = __ldcs(reinterpret_cast<const float4 *>(src + k0 + 4));
      x[0] = u.x; x[1] = u.y; x[2] = u.z; x[3] = u.w;
      x[4] = v.x; x[5] = v.y; x[6] = v.z; x[7] = v.w;
    } else {
#pragma unroll
      for (int e = 0; e < 8; e++) x[e] = k0 + e < g.K ? src[k0 + e] : 0.f;
    }
  };
  auto store = [&](int64_t i, const float (&x)[8]) {
    const int64_t rr = i / kc, k0 = (i - rr * kc) * 8;
    __align__(16) __nv_bfloat16 o[3][8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
      __nv_bfloat16 h[3];
      split1<LIMBS>(x[e], h);
#pragma unroll
      for (int l = 0; l < LIMBS; l++) o[l][e] = h[l];
    }
    __nv_bfloat16 *d = g.dst + rr * g.Kp + k0;
#pragma unroll
    for (int l = 0; l < LIMBS; l++)
      *reinterpret_cast<uint4 *>(d + l * per_limb) = *reinterpret_cast<const uint4 *>(o[l]);
  };
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += 2 * stride) {
    const bool two = i + stride < total;
    float x0[8], x1[8];
    load(i, x0);
    if (two) load(i + stride, x1);
    store(i, x0);
    if (two) store(i + stride, x1);
  }
}

// Rows whose k is strided (the b(w, t) operand, w contiguous): 32 x 32
// tiles through shared memory, read along the rows, written along k.
template <int LIMBS>
__global__ void __launch_bounds__(256) k_split_t(const SplitArgs g) {
  __shared__ float t[32][33];
  const int64_t rt = (g.rows + 31) / 32, kt = g.Kp / 32;
  const int64_t tiles = g.nb * rt * kt;
  const int64_t per_limb = g.nb * g.rows * g.Kp;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 warps
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int64_t z = tile / (rt * kt), rem = tile - z * rt * kt;
    const int64_t r0 = (rem / kt) * 32, k0 = (rem % kt) * 32;
    int64_t offs[MAXP];
    loop_offsets(g.L, z, offs);
    const float *src = g.src + offs[g.p];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; j++) {  // k = k0 + ty + 8j, row = r0 + tx (coalesced along rows)
      const int64_t k = k0 + ty + 8 * j, r = r0 + tx;
      t[ty + 8 * j][tx] = (k < g.K && r < g.rows) ? src[r * g.s_row + k * g.s_k] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; j++) {  // row = r0 + ty + 8j, k = k0 + tx (coalesced along k)
      const int64_t r = r0 + ty + 8 * j;
      if (r >= g.rows) continue;
      __nv_bfloat16 h[3];
      split1<LIMBS>(t[tx][ty + 8 * j], h);
      __nv_bfloat16 *d = g.dst + (z * g.rows + r) * g.Kp + k0 + tx;
#pragma unroll
      for (int l = 0; l < LIMBS; l++) d[l * per_limb] = h[l];
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

bool get_encode() {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  });
  return g_encode != nullptr;
}

bool make_map(CUtensorMap *map, void *ptr, int64_t kp, int64_t rows, uint32_t boxrows) {
  cuuint64_t gdim[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)TC_BK, boxrows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, gdim, gstride, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

bool all_zero_incs(const Loop &L, int p) {
  for (int k = 0; k < L.nd; k++)
    if (L.size[k] > 1 && L.inc[p][k] != 0) return false;
  return true;
}

template <int LIMBS>
pdlgb300_error tc_typed(const MMArgs &g, cudaStream_t s) {
  using C = TcCfg<LIMBS>;
  pdlgb300_error e = pgh::ok();
  if (!get_encode()) return pgh::err(PDLGB300_EFATAL, "cuTensorMapEncodeTiled unavailable");
  const int64_t Kp = (g.K + TC_BK - 1) / TC_BK * TC_BK;
  const int64_t nA = all_zero_incs(g.L, 0) ? 1 : g.batch;
  const int64_t nB = all_zero_incs(g.L, 1) ? 1 : g.batch;
  const size_t abytes = (size_t)LIMBS * nA * g.M * Kp * 2, bbytes = (size_t)LIMBS * nB * g.N * Kp * 2;
  void *scratch = nullptr;
  if (cudaMallocAsync(&scratch, abytes + bbytes + 256 + 16, s) != cudaSuccess) {
    cudaGetLastError();
    return pgh::err(PDLGB300_EFATAL, "matmult: no device memory for the bf16 limbs");
  }
  __nv_bfloat16 *al = (__nv_bfloat16 *)scratch;
  __nv_bfloat16 *bl = (__nv_bfloat16 *)((char *)scratch + ((abytes + 255) & ~(size_t)255));
  int *errp = (int *)((char *)bl + bbytes);
  errp = (int *)(((uintptr_t)errp + 15) & ~(uintptr_t)15);
  cudaMemsetAsync(errp, 0, sizeof(int), s);
  const int nsm = pgh::num_sms();
  // each operand's limbs: k contiguous -> k_split, else the transposing k_split_t
  auto split = [&](const SplitArgs &sg, int64_t rows, int64_t nb, int64_t sk) {
    if (sk == 1) {
      const int64_t n8 = nb * rows * (Kp / 8);
      const int64_t grid = std::min<int64_t>((n8 + 255) / 256, (int64_t)nsm * 64);
      k_split<LIMBS><<<(int)grid, 256, 0, s>>>(sg);
      pgh::record_kernel("k_split", grid, 256);
    } else {
      const int64_t tiles = nb * ((rows + 31) / 32) * (Kp / 32);
      const int64_t grid = std::min<int64_t>(tiles, (int64_t)nsm * 16);
      k_split_t<LIMBS><<<(int)grid, 256, 0, s>>>(sg);
      pgh::record_kernel("k_split_t", grid, 256);
    }
  };
  SplitArgs sa{reinterpret_cast<const float *>(g.a), al, g.M, g.K, Kp, nA, g.a_m, g.a_k, g.L, 0};
  split(sa, g.M, nA, g.a_k);
  SplitArgs sb{reinterpret_cast<const float *>(g.b), bl, g.N, g.K, Kp, nB, g.b_n, g.b_k, g.L, 1};
  split(sb, g.N, nB, g.b_k);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_split")) {
    cudaFreeAsync(scratch, s);
    return e;
  }
  CUtensorMap mA, mB;
  if (!make_map(&mA, al, Kp, LIMBS * nA * g.M, TC_M) ||
      !make_map(&mB, bl, Kp, LIMBS * nB * g.N, TC_N)) {
    cudaFreeAsync(scratch, s);
    return pgh::err(PDLGB300_EFATAL, "matmult: tensor map encoding failed");
  }
  TcArgs t;
  memset(&t, 0, sizeof t);
  t.c = g.c;
  t.M = g.M;
  t.N = g.N;
  t.K = g.K;
  t.Kp = Kp;
  t.c_n = g.c_n;
  t.c_m = g.c_m;
  t.nA = nA;
  t.nB = nB;
  t.L = g.L;
  t.err = errp;
  static bool attr_set[4] = {false, false, false, false};
  if (!attr_set[LIMBS]) {
    cudaFuncSetAttribute(k_mm_tc<LIMBS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
    attr_set[LIMBS] = true;
  }
  t.tiles_n = (g.N + TC_N - 1) / TC_N;
  t.tiles_m = (g.M + TC_M - 1) / TC_M;
  t.batch = g.batch;
  // one CTA per SM (the stages take most of its shared memory), each walking
  // tiles; a launch with fewer tiles than SMs has one tile per CTA
  dim3 grid((unsigned)std::min<int64_t>(t.tiles_n * t.tiles_m * t.batch, (int64_t)nsm));
  k_mm_tc<LIMBS><<<grid, 320, C::SMEM, s>>>(mA, mB, t);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_mm_tc")) {
    cudaFreeAsync(scratch, s);
    return e;
  }
  pgh::record_kernel(LIMBS == 3 ? "k_mm_tc_bf16x6" : "k_mm_tc_bf16x3", (int64_t)grid.x, 320);
  int herr = 0;
  cudaMemcpyAsync(&herr, errp, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(scratch, s);
  cudaError_t ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return pgh::err(PDLGB300_EFATAL, "matmult: %s", cudaGetErrorString(ce));
  if (herr) return pgh::err(PDLGB300_EFATAL, "matmult: tensor-core pipeline wait timed out");
  return e;
}

}  // namespace

bool matmult_tc_supported(const MMArgs &g) {
  return g.M > 0 && g.N > 0 && g.K > 0 && g.batch > 0 && g.batch <= 65535 &&
         !g.bad && g.M * (3 * g.batch) < (1LL << 31) && g.N * (3 * g.batch) < (1LL << 31) &&
         g.K < (1LL << 31);
}

pdlgb300_error launch_matmult_tc(int limbs, const MMArgs &g, cudaStream_t s) {
  return limbs == 3 ? tc_typed<3>(g, s) : tc_typed<2>(g, s);
}

}  // namespace pg
