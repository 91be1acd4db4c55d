// mm_simt.cu -- PDL::Primitive matmult (lib/PDL/Primitive.pd:191-264) on the
// CUDA cores: c(w,h) = sum_t a(t,h) b(w,t) over broadcast (batch) dims.
//
// Block tile 128 (h) x 128 (w), t-slab 8, 256 threads each owning 8x8
// outputs, shared-memory tiles double-buffered through registers.  Every
// output accumulates t in increasing order, the reference's order.  With
// fused == 0 each step rounds the product and then the sum (__fmul_rn,
// __fadd_rn): the same arithmetic as the reference's `cc += *ad * *bd`, so
// the result is bit-identical to the reference for every type.  fused == 1
// (float32 only) uses FFMA: the plain FP32 SIMT baseline.
#include "args.cuh"

namespace pg {
namespace {

constexpr int BM = 128, BN = 128, BK = 8, TM = 8, TN = 8, NT = 256;

template <class T, bool FUSED>
__device__ __forceinline__ T mac(T acc, T a, T b) {
  if constexpr (std::is_floating_point_v<T>) {
    if constexpr (FUSED) return fma(a, b, acc);
    else if constexpr (std::is_same_v<T, double>) return rn_add(acc, __dmul_rn(a, b));  // register-bound tile
    else return rn_add(acc, rn_mul(a, b));
  } else {
    return wadd<T>(acc, wmul<T>(a, b));
  }
}

template <class T, bool FUSED, bool BAD>
__global__ void __launch_bounds__(NT) k_mm_simt(const MMArgs g) {
  __shared__ T As[2][BK][BM];
  __shared__ T Bs[2][BK][BN];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
  int64_t offs[MAXP];
  loop_offsets(g.L, blockIdx.z, offs);
  const T *A = reinterpret_cast<const T *>(g.a) + offs[0];
  const T *B = reinterpret_cast<const T *>(g.b) + offs[1];
  T *C = reinterpret_cast<T *>(g.c) + offs[2];
  Bad<T> ba{from_bits<T>(g.abad), (bool)g.abad_isnan};
  Bad<T> bb{from_bits<T>(g.bbad), (bool)g.bbad_isnan};

  // loader mapping: A tile (BM x BK): thread loads 4 elements of row am,
  // k = ak..ak+3 ; B tile (BK x BN): row bk, n = bn..bn+3
  const int am = tid / 2, ak = (tid % 2) * 4;
  const int bk = tid / 32, bn = (tid % 32) * 4;
  T ra[4], rb[4];
  bool rba[4], rbb[4];

  auto load = [&](int64_t k0) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int64_t m = m0 + am, k = k0 + ak + j;
      bool in = m < g.M && k < g.K;
      T v = in ? A[k * g.a_k + m * g.a_m] : (T)0;
      ra[j] = v;
      rba[j] = BAD && in && ba.is(v);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int64_t k = k0 + bk, n = n0 + bn + j;
      bool in = k < g.K && n < g.N;
      T v = in ? B[n * g.b_n + k * g.b_k] : (T)0;
      rb[j] = v;
      rbb[j] = BAD && in && bb.is(v);
    }
  };
  // bad values: mark by storing into parallel shared flag arrays
  __shared__ unsigned char Af[2][BK][BM];
  __shared__ unsigned char Bf[2][BK][BN];
  auto store = [&](int buf) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      As[buf][ak + j][am] = ra[j];
      if (BAD) Af[buf][ak + j][am] = rba[j];
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      Bs[buf][bk][bn + j] = rb[j];
      if (BAD) Bf[buf][bk][bn + j] = rbb[j];
    }
  };

  T acc[TM][TN];
  bool badacc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) {
      acc[i][j] = (T)0;
      badacc[i][j] = false;
    }

  // The reference walks t in tiles of tsiz = 64 / sizeof(T) (a multiple of
  // BK for every type) and, in bad mode, starts each tile by reading the
  // partial sum back from c: one equal to c's badvalue is taken as bad and
  // left as it is (Primitive.pd matmult Code, `if ($ISBADVAR(cc,c))
  // continue`), including the zero it starts from when that badvalue is 0.
  constexpr int64_t TSIZ = 64 / sizeof(T);
  const Bad<T> bc{from_bits<T>(g.cbad), (bool)g.cbad_isnan};

  load(0);
  store(0);
  __syncthreads();
  int buf = 0;
  for (int64_t k0 = 0; k0 < g.K; k0 += BK) {
    if (BAD && k0 % TSIZ == 0) {
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) badacc[i][j] |= bc.is(acc[i][j]);
    }
    const bool more = k0 + BK < g.K;
    if (more) load(k0 + BK);
    const int kend = (int)(g.K - k0 < BK ? g.K - k0 : BK);
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      if (kk < kend) {
        T a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; i++) a[i] = As[buf][kk][ty * 4 + (i % 4) + (i / 4) * 64];
#pragma unroll
        for (int j = 0; j < TN; j++) b[j] = Bs[buf][kk][tx * 4 + (j % 4) + (j / 4) * 64];
#pragma unroll
        for (int i = 0; i < TM; i++)
#pragma unroll
          for (int j = 0; j < TN; j++) acc[i][j] = mac<T, FUSED>(acc[i][j], a[i], b[j]);
        if (BAD) {
#pragma unroll
          for (int i = 0; i < TM; i++) {
            bool fa = Af[buf][kk][ty * 4 + (i % 4) + (i / 4) * 64];
#pragma unroll
            for (int j = 0; j < TN; j++)
              badacc[i][j] |= fa | (bool)Bf[buf][kk][tx * 4 + (j % 4) + (j / 4) * 64];
          }
        }
      }
    }
    if (more) {
      store(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }
  const T cbad = bc.val;
#pragma unroll
  for (int i = 0; i < TM; i++) {
    int64_t m = m0 + ty * 4 + (i % 4) + (i / 4) * 64;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < TN; j++) {
      int64_t n = n0 + tx * 4 + (j % 4) + (j / 4) * 64;
      if (n >= g.N) continue;
      C[m * g.c_m + n * g.c_n] = (BAD && badacc[i][j]) ? cbad : acc[i][j];
    }
  }
}

template <class T, bool FUSED>
pdlgb300_error mm_typed(const MMArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.batch == 0 || g.M == 0 || g.N == 0) return e;
  dim3 grid((unsigned)((g.N + BN - 1) / BN), (unsigned)((g.M + BM - 1) / BM),
            (unsigned)g.batch);
  if (g.bad) k_mm_simt<T, FUSED, true><<<grid, NT, 0, s>>>(g);
  else k_mm_simt<T, FUSED, false><<<grid, NT, 0, s>>>(g);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_mm_simt")) return e;
  pgh::record_kernel(FUSED ? "k_mm_simt_ffma" : "k_mm_simt_exact",
                     (int64_t)grid.x * grid.y * grid.z, NT);
  return e;
}

}  // namespace

pdlgb300_error launch_matmult_simt(int dt, int fused, const MMArgs &g, cudaStream_t s) {
  if (g.batch > 65535)
    return pgh::err(PDLGB300_EUSERERROR, "matmult: more than 65535 broadcast matrices");
  if (dt == PDLGB300_F && fused) return mm_typed<float, true>(g, s);
  PG_DISPATCH(dt, return mm_typed<typename TT<DT>::T, false>(g, s));
  return pgh::err(PDLGB300_EUSERERROR, "matmult: unsupported type %d", dt);
}

}  // namespace pg
