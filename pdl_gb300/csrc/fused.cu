// fused.cu -- sumover(plus(mult(a, b), d)) in one pass: c() over a(n), b(n),
// d(n), each element computed exactly as the three reference ops compute it
// in sequence (lib/PDL/Ops.pd:133-153 for mult and plus with their bad-value
// rules, lib/PDL/Ufunc.pd:94-118 for sumover), without materialising the
// broadcast intermediates a*b and a*b+d.
//
// The common shape (a and d vary along one output dim, b along the other:
// an outer-product broadcast such as a(n,1,K) * b(n,J,1)) is tiled like a
// GEMM: each block owns 64x64 outputs, stages 32-deep slabs of a, b (and d)
// in shared memory, and each thread accumulates a 4x4 output tile, so every
// input element read from HBM is reused 64 times.  Integer work is order
// free and exact; float32 sums use compensated accumulation.
#include "args.cuh"
#include "f64sum.cuh"

namespace pg {
namespace {

template <class T, class Out, bool COMP> struct FAcc {
  using A = std::conditional_t<
      std::is_integral_v<Out>, uns_t<Out>,
      std::conditional_t<std::is_same_v<Out, float>,
                         std::conditional_t<COMP, float2, float>, double>>;
  __device__ static A zero() {
    A a;
    memset(&a, 0, sizeof a);
    return a;
  }
  __device__ static void add(A &a, T u) {
    if constexpr (std::is_integral_v<Out>) {
      a += (A)(Out)u;
    } else if constexpr (std::is_same_v<A, float2>) {
      float x = (float)u;
      float s = __fadd_rn(a.x, x);
      float bp = __fsub_rn(s, a.x);
      float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bp)), __fsub_rn(x, bp));
      a.x = s;
      a.y = __fadd_rn(a.y, e);
    } else {
      a = rn_add(a, (A)u);
    }
  }
  __device__ static Out value(const A &a) {
    if constexpr (std::is_same_v<A, float2>) return __fadd_rn(a.x, a.y);
    else return (Out)a;
  }
};

// One element of the chain.  Returns false when the element is skipped.
template <class T, bool BAD>
__device__ __forceinline__ bool chain(const FusedArgs &g, T va, T vb, T vd, const Bad<T> &ba,
                                      const Bad<T> &bb, const Bad<T> &bd, const Bad<T> &bt,
                                      T tbad, T ubad, T &u) {
  if constexpr (!BAD) {
    u = op_add<T>(op_mul<T>(va, vb), vd);
    return true;
  } else {
    const bool ft = g.fa || g.fb, fu = ft || g.fd;
    T t = ((g.fa && ba.is(va)) || (g.fb && bb.is(vb))) ? tbad : op_mul<T>(va, vb);
    u = ((ft && bt.is(t)) || (g.fd && bd.is(vd))) ? ubad : op_add<T>(t, vd);
    return !(fu && bt.is(u));  // sumover skips bad u (u's badvalue: the default)
  }
}

constexpr int FJ = 64, FK = 64, FT = 256;

template <class T, class Out, bool BAD, bool COMP, bool DA>
__global__ void __launch_bounds__(FT) k_fused_outer(const FusedArgs g) {
  using FA = FAcc<T, Out, COMP>;
  // slab depth; rows padded by one element so the transposing stores
  // (consecutive n across lanes) hit distinct banks
  constexpr int FN = sizeof(T) == 8 ? 16 : 32;
  __shared__ T sa[FN][FK + 1];
  __shared__ T sb[FN][FJ + 1];
  __shared__ T sd[DA ? 1 : FN][DA ? 1 : FK + 1];
  // float32 in bad-value mode with d = a: each staged value once -- zeroed where bad,
  // b's goodness as 0/1, good bits of each column over the slab (a ballot:
  // the staging lanes are the slab's i), the slab's largest magnitudes --
  // so that a slab whose products cannot reach the badvalue costs a pair
  // three float operations.  Rows of 16-byte chunks, chunk c of row i at
  // c ^ (i & 15), read four values at a time.
  // (with a separate d the copies would pass the 48 KB of static shared
  // memory; that case keeps the per-thread tests below)
  constexpr bool FPB = BAD && DA && std::is_same_v<T, float>;
  constexpr int ZN = FPB ? FN : 1, ZK = FPB ? FK : 4, ZJ = FPB ? FJ : 4;
  __shared__ __align__(16) T za[ZN][ZK];
  __shared__ __align__(16) T zd[(FPB && !DA) ? FN : 1][(FPB && !DA) ? FK : 4];
  __shared__ __align__(16) T zb[ZN][ZJ];
  __shared__ __align__(16) T zg[ZN][ZJ];
  __shared__ uint32_t mka[FPB ? FK : 1], mkb[FPB ? FJ : 1];
  __shared__ int s_max[2][3], s_fin[2];  // per slab parity: max |a|, |b|, |d| (float bits)
  auto swz = [](int i, int v) { return (((v >> 2) ^ (i & 15)) << 2) | (v & 3); };
  const int tid = threadIdx.x, tj = tid % 16, tk = tid / 16;
  const int64_t J = g.L.size[g.jdim], K = g.L.size[g.kdim];
  const int64_t j0 = (int64_t)blockIdx.x * FJ, k0 = (int64_t)blockIdx.y * FK;
  const int64_t a_k = g.L.inc[0][g.kdim], b_j = g.L.inc[1][g.jdim];
  const int64_t d_k = g.L.inc[2][g.kdim], d_j = g.L.inc[2][g.jdim];
  const T *A = reinterpret_cast<const T *>(g.a);
  const T *B = reinterpret_cast<const T *>(g.b);
  const T *D = reinterpret_cast<const T *>(g.d);
  Bad<T> ba{from_bits<T>(g.abad), (bool)g.abad_isnan};
  Bad<T> bb{from_bits<T>(g.bbad), (bool)g.bbad_isnan};
  Bad<T> bd{from_bits<T>(g.dbad), (bool)g.dbad_isnan};
  Bad<T> bt{from_bits<T>(g.tbad), (bool)g.tbad_isnan};
  const T tbad = from_bits<T>(g.tbad), ubad = from_bits<T>(g.ubad);
  typename FA::A acc[4][4];
  bool cnt[4][4];  // any good pair (sumover's flag), bad-value mode only
#pragma unroll
  for (int x = 0; x < 4; x++)
#pragma unroll
    for (int y = 0; y < 4; y++) {
      acc[x][y] = FA::zero();
      cnt[x][y] = false;
    }
  // Compensated float32: the pairs of one slab are summed plainly (FN
  // values, error below FN ulps of their magnitudes' sum), and each slab's
  // sum is added to the compensated accumulator: a pair costs one add, not
  // the seven of a compensated add.
  constexpr bool SLAB = std::is_same_v<typename FA::A, float2>;
  T part[4][4];
  if (FPB && tid < 2) {
    s_max[tid][0] = s_max[tid][1] = s_max[tid][2] = 0;
    s_fin[tid] = 1;
  }
  int par = 0;
  for (int64_t i0 = 0; i0 < g.n; i0 += FN, par ^= 1) {
    uint32_t gma[4] = {0, 0, 0, 0}, gmb[4] = {0, 0, 0, 0};  // fast path: good bits of the slab
    if constexpr (SLAB) {
#pragma unroll
      for (int y = 0; y < 4; y++)
#pragma unroll
        for (int x = 0; x < 4; x++) part[y][x] = (T)0;
    }
    __syncthreads();
    // stage: FN x FK of a (and d), FN x FJ of b; i fastest across threads
    float ma = 0.0f, mb = 0.0f, md = 0.0f;
    bool sfin = true;
    if (FPB && tid == 0) {
      // the other parity's flags were read before this slab began
      s_max[par ^ 1][0] = s_max[par ^ 1][1] = s_max[par ^ 1][2] = 0;
      s_fin[par ^ 1] = 1;
    }
    for (int idx = tid; idx < FN * FK; idx += FT) {
      int i = idx % FN, k = idx / FN;
      int64_t gi = i0 + i, gk = k0 + k;
      bool in = gi < g.n && gk < K;
      const T av = in ? A[gi * g.inc_a + gk * a_k] : (T)0;
      sa[i][k] = av;
      T dv = av;
      if constexpr (!DA) {
        dv = in ? D[gi * g.inc_d + gk * d_k] : (T)0;
        sd[i][k] = dv;
      }
      if constexpr (FPB) {
        // (FN = 32 and FT a multiple of 32: a warp stages one column k,
        // lane = i)
        const bool good = in && !(g.fa && ba.is(av)) && !(g.fd && bd.is(dv));
        const T a0 = good ? av : (T)0, d0 = good ? dv : (T)0;
        za[i][swz(i, k)] = a0;
        if constexpr (!DA) zd[i][swz(i, k)] = d0;
        const uint32_t m = __ballot_sync(0xffffffffu, good);
        if ((tid & 31) == 0) mka[k] = m;
        sfin = sfin && isfinite(a0) && isfinite(d0);
        ma = fmaxf(ma, fabsf(a0));
        md = fmaxf(md, fabsf(d0));
      }
    }
    for (int idx = tid; idx < FN * FJ; idx += FT) {
      int i = idx % FN, j = idx / FN;
      int64_t gi = i0 + i, gj = j0 + j;
      const bool in = gi < g.n && gj < J;
      const T bv = in ? B[gi * g.inc_b + gj * b_j] : (T)0;
      sb[i][j] = bv;
      if constexpr (FPB) {
        const bool good = in && !(g.fb && bb.is(bv));
        const T b0 = good ? bv : (T)0;
        zb[i][swz(i, j)] = b0;
        zg[i][swz(i, j)] = good ? (T)1 : (T)0;
        const uint32_t m = __ballot_sync(0xffffffffu, good);
        if ((tid & 31) == 0) mkb[j] = m;
        sfin = sfin && isfinite(b0);
        mb = fmaxf(mb, fabsf(b0));
      }
    }
    if constexpr (FPB) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, o));
        md = fmaxf(md, __shfl_xor_sync(0xffffffffu, md, o));
      }
      sfin = __all_sync(0xffffffffu, sfin);
      if ((tid & 31) == 0) {
        if (sfin) {
          atomicMax(&s_max[par][0], __float_as_int(ma));
          atomicMax(&s_max[par][1], __float_as_int(mb));
          atomicMax(&s_max[par][2], __float_as_int(md));
        } else {
          atomicAnd(&s_fin[par], 0);
        }
      }
    }
    __syncthreads();
    bool slab_fast = false;
    if constexpr (FPB) {
      // no product a*b nor sum a*b + d of the slab's good values can equal
      // the intermediates' badvalue: finite values give no NaN, and the
      // bound (rounded up, with a margin for the products' own rounding)
      // stays below a finite badvalue's magnitude
      if (s_fin[par]) {
        const float bound = __fmaf_ru(__int_as_float(s_max[par][0]), __int_as_float(s_max[par][1]),
                                      __int_as_float(s_max[par][2])) * (1.0f + 0x1p-20f);
        slab_fast = bt.isnan_ || bound < fabsf((float)tbad);
      }
    }
    if (slab_fast) {
      if constexpr (FPB) {
        const int iend = (int)(g.n - i0 < FN ? g.n - i0 : FN);
        for (int i = 0; i < iend; i++) {
          const float4 a4 = *reinterpret_cast<const float4 *>(&za[i][swz(i, tk * 4)]);
          const float4 b4 = *reinterpret_cast<const float4 *>(&zb[i][swz(i, tj * 4)]);
          const float4 g4 = *reinterpret_cast<const float4 *>(&zg[i][swz(i, tj * 4)]);
          float4 d4 = a4;
          if constexpr (!DA) d4 = *reinterpret_cast<const float4 *>(&zd[i][swz(i, tk * 4)]);
          const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
          const float gv[4] = {g4.x, g4.y, g4.z, g4.w}, dv[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
          for (int y = 0; y < 4; y++)
#pragma unroll
            for (int x = 0; x < 4; x++) {
              // the reference's two roundings, then the pair masked by b
              const float u = __fadd_rn(__fmul_rn(av[x], bv[y]), dv[x]);
              part[y][x] = __fmaf_rn(u, gv[y], part[y][x]);
            }
        }
#pragma unroll
        for (int y = 0; y < 4; y++)
#pragma unroll
          for (int x = 0; x < 4; x++)
            cnt[y][x] = cnt[y][x] || (mka[tk * 4 + x] & mkb[tj * 4 + y]) != 0;
      }
    } else {
    const int iend = (int)(g.n - i0 < FN ? g.n - i0 : FN);
    for (int i = 0; i < iend; i++) {
      T av[4], bv[4], dv[4];
#pragma unroll
      for (int x = 0; x < 4; x++) {
        av[x] = sa[i][tk * 4 + x];
        bv[x] = sb[i][tj * 4 + x];
        if constexpr (DA) dv[x] = av[x];
        else dv[x] = sd[i][tk * 4 + x];
      }
      if constexpr (!BAD && DA && std::is_integral_v<T>) {
        // a*b + a == a*(b+1) in wrapping arithmetic: one multiply-add
#pragma unroll
        for (int y = 0; y < 4; y++) {
          T b1 = wadd<T>(bv[y], (T)1);
#pragma unroll
          for (int x = 0; x < 4; x++) FA::add(acc[y][x], wmul<T>(av[x], b1));
        }
      } else if constexpr (BAD) {
        // the inputs' bad tests once per staged value, not per pair; the
        // intermediates' tests (t and u against their badvalue) per pair,
        // with the NaN mode fixed per launch
        const bool ft = g.fa || g.fb, fu = ft || g.fd;
        bool xa[4], xd[4], xb[4];
#pragma unroll
        for (int x = 0; x < 4; x++) {
          xa[x] = g.fa && ba.is(av[x]);
          xd[x] = g.fd && bd.is(dv[x]);
          xb[x] = g.fb && bb.is(bv[x]);
        }
        // Fast path: a bad a, b or d makes the pair's u bad (skipped); a
        // good pair is skipped only when t = a*b or u = t + d equals the
        // intermediates' badvalue.  Bounds from this step's good values
        // rule that out: |t| <= max|a| max|b| and |u| <= |t| + max|d|
        // (rounded up), below |badvalue|; with a NaN badvalue, finite good
        // values give finite-or-inf t and u, never NaN.  Then bad a and d
        // are zeroed once per value and a pair costs a product, a sum, a
        // select and the compensated add.
        bool ka[4];
        T a0[4], d0[4], b0[4];
        float ma = 0.0f, mb = 0.0f, md = 0.0f;
        bool fin = true;
#pragma unroll
        for (int x = 0; x < 4; x++) {
          ka[x] = xa[x] || xd[x];
          a0[x] = ka[x] ? (T)0 : av[x];
          d0[x] = ka[x] ? (T)0 : dv[x];
          b0[x] = xb[x] ? (T)0 : bv[x];
          ma = fmaxf(ma, fabsf((float)a0[x]));
          md = fmaxf(md, fabsf((float)d0[x]));
          mb = fmaxf(mb, fabsf((float)b0[x]));
          if constexpr (std::is_floating_point_v<T>)
            fin = fin && isfinite(a0[x]) && isfinite(d0[x]) && isfinite(b0[x]);
        }
        bool fast;
        if constexpr (std::is_floating_point_v<T>) {
          if (bt.isnan_) {
            fast = fin;
          } else {
            // (float bounds of double values are rounded to nearest: the
            // margin of 2^-20 covers that and the products' own rounding)
            const float bound = __fmaf_ru(ma, mb, md) * (1.0f + 0x1p-20f);
            fast = fin && bound < fabsf((float)tbad);
          }
        } else {
          fast = false;
        }
        if (fast) {
          // a pair is counted when its a, d and b are good: kept as bits
          // of this slab (bit i), tested once per slab
#pragma unroll
          for (int x = 0; x < 4; x++) {
            gma[x] |= (uint32_t)!ka[x] << i;
            gmb[x] |= (uint32_t)!xb[x] << i;
          }
          // (zeroed a and d make a pair with a bad a or d add 0 exactly; a bad
          // b is multiplied away -- u is finite here -- on one path for the
          // whole warp: lanes hold 16 different b groups, a branch on them
          // would diverge)
          T bg[4];
#pragma unroll
          for (int y = 0; y < 4; y++) bg[y] = xb[y] ? (T)0 : (T)1;
#pragma unroll
          for (int y = 0; y < 4; y++)
#pragma unroll
            for (int x = 0; x < 4; x++) {
              const T u = op_add<T>(op_mul<T>(a0[x], b0[y]), d0[x]);
              if constexpr (SLAB) part[y][x] = __fmaf_rn(u, bg[y], part[y][x]);
              else FA::add(acc[y][x], xb[y] ? (T)0 : u);
            }
        } else {
          auto pairs = [&](auto tnan) {
            constexpr bool TN = decltype(tnan)::value;
            auto isbt = [&](T v) { return TN ? (v != v) : (v == tbad); };
#pragma unroll
            for (int y = 0; y < 4; y++)
#pragma unroll
              for (int x = 0; x < 4; x++) {
                const T t = (xa[x] || xb[y]) ? tbad : op_mul<T>(av[x], bv[y]);
                const T u = ((ft && isbt(t)) || xd[x]) ? ubad : op_add<T>(t, dv[x]);
                if (!(fu && isbt(u))) {
                  FA::add(acc[y][x], u);
                  cnt[y][x] = true;
                }
              }
          };
          if (bt.isnan_) pairs(std::true_type{});
          else pairs(std::false_type{});
        }
      } else {
#pragma unroll
        for (int y = 0; y < 4; y++)
#pragma unroll
          for (int x = 0; x < 4; x++) {
            T u;
            if (chain<T, BAD>(g, av[x], bv[y], dv[x], ba, bb, bd, bt, tbad, ubad, u)) {
              if constexpr (SLAB && !BAD) part[y][x] = __fadd_rn(part[y][x], u);
              else FA::add(acc[y][x], u);
            }
          }
      }
    }
    }  // (the slab's values one thread at a time)
    if constexpr (SLAB) {
#pragma unroll
      for (int y = 0; y < 4; y++)
#pragma unroll
        for (int x = 0; x < 4; x++) FA::add(acc[y][x], part[y][x]);
    }
    if constexpr (BAD) {
#pragma unroll
      for (int y = 0; y < 4; y++)
#pragma unroll
        for (int x = 0; x < 4; x++) cnt[y][x] = cnt[y][x] || (gma[x] & gmb[y]) != 0;
    }
  }
  // write c(j, k): c's inc along the j dim and the k dim
  const int64_t c_j = g.L.inc[3][g.jdim], c_k = g.L.inc[3][g.kdim];
  Out *C = reinterpret_cast<Out *>(g.c);
  const Out cbad = from_bits<Out>(g.cbad);
#pragma unroll
  for (int y = 0; y < 4; y++) {
    int64_t j = j0 + tj * 4 + y;
    if (j >= J) continue;
#pragma unroll
    for (int x = 0; x < 4; x++) {
      int64_t k = k0 + tk * 4 + x;
      if (k >= K) continue;
      Out r = (BAD && !cnt[y][x]) ? cbad : FA::value(acc[y][x]);
      C[j * c_j + k * c_k] = r;
    }
  }
}

template <class T, class Out, bool BAD, bool COMP>
__global__ void k_fused_thread(const FusedArgs g) {
  using FA = FAcc<T, Out, COMP>;
  Bad<T> ba{from_bits<T>(g.abad), (bool)g.abad_isnan};
  Bad<T> bb{from_bits<T>(g.bbad), (bool)g.bbad_isnan};
  Bad<T> bd{from_bits<T>(g.dbad), (bool)g.dbad_isnan};
  Bad<T> bt{from_bits<T>(g.tbad), (bool)g.tbad_isnan};
  const T tbad = from_bits<T>(g.tbad), ubad = from_bits<T>(g.ubad);
  const Out cbad = from_bits<Out>(g.cbad);
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < g.rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    int64_t offs[MAXP];
    loop_offsets(g.L, row, offs);
    const T *a = reinterpret_cast<const T *>(g.a) + offs[0];
    const T *b = reinterpret_cast<const T *>(g.b) + offs[1];
    const T *d = reinterpret_cast<const T *>(g.d) + offs[2];
    auto acc = FA::zero();
    int64_t cnt = 0;
    for (int64_t i = 0; i < g.n; i++) {
      T u;
      if (chain<T, BAD>(g, a[i * g.inc_a], b[i * g.inc_b], d[i * g.inc_d], ba, bb, bd, bt,
                        tbad, ubad, u)) {
        FA::add(acc, u);
        cnt++;
      }
    }
    Out *c = reinterpret_cast<Out *>(g.c) + offs[3];
    *c = (BAD && cnt == 0) ? cbad : FA::value(acc);
  }
}

template <class T, class Out, bool COMP>
pdlgb300_error fused_typed(const FusedArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.rows == 0) return e;
  const bool bad = g.fa || g.fb || g.fd;
  if (g.outer) {
    dim3 grid((unsigned)((g.L.size[g.jdim] + FJ - 1) / FJ),
              (unsigned)((g.L.size[g.kdim] + FK - 1) / FK));
    if (bad) {
      if (g.d_is_a) k_fused_outer<T, Out, true, COMP, true><<<grid, FT, 0, s>>>(g);
      else k_fused_outer<T, Out, true, COMP, false><<<grid, FT, 0, s>>>(g);
    } else {
      if (g.d_is_a) k_fused_outer<T, Out, false, COMP, true><<<grid, FT, 0, s>>>(g);
      else k_fused_outer<T, Out, false, COMP, false><<<grid, FT, 0, s>>>(g);
    }
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_fused_outer")) return e;
    pgh::record_kernel("k_fused_outer", (int64_t)grid.x * grid.y, FT);
    return e;
  }
  int64_t grid = std::min<int64_t>((g.rows + 127) / 128, (int64_t)pgh::num_sms() * 64);
  if (bad) k_fused_thread<T, Out, true, COMP><<<(int)grid, 128, 0, s>>>(g);
  else k_fused_thread<T, Out, false, COMP><<<(int)grid, 128, 0, s>>>(g);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_fused_thread")) return e;
  pgh::record_kernel("k_fused_thread", grid, 128);
  return e;
}

}  // namespace

pdlgb300_error launch_fused_smp(int dt, const FusedArgs &g, cudaStream_t s) {
  PG_DISPATCH(dt, {
    using T = typename TT<DT>::T;
    using Out = typename TT<intplus(DT)>::T;
    if constexpr (std::is_same_v<Out, float>)
      if (g.f32_comp) return fused_typed<T, Out, true>(g, s);
    return fused_typed<T, Out, false>(g, s);
  });
  return pgh::err(PDLGB300_EUSERERROR, "sumover_mult_plus: unsupported type %d", dt);
}

}  // namespace pg
