// elem.cu -- PDL::Ops binary ops under broadcasting (lib/PDL/Ops.pd:104-153,
// 288-307: plus, mult, minus, divide, the comparisons, shifts and bit ops)
// and type conversion (lib/PDL/Core/pdlconv.c:163-172).
//
// One thread per output element along the innermost collapsed broadcast dim
// (coalesced), the outer dims flattened onto grid.y.  A fully contiguous
// operand set takes a 16-byte vectorised path.  Every product and sum is
// rounded exactly as the reference's C (no FMA contraction); integers wrap.
#include "biop.cuh"

namespace pg {

template <class T, int OP, bool BAD>
__device__ __forceinline__ T biop_elem(const BiopArgs &g, T va, T vb, const Bad<T> &ba,
                                       const Bad<T> &bb, T cbad, bool &anybad) {
  if constexpr (BAD) {
    if ((g.statebad_a && ba.is(va)) || (g.statebad_b && bb.is(vb))) {
      anybad = true;
      return cbad;
    }
  }
  return biop_apply<T, OP>(va, vb);
}

template <class T, int OP, bool BAD>
__global__ void __launch_bounds__(256) k_biop(const BiopArgs g) {
  const T *A = reinterpret_cast<const T *>(g.a);
  const T *B = reinterpret_cast<const T *>(g.b);
  T *C = reinterpret_cast<T *>(g.c);
  Bad<T> ba{from_bits<T>(g.abad), (bool)g.abad_isnan};
  Bad<T> bb{from_bits<T>(g.bbad), (bool)g.bbad_isnan};
  T cbad = from_bits<T>(g.cbad);
  bool anybad = false;
  const int64_t s0 = g.L.size[0];
  const int64_t outer = s0 ? g.L.total / s0 : 0;
  const int64_t ia = g.L.inc[0][0], ib = g.L.inc[1][0], ic = g.L.inc[2][0];
  for (int64_t o = blockIdx.y; o < outer; o += gridDim.y) {
    int64_t oa = 0, ob = 0, oc = 0, r = o;
    for (int k = 1; k < g.L.nd; k++) {
      int64_t s = g.L.size[k], q = r / s, i = r - q * s;
      r = q;
      oa += i * g.L.inc[0][k];
      ob += i * g.L.inc[1][k];
      oc += i * g.L.inc[2][k];
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < s0;
         i += (int64_t)gridDim.x * blockDim.x) {
      T va = A[oa + i * ia], vb = B[ob + i * ib];
      C[oc + i * ic] = biop_elem<T, OP, BAD>(g, va, vb, ba, bb, cbad, anybad);
    }
  }
  if (BAD && anybad) *g.setbad = 1;
}

// All three operands contiguous over the whole loop, 16-byte aligned.
template <class T, int OP, bool BAD>
__global__ void __launch_bounds__(256) k_biop_flat(const BiopArgs g) {
  constexpr int V = 16 / sizeof(T);
  struct alignas(16) Vec { T e[V]; };
  const Vec *A = reinterpret_cast<const Vec *>(g.a);
  const Vec *B = reinterpret_cast<const Vec *>(g.b);
  Vec *C = reinterpret_cast<Vec *>(g.c);
  Bad<T> ba{from_bits<T>(g.abad), (bool)g.abad_isnan};
  Bad<T> bb{from_bits<T>(g.bbad), (bool)g.bbad_isnan};
  T cbad = from_bits<T>(g.cbad);
  bool anybad = false;
  const int64_t nv = g.L.total / V;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv;
       i += (int64_t)gridDim.x * blockDim.x) {
    Vec va = A[i], vb = B[i], vc;
#pragma unroll
    for (int e = 0; e < V; e++)
      vc.e[e] = biop_elem<T, OP, BAD>(g, va.e[e], vb.e[e], ba, bb, cbad, anybad);
    C[i] = vc;
  }
  const T *As = reinterpret_cast<const T *>(g.a);
  const T *Bs = reinterpret_cast<const T *>(g.b);
  T *Cs = reinterpret_cast<T *>(g.c);
  for (int64_t i = nv * V + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.L.total;
       i += (int64_t)gridDim.x * blockDim.x)
    Cs[i] = biop_elem<T, OP, BAD>(g, As[i], Bs[i], ba, bb, cbad, anybad);
  if (BAD && anybad) *g.setbad = 1;
}

template <class T, int OP>
static pdlgb300_error biop_typed(const BiopArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const int64_t s0 = g.L.size[0];
  if (g.L.total == 0) return e;
  bool flat = g.L.nd == 1 && g.L.inc[0][0] == 1 && g.L.inc[1][0] == 1 &&
              g.L.inc[2][0] == 1 && ((uintptr_t)g.a % 16 == 0) &&
              ((uintptr_t)g.b % 16 == 0) && ((uintptr_t)g.c % 16 == 0);
  const int nsm = pgh::num_sms();
  if (flat) {
    int64_t nv = g.L.total / (16 / sizeof(T));
    int64_t grid = std::min<int64_t>((nv + 255) / 256, (int64_t)nsm * 16);
    if (grid < 1) grid = 1;
    if (g.bad) k_biop_flat<T, OP, true><<<(int)grid, 256, 0, s>>>(g);
    else k_biop_flat<T, OP, false><<<(int)grid, 256, 0, s>>>(g);
    if (!pgh::cuda_check(cudaGetLastError(), &e, "k_biop_flat")) return e;
    pgh::record_kernel("k_biop_flat", grid, 256);
    return e;
  }
  int64_t outer = g.L.total / s0;
  int64_t gx = std::min<int64_t>((s0 + 255) / 256, (int64_t)nsm * 8);
  int64_t gy = std::min<int64_t>(outer, 65535);
  if (gx * gy < nsm * 4 && outer > gy) gy = 65535;
  dim3 grid((unsigned)gx, (unsigned)gy);
  if (g.bad) k_biop<T, OP, true><<<grid, 256, 0, s>>>(g);
  else k_biop<T, OP, false><<<grid, 256, 0, s>>>(g);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_biop")) return e;
  pgh::record_kernel("k_biop", gx * gy, 256);
  return e;
}

template <class T, int OP>
static pdlgb300_error biop_code(const BiopArgs &g, cudaStream_t s) {
  if constexpr (biop_int_only<OP>() && !std::is_integral_v<T>)
    return pgh::err(PDLGB300_EUSERERROR, "bit operations need an integer type");
  else return biop_typed<T, OP>(g, s);
}

pdlgb300_error launch_biop(int op, int dt, const BiopArgs &g, cudaStream_t s) {
  PG_DISPATCH(dt, {
    using T = typename TT<DT>::T;
    switch (op) {
      case B_PLUS: return biop_code<T, B_PLUS>(g, s);
      case B_MULT: return biop_code<T, B_MULT>(g, s);
      case B_MINUS: return biop_code<T, B_MINUS>(g, s);
      case B_DIVIDE: return biop_code<T, B_DIVIDE>(g, s);
      case B_GT: return biop_code<T, B_GT>(g, s);
      case B_LT: return biop_code<T, B_LT>(g, s);
      case B_LE: return biop_code<T, B_LE>(g, s);
      case B_GE: return biop_code<T, B_GE>(g, s);
      case B_EQ: return biop_code<T, B_EQ>(g, s);
      case B_NE: return biop_code<T, B_NE>(g, s);
      case B_SHL: return biop_code<T, B_SHL>(g, s);
      case B_SHR: return biop_code<T, B_SHR>(g, s);
      case B_OR2: return biop_code<T, B_OR2>(g, s);
      case B_AND2: return biop_code<T, B_AND2>(g, s);
      case B_XOR: return biop_code<T, B_XOR>(g, s);
    }
  });
  return pgh::err(PDLGB300_EUSERERROR, "binary op: unsupported type %d or op %d", dt, op);
}

// ------------------------------------------------------------ conversion

template <class From, class To>
__device__ __forceinline__ To convert_value(From v) {
  if constexpr (std::is_unsigned_v<To> && std::is_floating_point_v<From>) {
    return (To)(long long)v;  // PDL: unsigned targets via (intmax_t)
  } else {
    return (To)v;
  }
}

template <class From, class To>
__global__ void __launch_bounds__(256) k_convert(const ConvArgs g) {
  const From *S = reinterpret_cast<const From *>(g.src);
  To *D = reinterpret_cast<To *>(g.dst);
  Bad<From> bs{from_bits<From>(g.sbad), (bool)g.sbad_isnan};
  To dbad = from_bits<To>(g.dbad);
  const int64_t s0 = g.L.size[0];
  const int64_t outer = s0 ? g.L.total / s0 : 0;
  for (int64_t o = blockIdx.y; o < outer; o += gridDim.y) {
    int64_t os = 0, od = 0, r = o;
    for (int k = 1; k < g.L.nd; k++) {
      int64_t sz = g.L.size[k], q = r / sz, i = r - q * sz;
      r = q;
      os += i * g.L.inc[0][k];
      od += i * g.L.inc[1][k];
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < s0;
         i += (int64_t)gridDim.x * blockDim.x) {
      From v = S[os + i * g.L.inc[0][0]];
      D[od + i * g.L.inc[1][0]] = (g.bad && bs.is(v)) ? dbad : convert_value<From, To>(v);
    }
  }
}

template <class From>
static pdlgb300_error convert_from(int to, const ConvArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.L.total == 0) return e;
  const int64_t s0 = g.L.size[0];
  int64_t outer = g.L.total / s0;
  int64_t gx = std::min<int64_t>((s0 + 255) / 256, (int64_t)pgh::num_sms() * 8);
  int64_t gy = std::min<int64_t>(outer, 65535);
  dim3 grid((unsigned)gx, (unsigned)gy);
  bool done = false;
  PG_DISPATCH(to, {
    k_convert<From, typename TT<DT>::T><<<grid, 256, 0, s>>>(g);
    done = true;
  });
  if (!done) return pgh::err(PDLGB300_EUSERERROR, "convert: unsupported type %d", to);
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_convert")) return e;
  pgh::record_kernel("k_convert", gx * gy, 256);
  return e;
}

pdlgb300_error launch_convert(int from, int to, const ConvArgs &g, cudaStream_t s) {
  PG_DISPATCH(from, return convert_from<typename TT<DT>::T>(to, g, s));
  return pgh::err(PDLGB300_EUSERERROR, "convert: unsupported type %d", from);
}

}  // namespace pg
