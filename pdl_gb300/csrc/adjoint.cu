// adjoint.cu -- the gradient reduction shared by the backward calls:
// out(o) = scale * sum over r of x(o, r) [* y(o, r)], where o walks the
// input's own dims and r the dims it was broadcast along (recomputed from
// the upstream gradient, nothing stored from the forward pass).
//
// float32 sums are compensated (the same float-float accumulator as the
// reductions), float64 sums plain FP64.  Three shapes of work:
//  * nothing to reduce (r is one element): one thread per output;
//  * r contiguous in x (a gradient summed along its dim 0): a warp per
//    output, lanes striding r with coalesced loads;
//  * otherwise (r strided, e.g. a bias broadcast along the rows of a
//    matrix): blocks of 32 outputs x 8 r-lanes, consecutive outputs on
//    consecutive lanes (coalesced when o is contiguous); when outputs are
//    too few to fill the GPU, r is split over several blocks whose partial
//    sums a second kernel adds in split order (deterministic).
#include "reduce.cuh"

namespace pg {
namespace {

template <class T> struct UAcc {
  using A = std::conditional_t<std::is_same_v<T, float>, FF, double>;
  __device__ static A zero() {
    A a;
    memset(&a, 0, sizeof a);
    return a;
  }
  __device__ static void add(A &a, T v) {
    if constexpr (std::is_same_v<T, float>) ff_add(a, v);
    else a = __dadd_rn(a, v);
  }
  __device__ static void merge(A &a, const A &b) {
    if constexpr (std::is_same_v<T, float>) ff_merge(a, b);
    else a = __dadd_rn(a, b);
  }
  __device__ static double value(const A &a) {
    if constexpr (std::is_same_v<T, float>) return (double)a.hi + (double)a.lo;
    else return a;
  }
};

template <class T, bool HASY>
__device__ __forceinline__ T term(const UnbArgs &g, const int64_t *oo, int64_t r) {
  const T *X = reinterpret_cast<const T *>(g.x);
  const T *Y = reinterpret_cast<const T *>(g.y);
  int64_t rx, ry;
  if (g.Lr.nd == 1) {
    rx = r * g.Lr.inc[0][0];
    ry = r * g.Lr.inc[1][0];
  } else {
    int64_t ro[MAXP];
    loop_offsets(g.Lr, r, ro);
    rx = ro[0];
    ry = ro[1];
  }
  T v = X[oo[0] + rx];
  if constexpr (HASY) v = op_mul<T>(v, Y[oo[1] + ry]);
  return v;
}

template <class T> __device__ __forceinline__ void put(const UnbArgs &g, int64_t off, double s) {
  reinterpret_cast<T *>(g.out)[off] = (T)(s * g.scale);
}

// r has one element: a scaled copy (sumover/average backward).
template <class T, bool HASY>
__global__ void __launch_bounds__(256) k_unb_map(const UnbArgs g) {
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < g.Lo.total;
       o += (int64_t)gridDim.x * blockDim.x) {
    int64_t oo[MAXP];
    loop_offsets(g.Lo, o, oo);
    put<T>(g, oo[2], (double)term<T, HASY>(g, oo, 0));
  }
}

// A warp per output, lanes along a contiguous r.
template <class T, bool HASY>
__global__ void __launch_bounds__(256) k_unb_rows(const UnbArgs g) {
  using U = UAcc<T>;
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t o = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); o < g.Lo.total;
       o += nw) {
    int64_t oo[MAXP];
    loop_offsets(g.Lo, o, oo);
    typename U::A a = U::zero();
    for (int64_t r = lane; r < g.Lr.total; r += 32) U::add(a, term<T, HASY>(g, oo, r));
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) U::merge(a, shfl_down_any(a, d));
    if (lane == 0) put<T>(g, oo[2], U::value(a));
  }
}

// 32 outputs x 8 r-lanes per block; blockIdx.y picks the r split.
template <class T, bool HASY>
__global__ void __launch_bounds__(256) k_unb_cols(const UnbArgs g) {
  using U = UAcc<T>;
  using A = typename U::A;
  __shared__ A part[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t o = (int64_t)blockIdx.x * 32 + tx;
  const int64_t chunk = (g.Lr.total + g.nsplit - 1) / g.nsplit;
  const int64_t lo = (int64_t)blockIdx.y * chunk;
  const int64_t hi = lo + chunk < g.Lr.total ? lo + chunk : g.Lr.total;
  A a = U::zero();
  int64_t oo[MAXP];
  if (o < g.Lo.total) {
    loop_offsets(g.Lo, o, oo);
    for (int64_t r = lo + ty; r < hi; r += 8) U::add(a, term<T, HASY>(g, oo, r));
  }
  part[ty][tx] = a;
  __syncthreads();
  if (ty == 0 && o < g.Lo.total) {
#pragma unroll
    for (int k = 1; k < 8; k++) U::merge(a, part[k][tx]);
    if (g.nsplit == 1) put<T>(g, oo[2], U::value(a));
    else reinterpret_cast<A *>(g.partials)[(int64_t)blockIdx.y * g.Lo.total + o] = a;
  }
}

// The splits' partial sums of each output, added in split order.
template <class T>
__global__ void __launch_bounds__(256) k_unb_combine(const UnbArgs g) {
  using U = UAcc<T>;
  using A = typename U::A;
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < g.Lo.total;
       o += (int64_t)gridDim.x * blockDim.x) {
    const A *p = reinterpret_cast<const A *>(g.partials);
    A a = p[o];
    for (int s = 1; s < g.nsplit; s++) U::merge(a, p[(int64_t)s * g.Lo.total + o]);
    int64_t oo[MAXP];
    loop_offsets(g.Lo, o, oo);
    put<T>(g, oo[2], U::value(a));
  }
}

template <class T, bool HASY>
pdlgb300_error launch_typed(UnbArgs g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  const int nsm = pgh::num_sms();
  const char *name;
  int64_t grid;
  if (g.Lr.total <= 1) {
    grid = std::min<int64_t>((g.Lo.total + 255) / 256, (int64_t)nsm * 32);
    k_unb_map<T, HASY><<<(int)grid, 256, 0, s>>>(g);
    name = "k_unb_map";
  } else if (g.Lr.nd == 1 && g.Lr.inc[0][0] == 1) {
    grid = std::min<int64_t>((g.Lo.total + 7) / 8, (int64_t)nsm * 64);
    k_unb_rows<T, HASY><<<(int)grid, 256, 0, s>>>(g);
    name = "k_unb_rows";
  } else {
    const int64_t ob = (g.Lo.total + 31) / 32;
    g.nsplit = 1;
    void *scratch = nullptr;
    if (ob < (int64_t)nsm * 4 && g.Lr.total >= 256) {
      // enough r splits to give every SM a few blocks, 64 r's at least each
      const int64_t want = ((int64_t)nsm * 4 + ob - 1) / ob;
      g.nsplit = (int)std::max<int64_t>(1, std::min<int64_t>(want, g.Lr.total / 64));
    }
    if (g.nsplit > 1) {
      const size_t bytes = (size_t)g.nsplit * g.Lo.total * sizeof(typename UAcc<T>::A);
      if (cudaMallocAsync(&scratch, bytes, s) != cudaSuccess) {
        cudaGetLastError();
        return pgh::err(PDLGB300_EFATAL, "backward: no device memory for partial sums");
      }
      g.partials = scratch;
    }
    dim3 gr((unsigned)ob, (unsigned)g.nsplit);
    k_unb_cols<T, HASY><<<gr, 256, 0, s>>>(g);
    grid = ob * g.nsplit;
    name = "k_unb_cols";
    if (g.nsplit > 1) {
      if (pgh::cuda_check(cudaGetLastError(), &e, name)) pgh::record_kernel(name, grid, 256);
      const int64_t gc = std::min<int64_t>((g.Lo.total + 255) / 256, (int64_t)nsm * 32);
      k_unb_combine<T><<<(int)gc, 256, 0, s>>>(g);
      cudaFreeAsync(scratch, s);
      name = "k_unb_combine";
      grid = gc;
    }
  }
  if (!pgh::cuda_check(cudaGetLastError(), &e, name)) return e;
  pgh::record_kernel(name, grid, 256);
  return e;
}

}  // namespace

pdlgb300_error launch_unbroadcast(int dt, const UnbArgs &g, cudaStream_t s) {
  if (g.Lo.total == 0) return pgh::ok();
  const bool hasy = g.y != nullptr;
  if (dt == PDLGB300_F) return hasy ? launch_typed<float, true>(g, s) : launch_typed<float, false>(g, s);
  if (dt == PDLGB300_D) return hasy ? launch_typed<double, true>(g, s) : launch_typed<double, false>(g, s);
  return pgh::err(PDLGB300_EUSERERROR, "backward: float or double only (type %d)", dt);
}

}  // namespace pg
