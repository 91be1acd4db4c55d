// adjoint.cu -- the gradient reduction shared by the backward calls:
// out(o) = scale * sum over r of x(o, r) [* y(o, r)], where o walks the
// input's own dims and r the dims it was broadcast along (recomputed from
// the upstream gradient, nothing stored from the forward pass).
#include "args.cuh"

namespace pg {
namespace {

template <class T, bool HASY>
__global__ void __launch_bounds__(256) k_unbroadcast(const UnbArgs g) {
  const T *X = reinterpret_cast<const T *>(g.x);
  const T *Y = reinterpret_cast<const T *>(g.y);
  T *O = reinterpret_cast<T *>(g.out);
  for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < g.Lo.total;
       o += (int64_t)gridDim.x * blockDim.x) {
    int64_t oo[MAXP];
    loop_offsets(g.Lo, o, oo);
    double s = 0.0;
    if (g.Lr.nd == 1) {
      const int64_t ix = g.Lr.inc[0][0], iy = g.Lr.inc[1][0];
      for (int64_t r = 0; r < g.Lr.total; r++) {
        double v = (double)X[oo[0] + r * ix];
        if (HASY) v *= (double)Y[oo[1] + r * iy];
        s += v;
      }
    } else {
      for (int64_t r = 0; r < g.Lr.total; r++) {
        int64_t ro[MAXP];
        loop_offsets(g.Lr, r, ro);
        double v = (double)X[oo[0] + ro[0]];
        if (HASY) v *= (double)Y[oo[1] + ro[1]];
        s += v;
      }
    }
    O[oo[2]] = (T)(s * g.scale);
  }
}

}  // namespace

pdlgb300_error launch_unbroadcast(int dt, const UnbArgs &g, cudaStream_t s) {
  pdlgb300_error e = pgh::ok();
  if (g.Lo.total == 0) return e;
  int64_t grid = std::min<int64_t>((g.Lo.total + 255) / 256, (int64_t)pgh::num_sms() * 32);
  const bool hasy = g.y != nullptr;
  if (dt == PDLGB300_F) {
    if (hasy) k_unbroadcast<float, true><<<(int)grid, 256, 0, s>>>(g);
    else k_unbroadcast<float, false><<<(int)grid, 256, 0, s>>>(g);
  } else if (dt == PDLGB300_D) {
    if (hasy) k_unbroadcast<double, true><<<(int)grid, 256, 0, s>>>(g);
    else k_unbroadcast<double, false><<<(int)grid, 256, 0, s>>>(g);
  } else {
    return pgh::err(PDLGB300_EUSERERROR, "backward: float or double only (type %d)", dt);
  }
  if (!pgh::cuda_check(cudaGetLastError(), &e, "k_unbroadcast")) return e;
  pgh::record_kernel("k_unbroadcast", grid, 256);
  return e;
}

}  // namespace pg
