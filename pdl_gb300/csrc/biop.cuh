// biop.cuh -- the element operation of each PDL::Ops binary op, shared by
// the broadcast kernel (elem.cu) and the fused expression reductions
// (expr.cu).
#pragma once
#include "args.cuh"

namespace pg {

// Binary op codes (lib/PDL/Ops.pd:288-307): each computes `$c() = $a() op
// $b()` in the working type T, as the reference's C does: integers wrap,
// floats are IEEE-rounded with no contraction, comparisons give 0 or 1,
// shifts and bit ops exist for integer types only.
enum BiopCode {
  B_PLUS, B_MULT, B_MINUS, B_DIVIDE, B_GT, B_LT, B_LE, B_GE, B_EQ, B_NE,
  B_SHL, B_SHR, B_OR2, B_AND2, B_XOR, B_NCODES
};

template <int OP> constexpr bool biop_int_only() {
  return OP == B_SHL || OP == B_SHR || OP == B_OR2 || OP == B_AND2 || OP == B_XOR;
}

template <class T, int OP>
__device__ __forceinline__ T biop_apply(T a, T b) {
  if constexpr (OP == B_PLUS) return op_add<T>(a, b);
  else if constexpr (OP == B_MULT) return op_mul<T>(a, b);
  else if constexpr (OP == B_MINUS) {
    if constexpr (std::is_floating_point_v<T>) return std::is_same_v<T, float> ? (T)__fsub_rn(a, b) : (T)__dsub_rn(a, b);
    else return (T)(uns_t<T>)((uns_t<T>)a - (uns_t<T>)b);
  } else if constexpr (OP == B_DIVIDE) {
    // integer division by zero (and the minimum over -1) has no defined
    // result in the reference's C; the GPU gives its own value there
    if constexpr (std::is_same_v<T, float>) return __fdiv_rn(a, b);
    else if constexpr (std::is_same_v<T, double>) return __ddiv_rn(a, b);
    else return (T)(a / b);
  } else if constexpr (OP == B_GT) return (T)(a > b);
  else if constexpr (OP == B_LT) return (T)(a < b);
  else if constexpr (OP == B_LE) return (T)(a <= b);
  else if constexpr (OP == B_GE) return (T)(a >= b);
  else if constexpr (OP == B_EQ) return (T)(a == b);
  else if constexpr (OP == B_NE) return (T)(a != b);
  else if constexpr (std::is_integral_v<T>) {
    // C's usual promotions, then back to T
    if constexpr (OP == B_SHL) return (T)(a << b);
    else if constexpr (OP == B_SHR) return (T)(a >> b);
    else if constexpr (OP == B_OR2) return (T)(a | b);
    else if constexpr (OP == B_AND2) return (T)(a & b);
    else return (T)(a ^ b);
  } else {
    return a;  // not instantiated: type selection gives bit ops an integer type
  }
}

}  // namespace pg
