// Forward-mode dual numbers for the hand-written adjoints: v carries the value, d one
// directional derivative.  Every formula of vs_common.cuh / vs_boundary.cuh is a template
// on its scalar type, so evaluating it on Dual<T> seeded with a unit tangent gives one
// column of its Jacobian.
#pragma once

#include "vs_common.cuh"

namespace vs {

template <typename T>
struct Dual {
  T v, d;
  __device__ Dual() : v(0), d(0) {}
  __device__ Dual(T a, T b) : v(a), d(b) {}
  template <typename U>
  __device__ Dual(U a) : v((T)a), d(0) {}
};
template <typename T>
__device__ __forceinline__ Dual<T> operator+(Dual<T> a, Dual<T> b) { return Dual<T>(a.v + b.v, a.d + b.d); }
template <typename T>
__device__ __forceinline__ Dual<T> operator-(Dual<T> a, Dual<T> b) { return Dual<T>(a.v - b.v, a.d - b.d); }
template <typename T>
__device__ __forceinline__ Dual<T> operator-(Dual<T> a) { return Dual<T>(-a.v, -a.d); }
template <typename T>
__device__ __forceinline__ Dual<T> operator*(Dual<T> a, Dual<T> b) {
  return Dual<T>(a.v * b.v, a.d * b.v + a.v * b.d);
}
template <typename T>
__device__ __forceinline__ Dual<T> operator/(Dual<T> a, Dual<T> b) {
  const T q = a.v / b.v;
  return Dual<T>(q, (a.d - q * b.d) / b.v);
}
template <typename T>
__device__ __forceinline__ Dual<T>& operator+=(Dual<T>& a, Dual<T> b) { return a = a + b; }

// the separately rounded products and sums of the shared formulas, on dual numbers
template <typename T>
__device__ __forceinline__ Dual<T> mul_rn(Dual<T> a, Dual<T> b) {
  return Dual<T>(mul_rn(a.v, b.v), a.d * b.v + a.v * b.d);
}
template <typename T>
__device__ __forceinline__ Dual<T> add_rn(Dual<T> a, Dual<T> b) { return Dual<T>(add_rn(a.v, b.v), a.d + b.d); }
template <typename T>
__device__ __forceinline__ Dual<T> sub_rn(Dual<T> a, Dual<T> b) { return Dual<T>(sub_rn(a.v, b.v), a.d - b.d); }

}  // namespace vs
