// Immersed-boundary device helpers shared by the per-op IB entry points and the fused
// IB step: the 1-D discrete delta kernels of vivsim/ib/kernels.py and the stencil
// geometry of vivsim/ib/stencil.py and vivsim/ib3d/stencil.py.
#pragma once

#include "vs_common.cuh"

namespace vs {

// The kernels are written with uncontracted operations (mul_rn / add_rn / sub_rn), so the
// fused body kernels and the per-operator kernels compute identical weights.

// Peskin 3-point, vivsim/ib/kernels.py:4-22
template <typename T>
__device__ __forceinline__ T delta_peskin3(T r) {
  const T a = fabs(r);
  if (a > T(1.5)) return T(0);
  const T aa = mul_rn(a, a);
  if (a < T(0.5)) return add_rn(T(1), sqrt(sub_rn(T(1), mul_rn(T(3), aa)))) / T(3);
  return sub_rn(sub_rn(T(5), mul_rn(T(3), a)), sqrt(sub_rn(add_rn(T(-2), mul_rn(T(6), a)), mul_rn(T(3), aa)))) /
         T(6);
}
// Peskin 4-point, vivsim/ib/kernels.py:25-43
template <typename T>
__device__ __forceinline__ T delta_peskin4(T r) {
  const T a = fabs(r);
  if (a > T(2)) return T(0);
  const T aa4 = mul_rn(T(4), mul_rn(a, a));
  if (a < T(1))
    return mul_rn(add_rn(sub_rn(T(3), mul_rn(T(2), a)), sqrt(sub_rn(add_rn(T(1), mul_rn(T(4), a)), aa4))), T(0.125));
  return mul_rn(sub_rn(sub_rn(T(5), mul_rn(T(2), a)), sqrt(sub_rn(add_rn(T(-7), mul_rn(T(12), a)), aa4))), T(0.125));
}
// Cosine 4-point, vivsim/ib/kernels.py:46-61
template <typename T>
__device__ __forceinline__ T delta_cosine4(T r) {
  const T a = fabs(r);
  if (a > T(2)) return T(0);
  return mul_rn(add_rn(T(1), cos(mul_rn(mul_rn((T)3.14159265358979323846, a), T(0.5)))), T(0.25));
}
template <typename T>
__device__ __forceinline__ T delta(int kernel, T r) {
  return kernel == VS_KERNEL_PESKIN3 ? delta_peskin3(r) : (kernel == VS_KERNEL_PESKIN4 ? delta_peskin4(r) : delta_cosine4(r));
}

// derivative of the delta kernels (ib/kernels.py), d phi / d r
template <typename T>
__device__ __forceinline__ T ddelta(int kernel, T r) {
  const T a = fabs(r), sg = r < T(0) ? T(-1) : T(1);
  if (kernel == VS_KERNEL_PESKIN4) {
    if (a >= T(2)) return T(0);
    if (a < T(1)) {
      const T q = sqrt((T(1) + T(4) * a) - T(4) * (a * a));
      return sg * T(0.125) * (T(-2) + (T(2) - T(4) * a) / q);
    }
    const T q = sqrt((T(-7) + T(12) * a) - T(4) * (a * a));
    return sg * T(0.125) * (T(-2) - (T(6) - T(4) * a) / q);
  }
  if (kernel == VS_KERNEL_PESKIN3) {
    if (a >= T(1.5)) return T(0);
    if (a < T(0.5)) return sg * (-(T(3) * a) / sqrt(T(1) - T(3) * (a * a))) / T(3);
    return sg * (T(-3) - (T(3) - T(3) * a) / sqrt((T(-2) + T(6) * a) - T(3) * (a * a))) / T(6);
  }
  if (a >= T(2)) return T(0);
  const T k = (T)3.14159265358979323846 * T(0.5);
  return sg * T(-0.25) * k * sin(k * a);
}

// floor() to int32 as in jnp.floor(x).astype(jnp.int32)
template <typename T>
__device__ __forceinline__ int ifloor(T x) { return (int)floor(x); }

}  // namespace vs

namespace vs {
// Views into the sorted (node, pair) CSR of a stencil: sorted keys and pair ids, segment
// heads, 0-based unique-node ids per sorted position, and the unique-node id of each pair.
struct IbCsrView {
  int32_t* skeys;
  int32_t* sids;
  int32_t* head;
  int32_t* uid;
  int32_t* pair_uid;
};
int ib_build_csr(const int32_t* I, int64_t P, int64_t n_grid, void* workspace, int m, int s, IbCsrView* out,
                 cudaStream_t st);

// Multi-direct forcing over the pair CSR in `workspace`; with csr_ready the CSR built by
// an earlier call for the same stencil indices is reused (defined in vs_ops_ib.cu).
int ib_mdf_run(int dtype, bool csr_ready, const void* grid_u, int c, int64_t n_grid, const void* W, const int32_t* I,
               int m, int s, const void* u_target, const void* ds, double ds_scalar, int n_iter, void* grid_force,
               void* marker_force, void* workspace, size_t workspace_bytes, void* stream);
}  // namespace vs
