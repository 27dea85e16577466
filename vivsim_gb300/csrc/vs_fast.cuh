// Division-free node physics for the fused grid kernel.
//
// Same mathematics as vs_common.cuh (and the reference), rearranged for instruction
// throughput: divisions by the lattice constants become multiplications by exact
// reciprocals (x / cs2 -> 3 x, x / cs2^2 -> 9 x), per-population divisions by feq use one
// hardware reciprocal each (float) and the velocity uses one reciprocal of rho.  Each
// rearrangement changes a result by about one unit in the last place; the per-operator
// kernels keep the reference's exact operation sequence.
#pragma once

#include "vs_common.cuh"

namespace vs {
namespace fast {

// float: one MUFU reciprocal (rcp.approx, within an ulp of 1/x); double: correctly rounded
template <typename T>
__device__ __forceinline__ T rcp(T x) {
  if constexpr (sizeof(T) == 4) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  } else {
    return __drcp_rn(x);
  }
}

template <class L, typename T>
__device__ __forceinline__ void macro(const T* f, T& rho, T* u) {
  T r = f[0];
#pragma unroll
  for (int i = 1; i < L::Q; ++i) r = r + f[i];
  rho = r;
  const T inv = rcp(r);
#pragma unroll
  for (int d = 0; d < L::D; ++d) {
    T m = T(0);
    bool first = true;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const int c = L::c(i, d);
      if (c == 0) continue;
      const T t = c > 0 ? f[i] : -f[i];
      m = first ? t : m + t;
      first = false;
    }
    u[d] = m * inv;
  }
}

// feq_i = rho w_i (1 + 3 cu + 4.5 cu^2 - 1.5 u^2); for D3Q19 this is the reference's
// 1 + cu/cs2 + cu^2/(2 cs2^2) - u^2/(2 cs2) with cs2 = 1/3.
template <class L, typename T>
__device__ __forceinline__ void equilibrium(T rho, const T* u, T* feq) {
  T usq = u[0] * u[0] + u[1] * u[1];
  if constexpr (L::D == 3) usq = usq + u[2] * u[2];
  const T base = T(1) - T(1.5) * usq;
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    T uc = T(0);
    bool first = true;
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      const int c = L::c(i, d);
      if (c == 0) continue;
      const T t = c > 0 ? u[d] : -u[d];
      uc = first ? t : uc + t;
      first = false;
    }
    const T rw = rho * L::template w<T>(i);
    feq[i] = rw * ((base + T(3) * uc) + T(4.5) * (uc * uc));
  }
}

// D2Q9 KBC (lbm/collision/kbc.py:10-60) with reciprocals of feq.
template <typename T>
__device__ __forceinline__ void collide_kbc(L9, T* f, const T* feq, const CollideParams<T>& p) {
  T fneq[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) fneq[i] = f[i] - feq[i];
  const T nsd = T(0.25) * (((fneq[1] - fneq[2]) + fneq[3]) - fneq[4]);
  const T ssd = T(0.25) * (((fneq[5] - fneq[6]) + fneq[7]) - fneq[8]);
  const T s[9] = {T(0), nsd, -nsd, nsd, -nsd, ssd, -ssd, ssd, -ssd};
  T h[9], ish = T(0), ihh = T(0);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    h[i] = fneq[i] - s[i];
    const T r = rcp(feq[i] + T(1e-20));
    ish = ish + (h[i] * s[i]) * r;
    ihh = ihh + (h[i] * h[i]) * r;
  }
  const T hg = p.inv_omega - (p.one_m_inv * ish) * rcp(ihh + T(1e-20));
#pragma unroll
  for (int i = 0; i < 9; ++i) f[i] = f[i] - p.omega * (s[i] + hg * h[i]);
}

// D3Q19 KBC (lbm3d/collision/kbc.py:8-42): the reference itself multiplies by 1/(feq+eps).
template <typename T>
__device__ __forceinline__ void collide_kbc(L19, T* f, const T* feq, const CollideParams<T>& p) {
  T n[19], s[19];
#pragma unroll
  for (int i = 0; i < 19; ++i) n[i] = f[i] - feq[i];
  projection19_any(n, s);
  T ish = T(0), ihh = T(0);
#pragma unroll
  for (int i = 0; i < 19; ++i) {
    const T h = n[i] - s[i];
    const T inv = rcp(feq[i] + T(1e-20));
    ish = ish + (h * s[i]) * inv;
    ihh = ihh + (h * h) * inv;
  }
  const T hg = p.inv_omega - (p.one_m_inv * ish) * rcp(ihh + T(1e-20));
#pragma unroll
  for (int i = 0; i < 19; ++i) f[i] = f[i] - p.omega * (s[i] + hg * (n[i] - s[i]));
}

// D2Q9 regularised (lbm/collision/reg.py:4-49) with reciprocal constants.
template <typename T>
__device__ __forceinline__ void collide_reg(L9, T* f, const T* feq, const CollideParams<T>& p) {
  T fneq[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) fneq[i] = f[i] - feq[i];
  const T diag_sum = ((fneq[5] + fneq[6]) + fneq[7]) + fneq[8];
  const T pxx = (fneq[1] + fneq[3]) + diag_sum;
  const T pyy = (fneq[2] + fneq[4]) + diag_sum;
  const T pxy = ((fneq[5] - fneq[6]) + fneq[7]) - fneq[8];
  const T tr = (pxx + pyy) * (T)(1.0 / 12.0);
  const T ax = (T(2) * pxx - pyy) * (T)(1.0 / 6.0);
  const T ay = (T(2) * pyy - pxx) * (T)(1.0 / 6.0);
  const T dp = tr + T(0.25) * pxy;
  const T dn = tr - T(0.25) * pxy;
  const T reg[9] = {T(-8) * tr, ax, ay, ax, ay, dp, dn, dp, dn};
#pragma unroll
  for (int i = 0; i < 9; ++i) f[i] = feq[i] + p.one_m_omega * reg[i];
}

template <class L, int COLL, typename T>
__device__ __forceinline__ void collide(T* f, const T* feq, const CollideParams<T>& p, const T* op) {
  if constexpr (COLL == VS_COLLIDE_BGK) collide_bgk<L>(f, feq, p);
  else if constexpr (COLL == VS_COLLIDE_KBC) fast::collide_kbc(L{}, f, feq, p);
  else if constexpr (COLL == VS_COLLIDE_REG) {
    if constexpr (L::Q == 9) fast::collide_reg(L9{}, f, feq, p);
    else vs::collide_reg(L19{}, f, feq, p);
  } else collide_mrt<L>(f, feq, op);
}

}  // namespace fast
}  // namespace vs
