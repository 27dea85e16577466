// Shared device code for the vivsim GB300 kernels: lattice tables, error plumbing and the
// per-node physics (moments, equilibria, collisions, forcing) of the D2Q9 and D3Q19 models.
//
// Every node-local formula follows the operation order of the reference function it
// restates (file:line cited per function), so that results agree with the reference to
// the last few ulps.  Layout everywhere: structure of arrays, f[q][node], node index
// n = (x * NY + y) * NZ + z with the last spatial axis contiguous.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vivsim_gb300.h"

namespace vs {

// ------------------------------------------------------------------ error plumbing
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);
#define VS_CHECK_LAUNCH(where)                                                   \
  do {                                                                           \
    cudaError_t _e = cudaGetLastError();                                         \
    if (_e != cudaSuccess) return ::vs::cuda_status(_e, where);                  \
  } while (0)
#define VS_REQUIRE(cond, ...)                                                    \
  do {                                                                           \
    if (!(cond)) {                                                               \
      ::vs::set_error(__VA_ARGS__);                                              \
      return VS_ERR_INVALID_ARG;                                                 \
    }                                                                            \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Correctly rounded products and sums that the compiler never contracts into an FMA, for
// the immersed-boundary arithmetic whose results must not depend on contraction choices.
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b) {
  if constexpr (sizeof(T) == 4) return __fmul_rn(a, b);
  else return __dmul_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b) {
  if constexpr (sizeof(T) == 4) return __fadd_rn(a, b);
  else return __dadd_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T sub_rn(T a, T b) {
  if constexpr (sizeof(T) == 4) return __fsub_rn(a, b);
  else return __dsub_rn(a, b);
}

inline unsigned grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  return (unsigned)(g < 1 ? 1 : g);
}

// ------------------------------------------------------------------ D2Q9 tables
// vivsim/lbm/lattice.py:39-61.  Numbering:  6 2 5 / 3 0 1 / 7 4 8.
__host__ __device__ constexpr int q9_cx(int i) {
  return (i == 1 || i == 5 || i == 8) ? 1 : (i == 3 || i == 6 || i == 7) ? -1 : 0;
}
__host__ __device__ constexpr int q9_cy(int i) {
  return (i == 2 || i == 5 || i == 6) ? 1 : (i == 4 || i == 7 || i == 8) ? -1 : 0;
}
__host__ __device__ constexpr int q9_opp(int i) {
  return i == 0 ? 0 : (i <= 4 ? ((i + 1) % 4) + 1 : ((i - 5 + 2) % 4) + 5);
}
// Weights are float32 literals in the reference; float64 math keeps those rounded values.
template <typename T>
__host__ __device__ constexpr T q9_w(int i) {
  return i == 0 ? (T)(float)(4.0 / 9.0) : (i <= 4 ? (T)(float)(1.0 / 9.0) : (T)(float)(1.0 / 36.0));
}

// ------------------------------------------------------------------ D3Q19 tables
// vivsim/lbm3d/lattice.py:39-67.
__host__ __device__ constexpr int q19_c(int i, int d) {
  // rows of D3Q19.c
  return d == 0 ? (i == 1 || i == 7 || i == 9 || i == 11 || i == 13)   ? 1
                  : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1
                                                                       : 0
       : d == 1 ? (i == 3 || i == 7 || i == 8 || i == 15 || i == 17)   ? 1
                  : (i == 4 || i == 9 || i == 10 || i == 16 || i == 18) ? -1
                                                                       : 0
                : (i == 5 || i == 11 || i == 12 || i == 15 || i == 16) ? 1
                  : (i == 6 || i == 13 || i == 14 || i == 17 || i == 18) ? -1
                                                                        : 0;
}
__host__ __device__ constexpr int q19_opp(int i) {
  return i == 0 ? 0 : (i <= 6 ? (i % 2 ? i + 1 : i - 1) : (i <= 10 ? 17 - i : (i <= 14 ? 25 - i : 33 - i)));
}
template <typename T>
__host__ __device__ constexpr T q19_w(int i) {
  return i == 0 ? (T)(float)(1.0 / 3.0) : (i <= 6 ? (T)(float)(1.0 / 18.0) : (T)(float)(1.0 / 36.0));
}

// Lattice descriptors used as template parameters.
struct L9 {
  static constexpr int Q = 9, D = 2;
  __host__ __device__ static constexpr int c(int i, int d) { return d == 0 ? q9_cx(i) : (d == 1 ? q9_cy(i) : 0); }
  __host__ __device__ static constexpr int opp(int i) { return q9_opp(i); }
  template <typename T>
  __host__ __device__ static constexpr T w(int i) { return q9_w<T>(i); }
};
struct L19 {
  static constexpr int Q = 19, D = 3;
  __host__ __device__ static constexpr int c(int i, int d) { return q19_c(i, d); }
  __host__ __device__ static constexpr int opp(int i) { return q19_opp(i); }
  template <typename T>
  __host__ __device__ static constexpr T w(int i) { return q19_w<T>(i); }
};

// ------------------------------------------------------------------ moments
// D2Q9: vivsim/lbm/basic.py:88-111 (direction groups right/left/up/down).
template <typename T>
__device__ __forceinline__ void macro(L9, const T* f, T& rho, T* u) {
  T r = f[0];
#pragma unroll
  for (int i = 1; i < 9; ++i) r = r + f[i];
  rho = r;
  u[0] = (((f[1] + f[5]) + f[8]) - ((f[3] + f[7]) + f[6])) / r;
  u[1] = (((f[2] + f[5]) + f[6]) - ((f[4] + f[7]) + f[8])) / r;
}

// D3Q19: vivsim/lbm3d/basic.py:90-106 (rho = sum f; u = c^T f / rho, summed in q order).
template <typename T>
__device__ __forceinline__ void macro(L19, const T* f, T& rho, T* u) {
  T r = f[0];
#pragma unroll
  for (int i = 1; i < 19; ++i) r = r + f[i];
  rho = r;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    T m = T(0);
    bool first = true;
#pragma unroll
    for (int i = 0; i < 19; ++i) {
      const int c = q19_c(i, d);
      if (c == 0) continue;
      const T t = c > 0 ? f[i] : -f[i];
      m = first ? t : m + t;
      first = false;
    }
    u[d] = m / r;
  }
}

// ------------------------------------------------------------------ equilibria
// D2Q9: feq_i = rho w_i (1 + 3 cu + 4.5 cu^2 - 1.5 u^2), vivsim/lbm/basic.py:114-135.
template <typename T>
__device__ __forceinline__ T feq_i(L9, int i, T rho, const T* u, T usq) {
  const int cx = q9_cx(i), cy = q9_cy(i);
  const T a = cx == 0 ? T(0) : (cx > 0 ? u[0] : -u[0]);
  const T b = cy == 0 ? T(0) : (cy > 0 ? u[1] : -u[1]);
  const T uc = a + b;
  return (rho * q9_w<T>(i)) * (((T(1) + T(3) * uc) + T(4.5) * (uc * uc)) - T(1.5) * usq);
}
template <typename T>
__device__ __forceinline__ T usq_of(L9, const T* u) { return u[0] * u[0] + u[1] * u[1]; }

// D3Q19: feq = rho w (1 + cu/cs2 + (cu)^2/(2 cs2^2) - u^2/(2 cs2)), vivsim/lbm3d/basic.py:109-130.
// cs2 = 1/3 enters as a (weakly typed) constant of the working precision, exactly as
// the reference's division by the Python float does.
template <typename T>
__device__ __forceinline__ T feq_i(L19, int i, T rho, const T* u, T usq) {
  T uc = T(0);
  bool first = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int c = q19_c(i, d);
    if (c == 0) continue;
    const T t = c > 0 ? u[d] : -u[d];
    uc = first ? t : uc + t;
    first = false;
  }
  const T cs2 = (T)(1.0 / 3.0);
  const T cs4 = (T)((1.0 / 3.0) * (1.0 / 3.0));
  return (rho * q19_w<T>(i)) * (((T(1) + uc / cs2) + (T(0.5) * (uc * uc)) / cs4) - (T(0.5) * usq) / cs2);
}
template <typename T>
__device__ __forceinline__ T usq_of(L19, const T* u) { return (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]; }

template <class L, typename T>
__device__ __forceinline__ void equilibrium(T rho, const T* u, T* feq) {
  const T usq = usq_of(L{}, u);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) feq[i] = feq_i(L{}, i, rho, u, usq);
}

// ------------------------------------------------------------------ collisions
// Scalars derived from omega are formed on the host in double precision and rounded to
// the working precision, as JAX does with the reference's Python-float omega.
template <typename T>
struct CollideParams {
  T omega;          // omega
  T one_m_omega;    // 1 - omega
  T inv_omega;      // 1 / omega
  T one_m_inv;      // 1 - 1 / omega
  const T* mrt;     // Q x Q row-major operator (device), collision_mrt only
};

// BGK: (1 - omega) f + omega feq, vivsim/lbm/basic.py:138-156.
template <class L, typename T>
__device__ __forceinline__ void collide_bgk(T* f, const T* feq, const CollideParams<T>& p) {
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = p.one_m_omega * f[i] + p.omega * feq[i];
}

// D2Q9 KBC, vivsim/lbm/collision/kbc.py:10-60.
template <typename T>
__device__ __forceinline__ void collide_kbc(L9, T* f, const T* feq, const CollideParams<T>& p) {
  T fneq[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) fneq[i] = f[i] - feq[i];
  const T nsd = ((fneq[1] - fneq[2]) + fneq[3]) - fneq[4];
  const T ssd = ((fneq[5] - fneq[6]) + fneq[7]) - fneq[8];
  const T a = nsd / T(4), b = -nsd / T(4), c = ssd / T(4), d = -ssd / T(4);
  T s[9] = {T(0), a, b, a, b, c, d, c, d};
  T h[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) h[i] = fneq[i] - s[i];
  T ish = T(0), ihh = T(0);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const T den = feq[i] + T(1e-20);
    ish = ish + (h[i] * s[i]) / den;
    ihh = ihh + (h[i] * h[i]) / den;
  }
  const T hg = p.inv_omega - (p.one_m_inv * ish) / (ihh + T(1e-20));
#pragma unroll
  for (int i = 0; i < 9; ++i) f[i] = f[i] - p.omega * (s[i] + hg * h[i]);
}

// D2Q9 regularised BGK via closed-form second-order moments, vivsim/lbm/collision/reg.py:4-49.
template <typename T>
__device__ __forceinline__ void collide_reg(L9, T* f, const T* feq, const CollideParams<T>& p) {
  T fneq[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) fneq[i] = f[i] - feq[i];
  const T diag_sum = ((fneq[5] + fneq[6]) + fneq[7]) + fneq[8];
  const T pxx = (fneq[1] + fneq[3]) + diag_sum;
  const T pyy = (fneq[2] + fneq[4]) + diag_sum;
  const T pxy = ((fneq[5] - fneq[6]) + fneq[7]) - fneq[8];
  const T tr = (pxx + pyy) / T(12);
  const T ax = (T(2) * pxx - pyy) / T(6);
  const T ay = (T(2) * pyy - pxx) / T(6);
  const T dp = tr + pxy / T(4);
  const T dn = tr - pxy / T(4);
  const T reg[9] = {T(-8) * tr, ax, ay, ax, ay, dp, dn, dp, dn};
#pragma unroll
  for (int i = 0; i < 9; ++i) f[i] = feq[i] + p.one_m_omega * reg[i];
}

// D3Q19 second-order (Hermite) projection of fneq, vivsim/lbm3d/collision/reg.py:10-41.
// The reference applies a 19x19 table; it equals w_q/(2 cs^4) (c_qa c_qb - cs^2 d_ab) Pi_ab
// with Pi = sum_r fneq_r c_ra c_rb, evaluated here through the six moments Pi_ab.
template <typename T>
__device__ __forceinline__ void projection19(const T* n, T* s) {
  const T dxy = (n[7] + n[10]) - (n[8] + n[9]);
  const T dxz = (n[11] + n[14]) - (n[12] + n[13]);
  const T dyz = (n[15] + n[18]) - (n[16] + n[17]);
  const T exy = ((n[7] + n[8]) + n[9]) + n[10];
  const T exz = ((n[11] + n[12]) + n[13]) + n[14];
  const T eyz = ((n[15] + n[16]) + n[17]) + n[18];
  const T pxx = (n[1] + n[2]) + (exy + exz);
  const T pyy = (n[3] + n[4]) + (exy + eyz);
  const T pzz = (n[5] + n[6]) + (exz + eyz);
  const T tr = (pxx + pyy) + pzz;
  // q = 0: w0/(2cs^4) * (-cs^2) tr = -tr/2
  s[0] = T(-0.5) * tr;
  // axis directions: w/(2cs^4) = 1/4; H = c c - cs^2 I  ->  (pxx - tr/3)/4 etc.
  const T third = (T)(1.0 / 3.0);
  const T ax = T(0.25) * (pxx - third * tr);
  const T ay = T(0.25) * (pyy - third * tr);
  const T az = T(0.25) * (pzz - third * tr);
  s[1] = ax; s[2] = ax; s[3] = ay; s[4] = ay; s[5] = az; s[6] = az;
  // diagonal directions: w/(2cs^4) = 1/8; (c c - cs^2 I):Pi = Pi_aa + Pi_bb + 2 s Pi_ab - tr/3
  const T eight = T(0.125);
  const T bxy = (pxx + pyy) - third * tr;
  const T bxz = (pxx + pzz) - third * tr;
  const T byz = (pyy + pzz) - third * tr;
  s[7] = eight * (bxy + T(2) * dxy);  s[10] = s[7];
  s[8] = eight * (bxy - T(2) * dxy);  s[9] = s[8];
  s[11] = eight * (bxz + T(2) * dxz); s[14] = s[11];
  s[12] = eight * (bxz - T(2) * dxz); s[13] = s[12];
  s[15] = eight * (byz + T(2) * dyz); s[18] = s[15];
  s[16] = eight * (byz - T(2) * dyz); s[17] = s[16];
}

// Entry (q, r) of the reference's 19x19 projection table, rounded to float32 as the
// reference declares it (vivsim/lbm3d/collision/reg.py:10-32): w_q/(2 cs^4) H_q : c_r c_r.
__host__ __device__ constexpr double p19_entry(int q, int r) {
  double s = 0.0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      s += ((double)(q19_c(q, a) * q19_c(q, b)) - (a == b ? 1.0 / 3.0 : 0.0)) * (double)(q19_c(r, a) * q19_c(r, b));
  const double wq = q == 0 ? 1.0 / 3.0 : (q <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
  return (double)(float)(wq / (2.0 * (1.0 / 3.0) * (1.0 / 3.0)) * s);
}

// In float64 the reference multiplies by the float32-rounded table, so the double kernels
// apply that table literally (sum over r in order); float kernels use the moment form.
template <typename T>
__device__ __forceinline__ void projection19_any(const T* n, T* s) {
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      T acc = T(0);
#pragma unroll
      for (int r = 1; r < 19; ++r) acc = r == 1 ? (T)p19_entry(q, r) * n[r] : acc + (T)p19_entry(q, r) * n[r];
      s[q] = acc;
    }
  } else {
    projection19(n, s);
  }
}

// D3Q19 regularised: feq + (1 - omega) P fneq, vivsim/lbm3d/collision/reg.py:44-62.
template <typename T>
__device__ __forceinline__ void collide_reg(L19, T* f, const T* feq, const CollideParams<T>& p) {
  T n[19], s[19];
#pragma unroll
  for (int i = 0; i < 19; ++i) n[i] = f[i] - feq[i];
  projection19_any(n, s);
#pragma unroll
  for (int i = 0; i < 19; ++i) f[i] = feq[i] + p.one_m_omega * s[i];
}

// D3Q19 KBC, vivsim/lbm3d/collision/kbc.py:8-42.
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
    const T inv = T(1) / (feq[i] + T(1e-20));
    ish = ish + (h * s[i]) * inv;
    ihh = ihh + (h * h) * inv;
  }
  const T hg = p.inv_omega - (p.one_m_inv * ish) / (ihh + T(1e-20));
#pragma unroll
  for (int i = 0; i < 19; ++i) f[i] = f[i] - p.omega * (s[i] + hg * (n[i] - s[i]));
}

// MRT: f + op (feq - f), vivsim/lbm/collision/mrt.py:66-88 and lbm3d/collision/mrt.py:88-98.
template <class L, typename T>
__device__ __forceinline__ void collide_mrt(T* f, const T* feq, const T* __restrict__ op) {
  T d[L::Q];
#pragma unroll
  for (int j = 0; j < L::Q; ++j) d[j] = feq[j] - f[j];
  T out[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    T acc = op[i * L::Q] * d[0];
#pragma unroll
    for (int j = 1; j < L::Q; ++j) acc = acc + op[i * L::Q + j] * d[j];
    out[i] = f[i] + acc;
  }
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = out[i];
}

template <class L, typename T>
__device__ __forceinline__ void collide(int kind, T* f, const T* feq, const CollideParams<T>& p) {
  switch (kind) {
    case VS_COLLIDE_BGK: collide_bgk<L>(f, feq, p); break;
    case VS_COLLIDE_KBC: collide_kbc(L{}, f, feq, p); break;
    case VS_COLLIDE_REG: collide_reg(L{}, f, feq, p); break;
    case VS_COLLIDE_MRT: collide_mrt<L>(f, feq, p.mrt); break;
    default: break;
  }
}

// ------------------------------------------------------------------ Guo force term
// D2Q9: w_i [gx (3 (cx - ux) + 9 cu cx) + gy (3 (cy - uy) + 9 cu cy)], vivsim/lbm/forcing/guo.py:6-35.
template <typename T>
__device__ __forceinline__ T guo_i(L9, int i, const T* g, const T* u) {
  const T cx = (T)q9_cx(i), cy = (T)q9_cy(i);
  const T uc = u[0] * cx + u[1] * cy;
  return q9_w<T>(i) * (g[0] * (T(3) * (cx - u[0]) + T(9) * (uc * cx)) +
                       g[1] * (T(3) * (cy - u[1]) + T(9) * (uc * cy)));
}
// D3Q19: w_i [3 (c.g - g.u) + 9 (c.g)(c.u)], vivsim/lbm3d/forcing/guo.py:13-38.
template <typename T>
__device__ __forceinline__ T guo_i(L19, int i, const T* g, const T* u) {
  T cu = T(0), cg = T(0);
  bool first = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int c = q19_c(i, d);
    if (c == 0) continue;
    const T tu = c > 0 ? u[d] : -u[d];
    const T tg = c > 0 ? g[d] : -g[d];
    cu = first ? tu : cu + tu;
    cg = first ? tg : cg + tg;
    first = false;
  }
  const T gu = (g[0] * u[0] + g[1] * u[1]) + g[2] * u[2];
  return q19_w<T>(i) * (T(3) * (cg - gu) + (T(9) * cg) * cu);
}

}  // namespace vs
