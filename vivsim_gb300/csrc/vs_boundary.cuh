// Face boundary conditions for one wall node (D2Q9 and D3Q19), shared by the per-op
// boundary entry point and the ordered face epilogue of the fused step.
//
// Restates vivsim/lbm/boundary/{_helpers,nee,nebb,eq,bb}.py and
// vivsim/lbm3d/boundary/{_helpers,nee,nebb,eq,bb}.py.  Scalar wall data that the
// reference combines as Python floats (double precision) are combined on the host and
// rounded once; array wall data are combined on the device in the working precision.
#pragma once

#include "vs_common.cuh"

namespace vs {

// loc -> normal axis / inward normal sign (lbm/lattice.py:62-109, lbm3d/lattice.py:68-125)
__host__ __device__ constexpr int loc_axis(int loc) { return loc < 2 ? 0 : (loc < 4 ? 1 : 2); }
__host__ __device__ constexpr int loc_sign(int loc) { return (loc % 2 == 0) ? 1 : -1; }

// D2Q9 face tables in the reference's listed order (order matters for pairing and rounding).
__host__ __device__ constexpr int f9_in(int loc, int k) {
  return loc == VS_LEFT ? (k == 0 ? 1 : k == 1 ? 5 : 8)
       : loc == VS_RIGHT ? (k == 0 ? 3 : k == 1 ? 7 : 6)
       : loc == VS_TOP ? (k == 0 ? 4 : k == 1 ? 7 : 8)
                       : (k == 0 ? 2 : k == 1 ? 5 : 6);
}
__host__ __device__ constexpr int f9_out(int loc, int k) {
  return loc == VS_LEFT ? (k == 0 ? 3 : k == 1 ? 7 : 6)
       : loc == VS_RIGHT ? (k == 0 ? 1 : k == 1 ? 5 : 8)
       : loc == VS_TOP ? (k == 0 ? 2 : k == 1 ? 5 : 6)
                       : (k == 0 ? 4 : k == 1 ? 7 : 8);
}
__host__ __device__ constexpr int f9_tan(int loc, int k) {
  return loc_axis(loc) == 0 ? (k == 0 ? 2 : 4) : (k == 0 ? 1 : 3);
}
__host__ __device__ constexpr int f9_ps(int loc, int k) {
  return loc_axis(loc) == 0 ? (k == 0 ? 2 : k == 1 ? 5 : 6) : (k == 0 ? 1 : k == 1 ? 5 : 8);
}
__host__ __device__ constexpr int f9_ns(int loc, int k) {
  return loc_axis(loc) == 0 ? (k == 0 ? 4 : k == 1 ? 7 : 8) : (k == 0 ? 3 : k == 1 ? 7 : 6);
}

template <typename T>
struct WallArgs {
  int kind, mode, loc;
  int n[3];            // grid dims (nz = 1 in 2-D)
  T rho;               // scalar wall density (rounded)
  T u[3];              // scalar wall velocity (rounded; force correction already applied)
  const T* rho_arr;    // optional per-node wall data (face shape)
  const T* u_arr[3];
  const T* f_pre;      // pre-streaming populations (BB / specular)
  int64_t pre_stride;  // population stride of f_pre (n_nodes, or the face size for a face buffer)
  int pre_face;        // 1: f_pre is a face buffer indexed by face node j
  // host-combined scalar terms (double math, rounded once)
  int un_scalar;       // wall velocity given as scalars (GIVEN / VELOCITY / FORCE_CORRECTED)
  int all_scalar;      // ... and rho_wall scalar too (GIVEN / FORCE_CORRECTED)
  T one_m_un;          // 1 - un
  T c23un, c16un, c05ut;  // 2/3 un, 1/6 un, 0.5 ut
  T t23, t16, t05;        // the same times rho_wall
  T b16p, b16m;           // 1/6 (un + ut), 1/6 (un - ut)
};

// Fill the host-side scalar fields of WallArgs from double wall data.
template <typename T>
inline void wall_args_scalars(WallArgs<T>& A, double rho, const double* u3, int dim) {
  const int a = loc_axis(A.loc), sg = loc_sign(A.loc);
  double un = sg * u3[a];
  double ut = dim == 2 ? sg * u3[1 - a] : 0.0;
  A.rho = (T)rho;
  for (int d = 0; d < 3; ++d) A.u[d] = (T)u3[d];
  A.one_m_un = (T)(1.0 - un);
  A.c23un = (T)(2.0 / 3.0 * un);
  A.c16un = (T)(1.0 / 6.0 * un);
  A.c05ut = (T)(0.5 * ut);
  A.t23 = (T)(2.0 / 3.0 * un * rho);
  A.t16 = (T)(1.0 / 6.0 * un * rho);
  A.t05 = (T)(0.5 * ut * rho);
  A.b16p = (T)(1.0 / 6.0 * (un + ut));
  A.b16m = (T)(1.0 / 6.0 * (un - ut));
}

__host__ __device__ inline int64_t face_size(int loc, const int* n) {
  const int a = loc_axis(loc);
  int64_t s = 1;
  for (int d = 0; d < 3; ++d)
    if (d != a) s *= n[d];
  return s;
}

// Node index of face node j at normal offset `depth` (0 = wall, 1 = neighbour).
__host__ __device__ inline int64_t face_node(int loc, const int* n, int64_t j, int depth) {
  const int a = loc_axis(loc), sg = loc_sign(loc);
  int c[3];
  const int b0 = a == 0 ? 1 : 0, b1 = a == 2 ? 1 : 2;
  c[a] = sg > 0 ? depth : n[a] - 1 - depth;
  c[b0] = (int)(j / n[b1]);
  c[b1] = (int)(j % n[b1]);
  return ((int64_t)c[0] * n[1] + c[1]) * n[2] + c[2];
}

// f0 + f_t0 + f_t1 + 2 (f_o0 + f_o1 + f_o2) (lbm/boundary/_helpers.py:124-135)
template <typename T>
__device__ __forceinline__ T rho_numerator(L9, int loc, const T* w) {
  return ((w[0] + w[f9_tan(loc, 0)]) + w[f9_tan(loc, 1)]) +
         T(2) * ((w[f9_out(loc, 0)] + w[f9_out(loc, 1)]) + w[f9_out(loc, 2)]);
}
// sum f_zero + 2 sum f_out (lbm3d/boundary/_helpers.py:37-44)
template <typename T>
__device__ __forceinline__ T rho_numerator(L19, int loc, const T* w) {
  const int a = loc_axis(loc), sg = loc_sign(loc);
  T z = T(0), o = T(0);
  bool fz = true, fo = true;
#pragma unroll
  for (int i = 0; i < 19; ++i) {
    const int c = q19_c(i, a);
    if (c == 0) { z = fz ? w[i] : z + w[i]; fz = false; }
    else if (c == -sg) { o = fo ? w[i] : o + w[i]; fo = false; }
  }
  return z + T(2) * o;
}

// Tangential wall velocity copied from the neighbour for a pressure boundary.
// D2Q9: (sum pos_side - sum neg_side) / rho_nb (lbm/boundary/_helpers.py:110-116)
template <typename T>
__device__ __forceinline__ void pressure_tangential(L9, int loc, const T* nb, T* u) {
  T r = nb[0];
#pragma unroll
  for (int i = 1; i < 9; ++i) r = r + nb[i];
  const T t = (((((nb[f9_ps(loc, 0)] - nb[f9_ns(loc, 0)]) + nb[f9_ps(loc, 1)]) - nb[f9_ns(loc, 1)]) +
                nb[f9_ps(loc, 2)]) - nb[f9_ns(loc, 2)]) / r;
  u[1 - loc_axis(loc)] = t;
}
// D3Q19: u of get_macroscopic(neighbour) (lbm3d/boundary/_helpers.py:76-80)
template <typename T>
__device__ __forceinline__ void pressure_tangential(L19, int loc, const T* nb, T* u) {
  T r, un[3];
  macro(L19{}, nb, r, un);
  const int a = loc_axis(loc);
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (d != a) u[d] = un[d];
}

// Compute the new wall populations of face node j.  `w` holds the wall node, `nb` the
// neighbour node (loaded only when the scheme needs it), `pre` the pre-stream wall node.
// Writes every population into out[] (unchanged ones copied from w).
template <class L, typename T>
__device__ __forceinline__ void bc_node(const WallArgs<T>& A, int64_t j, const T* w, const T* nb, const T* pre,
                                        T* out) {
  constexpr int Q = L::Q;
  const int a = loc_axis(A.loc), sg = loc_sign(A.loc);
  T rho = A.rho_arr ? A.rho_arr[j] : A.rho;
  T u[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) u[d] = A.u_arr[d] ? A.u_arr[d][j] : A.u[d];
  bool un_scalar = A.un_scalar && !(A.u_arr[0] || A.u_arr[1] || A.u_arr[2]);
  bool all_scalar = un_scalar && A.all_scalar && !A.rho_arr;
  if (A.mode == VS_WALL_VELOCITY) {
    const T omu = un_scalar ? A.one_m_un : T(1) - (sg > 0 ? u[a] : -u[a]);
    rho = rho_numerator(L{}, A.loc, w) / omu;
    all_scalar = false;
  } else if (A.mode == VS_WALL_PRESSURE) {
    const T nvs = T(1) - rho_numerator(L{}, A.loc, w) / rho;
    u[a] = sg > 0 ? nvs : -nvs;
    pressure_tangential(L{}, A.loc, nb, u);
    un_scalar = false;
    all_scalar = false;
  }
#pragma unroll
  for (int i = 0; i < Q; ++i) out[i] = w[i];
  if (A.kind == VS_BC_EQ || A.kind == VS_BC_NEE) {
    const T usq = usq_of(L{}, u);
    if (A.kind == VS_BC_EQ) {
#pragma unroll
      for (int i = 0; i < Q; ++i) out[i] = feq_i(L{}, i, rho, u, usq);
    } else {
      T rn, un[3];
      macro(L{}, nb, rn, un);
      const T usqn = usq_of(L{}, un);
#pragma unroll
      for (int i = 0; i < Q; ++i) out[i] = feq_i(L{}, i, rho, u, usq) + (nb[i] - feq_i(L{}, i, rn, un, usqn));
    }
    return;
  }
  if constexpr (L::Q == 9) {
    const T un = sg > 0 ? u[a] : -u[a];
    const T ut = sg > 0 ? u[1 - a] : -u[1 - a];
    if (A.kind == VS_BC_NEBB) {  // lbm/boundary/nebb.py:46-58
      const T shear = (T(0.5) * (w[f9_tan(A.loc, 0)] - w[f9_tan(A.loc, 1)])) * (T)sg;
      T nt, tt, n23;
      if (all_scalar) {
        nt = A.t16; tt = A.t05; n23 = A.t23;
      } else if (un_scalar) {
        nt = A.c16un * rho; tt = A.c05ut * rho; n23 = A.c23un * rho;
      } else {
        nt = ((T)(1.0 / 6.0) * un) * rho; tt = (T(0.5) * ut) * rho; n23 = ((T)(2.0 / 3.0) * un) * rho;
      }
      out[f9_in(A.loc, 0)] = w[f9_out(A.loc, 0)] + n23;
      out[f9_in(A.loc, 1)] = ((w[f9_out(A.loc, 1)] - shear) + nt) + tt;
      out[f9_in(A.loc, 2)] = ((w[f9_out(A.loc, 2)] + shear) + nt) - tt;
    } else {  // bounce-back / specular, lbm/boundary/bb.py:15-95
      T v0, v1, v2;
      if (un_scalar) {
        v0 = pre[f9_out(A.loc, 0)] + A.c23un;
        v1 = pre[f9_out(A.loc, 1)] + A.b16p;
        v2 = pre[f9_out(A.loc, 2)] + A.b16m;
      } else {
        v0 = pre[f9_out(A.loc, 0)] + (T)(2.0 / 3.0) * un;
        v1 = pre[f9_out(A.loc, 1)] + (T)(1.0 / 6.0) * (un + ut);
        v2 = pre[f9_out(A.loc, 2)] + (T)(1.0 / 6.0) * (un - ut);
      }
      out[f9_in(A.loc, 0)] = v0;
      if (A.kind == VS_BC_BB) {
        out[f9_in(A.loc, 1)] = v1; out[f9_in(A.loc, 2)] = v2;
      } else {
        out[f9_in(A.loc, 2)] = v1; out[f9_in(A.loc, 1)] = v2;
      }
    }
  } else {
    if (A.kind == VS_BC_NEBB) {  // lbm3d/boundary/nebb.py:16-32 (feq-difference form)
      const T usq = usq_of(L{}, u);
#pragma unroll
      for (int i = 0; i < 19; ++i) {
        if (q19_c(i, a) != sg) continue;
        const int o = q19_opp(i);
        out[i] = (w[o] + feq_i(L{}, i, rho, u, usq)) - feq_i(L{}, o, rho, u, usq);
      }
    } else {  // lbm3d/boundary/bb.py:20-53; in/out paired in listed (increasing) order
      T rp = pre[0];
#pragma unroll
      for (int i = 1; i < 19; ++i) rp = rp + pre[i];
      int outs[5], k = 0;
#pragma unroll
      for (int i = 0; i < 19; ++i)
        if (q19_c(i, a) == -sg) outs[k++] = i;
      k = 0;
#pragma unroll
      for (int i = 0; i < 19; ++i) {
        if (q19_c(i, a) != sg) continue;
        T cu = T(0);
        bool first = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int c = q19_c(i, d);
          if (c == 0) continue;
          const T t = c > 0 ? u[d] : -u[d];
          cu = first ? t : cu + t;
          first = false;
        }
        const T corr = (((T(2) * q19_w<T>(i)) * rp) * cu) / (T)(1.0 / 3.0);
        out[i] = pre[outs[k++]] + corr;
      }
    }
  }
}

// boundary_characteristic at one face node (lbm/boundary/cbc.py:14-53, lbm3d/boundary/cbc.py:
// 16-51) from the density r and normal velocity u of the wall (1) and the next two planes
// (2, 3); sg is the inward normal sign.  Every product and sum is rounded on its own, in
// the reference's order, so per-operator and fused callers agree to the bit.
template <typename T>
__device__ __forceinline__ void cbc_values(int sg, T cs, T r1, T r2, T r3, T u1, T u2, T u3, T& rho_next,
                                           T& un_next) {
  const T dc = (T)(-0.5 * sg);
  const T drho = mul_rn(dc, add_rn(sub_rn(mul_rn(T(3), r1), mul_rn(T(4), r2)), r3));
  const T dun = mul_rn(dc, add_rn(sub_rn(mul_rn(T(3), u1), mul_rn(T(4), u2)), u3));
  const T sgcs = mul_rn((T)sg, cs);
  const T cout = sub_rn(dun, mul_rn(sgcs / r1, drho));
  const T lout = mul_rn(sub_rn(u1, sgcs), cout);
  rho_next = sub_rn(r1, mul_rn(mul_rn(T(0.5), r1) / cs, lout));
  un_next = sub_rn(u1, mul_rn(T(0.5), lout));
}

// the reference's sound speed of each lattice: 1 / jnp.sqrt(3) (2-D), jnp.sqrt(1 / 3) (3-D)
template <typename T>
__host__ __device__ inline T cbc_cs(int dim) {
  return dim == 2 ? (T)1 / sqrt((T)3) : sqrt((T)(1.0 / 3.0));
}

template <class L>
__host__ __device__ constexpr bool bc_needs_neighbor(int kind, int mode) {
  return kind == VS_BC_NEE || mode == VS_WALL_PRESSURE;
}

}  // namespace vs
