// Vector-Jacobian products of the per-operator functions: the reverse-mode building blocks
// that let a caller differentiate an update step it composes itself from the reference's
// functions (the reference differentiates its jitted loop with jax.grad).
//
// Each entry point takes the forward inputs it needs and the cotangent of the output, and
// writes the cotangents of the inputs.  Node-local Jacobians come from forward-mode dual
// numbers evaluated on the same formulas the forward kernels use (vs_common.cuh,
// vs_boundary.cuh), so every collision model and boundary scheme has its exact transpose.
// Cotangents of scalar parameters (omega, wall values, spring constants) are reduced in a
// fixed order (vs_sum_ordered): the gradients are deterministic, run to run.
#include <cmath>

#include "vs_boundary.cuh"
#include "vs_dispatch.cuh"
#include "vs_dual.cuh"
#include "vs_ib.cuh"

namespace vs {
namespace {

constexpr int kB = 256;

__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// ------------------------------------------------------------------ streaming
// forward (lbm/basic.py:60-85): out_i(x) = f_i(x - c_i); transpose: g_f_i(x) = g_out_i(x + c_i)
template <class L, typename T>
__global__ void k_stream_vjp(const T* __restrict__ go, T* __restrict__ gi, int nx, int ny, int nz) {
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(p / ((int64_t)ny * nz));
    const int r = (int)(p - (int64_t)x * ny * nz);
    const int y = r / nz, z = r - y * nz;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const int xs = wrapi(x + L::c(i, 0), nx), ys = wrapi(y + L::c(i, 1), ny), zs = wrapi(z + L::c(i, 2), nz);
      gi[(int64_t)i * n + p] = go[(int64_t)i * n + ((int64_t)xs * ny + ys) * nz + zs];
    }
  }
}

// ------------------------------------------------------------------ moments
// rho = sum f, u = c^T f / rho: d rho / d f_i = 1, d u_d / d f_i = (c_id - u_d) / rho
template <class L, typename T>
__global__ void k_macro_vjp(const T* __restrict__ f, const T* __restrict__ grho, const T* __restrict__ gu,
                            T* __restrict__ gf, int64_t n) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  T fl[L::Q], rho, u[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int i = 0; i < L::Q; ++i) fl[i] = f[i * n + p];
  macro(L{}, fl, rho, u);
  const T gr = grho ? grho[p] : T(0);
  T g[3] = {T(0), T(0), T(0)};
  if (gu)
#pragma unroll
    for (int d = 0; d < L::D; ++d) g[d] = gu[d * n + p] / rho;
  T gdu = T(0);
#pragma unroll
  for (int d = 0; d < L::D; ++d) gdu += g[d] * u[d];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) {
    T acc = gr - gdu;
#pragma unroll
    for (int d = 0; d < L::D; ++d)
      if (L::c(i, d)) acc += L::c(i, d) > 0 ? g[d] : -g[d];
    gf[i * n + p] = acc;
  }
}

// ------------------------------------------------------------------ equilibrium
// D + 1 dual passes of feq_i (lbm/basic.py:114-135, lbm3d/basic.py:109-130)
template <class L, typename T>
__global__ void k_eq_vjp(const T* __restrict__ rho, const T* __restrict__ u, const T* __restrict__ gfeq,
                         T* __restrict__ grho, T* __restrict__ gu, int64_t n) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  T g[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) g[i] = gfeq[i * n + p];
  for (int k = 0; k <= L::D; ++k) {
    const Dual<T> r(rho[p], (T)(k == 0));
    Dual<T> ud[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) ud[d] = Dual<T>(d < L::D ? u[d * n + p] : T(0), (T)(k == d + 1));
    const Dual<T> usq = usq_of(L{}, ud);
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) acc += g[i] * feq_i(L{}, i, r, ud, usq).d;
    if (k == 0) grho[p] = acc;
    else gu[(k - 1) * n + p] = acc;
  }
}

// ------------------------------------------------------------------ collisions
template <class L, typename S>
__device__ __forceinline__ void collide_generic(int kind, S* f, const S* feq, S omega) {
  CollideParams<S> P;
  P.omega = omega;
  P.one_m_omega = S(1) - omega;
  P.inv_omega = S(1) / omega;
  P.one_m_inv = S(1) - S(1) / omega;
  P.mrt = nullptr;
  if (kind == VS_COLLIDE_KBC) collide_kbc(L{}, f, feq, P);
  else if (kind == VS_COLLIDE_REG) collide_reg(L{}, f, feq, P);
  else collide_bgk<L>(f, feq, P);
}

// 2Q + 1 dual passes (each population of f, of feq, and omega): g_f, g_feq, and the node's
// share of g_omega (lbm/basic.py:138-156, lbm/collision/{kbc,reg}.py, lbm3d/collision/*.py)
template <class L, typename T>
__global__ void k_collide_vjp(int kind, const T* __restrict__ f, const T* __restrict__ feq, T omega,
                              const T* __restrict__ gout, T* __restrict__ gf, T* __restrict__ gfeq,
                              T* __restrict__ gom, int64_t n) {
  constexpr int Q = L::Q;
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  T fl[Q], el[Q], g[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    fl[i] = f[i * n + p];
    el[i] = feq[i * n + p];
    g[i] = gout[i * n + p];
  }
  const int passes = gom ? 2 * Q + 1 : 2 * Q;
  for (int k = 0; k < passes; ++k) {
    Dual<T> fd[Q], ed[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      fd[i] = Dual<T>(fl[i], (T)(k == i));
      ed[i] = Dual<T>(el[i], (T)(k == Q + i));
    }
    collide_generic<L>(kind, fd, ed, Dual<T>(omega, (T)(k == 2 * Q)));
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) acc += g[i] * fd[i].d;
    if (k < Q) gf[k * n + p] = acc;
    else if (k < 2 * Q) gfeq[(k - Q) * n + p] = acc;
    else gom[p] = acc;
  }
}

// MRT (lbm/collision/mrt.py:66-88): out = f + A (feq - f); g_f = g - A^T g, g_feq = A^T g
template <class L, typename T>
struct OpArg {
  T a[L::Q * L::Q];
};
template <class L, typename T>
__global__ void k_mrt_vjp(const __grid_constant__ OpArg<L, T> A, const T* __restrict__ gout, T* __restrict__ gf,
                          T* __restrict__ gfeq, int64_t n) {
  constexpr int Q = L::Q;
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  T g[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) g[i] = gout[i * n + p];
#pragma unroll
  for (int j = 0; j < Q; ++j) {
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) acc += A.a[i * Q + j] * g[i];
    gfeq[j * n + p] = acc;
    gf[j * n + p] = g[j] - acc;
  }
}

// out[i * Q + j] = sum_nodes a_i(node) * (b1_j(node) - b0_j(node)) (b0 may be null): the
// cotangent of a Q x Q operator; one block per (i, j), summed in a fixed order
template <typename T>
__global__ void k_outer_sum(int Q, const T* __restrict__ a, const T* __restrict__ b1, const T* __restrict__ b0,
                            int64_t n, double* __restrict__ out) {
  const int i = blockIdx.x / Q, j = blockIdx.x - (blockIdx.x / Q) * Q;
  double acc = 0.0;
  for (int64_t p = threadIdx.x; p < n; p += blockDim.x) {
    const double b = (double)b1[j * n + p] - (b0 ? (double)b0[j * n + p] : 0.0);
    acc += (double)a[i * n + p] * b;
  }
  __shared__ double sh[kB];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// ------------------------------------------------------------------ forcing
// out = f + s guo(g, u) (lbm/forcing/edm.py:4-31, guo.py:6-59; s = 1 or 1 - omega / 2):
// g_f = g_out; 2 D dual passes of guo_i for g_g and g_u; g_s per node = g_out . guo
template <class L, typename T>
__global__ void k_forcing_vjp(const T* __restrict__ g, const T* __restrict__ u, T s, const T* __restrict__ gout,
                              T* __restrict__ gf, T* __restrict__ gg, T* __restrict__ gu, T* __restrict__ gs,
                              int64_t n) {
  constexpr int Q = L::Q, D = L::D;
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  T go[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    go[i] = gout[i * n + p];
    if (gf) gf[i * n + p] = go[i];
  }
  T gl[3] = {T(0), T(0), T(0)}, ul[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int d = 0; d < D; ++d) {
    gl[d] = g[d * n + p];
    ul[d] = u[d * n + p];
  }
  for (int k = 0; k < 2 * D; ++k) {
    Dual<T> gd[3], ud[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gd[d] = Dual<T>(gl[d], (T)(k == d));
      ud[d] = Dual<T>(ul[d], (T)(k == D + d));
    }
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) acc += go[i] * guo_i(L{}, i, gd, ud).d;
    if (k < D) gg[k * n + p] = s * acc;
    else gu[(k - D) * n + p] = s * acc;
  }
  if (gs) {
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) acc += go[i] * guo_i(L{}, i, gl, ul);
    gs[p] = acc;
  }
}

// Guo-MRT (lbm/forcing/guo.py:62-107): out = f + F guo(g, u); the cotangent of guo is F^T g_out
template <class L, typename T>
__global__ void k_guo_mrt_vjp(const __grid_constant__ OpArg<L, T> F, const T* __restrict__ g, const T* __restrict__ u,
                              const T* __restrict__ gout, T* __restrict__ gf, T* __restrict__ gg, T* __restrict__ gu,
                              T* __restrict__ guo_out, int64_t n) {
  constexpr int Q = L::Q, D = L::D;
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  T go[Q], gt[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    go[i] = gout[i * n + p];
    gf[i * n + p] = go[i];
  }
#pragma unroll
  for (int j = 0; j < Q; ++j) {
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) acc += F.a[i * Q + j] * go[i];
    gt[j] = acc;
  }
  T gl[3] = {T(0), T(0), T(0)}, ul[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int d = 0; d < D; ++d) {
    gl[d] = g[d * n + p];
    ul[d] = u[d * n + p];
  }
  for (int k = 0; k < 2 * D; ++k) {
    Dual<T> gd[3], ud[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      gd[d] = Dual<T>(gl[d], (T)(k == d));
      ud[d] = Dual<T>(ul[d], (T)(k == D + d));
    }
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) acc += gt[i] * guo_i(L{}, i, gd, ud).d;
    if (k < D) gg[k * n + p] = acc;
    else gu[(k - D) * n + p] = acc;
  }
  if (guo_out)
#pragma unroll
    for (int i = 0; i < Q; ++i) guo_out[i * n + p] = guo_i(L{}, i, gl, ul);
}

// ------------------------------------------------------------------ face boundaries
// One thread per face node: the boundary of vs_boundary.cuh on dual numbers, one pass per
// input (wall populations, neighbour populations where the scheme reads them, pre-stream
// populations for bounce-back, and the four wall values).  g_in starts as a copy of g_out;
// the wall row is replaced and the neighbour row accumulated (each face node owns its
// neighbour, so no two threads touch the same word).  gwall[4 * j + k]: the node's share
// of the cotangent of rho_wall, ux_wall, uy_wall, uz_wall.
template <typename T>
struct WallVjp {
  int kind, mode, loc, n[3];
  T rho, u[3];
};

template <class L, typename T>
__global__ void k_boundary_vjp(const __grid_constant__ WallVjp<T> W, const T* __restrict__ f,
                               const T* __restrict__ fpre, const T* __restrict__ gout, T* __restrict__ gin,
                               T* __restrict__ gpre, T* __restrict__ gwall, int64_t nf) {
  constexpr int Q = L::Q;
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= nf) return;
  const int64_t n = (int64_t)W.n[0] * W.n[1] * W.n[2];
  const int64_t pw = face_node(W.loc, W.n, j, 0), pn = face_node(W.loc, W.n, j, 1);
  const bool need_nb = bc_needs_neighbor<L>(W.kind, W.mode);
  const bool need_pre = W.kind == VS_BC_BB || W.kind == VS_BC_SPECULAR;
  T w[Q], nb[Q], pre[Q], g[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    w[i] = f[i * n + pw];
    nb[i] = need_nb ? f[i * n + pn] : T(0);
    pre[i] = need_pre ? fpre[i * n + pw] : T(0);
    g[i] = gout[i * n + pw];
  }
  WallArgs<Dual<T>> A{};
  A.kind = W.kind;
  A.mode = W.mode;
  A.loc = W.loc;
  for (int d = 0; d < 3; ++d) A.n[d] = W.n[d];
  A.un_scalar = 0;  // every wall term is formed on the device from rho and u
  A.all_scalar = 0;
  const int n_in = 3 * Q + 4;
  T gw[Q], gnb[Q], gp[Q], gv[4] = {T(0), T(0), T(0), T(0)};
  for (int k = 0; k < n_in; ++k) {
    const int grp = k / Q, idx = k - grp * Q;
    if (k < 3 * Q && ((grp == 1 && !need_nb) || (grp == 2 && !need_pre))) continue;
    Dual<T> wd[Q], nd[Q], pd[Q], out[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      wd[i] = Dual<T>(w[i], (T)(grp == 0 && idx == i));
      nd[i] = Dual<T>(nb[i], (T)(grp == 1 && idx == i));
      pd[i] = Dual<T>(pre[i], (T)(grp == 2 && idx == i));
    }
    const int kv = k - 3 * Q;  // wall value index 0..3 (k >= 3 Q)
    A.rho = Dual<T>(W.rho, (T)(kv == 0));
    for (int d = 0; d < 3; ++d) A.u[d] = Dual<T>(W.u[d], (T)(kv == d + 1));
    bc_node<L, Dual<T>>(A, j, wd, nd, pd, out);
    T acc = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) acc += g[i] * out[i].d;
    if (grp == 0) gw[idx] = acc;
    else if (grp == 1) gnb[idx] = acc;
    else if (grp == 2) gp[idx] = acc;
    else gv[kv] = acc;
  }
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    gin[i * n + pw] = gw[i];
    if (need_nb) gin[i * n + pn] = gout[i * n + pn] + gnb[i];
    if (need_pre && gpre) gpre[i * n + pw] = gp[i];
  }
  if (gwall)
#pragma unroll
    for (int k = 0; k < 4; ++k) gwall[4 * j + k] = gv[k];
}

// ------------------------------------------------------------------ immersed boundary
// out[m, s] = sum_c A[m, c] grid[c, I[m, s]]: the cotangent of the stencil weights, for
// interpolate (A = g_U, grid = u) and spread (A = marker values, grid = g_out)
template <typename T>
__global__ void k_pair_dot(const T* __restrict__ A, const T* __restrict__ grid, const int32_t* __restrict__ I, int m,
                           int s, int c, int64_t n_grid, T* __restrict__ out) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= (int64_t)m * s) return;
  const int mk = (int)(p / s);
  const int idx = I[p];
  T acc = T(0);
  if (idx >= 0 && idx < n_grid)
    for (int k = 0; k < c; ++k) acc += A[(int64_t)mk * c + k] * grid[(int64_t)k * n_grid + idx];
  out[p] = acc;
}

// get_ib_stencil (ib/stencil.py:7-51, ib3d/stencil.py:7-59): W = prod_d phi(node_d - X_d),
// floor() is piecewise constant, so g_X_d = sum_s g_W * (-phi'(r_d)) prod_{e != d} phi(r_e)
template <typename T>
__global__ void k_stencil_vjp(int kernel, int radius, int dim, const T* __restrict__ X, const T* __restrict__ Y,
                              const T* __restrict__ Z, const T* __restrict__ gW, T* __restrict__ gX,
                              T* __restrict__ gY, T* __restrict__ gZ, int m) {
  const int mk = blockIdx.x * blockDim.x + threadIdx.x;
  if (mk >= m) return;
  const int WD = 2 * radius;
  const T xs[3] = {X[mk], Y[mk], dim == 3 ? Z[mk] : T(0)};
  int ref[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) ref[d] = ifloor(xs[d]);
  const int S = dim == 2 ? WD * WD : WD * WD * WD;
  T acc[3] = {T(0), T(0), T(0)};
  for (int sidx = 0; sidx < S; ++sidx) {
    int o[3];
    if (dim == 2) {
      o[0] = sidx / WD;
      o[1] = sidx - o[0] * WD;
      o[2] = 0;
    } else {
      o[0] = sidx / (WD * WD);
      o[1] = (sidx / WD) % WD;
      o[2] = sidx % WD;
    }
    T ph[3], dph[3];
    for (int d = 0; d < dim; ++d) {
      const T r = (T)(ref[d] + o[d] - radius + 1) - xs[d];
      ph[d] = delta(kernel, r);
      dph[d] = ddelta(kernel, r);
    }
    const T gw = gW[(int64_t)mk * S + sidx];
    for (int d = 0; d < dim; ++d) {
      T prod = -dph[d];
      for (int e = 0; e < dim; ++e)
        if (e != d) prod *= ph[e];
      acc[d] += gw * prod;
    }
  }
  gX[mk] = acc[0];
  gY[mk] = acc[1];
  if (dim == 3) gZ[mk] = acc[2];
}

// ------------------------------------------------------------------ Newmark
// dyn.py:5-51 (scalar branch :42-45, matrix branch :36-41).  Outputs g_a, g_v, g_d, g_h per
// DOF and (scalar branch) the cotangents of m, k, c summed over the DOFs, in gmkc[3].
template <typename T>
__global__ void k_newmark_vjp(int ndof, int matrix, const T* a, const T* v, const T* d, const T* h, const T* mm,
                              const T* km, const T* cm, double m, double k, double c, double dt, double gamma,
                              double beta, const T* gan, const T* gvn, const T* gdn, T* ga, T* gv, T* gd, T* gh,
                              T* gmkc, T* gmat) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const T c1 = (T)(gamma * dt), c2 = (T)(beta * dt * dt);
  const T k1 = (T)(dt * (1 - gamma)), k2 = (T)(dt * dt * (0.5 - beta)), tdt = (T)dt;
  T v1[8], v2[8], G[8], an[8];
  for (int i = 0; i < ndof; ++i) {
    v1[i] = v[i] + k1 * a[i];
    v2[i] = (d[i] + tdt * v[i]) + k2 * a[i];
    G[i] = (gan ? gan[i] : T(0)) + c1 * (gvn ? gvn[i] : T(0)) + c2 * (gdn ? gdn[i] : T(0));
  }
  T gv1[8], gv2[8];
  if (!matrix) {
    const T den = (T)(m + gamma * dt * c + beta * dt * dt * k);
    T gm = T(0), gk = T(0), gc = T(0);
    for (int i = 0; i < ndof; ++i) {
      an[i] = ((h[i] - (T)c * v1[i]) - (T)k * v2[i]) / den;
      const T gr = G[i] / den;  // cotangent of the right-hand side
      gh[i] = gr;
      gv1[i] = (gvn ? gvn[i] : T(0)) - (T)c * gr;
      gv2[i] = (gdn ? gdn[i] : T(0)) - (T)k * gr;
      const T gden = -gr * an[i];
      gm += gden;
      gc += c1 * gden - gr * v1[i];
      gk += c2 * gden - gr * v2[i];
    }
    if (gmkc) {
      gmkc[0] = gm;
      gmkc[1] = gk;
      gmkc[2] = gc;
    }
  } else {
    // A an = h - C v1 - K v2 with A = M + c1 C + c2 K: solve A^T r = G (partial pivoting)
    T At[8][9], Af[8][9];
    for (int i = 0; i < ndof; ++i) {
      T cv = T(0), kv = T(0);
      for (int j = 0; j < ndof; ++j) {
        Af[i][j] = (mm[i * ndof + j] + c1 * cm[i * ndof + j]) + c2 * km[i * ndof + j];
        At[j][i] = Af[i][j];
        cv += cm[i * ndof + j] * v1[j];
        kv += km[i * ndof + j] * v2[j];
      }
      Af[i][ndof] = (h[i] - cv) - kv;
      At[i][ndof] = G[i];
    }
    auto solve = [&](T (*Mx)[9], T* x) {
      for (int col = 0; col < ndof; ++col) {
        int piv = col;
        for (int r = col + 1; r < ndof; ++r)
          if (fabs(Mx[r][col]) > fabs(Mx[piv][col])) piv = r;
        if (piv != col)
          for (int q = 0; q <= ndof; ++q) {
            const T t = Mx[col][q];
            Mx[col][q] = Mx[piv][q];
            Mx[piv][q] = t;
          }
        for (int r = col + 1; r < ndof; ++r) {
          const T fct = Mx[r][col] / Mx[col][col];
          for (int q = col; q <= ndof; ++q) Mx[r][q] -= fct * Mx[col][q];
        }
      }
      for (int r = ndof - 1; r >= 0; --r) {
        T acc = Mx[r][ndof];
        for (int q = r + 1; q < ndof; ++q) acc -= Mx[r][q] * x[q];
        x[r] = acc / Mx[r][r];
      }
    };
    T r[8];
    solve(Af, an);
    solve(At, r);
    for (int i = 0; i < ndof; ++i) {
      gh[i] = r[i];
      T cr = T(0), kr = T(0);
      for (int j = 0; j < ndof; ++j) {
        cr += cm[j * ndof + i] * r[j];
        kr += km[j * ndof + i] * r[j];
      }
      gv1[i] = (gvn ? gvn[i] : T(0)) - cr;
      gv2[i] = (gdn ? gdn[i] : T(0)) - kr;
    }
    if (gmat)  // g_M, g_K, g_C (ndof x ndof each, row-major, in that order)
      for (int i = 0; i < ndof; ++i)
        for (int j = 0; j < ndof; ++j) {
          const T gA = -r[i] * an[j];
          gmat[i * ndof + j] = gA;
          gmat[ndof * ndof + i * ndof + j] = c2 * gA - r[i] * v2[j];
          gmat[2 * ndof * ndof + i * ndof + j] = c1 * gA - r[i] * v1[j];
        }
  }
  for (int i = 0; i < ndof; ++i) {
    gv[i] = gv1[i] + tdt * gv2[i];
    gd[i] = gv2[i];
    ga[i] = k1 * gv1[i] + k2 * gv2[i];
  }
}

// ------------------------------------------------------------------ ordered sums
// Two passes with a fixed association: block b sums elements b, b + B, ... of a strided
// loop in thread order and a fixed tree; one block then sums the block results.  The
// result does not depend on scheduling, so repeated calls give the same bits.
constexpr int kSumBlocks = 256;
template <typename T>
__global__ void k_sum_partial(const T* __restrict__ x, int64_t n, int64_t stride, double* __restrict__ part) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)x[i * stride];
  __shared__ double sh[kB];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_sum_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  __shared__ double sh[kSumBlocks];
  sh[threadIdx.x] = (int)threadIdx.x < nb ? part[threadIdx.x] : 0.0;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

template <class L, typename T>
OpArg<L, T> op_arg(const double* host) {
  OpArg<L, T> A;
  for (int i = 0; i < L::Q * L::Q; ++i) A.a[i] = (T)host[i];
  return A;
}

}  // namespace
}  // namespace vs

using namespace vs;

extern "C" {

int vs_streaming_vjp(int q, int dtype, const void* g_out, void* g_in, int nx, int ny, int nz, void* stream) {
  VS_REQUIRE(g_out && g_in && g_out != g_in && nx > 0 && ny > 0, "vs_streaming_vjp: bad arguments");
  const int nzz = q == 9 ? 1 : nz;
  VS_REQUIRE(nzz > 0, "vs_streaming_vjp: bad nz");
  const int64_t n = (int64_t)nx * ny * nzz;
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    const int64_t b = (n + kB - 1) / kB;
    k_stream_vjp<L, T><<<(unsigned)(b < 65535 * 8 ? b : 65535 * 8), kB, 0, as_stream(stream)>>>(
        (const T*)g_out, (T*)g_in, nx, ny, nzz);
    VS_CHECK_LAUNCH("vs_streaming_vjp");
    return VS_OK;
  });
}

int vs_macroscopic_vjp(int q, int dtype, const void* f, const void* g_rho, const void* g_u, void* g_f, int64_t n,
                       void* stream) {
  VS_REQUIRE(f && g_f && n > 0 && (g_rho || g_u), "vs_macroscopic_vjp: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_macro_vjp<L, T><<<grid_for(n, kB), kB, 0, as_stream(stream)>>>((const T*)f, (const T*)g_rho, (const T*)g_u,
                                                                      (T*)g_f, n);
    VS_CHECK_LAUNCH("vs_macroscopic_vjp");
    return VS_OK;
  });
}

int vs_equilibrium_vjp(int q, int dtype, const void* rho, const void* u, const void* g_feq, void* g_rho, void* g_u,
                       int64_t n, void* stream) {
  VS_REQUIRE(rho && u && g_feq && g_rho && g_u && n > 0, "vs_equilibrium_vjp: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_eq_vjp<L, T><<<grid_for(n, kB), kB, 0, as_stream(stream)>>>((const T*)rho, (const T*)u, (const T*)g_feq,
                                                                   (T*)g_rho, (T*)g_u, n);
    VS_CHECK_LAUNCH("vs_equilibrium_vjp");
    return VS_OK;
  });
}

int vs_collision_vjp(int q, int dtype, int kind, const void* f, const void* feq, double omega, const void* g_out,
                     void* g_f, void* g_feq, void* g_omega_node, int64_t n, void* stream) {
  VS_REQUIRE(f && feq && g_out && g_f && g_feq && n > 0, "vs_collision_vjp: bad arguments");
  VS_REQUIRE(kind == VS_COLLIDE_BGK || kind == VS_COLLIDE_KBC || kind == VS_COLLIDE_REG,
             "vs_collision_vjp: kind must be BGK, KBC or REG (MRT: vs_collision_mrt_vjp)");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_collide_vjp<L, T><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(kind, (const T*)f, (const T*)feq, (T)omega,
                                                                          (const T*)g_out, (T*)g_f, (T*)g_feq,
                                                                          (T*)g_omega_node, n);
    VS_CHECK_LAUNCH("vs_collision_vjp");
    return VS_OK;
  });
}

int vs_collision_mrt_vjp(int q, int dtype, const void* f, const void* feq, const double* op_host, const void* g_out,
                         void* g_f, void* g_feq, double* g_op, int64_t n, void* stream) {
  VS_REQUIRE(f && feq && op_host && g_out && g_f && g_feq && n > 0, "vs_collision_mrt_vjp: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    cudaStream_t st = as_stream(stream);
    k_mrt_vjp<L, T><<<grid_for(n, kB), kB, 0, st>>>(op_arg<L, T>(op_host), (const T*)g_out, (T*)g_f, (T*)g_feq, n);
    if (g_op)  // g_A[i][j] = sum_nodes g_i (feq_j - f_j)
      k_outer_sum<T><<<L::Q * L::Q, kB, 0, st>>>(L::Q, (const T*)g_out, (const T*)feq, (const T*)f, n, g_op);
    VS_CHECK_LAUNCH("vs_collision_mrt_vjp");
    return VS_OK;
  });
}

int vs_forcing_vjp(int q, int dtype, int kind, const void* g, const void* u, double omega, const void* g_out,
                   void* g_f, void* g_g, void* g_u, void* g_scale_node, int64_t n, void* stream) {
  VS_REQUIRE(g && u && g_out && g_g && g_u && n > 0, "vs_forcing_vjp: bad arguments");
  VS_REQUIRE(kind == VS_FORCE_EDM || kind == VS_FORCE_GUO_BGK, "vs_forcing_vjp: kind must be EDM or GUO_BGK");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    const T s = kind == VS_FORCE_EDM ? T(1) : (T)(1.0 - 0.5 * omega);
    k_forcing_vjp<L, T><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(
        (const T*)g, (const T*)u, s, (const T*)g_out, (T*)g_f, (T*)g_g, (T*)g_u, (T*)g_scale_node, n);
    VS_CHECK_LAUNCH("vs_forcing_vjp");
    return VS_OK;
  });
}

int vs_forcing_guo_mrt_vjp(int q, int dtype, const void* g, const void* u, const double* op_host, const void* g_out,
                           void* g_f, void* g_g, void* g_u, void* guo_scratch, double* g_op, int64_t n, void* stream) {
  VS_REQUIRE(g && u && op_host && g_out && g_f && g_g && g_u && n > 0, "vs_forcing_guo_mrt_vjp: bad arguments");
  VS_REQUIRE(!g_op || guo_scratch, "vs_forcing_guo_mrt_vjp: the operator's cotangent needs guo_scratch (q x n)");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    cudaStream_t st = as_stream(stream);
    k_guo_mrt_vjp<L, T><<<grid_for(n, 128), 128, 0, st>>>(op_arg<L, T>(op_host), (const T*)g, (const T*)u,
                                                           (const T*)g_out, (T*)g_f, (T*)g_g, (T*)g_u,
                                                           g_op ? (T*)guo_scratch : nullptr, n);
    if (g_op)  // g_F[i][j] = sum_nodes g_out_i guo_j
      k_outer_sum<T><<<L::Q * L::Q, kB, 0, st>>>(L::Q, (const T*)g_out, (const T*)guo_scratch, nullptr, n, g_op);
    VS_CHECK_LAUNCH("vs_forcing_guo_mrt_vjp");
    return VS_OK;
  });
}

int vs_boundary_vjp(int q, int dtype, int kind, int mode, int loc, const void* f_in, const void* f_before_stream,
                    const void* g_out, void* g_in, void* g_before_stream, void* g_wall_node, int nx, int ny, int nz,
                    double rho_wall, double ux_wall, double uy_wall, double uz_wall, void* stream) {
  VS_REQUIRE(f_in && g_out && g_in && g_in != g_out, "vs_boundary_vjp: bad arguments");
  VS_REQUIRE(kind >= VS_BC_NEE && kind <= VS_BC_SPECULAR, "vs_boundary_vjp: bad kind %d", kind);
  VS_REQUIRE(mode >= VS_WALL_GIVEN && mode <= VS_WALL_PRESSURE,
             "vs_boundary_vjp: mode must be given, velocity or pressure (a force-corrected wall is a given wall "
             "with corrected velocity)");
  VS_REQUIRE(!((kind == VS_BC_BB || kind == VS_BC_SPECULAR) && !f_before_stream),
             "vs_boundary_vjp: bounce-back needs f_before_stream");
  const int dim = q == 9 ? 2 : 3;
  VS_REQUIRE(loc >= 0 && loc < 2 * dim, "vs_boundary_vjp: loc %d invalid", loc);
  const int nn[3] = {nx, ny, q == 9 ? 1 : nz};
  VS_REQUIRE(nx >= 3 && ny >= 3 && (q == 9 || nz >= 3), "vs_boundary_vjp: grid too small");
  const int64_t n = (int64_t)nn[0] * nn[1] * nn[2];
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemcpyAsync(g_in, g_out, sizeof(T) * L::Q * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && g_before_stream) e = cudaMemsetAsync(g_before_stream, 0, sizeof(T) * L::Q * n, s);
    if (e != cudaSuccess) return cuda_status(e, "vs_boundary_vjp copy");
    WallVjp<T> W{};
    W.kind = kind;
    W.mode = mode;
    W.loc = loc;
    for (int d = 0; d < 3; ++d) W.n[d] = nn[d];
    W.rho = (T)rho_wall;
    W.u[0] = (T)ux_wall;
    W.u[1] = (T)uy_wall;
    W.u[2] = (T)uz_wall;
    const int64_t nf = face_size(loc, nn);
    k_boundary_vjp<L, T><<<grid_for(nf, 64), 64, 0, s>>>(W, (const T*)f_in, (const T*)f_before_stream,
                                                         (const T*)g_out, (T*)g_in, (T*)g_before_stream,
                                                         (T*)g_wall_node, nf);
    VS_CHECK_LAUNCH("vs_boundary_vjp");
    return VS_OK;
  });
}

int vs_ib_pair_dot(int dtype, const void* A, const void* grid, int c, int64_t n_grid, const int32_t* I, int m, int s,
                   void* out, void* stream) {
  VS_REQUIRE(A && grid && I && out && c > 0 && m > 0 && s > 0 && n_grid > 0, "vs_ib_pair_dot: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_pair_dot<T><<<grid_for((int64_t)m * s, kB), kB, 0, as_stream(stream)>>>((const T*)A, (const T*)grid, I, m, s, c,
                                                                               n_grid, (T*)out);
    VS_CHECK_LAUNCH("vs_ib_pair_dot");
    return VS_OK;
  });
}

int vs_ib_stencil_vjp(int kernel, int radius, int dtype, int dim, const void* x, const void* y, const void* z,
                      const void* g_W, void* g_x, void* g_y, void* g_z, int m, void* stream) {
  VS_REQUIRE(x && y && g_W && g_x && g_y && m > 0 && (dim == 2 || (dim == 3 && z && g_z)),
             "vs_ib_stencil_vjp: bad arguments");
  VS_REQUIRE(radius >= 1 && radius <= 3, "vs_ib_stencil_vjp: radius must be 1..3");
  VS_REQUIRE(kernel >= VS_KERNEL_PESKIN3 && kernel <= VS_KERNEL_COSINE4, "vs_ib_stencil_vjp: bad kernel");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_stencil_vjp<T><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>(kernel, radius, dim, (const T*)x, (const T*)y,
                                                                       (const T*)z, (const T*)g_W, (T*)g_x, (T*)g_y,
                                                                       (T*)g_z, m);
    VS_CHECK_LAUNCH("vs_ib_stencil_vjp");
    return VS_OK;
  });
}

int vs_newmark_vjp(int dtype, int ndof, const void* a, const void* v, const void* d, const void* h, double m, double k,
                   double c, const void* m_mat, const void* k_mat, const void* c_mat, double dt, double gamma,
                   double beta, const void* g_a_next, const void* g_v_next, const void* g_d_next, void* g_a,
                   void* g_v, void* g_d, void* g_h, void* g_mkc, void* g_mats, void* stream) {
  VS_REQUIRE(a && v && d && h && g_a && g_v && g_d && g_h, "vs_newmark_vjp: null argument");
  VS_REQUIRE(ndof >= 1 && ndof <= 8, "vs_newmark_vjp: ndof must be 1..8");
  const int matrix = m_mat != nullptr;
  VS_REQUIRE(!matrix || (k_mat && c_mat), "vs_newmark_vjp: matrix form needs m, k and c matrices");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_newmark_vjp<T><<<1, 32, 0, as_stream(stream)>>>(
        ndof, matrix, (const T*)a, (const T*)v, (const T*)d, (const T*)h, (const T*)m_mat, (const T*)k_mat,
        (const T*)c_mat, m, k, c, dt, gamma, beta, (const T*)g_a_next, (const T*)g_v_next, (const T*)g_d_next, (T*)g_a,
        (T*)g_v, (T*)g_d, (T*)g_h, (T*)g_mkc, (T*)g_mats);
    VS_CHECK_LAUNCH("vs_newmark_vjp");
    return VS_OK;
  });
}

int vs_sum_ordered(int dtype, const void* x, int64_t n, int64_t stride, double* scratch, double* out, void* stream) {
  VS_REQUIRE(x && scratch && out && n >= 0 && stride >= 1, "vs_sum_ordered: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    cudaStream_t st = as_stream(stream);
    k_sum_partial<T><<<kSumBlocks, kB, 0, st>>>((const T*)x, n, stride, scratch);
    k_sum_final<<<1, kSumBlocks, 0, st>>>(scratch, kSumBlocks, out);
    VS_CHECK_LAUNCH("vs_sum_ordered");
    return VS_OK;
  });
}

}  // extern "C"
