// Discrete adjoint of the 2-D cylinder VIV step (D2Q9 BGK, exact-difference forcing,
// multi-direct-forcing immersed boundary on a spring-mounted rigid cylinder, Newmark,
// equilibrium inflow, pressure non-equilibrium-extrapolation outflow, periodic y).
//
// Forward step (examples/2d/vortex_induced_vibration.py:96-148, with BGK collision):
//   rho, u = get_macroscopic(f);  f1 = (1 - w) f + w feq(rho, u)
//   X = X0 + d;  W = kernel(node - X) (ib/stencil.py:7-51)
//   U0 = interp(u);  k = 0..n_iter-1:  Fs_k = (v - U_k) 2 ds,  Ft += Fs_k,
//                                     U_k+1 = U_k + interp(0.5 spread(Fs_k))   (ib/mdf.py)
//   g = spread(Ft);  h = -sum Ft + a A;  Newmark (dyn.py:5-51) on the free DOFs
//   f2 = f1 + guo(g, u) (lbm/forcing/edm.py);  f3 = stream(f2);  f' = nee_p(eq(f3))
// The reverse sweep runs these in reverse with hand-derived transposes:
//   k_adj_bc    the outflow boundary (its 9 x 18 local Jacobian by forward-mode dual numbers)
//               and the inflow boundary (zeroes the wall adjoint, accumulates d/dU0)
//   k_adj_body  one CTA: recomputes the body's forward MDF, then Newmark^T, spread^T =
//               interpolation, the MDF iterations in reverse, interp^T = spread, and the
//               derivative of the weights with respect to the marker positions
//   k_adj_grid  per node: reverse streaming (pull) fused with the transposed Jacobian of
//               collision + forcing, plus the d/domega reduction
// f is checkpointed every `checkpoint_every` steps; each segment is recomputed forward
// (keeping its states) before its reverse sweep, so memory is (steps / C + C) grids.
#include <cmath>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "vs_boundary.cuh"
#include "vs_dispatch.cuh"
#include "vs_dual.cuh"
#include "vs_ib.cuh"

namespace vs {
namespace adj {

// dual numbers: vs_dual.cuh
using vs::Dual;

// feq_i(rho, u) in the reference's form (lbm/basic.py:114-135), generic scalar S
template <typename S, typename T>
__device__ __forceinline__ void feq9(S rho, S ux, S uy, S* out) {
  const S usq = ux * ux + uy * uy;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const S uc = ux * S((T)q9_cx(i)) + uy * S((T)q9_cy(i));
    out[i] = (rho * S(q9_w<T>(i))) * (((S(1) + S(3) * uc) + S(4.5) * (uc * uc)) - S(1.5) * usq);
  }
}

// boundary_pressure_nee at the right wall for one face node (lbm/boundary/nee.py:19-60,
// _helpers.py:98-121, 200-217): wall populations w, neighbour populations nb -> out
template <typename S, typename T>
__device__ __forceinline__ void pnee_right(const S* w, const S* nb, T rho_w, S* out) {
  constexpr int loc = VS_RIGHT;
  const S num = rho_numerator(L9{}, loc, w);
  const S nvs = S(1) - num / S(rho_w);
  S u[2];
  u[0] = S(loc_sign(loc)) * nvs;
  pressure_tangential(L9{}, loc, nb, u);
  S fw[9], fe[9], rn, un[2];
  feq9<S, T>(S(rho_w), u[0], u[1], fw);
  macro(L9{}, nb, rn, un);
  feq9<S, T>(rn, un[0], un[1], fe);
#pragma unroll
  for (int i = 0; i < 9; ++i) out[i] = fw[i] + (nb[i] - fe[i]);
}

// The collision of the step on scalar type S (T, or Dual<T> for derivatives): BGK, KBC,
// regularised (vs_common.cuh restatements of lbm/collision/*.py) or MRT with operator op
// (its derivative with respect to omega in dop, for the dual part).
template <typename S, typename T>
__device__ __forceinline__ void collide_any(int kind, S* f, const S* fe, S omega, const T* op, const T* dop) {
  if (kind == VS_COLLIDE_MRT) {
    S d[9], out[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) d[j] = fe[j] - f[j];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      S acc = S(0);
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        S o;
        if constexpr (std::is_same<S, T>::value) o = op[i * 9 + j];
        else o = S(op[i * 9 + j], dop[i * 9 + j] * omega.d);  // omega.d seeds d/domega
        acc = j == 0 ? o * d[j] : acc + o * d[j];
      }
      out[i] = f[i] + acc;
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) f[i] = out[i];
    return;
  }
  CollideParams<S> P;
  P.omega = omega;
  P.one_m_omega = S(1) - omega;
  P.inv_omega = S(1) / omega;
  P.one_m_inv = S(1) - S(1) / omega;
  P.mrt = nullptr;
  if (kind == VS_COLLIDE_KBC) collide_kbc(L9{}, f, fe, P);
  else if (kind == VS_COLLIDE_REG) collide_reg(L9{}, f, fe, P);
  else collide_bgk<L9>(f, fe, P);
}

// post-collision populations of node (x, y) without body force
template <typename T>
__device__ __forceinline__ void post_collide(const T* __restrict__ f, int64_t n, int ny, int x, int y, T omega,
                                             T* out, int kind, const T* op) {
  const int64_t p = (int64_t)x * ny + y;
  T r, u[2], fe[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) out[i] = f[i * n + p];
  macro(L9{}, out, r, u);
  feq9<T, T>(r, u[0], u[1], fe);
  collide_any<T, T>(kind, out, fe, omega, op, op);
}

// lambda_f and d/domega of one node for collision + exact-difference forcing, by forward-mode
// dual numbers (10 passes: the 9 populations and omega): the transposed Jacobian of any
// collision model of the reference.  g is the node's body force.
template <typename T>
__device__ __forceinline__ void node_adjoint_dual(const T* f, T g0, T g1, const T* l2, T omega, int kind, const T* op,
                                                  const T* dop, T* lam_f, T& lomega) {
  for (int k = 0; k < 10; ++k) {
    Dual<T> fd[9], r, u[2], fe[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) fd[i] = Dual<T>(f[i], (T)(k == i));
    macro(L9{}, fd, r, u);
    feq9<Dual<T>, T>(r, u[0], u[1], fe);
    const Dual<T> om(omega, (T)(k == 9));
    collide_any<Dual<T>, T>(kind, fd, fe, om, op, dop);
    const Dual<T> gd[2] = {Dual<T>(g0, T(0)), Dual<T>(g1, T(0))};
    T sum = T(0);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const Dual<T> out = fd[i] + guo_i(L9{}, i, gd, u);
      sum += l2[i] * out.d;
    }
    if (k < 9) lam_f[k] = sum;
    else lomega = sum;
  }
}

template <typename T>
struct GridArgs {
  const T* f;   // populations at the start of the step (9, nx, ny)
  T* lam;       // in: adjoint of the step's output; k_adj_bc rewrites its wall columns
  T* lam_out;   // out: adjoint of f
  T* g;         // body force of the step on the full grid (2, nx, ny), zero off the stencils
  T* lu;        // adjoint of u from the immersed boundary (2, nx, ny); both reset to zero here
  int nx, ny;
  T omega, U0, rho_out;
  double* acc;  // [0] d/dU0 (boundaries), [1] d/domega
  double* acc_bc; // per-block partial sums of the inflow's d/dU0 (one slot per boundary block)
  double* acc_w;  // per-block partial sums of d/domega (one slot per grid-adjoint block)
  int slot0;      // first slot of this launch
  int mode;       // 0: every node; 1: outside the body's window; 2: the window only
  const T* wstate;  // body state of the step (displacement -> window origin)
  double lo0, lo1;  // smallest marker x, y (plan precision)
  int R, cap[2];    // stencil half-width; window extent
  int kind;         // collision model (VS_COLLIDE_*)
  const T* op;      // MRT operator (device, 9 x 9) and its derivative with respect to omega
  const T* dop;
};

__device__ __forceinline__ int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// block sum of v into part[blockIdx.x] (a fixed tree per block; the host sums the block
// slots in order, so the result does not depend on scheduling)
template <int NT>
__device__ __forceinline__ void block_accumulate(double v, double* part) {
  __shared__ double red[NT / 32];
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int k = 0; k < NT / 32; ++k) s += red[k];
    part[blockIdx.x] = s;
  }
}

// Boundary adjoint.  Forward order: f_a = eq_left(f3), f' = nee_p_right(f_a); reverse: the
// right wall and neighbour columns, then the left wall.  A block handles kRows face rows:
// phase 1 rebuilds the streamed wall and neighbour populations (one thread per row and
// population), phase 2 evaluates the 18 Jacobian columns of the outflow boundary by
// forward-mode dual numbers (one thread per row and input), phase 3 writes the adjoints.
constexpr int kRows = 8;

template <typename T>
__global__ void __launch_bounds__(kRows * 18) k_adj_bc(GridArgs<T> A) {
  __shared__ T w[kRows][9], nb[kRows][9], lo[kRows][9], col[kRows][18];
  const int nx = A.nx, ny = A.ny;
  const int64_t n = (int64_t)nx * ny;
  const int r = threadIdx.x / 18, k = threadIdx.x % 18;
  const int y = blockIdx.x * kRows + r;
  const bool live = y < ny;
  if (live && k < 9) {
    // streamed population k at the wall (x = nx-1) and at its neighbour (x = nx-2)
    T src[9];
    post_collide(A.f, n, ny, wrap(nx - 1 - q9_cx(k), nx), wrap(y - q9_cy(k), ny), A.omega, src, A.kind, A.op);
    w[r][k] = src[k];
    post_collide(A.f, n, ny, nx - 2 - q9_cx(k), wrap(y - q9_cy(k), ny), A.omega, src, A.kind, A.op);
    nb[r][k] = src[k];
    lo[r][k] = A.lam[k * n + (int64_t)(nx - 1) * ny + y];
  }
  __syncthreads();
  if (live) {
    Dual<T> dw[9], dn[9], o[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      dw[i] = Dual<T>(w[r][i], (T)(k == i));
      dn[i] = Dual<T>(nb[r][i], (T)(k == 9 + i));
    }
    pnee_right<Dual<T>, T>(dw, dn, A.rho_out, o);
    T sum = T(0);
#pragma unroll
    for (int i = 0; i < 9; ++i) sum += lo[r][i] * o[i].d;
    col[r][k] = sum;
  }
  __syncthreads();
  double dU0 = 0.0;
  if (live && k < 9) {
    const int64_t pw = (int64_t)(nx - 1) * ny + y, pn = (int64_t)(nx - 2) * ny + y;
    A.lam[k * n + pw] = col[r][k];  // the wall values were replaced: only the new path remains
    A.lam[k * n + pn] = A.lam[k * n + pn] + col[r][9 + k];
    // left wall: f = feq(1, (U0, 0)) replaced every population (lbm/boundary/eq.py:25-56)
    const T cx = (T)q9_cx(k);
    const T dfeq = q9_w<T>(k) * ((T(3) * cx + T(9) * (cx * A.U0) * cx) - T(3) * A.U0);
    const int64_t p0 = k * n + y;
    dU0 = (double)(A.lam[p0] * dfeq);
    A.lam[p0] = T(0);
  }
  // block sum of the inflow term (rows x populations) in a fixed order
  __shared__ double red[kRows * 18];
  red[threadIdx.x] = dU0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int i = 0; i < kRows * 18; ++i) sum += red[i];
    A.acc_bc[blockIdx.x] += sum;  // this block's slot; the steps run in order
  }
}

// Grid adjoint, one thread per node: pull the streamed adjoint, then the transposed
// Jacobian of BGK collision + exact-difference forcing at this node.
template <typename T>
__global__ void __launch_bounds__(256) k_adj_grid(GridArgs<T> A) {
  const int nx = A.nx, ny = A.ny;
  const int64_t n = (int64_t)nx * ny;
  // the body's stencil window of this step (from its displacement), which the body adjoint
  // feeds: mode 1 does every node outside it, mode 2 the window only, mode 0 everything
  int wx0 = 0, wy0 = 0;
  if (A.mode) {
    wx0 = ifloor((T)A.lo0 + A.wstate[6]) - A.R + 1;
    wy0 = ifloor((T)A.lo1 + A.wstate[7]) - A.R + 1;
  }
  int x, y;
  bool live;
  if (A.mode == 2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    live = k < A.cap[0] * A.cap[1];
    x = wx0 + (live ? k / A.cap[1] : 0);
    y = wy0 + (live ? k % A.cap[1] : 0);
    live = live && x >= 0 && x < nx && y >= 0 && y < ny;
  } else {
    x = blockIdx.y;
    y = blockIdx.x * blockDim.x + threadIdx.x;
    live = y < ny;
    if (A.mode == 1 && x >= wx0 && x < wx0 + A.cap[0] && y >= wy0 && y < wy0 + A.cap[1]) live = false;
  }
  T dw = T(0);
  if (live) {
    const int64_t p = (int64_t)x * ny + y;
    T f[9], l2[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      f[i] = A.f[i * n + p];
      l2[i] = A.lam[i * n + (int64_t)wrap(x + q9_cx(i), nx) * ny + wrap(y + q9_cy(i), ny)];
    }
    T r, u[2], fe[9];
    macro(L9{}, f, r, u);
    feq9<T, T>(r, u[0], u[1], fe);
    const T ir = T(1) / r;
    T g0 = T(0), g1 = T(0), lu0 = T(0), lu1 = T(0);
    if (A.mode != 1) {  // only the window carries body force and the interpolation adjoint
      g0 = A.g[p];
      g1 = A.g[n + p];
      lu0 = A.lu[p];
      lu1 = A.lu[n + p];
      // leave the body fields zero for the next (earlier) step, which writes only its stencils
      if (g0 != T(0) || g1 != T(0) || lu0 != T(0) || lu1 != T(0)) {
        A.g[p] = T(0);
        A.g[n + p] = T(0);
        A.lu[p] = T(0);
        A.lu[n + p] = T(0);
      }
    }
    if (A.kind != VS_COLLIDE_BGK) {
      // other collision models: transposed Jacobian by dual numbers, plus the immersed
      // boundary's lambda_u through u = m / rho
      T lf[9], lom;
      node_adjoint_dual<T>(f, g0, g1, l2, A.omega, A.kind, A.op, A.dop, lf, lom);
      dw = lom;
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        const T cx = (T)q9_cx(j), cy = (T)q9_cy(j);
        A.lam_out[j * n + p] = lf[j] + (lu0 * (cx - u[0]) + lu1 * (cy - u[1])) * ir;
      }
    } else {
    T lrho = T(0);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const T cx = (T)q9_cx(i), cy = (T)q9_cy(i), wi = q9_w<T>(i);
      const T cu = cx * u[0] + cy * u[1], cg = cx * g0 + cy * g1;
      // forcing term: d/du_a of w_i (3 (c_i - u).g + 9 (c_i.u)(c_i.g))
      lu0 += l2[i] * wi * (T(-3) * g0 + T(9) * cg * cx);
      lu1 += l2[i] * wi * (T(-3) * g1 + T(9) * cg * cy);
      // collision: omega feq_i(rho, u)
      const T lf = A.omega * l2[i];
      lrho += lf * fe[i] * ir;
      const T rw = r * wi;
      lu0 += lf * rw * ((T(3) * cx + T(9) * cu * cx) - T(3) * u[0]);
      lu1 += lf * rw * ((T(3) * cy + T(9) * cu * cy) - T(3) * u[1]);
      dw += l2[i] * (fe[i] - f[i]);
    }
    lu0 *= ir;
    lu1 *= ir;
#pragma unroll
    for (int j = 0; j < 9; ++j) {
      const T cx = (T)q9_cx(j), cy = (T)q9_cy(j);
      A.lam_out[j * n + p] = (T(1) - A.omega) * l2[j] + lrho + (lu0 * (cx - u[0]) + lu1 * (cy - u[1]));
    }
    }
  }
  {
    // per-block partial of d/domega in its own slot (no contention; summed at the end)
    __shared__ double red[8];
    double v = (double)dw;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double sum = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) sum += red[k];
      A.acc_w[A.slot0 + blockIdx.y * gridDim.x + blockIdx.x] += sum;
    }
  }
}

// d/dU0 of the initial state f = feq(1, (U0, 0)) everywhere
template <typename T>
__global__ void __launch_bounds__(256) k_adj_initial(const T* __restrict__ lam, int64_t n, T U0, double* acc) {
  double s = 0.0;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const T cx = (T)q9_cx(i);
      s += (double)(lam[i * n + p] * (q9_w<T>(i) * ((T(3) * cx + T(9) * (cx * U0) * cx) - T(3) * U0)));
    }
  }
  block_accumulate<256>(s, acc);
}

// ------------------------------------------------------------------ body adjoint
template <typename T>
struct BodyArgs {
  const T* f;       // populations at the start of the step
  const T* lam;     // adjoint of the streamed populations (after k_adj_bc)
  T* g;             // out: forward body force at the stencil nodes (2, nx, ny)
  T* lu;            // out: adjoint of u at the stencil nodes (2, nx, ny)
  const T* state;   // body state at the start of the step: a[3], v[3], d[3], h[3]
  T* lstate;        // in: adjoint of the state after the step (a, v, d: 3 each); out: before
  const T* X0;      // (M) marker x, (M) marker y
  int nx, ny, M, kernel, n_iter;
  T ds2;            // 2 ds
  T wobj;           // weight of the x force in the objective, for steps >= obj_start
  const int* seg_start;  // first step of the segment (device), so a graph can replay it
  int j, obj_start;      // this step's index in its segment
  int chain_k;           // markers share stencil nodes only within +-chain_k in marker order (0: any)
  T k1, k2, c1, c2, dt, damp, stiff, den, area;
  int free_dof[2];
  double* dK;       // d/dstiffness
  double* dX;       // (2 M): d/dX0, d/dY0
};

constexpr int kAdjBodyThreads = 1024;

// Node sum over the pairs that reach the node (nx_, ny_) of a pair: sum_p W_p F[m_p] (both
// components), the contributing markers given by the pair's bit mask (NW 64-bit words,
// bit i = marker i), taken in increasing marker order.
template <typename T, int WD>
__device__ __forceinline__ void node_sum(int nx_, int ny_, const unsigned long long* mask, int NW, const int* fxy,
                                         const T* W, const T* F, T& s0, T& s1) {
  constexpr int S = WD * WD;
  s0 = T(0);
  s1 = T(0);
  for (int w = 0; w < NW; ++w) {
    unsigned long long b = mask[w];
    while (b) {
      const int i = w * 64 + __ffsll((long long)b) - 1;
      b &= b - 1;
      const T wt = W[i * S + (nx_ - fxy[2 * i]) * WD + (ny_ - fxy[2 * i + 1])];
      s0 += F[2 * i] * wt;
      s1 += F[2 * i + 1] * wt;
    }
  }
}

// sum of v over the S consecutive threads of one marker's stencil pairs, complete in the
// group's first lane (S a power of two up to 32)
template <typename T, int S>
__device__ __forceinline__ T group_sum(T v) {
  static_assert(S <= 32 && (S & (S - 1)) == 0, "stencil groups of a power of two up to 32");
  const unsigned lane = threadIdx.x & 31, base = lane & ~(unsigned)(S - 1);
  const unsigned gm = S == 32 ? 0xffffffffu : (((1u << S) - 1u) << base);
#pragma unroll
  for (int o = S / 2; o >= 1; o >>= 1) v += __shfl_down_sync(gm, v, o, S);
  return v;
}

template <typename T, int R>
__global__ void __launch_bounds__(kAdjBodyThreads) k_adj_body(BodyArgs<T> A) {
  constexpr int WD = 2 * R, S = WD * WD;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int M = A.M, P = M * S, NI = A.n_iter > 0 ? A.n_iter : 0, NF = NI > 0 ? NI : 1;
  const int nx = A.nx, ny = A.ny;
  const int64_t n = (int64_t)nx * ny;
  T* W = (T*)smem;             // [P] weights
  T* dWx = W + P;              // [P] dW/dX of the marker
  T* dWy = dWx + P;            // [P] dW/dY
  T* lW = dWy + P;             // [P] adjoint of the weight
  T* un = lW + P;              // [2P] u at the pair's node
  T* lg = un + 2 * P;          // [2P] adjoint of g at the pair's node
  T* nmu = lg + 2 * P;         // [2P] nodeval(mu) at the pair's node
  T* Fs = nmu + 2 * P;         // [NF][2M] force steps; in reverse their adjoints
  T* Ft = Fs + 2 * M * NF;     // [2M]
  T* U = Ft + 2 * M;           // [2M]
  T* mu = U + 2 * M;           // [2M] adjoint of U_k (read)
  T* mu2 = mu + 2 * M;         // [2M] adjoint of U_k (written)
  T* lFt = mu2 + 2 * M;        // [2M] adjoint of Ft
  T* lFs = lFt + 2 * M;        // [NF][2M] adjoints of the force steps
  T* red = lFs + 2 * M * NF;   // [8] a, v, d, h adjoints
  const int NW = (M + 63) / 64;
  unsigned long long* cm = (unsigned long long*)(((uintptr_t)(red + 8) + 7) & ~(uintptr_t)7);  // [P][NW]
  int* fxy = (int*)(cm + (size_t)P * NW);  // [2M] stencil corners
  {
    unsigned have;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(have));
    if ((size_t)((const unsigned char*)(fxy + 2 * M) - smem) > have) return;  // host sizing error: no work
  }
  const int step = *A.seg_start + A.j;
  const T wobj = step >= A.obj_start ? A.wobj : T(0);

  const T a[2] = {A.state[0], A.state[1]}, v[2] = {A.state[3], A.state[4]}, d[2] = {A.state[6], A.state[7]};
  // markers (dyn.py:68-81), weights and their position derivatives, u and lambda_g at the nodes
  for (int p = tid; p < P; p += nt) {
    const int m = p / S, s = p - m * S, ix = s / WD, iy = s - ix * WD;
    const T xm = A.X0[m] + d[0], ym = A.X0[M + m] + d[1];
    const int fx = ifloor(xm), fy = ifloor(ym);
    if (s == 0) {
      fxy[2 * m] = fx - R + 1;
      fxy[2 * m + 1] = fy - R + 1;
    }
    const T rx = (T)(fx + ix - R + 1) - xm, ry = (T)(fy + iy - R + 1) - ym;
    const T px = delta(A.kernel, rx), py = delta(A.kernel, ry);
    W[p] = px * py;
    dWx[p] = -ddelta(A.kernel, rx) * py;
    dWy[p] = -px * ddelta(A.kernel, ry);
    lW[p] = T(0);
    const int gx = fx + ix - R + 1, gy = fy + iy - R + 1;
    // a forward run that succeeded kept every stencil inside the grid; clamp so that a
    // caller's inconsistent state cannot read outside it
    const int gxc = min(max(gx, 0), nx - 1), gyc = min(max(gy, 0), ny - 1);
    const int64_t q = (int64_t)gxc * ny + gyc;
    T fl[9], r, uu[2];
#pragma unroll
    for (int i = 0; i < 9; ++i) fl[i] = A.f[i * n + q];
    macro(L9{}, fl, r, uu);
    un[2 * p] = uu[0];
    un[2 * p + 1] = uu[1];
    // lambda_g = sum_i lambda2_i d guo_i / d g, lambda2 pulled from the streamed adjoint
    T l0 = T(0), l1 = T(0);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const T cx = (T)q9_cx(i), cy = (T)q9_cy(i), wi = q9_w<T>(i);
      const T l = A.lam[i * n + (int64_t)wrap(gxc + q9_cx(i), nx) * ny + wrap(gyc + q9_cy(i), ny)];
      const T cu = cx * uu[0] + cy * uu[1];
      l0 += l * wi * (T(3) * (cx - uu[0]) + T(9) * cu * cx);
      l1 += l * wi * (T(3) * (cy - uu[1]) + T(9) * cu * cy);
    }
    lg[2 * p] = l0;
    lg[2 * p + 1] = l1;
  }
  __syncthreads();
  // contributors of each pair's node
  for (int p = tid; p < P; p += nt) {
    const int m = p / S, s = p - m * S, ix = s / WD, iy = s - ix * WD;
    const int gx = fxy[2 * m] + ix, gy = fxy[2 * m + 1] + iy;
    for (int w = 0; w < NW; ++w) cm[(size_t)p * NW + w] = 0ull;
    // candidates: the whole marker set, or the cyclic neighbourhood m-K..m+K
    const int K = A.chain_k, nc = (K > 0 && 2 * K + 1 < M) ? 2 * K + 1 : M;
    for (int b = 0; b < nc; ++b) {
      int i = nc == M ? b : m - K + b;
      i = i < 0 ? i + M : (i >= M ? i - M : i);
      const unsigned dx = (unsigned)(gx - fxy[2 * i]), dy = (unsigned)(gy - fxy[2 * i + 1]);
      if (dx < (unsigned)WD && dy < (unsigned)WD) cm[(size_t)p * NW + (i >> 6)] |= 1ull << (i & 63);
    }
  }
  __syncthreads();
  // forward MDF (ib/mdf.py:38-64), every force step kept; one thread per pair, the
  // interpolation sums reduced within each marker's group of S threads
  for (int p = tid; p < P; p += nt) {
    const int m = p / S, s = p - m * S;
    const T a0 = group_sum<T, S>(W[p] * un[2 * p]), a1 = group_sum<T, S>(W[p] * un[2 * p + 1]);
    if (s == 0) {
      const T acc[2] = {a0, a1};
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        U[2 * m + c] = acc[c];
        const T fs = (v[c] - acc[c]) * A.ds2;
        Fs[2 * m + c] = fs;
        Ft[2 * m + c] = NI > 0 ? fs : T(0);
      }
    }
  }
  __syncthreads();
  for (int k = 0; k + 1 < NI; ++k) {
    const T* F = Fs + 2 * M * k;
    for (int p = tid; p < P; p += nt) {
      const int m = p / S, s = p - m * S, ix = s / WD, iy = s - ix * WD;
      T n0, n1;  // spread(F_k) at the pair's node
      node_sum<T, WD>(fxy[2 * m] + ix, fxy[2 * m + 1] + iy, cm + (size_t)p * NW, NW, fxy, W, F, n0, n1);
      const T a0 = group_sum<T, S>(W[p] * (T(0.5) * n0)), a1 = group_sum<T, S>(W[p] * (T(0.5) * n1));
      if (s == 0) {
        const T acc[2] = {a0, a1};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const T uq = U[2 * m + c] + acc[c];
          U[2 * m + c] = uq;
          const T fs = (v[c] - uq) * A.ds2;
          Fs[2 * M * (k + 1) + 2 * m + c] = fs;
          Ft[2 * m + c] = Ft[2 * m + c] + fs;
        }
      }
    }
    __syncthreads();
  }
  // g = spread(Ft) at the stencil nodes, for the grid adjoint's forcing Jacobian
  for (int p = tid; p < P; p += nt) {
    const int m = p / S, s = p - m * S, ix = s / WD, iy = s - ix * WD;
    const int gx = fxy[2 * m] + ix, gy = fxy[2 * m + 1] + iy;
    T s0, s1;
    node_sum<T, WD>(gx, gy, cm + (size_t)p * NW, NW, fxy, W, Ft, s0, s1);
    if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
    const int64_t q = (int64_t)gx * ny + gy;
    A.g[q] = s0;
    A.g[n + q] = s1;
  }
  // h = -sum Ft + a A (dyn.py:126-136, vortex_induced_vibration.py:136) and the Newmark
  // transpose (dyn.py:5-51); the objective weights h_x
  T hsum[2] = {T(0), T(0)};
  if (tid < 32) {  // sum of -Ft over the markers, warp 0 in a fixed tree
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      T acc = T(0);
      for (int m = tid; m < M; m += 32) acc += -Ft[2 * m + c];
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      hsum[c] = acc;
    }
  }
  if (tid == 0) {
    T h[2];
    for (int c = 0; c < 2; ++c) h[c] = hsum[c] + a[c] * A.area;
    double dK = 0.0;
    for (int c = 0; c < 2; ++c) {
      const T la1 = A.lstate[c], lv1 = A.lstate[3 + c], ld1 = A.lstate[6 + c];
      T la, lv, ld, lh;
      if (A.free_dof[c]) {
        const T v1 = v[c] + A.k1 * a[c];
        const T v2 = (d[c] + A.dt * v[c]) + A.k2 * a[c];
        const T an = ((h[c] - A.damp * v1) - A.stiff * v2) / A.den;
        const T lan = la1 + A.c1 * lv1 + A.c2 * ld1;  // a' feeds v' = c1 a' + v1, d' = c2 a' + v2
        const T lv1_ = lv1 - lan * A.damp / A.den;
        const T lv2_ = ld1 - lan * A.stiff / A.den;
        lh = lan / A.den;
        dK += (double)(lan * ((-v2 - an * A.c2) / A.den));  // den = m + c1 c + c2 k
        la = A.k1 * lv1_ + A.k2 * lv2_;
        lv = lv1_ + A.dt * lv2_;
        ld = lv2_;
      } else {
        la = la1;
        lv = lv1;
        ld = ld1;
        lh = T(0);
      }
      if (c == 0) lh += wobj;
      red[c] = la + A.area * lh;
      red[2 + c] = lv;
      red[4 + c] = ld;
      red[6 + c] = lh;
    }
    if (dK != 0.0) atomicAdd(A.dK, dK);
  }
  __syncthreads();
  // lambda_Ft = interp(lambda_g) - lambda_h; mu_NI-1 = 0
  for (int p = tid; p < P; p += nt) {
    const int m = p / S, s = p - m * S;
    const T a0 = group_sum<T, S>(W[p] * lg[2 * p]), a1 = group_sum<T, S>(W[p] * lg[2 * p + 1]);
    if (s == 0) {
      lFt[2 * m] = a0 - red[6];
      lFt[2 * m + 1] = a1 - red[7];
      mu[2 * m] = T(0);
      mu[2 * m + 1] = T(0);
    }
  }
  __syncthreads();
  // MDF in reverse: for k = NI-1 .. 0 (one pass per iteration, mu double-buffered)
  //   lambda_Fs_k = lambda_Ft + [k < NI-1] 0.5 interp(nodeval(mu_k+1))
  //   lambda_W   += [k < NI-1] 0.5 (mu_k+1,m . nodeval(Fs_k) + Fs_k,m . nodeval(mu_k+1))
  //   mu_k = mu_k+1 - 2 ds lambda_Fs_k
  T* mr = mu;
  T* mw = mu2;
  for (int k = NI - 1; k >= 0; --k) {
    const T* F = Fs + 2 * M * k;
    for (int p = tid; p < P; p += nt) {
      const int m = p / S, s = p - m * S, ix = s / WD, iy = s - ix * WD;
      T a0 = T(0), a1 = T(0);
      if (k + 1 < NI) {
        const int gx = fxy[2 * m] + ix, gy = fxy[2 * m + 1] + iy;
        T m0, m1, f0, f1;
        node_sum<T, WD>(gx, gy, cm + (size_t)p * NW, NW, fxy, W, mr, m0, m1);
        node_sum<T, WD>(gx, gy, cm + (size_t)p * NW, NW, fxy, W, F, f0, f1);
        lW[p] += T(0.5) * ((mr[2 * m] * f0 + mr[2 * m + 1] * f1) + (F[2 * m] * m0 + F[2 * m + 1] * m1));
        a0 = W[p] * (T(0.5) * m0);
        a1 = W[p] * (T(0.5) * m1);
      }
      a0 = group_sum<T, S>(a0);
      a1 = group_sum<T, S>(a1);
      if (s == 0) {
        const T acc[2] = {a0, a1};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const T lfs = lFt[2 * m + c] + acc[c];
          lFs[2 * M * k + 2 * m + c] = lfs;
          mw[2 * m + c] = mr[2 * m + c] - A.ds2 * lfs;
        }
      }
    }
    __syncthreads();
    T* t = mr;
    mr = mw;
    mw = t;
  }
  // lambda_v: every force step targets the body velocity
  if (tid < 32) {  // warp 0, fixed tree
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      T acc = T(0);
      for (int k = 0; k < NI; ++k)
        for (int m = tid; m < M; m += 32) acc += A.ds2 * lFs[2 * M * k + 2 * m + c];
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      if (tid == 0) red[2 + c] += acc;
    }
  }
  // interp^T: lambda_u at the nodes = nodeval(mu_0); weight adjoints of U0 = interp(u) and
  // of g = spread(Ft); then the marker position adjoints (X = X0 + d), summed per group
  for (int p = tid; p < P; p += nt) {
    const int m = p / S, s = p - m * S, ix = s / WD, iy = s - ix * WD;
    const int gx = fxy[2 * m] + ix, gy = fxy[2 * m + 1] + iy;
    T n0, n1;
    node_sum<T, WD>(gx, gy, cm + (size_t)p * NW, NW, fxy, W, mr, n0, n1);
    if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) {
      const int64_t q = (int64_t)gx * ny + gy;
      A.lu[q] = n0;
      A.lu[n + q] = n1;
    }
    const T lw = lW[p] + (mr[2 * m] * un[2 * p] + mr[2 * m + 1] * un[2 * p + 1]) +
                 (Ft[2 * m] * lg[2 * p] + Ft[2 * m + 1] * lg[2 * p + 1]);
    const T gxm = group_sum<T, S>(lw * dWx[p]), gym = group_sum<T, S>(lw * dWy[p]);
    if (s == 0) {
      lFt[2 * m] = gxm;  // lambda_Ft is no longer needed: reuse it for the position adjoints
      lFt[2 * m + 1] = gym;
      atomicAdd(A.dX + m, (double)gxm);
      atomicAdd(A.dX + M + m, (double)gym);
    }
  }
  __syncthreads();
  if (tid < 32) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      T acc = T(0);
      for (int m = tid; m < M; m += 32) acc += lFt[2 * m + c];
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
      if (tid == 0) {
        A.lstate[c] = red[c];
        A.lstate[3 + c] = red[2 + c];
        A.lstate[6 + c] = red[4 + c] + acc;
      }
    }
  }
}

template <typename T>
static size_t adj_body_smem(int M, int R, int n_iter) {
  const size_t S = 4 * R * R, P = M * S, NF = n_iter > 0 ? n_iter : 1, NW = (M + 63) / 64;
  return sizeof(T) * (4 * P + 6 * P + 4 * M * NF + 10 * (size_t)M + 8) + 8 + 8 * P * NW + sizeof(int) * 2 * M + 16;
}

}  // namespace adj
}  // namespace vs

// ------------------------------------------------------------------ plan
struct vs_adjoint_plan {
  vs_adjoint_cfg cfg;
  vs_lattice_plan* lat = nullptr;
  vs_body_plan* body = nullptr;
  int64_t n = 0;
  int M = 0, S = 0, C = 0, n_ck = 0;
  size_t ts = 4;
  double omega = 0, ds = 0;
  std::vector<double> theta;       // marker angles
  void* d_f0 = nullptr;            // initial populations
  void* d_fa = nullptr;
  void* d_fb = nullptr;
  void* d_ck = nullptr;            // checkpoints: n_ck x (9 n)
  void* d_ck_state = nullptr;      // n_ck x 12
  void* d_seg[2] = {nullptr, nullptr};        // (C + 1) x (9 n): recomputed segments (two in flight)
  void* d_seg_state[2] = {nullptr, nullptr};  // (C + 1) x 12
  int* d_seg_start = nullptr;      // [2] first step of the segment in each buffer
  cudaStream_t rec = nullptr;      // recompute stream (runs the next segment's forward)
  cudaStream_t aux = nullptr;      // boundary adjoint, concurrent with the body adjoint
  cudaEvent_t ev_rec[2] = {}, ev_rev[2] = {}, ev_f = nullptr, ev_b = nullptr;
  cudaGraphExec_t g_rec[2] = {}, g_rev[2] = {};
  cudaStream_t g_stream = nullptr;
  void* d_lam[2] = {nullptr, nullptr};
  void* d_g = nullptr;             // 2 n
  void* d_lu = nullptr;            // 2 n
  void* d_lstate = nullptr;        // 12
  void* d_X0 = nullptr;            // 2 M
  void* d_hist = nullptr;          // n_steps x 3
  double* d_acc = nullptr;         // [0] dU0 (boundary), [1] domega, [2] dK, [3] dU0 (initial state), [4..] dX0, dY0
  double* d_acc_w = nullptr;       // per-block partial sums of d/domega (grid adjoint)
  double* d_acc_bc = nullptr;      // per-block partial sums of the inflow's d/dU0 (boundary adjoint)
  double* d_acc_init = nullptr;    // per-block partial sums of d/dU0 through the initial state
  int n_acc_bc = 0;
  int n_accw = 0, n_accw_grid = 0; // all slots; slots of the outside-window launch
  double lo[2] = {0, 0};           // smallest marker x, y (plan precision)
  void* d_op = nullptr;            // MRT operator and its omega derivative (9 x 9 each)
  int wcap[2] = {0, 0};            // extent of the body's stencil window
  int have_ck = 0;
  size_t body_smem = 0;
  int chain_k = 0;  // see BodyArgs::chain_k
};

namespace vs {
namespace adj {

static void free_plan(vs_adjoint_plan* p) {
  if (p->body) vs_body_plan_destroy(p->body);
  if (p->lat) vs_lattice_plan_destroy(p->lat);
  if (p->d_acc_w) cudaFree(p->d_acc_w);
  if (p->d_acc_bc) cudaFree(p->d_acc_bc);
  if (p->d_acc_init) cudaFree(p->d_acc_init);
  if (p->d_op) cudaFree(p->d_op);
  void* bufs[] = {p->d_f0,  p->d_fa,       p->d_fb,     p->d_ck,        p->d_ck_state, p->d_seg[0],
                  p->d_seg[1], p->d_seg_state[0], p->d_seg_state[1], p->d_lam[0], p->d_lam[1], p->d_g,
                  p->d_lu,  p->d_lstate,  p->d_X0,     p->d_hist,      p->d_acc,      p->d_seg_start};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (int k = 0; k < 2; ++k) {
    if (p->g_rec[k]) cudaGraphExecDestroy(p->g_rec[k]);
    if (p->g_rev[k]) cudaGraphExecDestroy(p->g_rev[k]);
    if (p->ev_rec[k]) cudaEventDestroy(p->ev_rec[k]);
    if (p->ev_rev[k]) cudaEventDestroy(p->ev_rev[k]);
  }
  if (p->ev_f) cudaEventDestroy(p->ev_f);
  if (p->ev_b) cudaEventDestroy(p->ev_b);
  if (p->rec) cudaStreamDestroy(p->rec);
  if (p->aux) cudaStreamDestroy(p->aux);
  delete p;
}

template <typename T>
static void host_equilibrium(double U0, int64_t n, std::vector<T>& f) {
  f.resize(9 * n);
  for (int i = 0; i < 9; ++i) {
    const double cx = q9_cx(i);
    const double w = (double)(float)(i == 0 ? 4.0 / 9 : (i <= 4 ? 1.0 / 9 : 1.0 / 36));
    const T uc = (T)(cx * U0), usq = (T)U0 * (T)U0;
    const T v = ((T)1 * (T)w) * ((((T)1 + (T)3 * uc) + (T)4.5 * (uc * uc)) - (T)1.5 * usq);
    for (int64_t p = 0; p < n; ++p) f[i * n + p] = v;
  }
}

__global__ void k_set_int(int* p, int v) { *p = v; }

// Forward recomputation of segment sg into buffer b (states kept), on stream `st`:
// the restore (checkpoint copy, device-side body state) and then `len` fused steps.
template <typename T>
static int recompute_steps(vs_adjoint_plan* P, int b, int len, cudaStream_t st) {
  const int64_t n = P->n;
  T* seg = (T*)P->d_seg[b];
  T* sst = (T*)P->d_seg_state[b];
  void* state_dev = nullptr;
  int rc = vs_body_state_device(P->body, &state_dev);
  if (rc) return rc;
  for (int j = 0; j < len; ++j) {
    cudaError_t e = cudaMemcpyAsync(sst + 12 * j, state_dev, sizeof(T) * 12, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward state copy");
    rc = vs_step(P->lat, P->body, seg + (size_t)j * 9 * n, seg + (size_t)(j + 1) * 9 * n, nullptr, st);
    if (rc) return rc;
  }
  return VS_OK;
}

// Reverse sweep over `len` steps of buffer b (steps seg_start[b] + len-1 .. seg_start[b]),
// starting from adjoint buffer `cur`; returns the final buffer index through *cur.
template <typename T>
static int reverse_steps(vs_adjoint_plan* P, int b, int len, int* cur, cudaStream_t st) {
  const vs_adjoint_cfg& c = P->cfg;
  const int64_t n = P->n;
  const T* seg = (const T*)P->d_seg[b];
  const T* sst = (const T*)P->d_seg_state[b];
  const double k1 = 0.5, k2 = 0.25, c1 = 0.5, c2 = 0.25;  // Newmark beta 1/4, gamma 1/2, dt 1
  const double den = c.mass + c1 * c.damping + c2 * c.stiffness;
  for (int j = len - 1; j >= 0; --j) {
    const T* fj = seg + (size_t)j * 9 * n;
    GridArgs<T> G{};
    G.f = fj;
    G.lam = (T*)P->d_lam[*cur];
    G.lam_out = (T*)P->d_lam[1 - *cur];
    G.g = (T*)P->d_g;
    G.lu = (T*)P->d_lu;
    G.nx = c.nx;
    G.ny = c.ny;
    G.omega = (T)P->omega;
    G.U0 = (T)c.U0;
    G.rho_out = (T)c.rho_out;
    G.acc = P->d_acc;
    G.acc_w = P->d_acc_w;
    G.acc_bc = P->d_acc_bc;
    G.kind = c.collision;
    G.op = (const T*)P->d_op;
    G.dop = (const T*)P->d_op + 81;
    // the boundary adjoint touches the x = 0, nx-2, nx-1 columns only, the body adjoint
    // reads the stencils (kept clear of them): run them side by side
    cudaError_t e = cudaEventRecord(P->ev_f, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(P->aux, P->ev_f, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward fork");
    k_adj_bc<T><<<(c.ny + kRows - 1) / kRows, kRows * 18, 0, P->aux>>>(G);
    BodyArgs<T> B{};
    B.f = fj;
    B.lam = (const T*)P->d_lam[*cur];
    B.g = (T*)P->d_g;
    B.lu = (T*)P->d_lu;
    B.state = sst + 12 * j;
    B.lstate = (T*)P->d_lstate;
    B.X0 = (const T*)P->d_X0;
    B.nx = c.nx;
    B.ny = c.ny;
    B.M = P->M;
    B.kernel = c.kernel;
    B.n_iter = c.n_iter;
    B.ds2 = (T)P->ds * T(2);
    B.wobj = (T)(1.0 / (double)(c.n_steps - c.obj_start));
    B.seg_start = P->d_seg_start + b;
    B.chain_k = P->chain_k;
    B.j = j;
    B.obj_start = c.obj_start;
    B.k1 = (T)k1; B.k2 = (T)k2; B.c1 = (T)c1; B.c2 = (T)c2; B.dt = T(1);
    B.damp = (T)c.damping; B.stiff = (T)c.stiffness; B.den = (T)den; B.area = (T)c.added_mass_area;
    B.free_dof[0] = 0;
    B.free_dof[1] = 1;
    B.dK = P->d_acc + 2;
    B.dX = P->d_acc + 4;
    switch (c.radius) {
      case 1: k_adj_body<T, 1><<<1, kAdjBodyThreads, P->body_smem, st>>>(B); break;
      case 2: k_adj_body<T, 2><<<1, kAdjBodyThreads, P->body_smem, st>>>(B); break;
      default: k_adj_body<T, 2><<<1, kAdjBodyThreads, P->body_smem, st>>>(B); break;
    }
    // window nodes only after the body adjoint: the rest runs beside it (after the boundary
    // adjoint, which it also needs)
    G.wstate = sst + 12 * j;
    G.lo0 = P->lo[0];
    G.lo1 = P->lo[1];
    G.R = c.radius;
    G.cap[0] = P->wcap[0];
    G.cap[1] = P->wcap[1];
    G.mode = 1;
    G.slot0 = 0;
    k_adj_grid<T><<<dim3(grid_for(c.ny, 256), c.nx), 256, 0, P->aux>>>(G);
    e = cudaEventRecord(P->ev_b, P->aux);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, P->ev_b, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward join");
    G.mode = 2;
    G.slot0 = P->n_accw_grid;
    k_adj_grid<T><<<grid_for((int64_t)P->wcap[0] * P->wcap[1], 256), 256, 0, st>>>(G);
    VS_CHECK_LAUNCH("vs_adjoint_backward kernels");
    *cur = 1 - *cur;
  }
  return VS_OK;
}

// Captures fn(stream) into *g once (replayed afterwards).
template <class F>
static int capture(cudaGraphExec_t* g, cudaStream_t st, F&& fn) {
  if (*g) return VS_OK;
  cudaGraph_t gr = nullptr;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_status(e, "vs_adjoint capture");
  const int rc = fn();
  e = cudaStreamEndCapture(st, &gr);
  if (rc) {
    if (gr) cudaGraphDestroy(gr);
    return rc;
  }
  if (e != cudaSuccess) return cuda_status(e, "vs_adjoint end capture");
  e = cudaGraphInstantiate(g, gr, 0);
  cudaGraphDestroy(gr);
  return cuda_status(e, "vs_adjoint instantiate");
}

// Reverse sweep.  Segments are recomputed on P->rec one ahead of the reverse sweep on st
// (double-buffered), so the forward recomputation of segment sg-1 overlaps the adjoint of
// segment sg.  Full segments of an even length replay CUDA graphs.
template <typename T>
static int backward_t(vs_adjoint_plan* P, cudaStream_t st) {
  const vs_adjoint_cfg& c = P->cfg;
  const int64_t n = P->n;
  const int N = c.n_steps, C = P->C;
  const size_t fb = sizeof(T) * 9 * n;
  if (P->g_stream != st) {  // graphs are tied to the stream they were captured for
    for (int k = 0; k < 2; ++k) {
      if (P->g_rec[k]) cudaGraphExecDestroy(P->g_rec[k]);
      if (P->g_rev[k]) cudaGraphExecDestroy(P->g_rev[k]);
      P->g_rec[k] = P->g_rev[k] = nullptr;
    }
    P->g_stream = st;
  }
  cudaError_t e = cudaMemsetAsync(P->d_acc, 0, sizeof(double) * (4 + 2 * P->M), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(P->d_acc_w, 0, sizeof(double) * P->n_accw, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(P->d_acc_bc, 0, sizeof(double) * P->n_acc_bc, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(P->d_lam[0], 0, fb, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(P->d_lstate, 0, sizeof(T) * 12, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(P->d_g, 0, sizeof(T) * 2 * n, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(P->d_lu, 0, sizeof(T) * 2 * n, st);
  if (e == cudaSuccess) e = cudaEventRecord(P->ev_f, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(P->rec, P->ev_f, 0);
  if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward");
  const bool graphs = C % 2 == 0 && st != nullptr;
  bool rev_pending[2] = {false, false};
  auto launch_recompute = [&](int sg) -> int {
    const int b = sg & 1, s0 = sg * C, len = (N - s0) < C ? (N - s0) : C;
    cudaStream_t rs = P->rec;
    cudaError_t e2 = cudaSuccess;
    if (rev_pending[b]) e2 = cudaStreamWaitEvent(rs, P->ev_rev[b], 0);  // buffer b free again
    if (e2 == cudaSuccess)
      e2 = cudaMemcpyAsync(P->d_seg[b], (const char*)P->d_ck + (size_t)sg * fb, fb, cudaMemcpyDeviceToDevice, rs);
    if (e2 != cudaSuccess) return cuda_status(e2, "vs_adjoint_backward restore");
    int rc = vs_body_set_state_device(P->body, (const char*)P->d_ck_state + (size_t)sg * 12 * sizeof(T), rs);
    if (rc) return rc;
    k_set_int<<<1, 1, 0, rs>>>(P->d_seg_start + b, s0);
    if (graphs && len == C) {
      rc = capture(&P->g_rec[b], rs, [&]() { return recompute_steps<T>(P, b, C, rs); });
      if (rc) return rc;
      e2 = cudaGraphLaunch(P->g_rec[b], rs);
      if (e2 != cudaSuccess) return cuda_status(e2, "vs_adjoint_backward recompute graph");
    } else {
      rc = recompute_steps<T>(P, b, len, rs);
      if (rc) return rc;
    }
    e2 = cudaEventRecord(P->ev_rec[b], rs);
    return e2 == cudaSuccess ? VS_OK : cuda_status(e2, "vs_adjoint_backward event");
  };
  int rc = launch_recompute(P->n_ck - 1);
  if (rc) return rc;
  int cur = 0;
  for (int sg = P->n_ck - 1; sg >= 0; --sg) {
    const int b = sg & 1, s0 = sg * C, len = (N - s0) < C ? (N - s0) : C;
    e = cudaStreamWaitEvent(st, P->ev_rec[b], 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward wait");
    if (sg > 0) {
      rc = launch_recompute(sg - 1);  // overlaps the reverse sweep below
      if (rc) return rc;
    }
    if (graphs && len == C && cur == 0) {
      rc = capture(&P->g_rev[b], st, [&]() {
        int cc = 0;
        return reverse_steps<T>(P, b, C, &cc, st);
      });
      if (rc) return rc;
      e = cudaGraphLaunch(P->g_rev[b], st);
      if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward reverse graph");
    } else {
      rc = reverse_steps<T>(P, b, len, &cur, st);
      if (rc) return rc;
    }
    e = cudaEventRecord(P->ev_rev[b], st);
    if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward event");
    rev_pending[b] = true;
  }
  k_adj_initial<T><<<256, 256, 0, st>>>((const T*)P->d_lam[cur], n, (T)c.U0, P->d_acc_init);
  VS_CHECK_LAUNCH("vs_adjoint_backward initial state");
  return VS_OK;
}

}  // namespace adj
}  // namespace vs

using namespace vs;
using namespace vs::adj;

extern "C" {

int vs_adjoint_plan_create(const vs_adjoint_cfg* cfg, vs_adjoint_plan** out) {
  VS_REQUIRE(cfg && out, "vs_adjoint_plan_create: null argument");
  VS_REQUIRE(cfg->dtype == VS_F32 || cfg->dtype == VS_F64, "vs_adjoint_plan_create: bad dtype");
  VS_REQUIRE(cfg->nx >= 16 && cfg->ny >= 16, "vs_adjoint_plan_create: grid too small");
  VS_REQUIRE(cfg->n_markers >= 3 && cfg->offsets_host, "vs_adjoint_plan_create: markers and offsets needed");
  VS_REQUIRE(cfg->n_steps >= 1 && cfg->checkpoint_every >= 1, "vs_adjoint_plan_create: steps / checkpoints");
  VS_REQUIRE(cfg->obj_start >= 0 && cfg->obj_start < cfg->n_steps, "vs_adjoint_plan_create: objective window");
  VS_REQUIRE(cfg->radius >= 1 && cfg->radius <= 2, "vs_adjoint_plan_create: radius 1 or 2");
  VS_REQUIRE(cfg->U0 > 0 && cfg->D > 0 && cfg->Re > 0, "vs_adjoint_plan_create: U0, D, Re must be positive");
  VS_REQUIRE(cfg->collision >= VS_COLLIDE_BGK && cfg->collision <= VS_COLLIDE_REG,
             "vs_adjoint_plan_create: bad collision %d", cfg->collision);
  vs_adjoint_plan* P = new (std::nothrow) vs_adjoint_plan();
  if (!P) {
    set_error("out of host memory");
    return VS_ERR_INVALID_ARG;
  }
  P->cfg = *cfg;
  P->cfg.offsets_host = nullptr;
  P->n = (int64_t)cfg->nx * cfg->ny;
  P->M = cfg->n_markers;
  P->S = 4 * cfg->radius * cfg->radius;
  P->C = cfg->checkpoint_every;
  P->n_ck = (cfg->n_steps + P->C - 1) / P->C;
  P->ts = cfg->dtype == VS_F64 ? 8 : 4;
  const double nu = cfg->U0 * cfg->D / cfg->Re;
  P->omega = 1.0 / (3.0 * nu + 0.5);
  P->ds = M_PI * cfg->D / cfg->n_markers;
  auto fail = [&](int rc) {
    free_plan(P);
    return rc;
  };
  // markers on the circle, radius D/2 + offset
  const int M = P->M;
  std::vector<double> X(M), Y(M);
  P->theta.resize(M);
  double rmax = 0;
  for (int m = 0; m < M; ++m) {
    P->theta[m] = 2 * M_PI * m / M;
    const double r = 0.5 * cfg->D + cfg->offsets_host[m];
    rmax = r > rmax ? r : rmax;
    X[m] = cfg->cx + r * cos(P->theta[m]);
    Y[m] = cfg->cy + r * sin(P->theta[m]);
  }
  {
    // cyclic index distance bound between markers that can share a stencil node under a
    // translation (|dx| < 2R and |dy| < 2R); 0 when it does not pay
    const double lim = 2.0 * cfg->radius + 1e-3;
    int K = 0;
    for (int i = 0; i < M; ++i)
      for (int j = i + 1; j < M; ++j)
        if (fabs(X[i] - X[j]) < lim && fabs(Y[i] - Y[j]) < lim) {
          const int dd = j - i, cyc = dd < M - dd ? dd : M - dd;
          K = cyc > K ? cyc : K;
        }
    P->chain_k = 2 * K + 1 < M ? K : 0;
  }
  if (cfg->cx - rmax - cfg->radius - 2 < 4 || cfg->cx + rmax + cfg->radius + 2 > cfg->nx - 5) {
    set_error("vs_adjoint_plan_create: the body's stencils must stay clear of the x = 0 / nx-1 boundaries");
    return fail(VS_ERR_INVALID_ARG);
  }
  // the forward step: fused lattice + body plans
  vs_lattice_cfg lc;
  memset(&lc, 0, sizeof(lc));
  lc.q = 9;
  lc.dtype = cfg->dtype;
  lc.nx = cfg->nx;
  lc.ny = cfg->ny;
  lc.nz = 1;
  lc.collision = cfg->collision;
  if (cfg->collision == VS_COLLIDE_MRT)
    for (int i = 0; i < 81; ++i) lc.mrt_op[i] = cfg->mrt_op[i];
  lc.omega = P->omega;
  lc.forcing = VS_FORCE_EDM;
  lc.n_bc = 2;
  lc.bc[0].kind = VS_BC_EQ;
  lc.bc[0].mode = VS_WALL_GIVEN;
  lc.bc[0].loc = VS_LEFT;
  lc.bc[0].rho = 1.0;
  lc.bc[0].ux = cfg->U0;
  lc.bc[1].kind = VS_BC_NEE;
  lc.bc[1].mode = VS_WALL_PRESSURE;
  lc.bc[1].loc = VS_RIGHT;
  lc.bc[1].rho = cfg->rho_out;
  lc.variant = VS_GRID_PLAIN;
  int rc = vs_lattice_plan_create(&lc, &P->lat);
  if (rc) return fail(rc);
  vs_body_cfg bc;
  memset(&bc, 0, sizeof(bc));
  bc.dim = 2;
  bc.dtype = cfg->dtype;
  bc.n_markers = M;
  bc.x0_host = X.data();
  bc.y0_host = Y.data();
  bc.ds_scalar = P->ds;
  bc.kernel = cfg->kernel;
  bc.radius = cfg->radius;
  bc.n_iter = cfg->n_iter;
  bc.moving = 1;
  bc.free_dof[1] = 1;
  bc.mass = cfg->mass;
  bc.stiffness = cfg->stiffness;
  bc.damping = cfg->damping;
  bc.added_mass_area = cfg->added_mass_area;
  rc = vs_body_plan_create(&bc, P->lat, &P->body);
  if (rc) return fail(rc);
  const size_t ts = P->ts, fbytes = ts * 9 * P->n;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  alloc(&P->d_f0, fbytes);
  alloc(&P->d_fa, fbytes);
  alloc(&P->d_fb, fbytes);
  alloc(&P->d_ck, fbytes * P->n_ck);
  alloc(&P->d_ck_state, ts * 12 * P->n_ck);
  for (int k = 0; k < 2; ++k) {
    alloc(&P->d_seg[k], fbytes * (P->C + 1));
    alloc(&P->d_seg_state[k], ts * 12 * (P->C + 1));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->ev_rec[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->ev_rev[k], cudaEventDisableTiming);
  }
  alloc((void**)&P->d_seg_start, sizeof(int) * 2);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->rec, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->aux, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->ev_f, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->ev_b, cudaEventDisableTiming);
  alloc(&P->d_lam[0], fbytes);
  alloc(&P->d_lam[1], fbytes);
  alloc(&P->d_g, ts * 2 * P->n);
  alloc(&P->d_lu, ts * 2 * P->n);
  alloc(&P->d_lstate, ts * 12);
  alloc(&P->d_X0, ts * 2 * M);
  alloc(&P->d_hist, ts * 3 * cfg->n_steps);
  alloc((void**)&P->d_acc, sizeof(double) * (4 + 2 * M));
  alloc(&P->d_op, ts * 162);
  {
    double lx = 1e300, ly = 1e300, hx = -1e300, hy = -1e300;
    for (int m = 0; m < M; ++m) {
      lx = X[m] < lx ? X[m] : lx;
      ly = Y[m] < ly ? Y[m] : ly;
      hx = X[m] > hx ? X[m] : hx;
      hy = Y[m] > hy ? Y[m] : hy;
    }
    const bool f32 = cfg->dtype == VS_F32;
    P->lo[0] = f32 ? (double)(float)lx : lx;
    P->lo[1] = f32 ? (double)(float)ly : ly;
    // floor(hi + d) - floor(lo + d) <= floor(hi) - floor(lo) + 1, plus the stencil width
    P->wcap[0] = (int)(floor(hx) - floor(lx)) + 2 * cfg->radius + 1;
    P->wcap[1] = (int)(floor(hy) - floor(ly)) + 2 * cfg->radius + 1;
  }
  P->n_accw_grid = (int)grid_for(cfg->ny, 256) * cfg->nx;
  P->n_accw = P->n_accw_grid + (int)grid_for((int64_t)P->wcap[0] * P->wcap[1], 256);
  alloc((void**)&P->d_acc_w, sizeof(double) * P->n_accw);
  P->n_acc_bc = (cfg->ny + kRows - 1) / kRows;
  alloc((void**)&P->d_acc_bc, sizeof(double) * P->n_acc_bc);
  alloc((void**)&P->d_acc_init, sizeof(double) * 256);
  if (e != cudaSuccess) return fail(cuda_status(e, "vs_adjoint_plan_create"));
  rc = dispatch_t(cfg->dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    std::vector<T> f0, x0(2 * M);
    host_equilibrium<T>(cfg->U0, P->n, f0);
    for (int m = 0; m < M; ++m) {
      x0[m] = (T)X[m];
      x0[M + m] = (T)Y[m];
    }
    std::vector<T> ops(162);
    for (int i = 0; i < 81; ++i) {
      ops[i] = (T)cfg->mrt_op[i];
      ops[81 + i] = (T)cfg->mrt_dop[i];
    }
    cudaError_t e2 = cudaMemcpy(P->d_f0, f0.data(), fbytes, cudaMemcpyHostToDevice);
    if (e2 == cudaSuccess) e2 = cudaMemcpy(P->d_op, ops.data(), ts * 162, cudaMemcpyHostToDevice);
    if (e2 == cudaSuccess) e2 = cudaMemcpy(P->d_X0, x0.data(), ts * 2 * M, cudaMemcpyHostToDevice);
    if (e2 != cudaSuccess) return cuda_status(e2, "vs_adjoint_plan_create upload");
    P->body_smem = adj_body_smem<T>(M, cfg->radius, cfg->n_iter);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if ((int64_t)P->body_smem > optin) {
      set_error("vs_adjoint_plan_create: %d markers need %zu bytes of shared memory", M, P->body_smem);
      return VS_ERR_UNSUPPORTED;
    }
    switch (cfg->radius) {
      case 1: e2 = cudaFuncSetAttribute(k_adj_body<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin); break;
      case 2: e2 = cudaFuncSetAttribute(k_adj_body<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin); break;
      default: e2 = cudaFuncSetAttribute(k_adj_body<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin); break;
    }
    return cuda_status(e2, "vs_adjoint_plan_create attribute");
  });
  if (rc) return fail(rc);
  *out = P;
  return VS_OK;
}

int vs_adjoint_plan_destroy(vs_adjoint_plan* plan) {
  if (plan) free_plan(plan);
  return VS_OK;
}

int vs_adjoint_forward(vs_adjoint_plan* P, int keep_checkpoints, double* J_out, void* stream) {
  VS_REQUIRE(P, "vs_adjoint_forward: null plan");
  cudaStream_t st = as_stream(stream);
  const vs_adjoint_cfg& c = P->cfg;
  const size_t ts = P->ts, fbytes = ts * 9 * P->n;
  double zero[12] = {0};
  int rc = vs_body_set_state(P->body, zero, stream);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(P->d_fa, P->d_f0, fbytes, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_forward");
  void* state_dev = nullptr;
  rc = vs_body_state_device(P->body, &state_dev);
  if (rc) return rc;
  void* fa = P->d_fa;
  void* fbuf = P->d_fb;
  for (int s = 0, k = 0; s < c.n_steps; s += P->C, ++k) {
    const int len = (c.n_steps - s) < P->C ? (c.n_steps - s) : P->C;
    if (keep_checkpoints) {
      e = cudaMemcpyAsync((char*)P->d_ck + (size_t)k * fbytes, fa, fbytes, cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync((char*)P->d_ck_state + (size_t)k * 12 * ts, state_dev, 12 * ts, cudaMemcpyDeviceToDevice,
                            st);
      if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_forward checkpoint");
    }
    rc = vs_run(P->lat, P->body, fa, fbuf, len, (char*)P->d_hist + (size_t)s * 3 * ts, stream);
    if (rc) return rc;
    if (len % 2 == 1) {
      void* t = fa;
      fa = fbuf;
      fbuf = t;
    }
  }
  std::vector<unsigned char> h(ts * 3 * c.n_steps);
  e = cudaMemcpyAsync(h.data(), P->d_hist, h.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_forward history");
  double J = 0;
  for (int s = c.obj_start; s < c.n_steps; ++s)
    J += ts == 8 ? ((double*)h.data())[3 * s] : (double)((float*)h.data())[3 * s];
  J /= (double)(c.n_steps - c.obj_start);
  if (J_out) *J_out = J;
  P->have_ck = keep_checkpoints ? 1 : 0;
  double st_h[12];
  return vs_body_get_state(P->body, st_h, stream);  // surfaces a body that left its window
}

int vs_adjoint_backward(vs_adjoint_plan* P, double seed, double* grad_U0, double* grad_K, double* grad_offsets,
                        void* stream) {
  VS_REQUIRE(P, "vs_adjoint_backward: null plan");
  VS_REQUIRE(P->have_ck, "vs_adjoint_backward: run vs_adjoint_forward with keep_checkpoints first");
  cudaStream_t st = as_stream(stream);
  const int rc = dispatch_t(P->cfg.dtype, [&](auto t) -> int {
    return backward_t<typename decltype(t)::type>(P, st);
  });
  if (rc) return rc;
  const int M = P->M;
  std::vector<double> acc(4 + 2 * M), accw(P->n_accw), accbc(P->n_acc_bc), accinit(256);
  cudaError_t e = cudaMemcpyAsync(acc.data(), P->d_acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(accw.data(), P->d_acc_w, sizeof(double) * accw.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(accbc.data(), P->d_acc_bc, sizeof(double) * accbc.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(accinit.data(), P->d_acc_init, sizeof(double) * 256, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "vs_adjoint_backward result");
  // block partials summed in a fixed order: the gradients are the same bits run to run
  for (double v : accw) acc[1] += v;      // d/domega
  for (double v : accbc) acc[0] += v;     // d/dU0 through the inflow boundary
  for (double v : accinit) acc[3] += v;   // d/dU0 through the initial state
  const vs_adjoint_cfg& c = P->cfg;
  const double domega = -3.0 * (c.D / c.Re) * P->omega * P->omega;
  if (grad_U0) *grad_U0 = seed * (acc[0] + acc[3] + acc[1] * domega);
  if (grad_K) *grad_K = seed * acc[2];
  if (grad_offsets)
    for (int m = 0; m < M; ++m)
      grad_offsets[m] = seed * (acc[4 + m] * cos(P->theta[m]) + acc[4 + M + m] * sin(P->theta[m]));
  double st_h[12];
  return vs_body_get_state(P->body, st_h, stream);
}

}  // extern "C"
