// Per-operator LBM kernels: one entry point per pure function of vivsim.lbm / vivsim.lbm3d.
// These are the drop-in replacements for the individual reference functions; the fused
// time step lives in vs_step.cu.
#include <math.h>

#include "vs_boundary.cuh"
#include "vs_dispatch.cuh"

namespace vs {

// ------------------------------------------------------------------ pointwise kernels
template <class L, typename T>
__global__ void k_macro(const T* __restrict__ f, T* __restrict__ rho, T* __restrict__ u, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    T fl[L::Q];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) fl[i] = f[i * n + p];
    T r, uu[3];
    macro(L{}, fl, r, uu);
    rho[p] = r;
#pragma unroll
    for (int d = 0; d < L::D; ++d) u[d * n + p] = uu[d];
  }
}

template <class L, typename T>
__global__ void k_equilibrium(const T* __restrict__ rho, const T* __restrict__ u, T* __restrict__ feq, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    T uu[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int d = 0; d < L::D; ++d) uu[d] = u[d * n + p];
    const T r = rho[p];
    const T usq = usq_of(L{}, uu);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) feq[i * n + p] = feq_i(L{}, i, r, uu, usq);
  }
}

template <class L, typename T>
struct OpMatrix {
  T m[L::Q * L::Q];
};

template <class L, typename T>
__global__ void k_collision(int kind, const T* __restrict__ f, const T* __restrict__ feq, CollideParams<T> cp,
                            OpMatrix<L, T> op, T* __restrict__ out, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    T fl[L::Q], fe[L::Q];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      fl[i] = f[i * n + p];
      fe[i] = feq[i * n + p];
    }
    if (kind == VS_COLLIDE_MRT)
      collide_mrt<L>(fl, fe, op.m);
    else
      collide<L>(kind, fl, fe, cp);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) out[i * n + p] = fl[i];
  }
}

// mode 0: guo term only; 1: f + scale * guo; 2: f + op guo
template <class L, typename T>
__global__ void k_forcing(int mode, const T* __restrict__ f, const T* __restrict__ g, const T* __restrict__ u,
                          T scale, OpMatrix<L, T> op, T* __restrict__ out, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    T uu[3] = {T(0), T(0), T(0)}, gg[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int d = 0; d < L::D; ++d) {
      uu[d] = u[d * n + p];
      gg[d] = g[d * n + p];
    }
    T gl[L::Q];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) gl[i] = guo_i(L{}, i, gg, uu);
    if (mode == 0) {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) out[i * n + p] = gl[i];
    } else if (mode == 1) {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) out[i * n + p] = f[i * n + p] + (scale == T(1) ? gl[i] : gl[i] * scale);
    } else {
#pragma unroll
      for (int i = 0; i < L::Q; ++i) {
        T acc = op.m[i * L::Q] * gl[0];
#pragma unroll
        for (int j = 1; j < L::Q; ++j) acc = acc + op.m[i * L::Q + j] * gl[j];
        out[i * n + p] = f[i * n + p] + acc;
      }
    }
  }
}

template <typename T>
__global__ void k_velocity_correction(int dim, const T* __restrict__ g, const T* __restrict__ rho, T* __restrict__ out,
                                      int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    for (int d = 0; d < dim; ++d) out[d * n + p] = (g[d * n + p] * T(0.5)) / rho[p];
}

// ------------------------------------------------------------------ streaming
// out_i(x) = f_i(x - c_i) with periodic wrap on every axis (lbm/basic.py:60-85).
template <class L, typename T>
__global__ void k_streaming(const T* __restrict__ f, T* __restrict__ out, int nx, int ny, int nz) {
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(p % nz);
    const int y = (int)((p / nz) % ny);
    const int x = (int)(p / ((int64_t)nz * ny));
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      int xs = x - L::c(i, 0), ys = y - L::c(i, 1), zs = z - L::c(i, 2);
      xs += xs < 0 ? nx : (xs >= nx ? -nx : 0);
      ys += ys < 0 ? ny : (ys >= ny ? -ny : 0);
      zs += zs < 0 ? nz : (zs >= nz ? -nz : 0);
      out[i * n + p] = f[i * n + ((int64_t)xs * ny + ys) * nz + zs];
    }
  }
}

// ------------------------------------------------------------------ boundaries
template <class L, typename T>
__global__ void k_boundary(WallArgs<T> A, const T* __restrict__ fin, T* fout) {
  const int64_t n = (int64_t)A.n[0] * A.n[1] * A.n[2];
  const int64_t nf = face_size(A.loc, A.n);
  const bool need_nb = bc_needs_neighbor<L>(A.kind, A.mode);
  const bool need_pre = A.kind == VS_BC_BB || A.kind == VS_BC_SPECULAR;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nf; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pw = face_node(A.loc, A.n, j, 0);
    T w[L::Q], nb[L::Q], pre[L::Q], out[L::Q];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) w[i] = fin[i * n + pw];
    if (need_nb) {
      const int64_t pn = face_node(A.loc, A.n, j, 1);
#pragma unroll
      for (int i = 0; i < L::Q; ++i) nb[i] = fin[i * n + pn];
    }
    if (need_pre) {
      const int64_t pp = A.pre_face ? j : pw;
#pragma unroll
      for (int i = 0; i < L::Q; ++i) pre[i] = A.f_pre[i * A.pre_stride + pp];
    }
    bc_node<L, T>(A, j, w, nb, pre, out);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) fout[i * n + pw] = out[i];
  }
}

template <class L, typename T>
__global__ void k_obstacle_bb(const T* __restrict__ fin, T* __restrict__ fout, const uint8_t* __restrict__ mask,
                              int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const bool m = mask[p] != 0;
    T v[L::Q];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) v[i] = fin[i * n + p];
#pragma unroll
    for (int i = 0; i < L::Q; ++i) fout[i * n + p] = m ? v[L::opp(i)] : v[i];
  }
}

// Non-reflective characteristic update of (rho, u) on a face (lbm/boundary/cbc.py:14-53,
// lbm3d/boundary/cbc.py:16-51).
template <typename T>
__global__ void k_characteristic(int dim, int loc, const T* __restrict__ rho, const T* __restrict__ u, int nx, int ny,
                                 int nz, T* __restrict__ rho_next, T* __restrict__ u_next) {
  const int nn[3] = {nx, ny, nz};
  const int64_t n = (int64_t)nx * ny * nz;
  const int64_t nf = face_size(loc, nn);
  const int a = loc_axis(loc), sg = loc_sign(loc);
  const T cs = cbc_cs<T>(dim);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nf; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p0 = face_node(loc, nn, j, 0), p1 = face_node(loc, nn, j, 1), p2 = face_node(loc, nn, j, 2);
    T rn, un;
    cbc_values<T>(sg, cs, rho[p0], rho[p1], rho[p2], u[a * n + p0], u[a * n + p1], u[a * n + p2], rn, un);
    rho_next[j] = rn;
    for (int d = 0; d < dim; ++d) u_next[d * nf + j] = d == a ? un : u[d * n + p0];
  }
}

// ------------------------------------------------------------------ host helpers
template <class L, typename T>
OpMatrix<L, T> op_from_host(const double* h) {
  OpMatrix<L, T> m;
  for (int i = 0; i < L::Q * L::Q; ++i) m.m[i] = h ? (T)h[i] : T(0);
  return m;
}

template <typename T>
CollideParams<T> collide_params(double omega) {
  CollideParams<T> p;
  p.omega = (T)omega;
  p.one_m_omega = (T)(1.0 - omega);
  p.inv_omega = (T)(1.0 / omega);
  p.one_m_inv = (T)(1.0 - 1.0 / omega);
  p.mrt = nullptr;
  return p;
}

static const int kBlock = 256;

}  // namespace vs

using namespace vs;

extern "C" {

int vs_streaming(int q, int dtype, const void* f, void* out, int nx, int ny, int nz, void* stream) {
  VS_REQUIRE(f && out && f != out, "vs_streaming: f and out must be distinct device pointers");
  VS_REQUIRE(nx > 0 && ny > 0 && nz > 0 && (q == 19 || nz == 1), "vs_streaming: bad grid %d x %d x %d", nx, ny, nz);
  const int64_t n = (int64_t)nx * ny * nz;
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_streaming<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>((const T*)f, (T*)out, nx, ny, nz);
    VS_CHECK_LAUNCH("vs_streaming");
    return VS_OK;
  });
}

int vs_get_macroscopic(int q, int dtype, const void* f, void* rho, void* u, int64_t n, void* stream) {
  VS_REQUIRE(f && rho && u && n > 0, "vs_get_macroscopic: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_macro<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>((const T*)f, (T*)rho, (T*)u, n);
    VS_CHECK_LAUNCH("vs_get_macroscopic");
    return VS_OK;
  });
}

int vs_get_equilibrium(int q, int dtype, const void* rho, const void* u, void* feq, int64_t n, void* stream) {
  VS_REQUIRE(rho && u && feq && n > 0, "vs_get_equilibrium: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_equilibrium<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>((const T*)rho, (const T*)u, (T*)feq, n);
    VS_CHECK_LAUNCH("vs_get_equilibrium");
    return VS_OK;
  });
}

int vs_collision(int q, int dtype, int kind, const void* f, const void* feq, double omega, void* out, int64_t n,
                 void* stream) {
  VS_REQUIRE(f && feq && out && n > 0, "vs_collision: bad arguments");
  VS_REQUIRE(kind == VS_COLLIDE_BGK || kind == VS_COLLIDE_KBC || kind == VS_COLLIDE_REG,
             "vs_collision: kind must be BGK, KBC or REG (use vs_collision_mrt for MRT)");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_collision<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>(
        kind, (const T*)f, (const T*)feq, collide_params<T>(omega), op_from_host<L, T>(nullptr), (T*)out, n);
    VS_CHECK_LAUNCH("vs_collision");
    return VS_OK;
  });
}

int vs_collision_mrt(int q, int dtype, const void* f, const void* feq, const double* op_host, void* out, int64_t n,
                     void* stream) {
  VS_REQUIRE(f && feq && out && op_host && n > 0, "vs_collision_mrt: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_collision<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>(
        VS_COLLIDE_MRT, (const T*)f, (const T*)feq, collide_params<T>(1.0), op_from_host<L, T>(op_host), (T*)out, n);
    VS_CHECK_LAUNCH("vs_collision_mrt");
    return VS_OK;
  });
}

int vs_guo_forcing_term(int q, int dtype, const void* g, const void* u, void* out, int64_t n, void* stream) {
  VS_REQUIRE(g && u && out && n > 0, "vs_guo_forcing_term: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_forcing<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>(
        0, nullptr, (const T*)g, (const T*)u, T(1), op_from_host<L, T>(nullptr), (T*)out, n);
    VS_CHECK_LAUNCH("vs_guo_forcing_term");
    return VS_OK;
  });
}

int vs_forcing(int q, int dtype, int kind, const void* f, const void* g, const void* u, double omega, void* out,
               int64_t n, void* stream) {
  VS_REQUIRE(f && g && u && out && n > 0, "vs_forcing: bad arguments");
  VS_REQUIRE(kind == VS_FORCE_EDM || kind == VS_FORCE_GUO_BGK, "vs_forcing: kind must be EDM or GUO_BGK");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    const T scale = kind == VS_FORCE_EDM ? T(1) : (T)(1.0 - 0.5 * omega);
    k_forcing<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>(
        1, (const T*)f, (const T*)g, (const T*)u, scale, op_from_host<L, T>(nullptr), (T*)out, n);
    VS_CHECK_LAUNCH("vs_forcing");
    return VS_OK;
  });
}

int vs_forcing_guo_mrt(int q, int dtype, const void* f, const void* g, const void* u, const double* op_host, void* out,
                       int64_t n, void* stream) {
  VS_REQUIRE(f && g && u && out && op_host && n > 0, "vs_forcing_guo_mrt: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_forcing<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>(
        2, (const T*)f, (const T*)g, (const T*)u, T(1), op_from_host<L, T>(op_host), (T*)out, n);
    VS_CHECK_LAUNCH("vs_forcing_guo_mrt");
    return VS_OK;
  });
}

int vs_velocity_correction(int q, int dtype, const void* g, const void* rho, void* out, int64_t n, void* stream) {
  VS_REQUIRE(g && rho && out && n > 0, "vs_velocity_correction: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_velocity_correction<T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>(L::D, (const T*)g, (const T*)rho,
                                                                                     (T*)out, n);
    VS_CHECK_LAUNCH("vs_velocity_correction");
    return VS_OK;
  });
}

int vs_boundary(int q, int dtype, int kind, int mode, int loc, const void* f_in, void* f_out,
                const void* f_before_stream, int nx, int ny, int nz, const vs_wall* wall, void* stream) {
  VS_REQUIRE(f_in && f_out && wall, "vs_boundary: null argument");
  VS_REQUIRE(kind >= VS_BC_NEE && kind <= VS_BC_SPECULAR, "vs_boundary: bad kind %d", kind);
  VS_REQUIRE(mode >= VS_WALL_GIVEN && mode <= VS_WALL_FORCE_CORRECTED, "vs_boundary: bad mode %d", mode);
  VS_REQUIRE(!((kind == VS_BC_BB || kind == VS_BC_SPECULAR) && mode != VS_WALL_GIVEN),
             "vs_boundary: bounce-back has no velocity/pressure/force-corrected form");
  VS_REQUIRE(!((kind == VS_BC_BB || kind == VS_BC_SPECULAR) && !f_before_stream),
             "vs_boundary: bounce-back needs f_before_stream");
  const int dim = q == 9 ? 2 : 3;
  VS_REQUIRE(loc >= 0 && loc < 2 * dim, "vs_boundary: loc %d invalid for D%dQ%d", loc, dim, q);
  const int nn[3] = {nx, ny, q == 9 ? 1 : nz};
  VS_REQUIRE(nx >= 3 && ny >= 3 && (q == 9 || nz >= 3), "vs_boundary: grid too small");
  const int64_t n = (int64_t)nn[0] * nn[1] * nn[2];
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    cudaStream_t s = as_stream(stream);
    if (f_out != f_in) {
      cudaError_t e = cudaMemcpyAsync(f_out, f_in, sizeof(T) * L::Q * n, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return cuda_status(e, "vs_boundary copy");
    }
    WallArgs<T> A{};
    A.kind = kind;
    A.mode = mode;
    A.loc = loc;
    for (int d = 0; d < 3; ++d) A.n[d] = nn[d];
    double rho = wall->rho, u3[3] = {wall->ux, wall->uy, wall->uz};
    if (mode == VS_WALL_FORCE_CORRECTED) {
      const double g3[3] = {wall->gx, wall->gy, wall->gz};
      for (int d = 0; d < 3; ++d) u3[d] = u3[d] - (g3[d] * 0.5) / rho;
    }
    A.un_scalar = mode != VS_WALL_PRESSURE;
    A.all_scalar = mode == VS_WALL_GIVEN || mode == VS_WALL_FORCE_CORRECTED;
    wall_args_scalars(A, rho, u3, dim);
    A.rho_arr = (const T*)wall->rho_arr;
    A.u_arr[0] = (const T*)wall->ux_arr;
    A.u_arr[1] = (const T*)wall->uy_arr;
    A.u_arr[2] = q == 9 ? nullptr : (const T*)wall->uz_arr;
    A.f_pre = (const T*)f_before_stream;
    A.pre_stride = n;
    A.pre_face = 0;
    const int64_t nf = face_size(loc, nn);
    k_boundary<L, T><<<grid_for(nf, 128), 128, 0, s>>>(A, (const T*)f_in, (T*)f_out);
    VS_CHECK_LAUNCH("vs_boundary");
    return VS_OK;
  });
}

int vs_obstacle_bounce_back(int q, int dtype, const void* f_in, void* f_out, const uint8_t* mask, int64_t n,
                            void* stream) {
  VS_REQUIRE(f_in && f_out && mask && n > 0, "vs_obstacle_bounce_back: bad arguments");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_obstacle_bb<L, T><<<grid_for(n, kBlock), kBlock, 0, as_stream(stream)>>>((const T*)f_in, (T*)f_out, mask, n);
    VS_CHECK_LAUNCH("vs_obstacle_bounce_back");
    return VS_OK;
  });
}

int vs_boundary_characteristic(int q, int dtype, int loc, const void* rho, const void* u, int nx, int ny, int nz,
                               void* rho_next, void* u_next, void* stream) {
  VS_REQUIRE(rho && u && rho_next && u_next, "vs_boundary_characteristic: null argument");
  const int dim = q == 9 ? 2 : 3;
  VS_REQUIRE(loc >= 0 && loc < 2 * dim, "loc must be one of: %s",
             dim == 2 ? "'left', 'right', 'top', 'bottom'" : "'left', 'right', 'bottom', 'top', 'back', 'front'");
  const int nn[3] = {nx, ny, q == 9 ? 1 : nz};
  VS_REQUIRE(nn[loc_axis(loc)] >= 3, "vs_boundary_characteristic: need 3 nodes along the normal");
  return dispatch(q, dtype, [&](auto l, auto t) -> int {
    using T = typename decltype(t)::type;
    const int64_t nf = face_size(loc, nn);
    k_characteristic<T><<<grid_for(nf, 128), 128, 0, as_stream(stream)>>>(dim, loc, (const T*)rho, (const T*)u, nn[0],
                                                                          nn[1], nn[2], (T*)rho_next, (T*)u_next);
    VS_CHECK_LAUNCH("vs_boundary_characteristic");
    return VS_OK;
  });
}

}  // extern "C"
