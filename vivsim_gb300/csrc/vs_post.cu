// Flow diagnostics of vivsim/post.py on the device: velocity gradient, vorticity,
// divergence, strain rate, kinetic energy, enstrophy, Q-criterion.
//
// Derivatives follow jnp.gradient (edge_order 1, unit spacing): central differences
// (u[i+1] - u[i-1]) / 2 inside, one-sided u[1] - u[0] and u[n-1] - u[n-2] at the two ends
// of every axis (no periodic wrap).  One thread per node evaluates the whole velocity
// gradient from its neighbours (read from u, or computed from the populations f when
// from_f is set, which saves the separate get_macroscopic pass) and writes the requested
// field.  The domain means reduce per block in a fixed order and add the block sums to a
// double accumulator.
#include <type_traits>

#include "vs_dispatch.cuh"

namespace vs {
namespace post {

template <typename T, int D>
struct Ctx {
  const T* u;  // (D, n) velocity, or null
  const T* f;  // (Q, n) populations, or null
  int n[3];
  int64_t nn;
};

// velocity vector at node (x, y, z): read from u, or from the populations (get_macroscopic)
template <typename T, int D>
__device__ __forceinline__ void vel(const Ctx<T, D>& C, int x, int y, int z, T* out) {
  const int64_t p = ((int64_t)x * C.n[1] + y) * C.n[2] + z;
  if (C.u) {
#pragma unroll
    for (int c = 0; c < D; ++c) out[c] = C.u[c * C.nn + p];
    return;
  }
  constexpr int Q = D == 2 ? 9 : 19;
  using L = typename std::conditional<D == 2, L9, L19>::type;
  T fl[Q], r, uu[3] = {T(0), T(0), T(0)};
#pragma unroll
  for (int i = 0; i < Q; ++i) fl[i] = __ldg(C.f + i * C.nn + p);
  macro(L{}, fl, r, uu);
#pragma unroll
  for (int c = 0; c < D; ++c) out[c] = uu[c];
}

template <typename T, int D>
__global__ void __launch_bounds__(256) k_post(Ctx<T, D> C, int what, T* __restrict__ out, double* acc) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double contrib = 0.0;
  if (p < C.nn) {
    const int z = D == 3 ? (int)(p % C.n[2]) : 0;
    const int y = (int)((p / C.n[2]) % C.n[1]);
    const int x = (int)(p / ((int64_t)C.n[1] * C.n[2]));
    T u[3] = {T(0), T(0), T(0)};
    T G[3][3];
    const bool need_grad = what != VS_POST_VELOCITY_MAGNITUDE && what != VS_POST_KINETIC_ENERGY &&
                           what != VS_POST_MEAN_KINETIC_ENERGY;
    if (!need_grad) {
      vel<T, D>(C, x, y, z, u);
    } else {
      // G[i][a] = d u_i / d x_a as jnp.gradient: (u[+1] - u[-1]) / 2 inside, one-sided at the ends
      const int co[3] = {x, y, z};
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const int i = co[a], N = C.n[a];
        if (N < 2) {
#pragma unroll
          for (int c = 0; c < D; ++c) G[c][a] = T(0);
          continue;
        }
        const int lo = i == 0 ? 0 : (i == N - 1 ? N - 2 : i - 1);
        const int hi = i == 0 ? 1 : (i == N - 1 ? N - 1 : i + 1);
        int cl[3] = {x, y, z}, ch[3] = {x, y, z};
        cl[a] = lo;
        ch[a] = hi;
        T uL[3], uR[3];
        vel<T, D>(C, cl[0], cl[1], cl[2], uL);
        vel<T, D>(C, ch[0], ch[1], ch[2], uR);
        const bool inner = i > 0 && i < N - 1;
#pragma unroll
        for (int c = 0; c < D; ++c) G[c][a] = inner ? (uR[c] - uL[c]) / T(2) : uR[c] - uL[c];
      }
    }
    const int64_t nn = C.nn;
    switch (what) {
      case VS_POST_VELOCITY_MAGNITUDE: {  // jnp.linalg.norm(u, axis=0)
        T s = u[0] * u[0];
        for (int c = 1; c < D; ++c) s = s + u[c] * u[c];
        out[p] = sqrt(s);
        break;
      }
      case VS_POST_KINETIC_ENERGY:
      case VS_POST_MEAN_KINETIC_ENERGY: {  // 0.5 * sum(u**2, axis=0)
        T s = u[0] * u[0];
        for (int c = 1; c < D; ++c) s = s + u[c] * u[c];
        const T ke = T(0.5) * s;
        if (what == VS_POST_KINETIC_ENERGY) out[p] = ke;
        else contrib = (double)ke;
        break;
      }
      case VS_POST_VELOCITY_GRADIENT:  // (dim, dim, *spatial), G[i][j] = du_i/dx_j
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) out[(i * D + j) * nn + p] = G[i][j];
        break;
      case VS_POST_STRAIN_RATE:  // 0.5 (G + G^T)
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) out[(i * D + j) * nn + p] = T(0.5) * (G[i][j] + G[j][i]);
        break;
      case VS_POST_STRAIN_RATE_MAGNITUDE: {  // sqrt(sum_ij S_ij S_ij)
        T s = T(0);
        bool first = true;
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) {
            const T sij = T(0.5) * (G[i][j] + G[j][i]);
            s = first ? sij * sij : s + sij * sij;
            first = false;
          }
        out[p] = sqrt(s);
        break;
      }
      case VS_POST_DIVERGENCE: {  // sum_i du_i/dx_i
        T s = G[0][0];
        for (int i = 1; i < D; ++i) s = s + G[i][i];
        out[p] = s;
        break;
      }
      case VS_POST_Q_CRITERION: {  // -0.5 sum_ij G_ij G_ji
        T s = T(0);
        bool first = true;
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) {
            s = first ? G[i][j] * G[j][i] : s + G[i][j] * G[j][i];
            first = false;
          }
        out[p] = T(-0.5) * s;
        break;
      }
      default: {  // vorticity and what derives from it
        T w[3];
        int nw = 1;
        if (D == 2) {
          w[0] = G[1][0] - G[0][1];  // dv/dx - du/dy
        } else {
          w[0] = G[2][1] - G[1][2];  // dw/dy - dv/dz
          w[1] = G[0][2] - G[2][0];  // du/dz - dw/dx
          w[2] = G[1][0] - G[0][1];  // dv/dx - du/dy
          nw = 3;
        }
        if (what == VS_POST_VORTICITY) {
          for (int k = 0; k < nw; ++k) out[k * nn + p] = w[k];
        } else {
          T s = w[0] * w[0];
          for (int k = 1; k < nw; ++k) s = s + w[k] * w[k];
          if (what == VS_POST_VORTICITY_MAGNITUDE) out[p] = nw == 1 ? fabs(w[0]) : sqrt(s);
          else if (what == VS_POST_ENSTROPHY) out[p] = T(0.5) * s;
          else contrib = (double)(T(0.5) * s);  // VS_POST_MEAN_ENSTROPHY
        }
      }
    }
  }
  if (acc) {
    __shared__ double red[8];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) contrib += __shfl_down_sync(0xffffffffu, contrib, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = contrib;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
      atomicAdd(acc, s);
    }
  }
}

template <typename T>
__global__ void k_pressure(const T* __restrict__ rho, int64_t n, T cs2, T* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    out[p] = rho[p] * cs2;
}

static int out_components(int what, int dim) {
  switch (what) {
    case VS_POST_VELOCITY_GRADIENT:
    case VS_POST_STRAIN_RATE: return dim * dim;
    case VS_POST_VORTICITY: return dim == 2 ? 1 : 3;
    default: return 1;
  }
}

}  // namespace post
}  // namespace vs

using namespace vs;
using namespace vs::post;

extern "C" {

int vs_post(int q, int dtype, int what, const void* u, const void* f, int nx, int ny, int nz, void* out,
            double* sum_dev, void* stream) {
  VS_REQUIRE(q == 9 || q == 19, "vs_post: q must be 9 or 19");
  VS_REQUIRE((u != nullptr) != (f != nullptr), "vs_post: pass exactly one of u and f");
  VS_REQUIRE(what >= VS_POST_VELOCITY_MAGNITUDE && what <= VS_POST_MEAN_ENSTROPHY, "vs_post: bad field %d", what);
  const bool mean = what == VS_POST_MEAN_KINETIC_ENERGY || what == VS_POST_MEAN_ENSTROPHY;
  VS_REQUIRE(mean ? sum_dev != nullptr : out != nullptr, "vs_post: output missing");
  const int dim = q == 9 ? 2 : 3;
  if (dim == 2) nz = 1;
  VS_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1, "vs_post: bad grid");
  const int64_t n = (int64_t)nx * ny * nz;
  cudaStream_t st = as_stream(stream);
  double* acc = mean ? sum_dev : nullptr;
  if (mean) {
    cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(double), st);
    if (e != cudaSuccess) return cuda_status(e, "vs_post accumulator");
  }
  int rc = dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    auto go = [&](auto dd) {
      constexpr int D = decltype(dd)::value;
      Ctx<T, D> C{};
      C.u = (const T*)u;
      C.f = (const T*)f;
      C.n[0] = nx;
      C.n[1] = ny;
      C.n[2] = nz;
      C.nn = n;
      k_post<T, D><<<grid_for(n, 256), 256, 0, st>>>(C, what, (T*)out, acc);
    };
    if (dim == 2) go(std::integral_constant<int, 2>{});
    else go(std::integral_constant<int, 3>{});
    VS_CHECK_LAUNCH("vs_post");
    return VS_OK;
  });
  return rc;
}

int vs_post_pressure(int dtype, const void* rho, int64_t n, double cs2, void* out, void* stream) {
  VS_REQUIRE(rho && out && n > 0, "vs_post_pressure: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_pressure<T><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>((const T*)rho, n, (T)cs2, (T*)out);
    VS_CHECK_LAUNCH("vs_post_pressure");
    return VS_OK;
  });
}

int vs_post_components(int q, int what) { return out_components(what, q == 9 ? 2 : 3); }

}  // extern "C"
