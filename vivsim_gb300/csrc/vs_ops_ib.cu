// Per-operator immersed-boundary and rigid-body kernels: one entry point per function of
// vivsim.ib / vivsim.ib3d / vivsim.dyn.
//
// Spreading is deterministic: the (node, pair) keys of all marker-stencil pairs are
// radix-sorted stably, so the contributions to a node are summed in increasing
// (marker, stencil point) order — the order of the reference's scatter-add — by one
// thread per node, with no floating-point atomics.
#include <cuda.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <mutex>

#include "vs_dispatch.cuh"
#include "vs_ib.cuh"

namespace vs {

// device-side status word: bit 0 = stencil index out of range
__device__ unsigned int g_ib_status = 0;

template <typename T>
__global__ void k_ib_kernel(int kernel, const T* __restrict__ r, T* __restrict__ out, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    out[p] = delta(kernel, r[p]);
}

// get_ib_stencil, vivsim/ib/stencil.py:7-51: one thread per (marker, stencil point),
// offsets -r+1..r, s = ix * 2r + iy (meshgrid 'ij').
template <typename T>
__global__ void k_stencil_2d(int kernel, int radius, const T* __restrict__ mx, const T* __restrict__ my, int m, int ny,
                             T* __restrict__ W, int32_t* __restrict__ I) {
  const int w = 2 * radius, s = w * w;
  const int64_t total = (int64_t)m * s;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int mk = (int)(p / s), k = (int)(p % s);
    const int ox = k / w - radius + 1, oy = k % w - radius + 1;
    const T x = mx[mk], y = my[mk];
    const int sx = ifloor(x) + ox, sy = ifloor(y) + oy;
    W[p] = delta(kernel, (T)sx - x) * delta(kernel, (T)sy - y);
    I[p] = sx * ny + sy;
  }
}

// ib3d.get_ib_stencil, vivsim/ib3d/stencil.py:7-59: s = (ix * 2r + iy) * 2r + iz.
template <typename T>
__global__ void k_stencil_3d(int kernel, int radius, const T* __restrict__ X, int m, int ny, int nz,
                             T* __restrict__ W, int32_t* __restrict__ I) {
  const int w = 2 * radius, s = w * w * w;
  const int64_t total = (int64_t)m * s;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int mk = (int)(p / s), k = (int)(p % s);
    const int ox = k / (w * w) - radius + 1, oy = (k / w) % w - radius + 1, oz = k % w - radius + 1;
    const T x = X[3 * mk], y = X[3 * mk + 1], z = X[3 * mk + 2];
    const int sx = ifloor(x) + ox, sy = ifloor(y) + oy, sz = ifloor(z) + oz;
    W[p] = (delta(kernel, (T)sx - x) * delta(kernel, (T)sy - y)) * delta(kernel, (T)sz - z);
    I[p] = sx * (ny * nz) + sy * nz + sz;
  }
}

// interpolate, vivsim/ib/stencil.py:54-78: out[m][c] = sum_s W[m][s] grid[c][I[m][s]], s in order.
template <typename T>
__global__ void k_interpolate(const T* __restrict__ grid, int c, int64_t n_grid, const T* __restrict__ W,
                              const int32_t* __restrict__ I, int m, int s, T* __restrict__ out) {
  const int64_t total = (int64_t)m * c;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int mk = (int)(p / c), cc = (int)(p % c);
    T acc = T(0);
    for (int k = 0; k < s; ++k) {
      const int32_t idx = I[(int64_t)mk * s + k];
      T v = T(0);
      if (idx >= 0 && idx < n_grid) v = grid[cc * n_grid + idx];
      else atomicOr(&g_ib_status, 1u);
      const T t = W[(int64_t)mk * s + k] * v;
      acc = k == 0 ? t : acc + t;
    }
    out[p] = acc;
  }
}

// ------------------------------------------------------------------ CSR build
__global__ void k_iota_keys(const int32_t* __restrict__ I, int64_t P, int32_t* __restrict__ keys,
                            int32_t* __restrict__ ids, int64_t n_grid) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
    int32_t k = I[p];
    if (k < 0 || k >= n_grid) {
      atomicOr(&g_ib_status, 1u);
      k = -1;  // sorted first, skipped by the reductions (out-of-range contributions are dropped)
    }
    keys[p] = k;
    ids[p] = (int32_t)p;
  }
}

// head[k] = 1 where a new node starts in the sorted key list; uid[k] = running count - 1.
__global__ void k_heads(const int32_t* __restrict__ skeys, int64_t P, int32_t* __restrict__ head) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
    head[p] = (skeys[p] >= 0 && (p == 0 || skeys[p] != skeys[p - 1])) ? 1 : 0;
}

// One thread per sorted position that starts a segment: sums the segment in order.
// mode 0: grid_out[c][node] = grid_in[c][node] + sum F[m][c] W[p]  (spread onto a grid)
// mode 1: nodes[c][uid] = scale * sum F[m][c] W[p]                 (compact node buffer)
template <typename T>
__global__ void k_segment_sum(int mode, const int32_t* __restrict__ skeys, const int32_t* __restrict__ sids,
                              const int32_t* __restrict__ head, const int32_t* __restrict__ uid, int64_t P,
                              const T* __restrict__ F, const T* __restrict__ W, int c, int s, const T* grid_in,
                              T* grid_out, int64_t n_grid, T* __restrict__ nodes, int64_t n_nodes, T scale) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
    if (!head[p]) continue;
    const int32_t key = skeys[p];
    for (int cc = 0; cc < c; ++cc) {
      T acc = mode == 0 ? grid_in[cc * n_grid + key] : T(0);
      bool first = mode != 0;
      for (int64_t q = p; q < P && skeys[q] == key; ++q) {
        const int32_t id = sids[q];
        const T t = F[(int64_t)(id / s) * c + cc] * W[id];
        acc = first ? t : acc + t;
        first = false;
      }
      if (mode == 0)
        grid_out[cc * n_grid + key] = acc;
      else
        nodes[cc * n_nodes + uid[p]] = acc * scale;
    }
  }
}

// pair -> unique node id (inverse of the sort permutation)
__global__ void k_pair_uid(const int32_t* __restrict__ sids, const int32_t* __restrict__ skeys,
                           const int32_t* __restrict__ uid, int64_t P, int32_t* __restrict__ pair_uid) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
    pair_uid[sids[p]] = skeys[p] >= 0 ? uid[p] : -1;
}

// MDF marker update (vivsim/ib/mdf.py:41-56), one thread per (marker, component):
//   first: U = interp(grid_u)   else: U += interp(nodes)   (nodes already hold 0.5 * spread)
//   F_step = (U_target - U) * (2 ds);  F_total = F_step (first, if any iteration) or += F_step
//   write_force: marker_force = -F_total
template <typename T>
__global__ void k_mdf_marker(int first, int use_step, int write_force, const T* __restrict__ grid_u, int64_t n_grid,
                             const T* __restrict__ nodes, int64_t n_nodes, const int32_t* __restrict__ I,
                             const int32_t* __restrict__ pair_uid, const T* __restrict__ W, int m, int s, int c,
                             const T* __restrict__ ut, const T* __restrict__ ds, T ds_scalar, T* __restrict__ U,
                             T* __restrict__ Fstep, T* __restrict__ Ftot, T* __restrict__ marker_force) {
  const int64_t total = (int64_t)m * c;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int mk = (int)(p / c), cc = (int)(p % c);
    T acc = T(0);
    for (int k = 0; k < s; ++k) {
      const int64_t pk = (int64_t)mk * s + k;
      T v = T(0);
      if (first) {
        const int32_t idx = I[pk];
        if (idx >= 0 && idx < n_grid) v = grid_u[cc * n_grid + idx];
      } else {
        const int32_t id = pair_uid[pk];
        if (id >= 0) v = nodes[cc * n_nodes + id];
      }
      const T t = W[pk] * v;
      acc = k == 0 ? t : acc + t;
    }
    const T u = first ? acc : U[p] + acc;
    U[p] = u;
    const T d2 = (ds ? ds[mk] : ds_scalar) * T(2);
    const T fs = (ut[p] - u) * d2;
    Fstep[p] = fs;
    const T ft = first ? (use_step ? fs : T(0)) : Ftot[p] + fs;
    Ftot[p] = ft;
    if (write_force) marker_force[p] = -ft;
  }
}

template <typename T>
__global__ void k_copy(const T* __restrict__ a, T* __restrict__ b, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    b[p] = a[p];
}

// ------------------------------------------------------------------ workspace
struct IbWorkspace {
  int32_t *keys, *ids, *skeys, *sids, *head, *uid, *pair_uid;
  void* cub_tmp;
  size_t cub_bytes;
  char* tail;  // float scratch (U, Fstep, Ftot, nodes) for MDF
  size_t total;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// CUB scratch for the pair sort and the head scan (the larger of the two).
static size_t cub_sort_bytes(int64_t P) {
  size_t sort_bytes = 0, scan_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, (const int32_t*)nullptr, (int32_t*)nullptr,
                                  (const int32_t*)nullptr, (int32_t*)nullptr, (int)P);
  cub::DeviceScan::InclusiveSum(nullptr, scan_bytes, (const int32_t*)nullptr, (int32_t*)nullptr, (int)P);
  return sort_bytes > scan_bytes ? sort_bytes : scan_bytes;
}

// Float scratch for MDF: U, Fstep, Ftot (m*c each) + compact nodes (c * P) in double.
static size_t mdf_float_bytes(int m, int s) {
  const int64_t P = (int64_t)m * s;
  return align256(sizeof(double) * 3 * (int64_t)m * 3) + align256(sizeof(double) * 3 * P);
}

static size_t ws_bytes(int m, int s) {
  const int64_t P = (int64_t)m * s;
  size_t b = 0;
  b += 7 * align256(sizeof(int32_t) * P);
  b += align256(cub_sort_bytes(P));
  b += mdf_float_bytes(m, s);
  return b;
}

// Lays the workspace out from base.  with_tail = false lays out only what a spread uses
// (the pair arrays and the CUB storage) and forms no pointer beyond them.
static IbWorkspace carve(void* base, int m, int s, bool with_tail = true) {
  const int64_t P = (int64_t)m * s;
  IbWorkspace w{};
  char* p = (char*)base;
  int32_t** arrs[7] = {&w.keys, &w.ids, &w.skeys, &w.sids, &w.head, &w.uid, &w.pair_uid};
  size_t off = 0;
  for (auto a : arrs) {
    *a = (int32_t*)(p + off);
    off += align256(sizeof(int32_t) * P);
  }
  w.cub_bytes = align256(cub_sort_bytes(P));
  w.cub_tmp = p + off;
  off += w.cub_bytes;
  w.tail = nullptr;
  if (with_tail) {
    w.tail = p + off;
    off += mdf_float_bytes(m, s);
  }
  w.total = off;
  return w;
}

// Sort (node, pair) keys and build segment heads / unique ids.  Returns the status.
static int build_csr(const int32_t* I, int64_t P, int64_t n_grid, IbWorkspace& w, cudaStream_t st) {
  const int B = 256;
  k_iota_keys<<<grid_for(P, B), B, 0, st>>>(I, P, w.keys, w.ids, n_grid);
  size_t tb = w.cub_bytes;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(w.cub_tmp, tb, w.keys, w.skeys, w.ids, w.sids, (int)P, 0,
                                                  32, st);
  if (e != cudaSuccess) return cuda_status(e, "ib csr sort");
  k_heads<<<grid_for(P, B), B, 0, st>>>(w.skeys, P, w.head);
  // inclusive scan of heads -> uid + 1 (reuse CUB scan through a simple kernel-free path:
  // one block prefix sum is enough for the sizes the per-op API sees, so use a
  // device-wide scan)
  size_t sb = 0;
  cub::DeviceScan::InclusiveSum(nullptr, sb, w.head, w.uid, (int)P);
  if (sb > w.cub_bytes) {
    set_error("ib csr: scan scratch larger than reserved (%zu > %zu)", sb, w.cub_bytes);
    return VS_ERR_INVALID_ARG;
  }
  e = cub::DeviceScan::InclusiveSum(w.cub_tmp, sb, w.head, w.uid, (int)P, st);
  if (e != cudaSuccess) return cuda_status(e, "ib csr scan");
  VS_CHECK_LAUNCH("ib csr");
  return VS_OK;
}

__global__ void k_uid_minus_one(int32_t* uid, int64_t P);

// Sorted pair CSR of a static stencil, built in `workspace` (vivsim_gb300 fixed bodies).
int ib_build_csr(const int32_t* I, int64_t P, int64_t n_grid, void* workspace, int m, int s, IbCsrView* out,
                 cudaStream_t st) {
  IbWorkspace w = carve(workspace, m, s);
  int rc = build_csr(I, P, n_grid, w, st);
  if (rc) return rc;
  k_uid_minus_one<<<grid_for(P, 256), 256, 0, st>>>(w.uid, P);
  k_pair_uid<<<grid_for(P, 256), 256, 0, st>>>(w.sids, w.skeys, w.uid, P, w.pair_uid);
  VS_CHECK_LAUNCH("ib_build_csr");
  out->skeys = w.skeys;
  out->sids = w.sids;
  out->head = w.head;
  out->uid = w.uid;
  out->pair_uid = w.pair_uid;
  return VS_OK;
}

__global__ void k_uid_minus_one(int32_t* uid, int64_t P) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
    uid[p] -= 1;
}

// ------------------------------------------------------------------ dynamics
// Newmark-beta, vivsim/dyn.py:5-51.
template <typename T>
__global__ void k_newmark(int ndof, int matrix, const T* a, const T* v, const T* d, const T* h, const T* m,
                          const T* k, const T* c, T sc, T sk, T sden, double dt, double gamma, double beta, T* an,
                          T* vn, T* dn) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const T c1 = (T)(gamma * dt), c2 = (T)(beta * dt * dt);
  const T k1 = (T)(dt * (1 - gamma)), k2 = (T)(dt * dt * (0.5 - beta)), tdt = (T)dt;
  T v1[8], v2[8], res[8];
  for (int i = 0; i < ndof; ++i) {
    v1[i] = v[i] + k1 * a[i];
    v2[i] = (d[i] + tdt * v[i]) + k2 * a[i];
  }
  if (!matrix) {
    // scalar branch (dyn.py:42-45): m, k, c are Python floats, the denominator is
    // formed in double precision and rounded once
    for (int i = 0; i < ndof; ++i) res[i] = ((h[i] - sc * v1[i]) - sk * v2[i]) / sden;
  } else {
    // solve (m + c1 c + c2 k) x = h - c v1 - k v2 by Gaussian elimination with partial pivoting
    T A[8][9];
    for (int i = 0; i < ndof; ++i) {
      T cv = T(0), kv = T(0);
      for (int j = 0; j < ndof; ++j) {
        A[i][j] = (m[i * ndof + j] + c1 * c[i * ndof + j]) + c2 * k[i * ndof + j];
        cv = cv + c[i * ndof + j] * v1[j];
        kv = kv + k[i * ndof + j] * v2[j];
      }
      A[i][ndof] = (h[i] - cv) - kv;
    }
    for (int col = 0; col < ndof; ++col) {
      int piv = col;
      for (int r = col + 1; r < ndof; ++r)
        if (fabs(A[r][col]) > fabs(A[piv][col])) piv = r;
      for (int j = 0; j <= ndof; ++j) {
        T t = A[col][j]; A[col][j] = A[piv][j]; A[piv][j] = t;
      }
      for (int r = col + 1; r < ndof; ++r) {
        const T f = A[r][col] / A[col][col];
        for (int j = col; j <= ndof; ++j) A[r][j] = A[r][j] - f * A[col][j];
      }
    }
    for (int i = ndof - 1; i >= 0; --i) {
      T acc = A[i][ndof];
      for (int j = i + 1; j < ndof; ++j) acc = acc - A[i][j] * res[j];
      res[i] = acc / A[i][i];
    }
  }
  for (int i = 0; i < ndof; ++i) {
    an[i] = res[i];
    vn[i] = c1 * res[i] + v1[i];
    dn[i] = c2 * res[i] + v2[i];
  }
}

template <typename T>
__global__ void k_coords_2dof(const T* x0, const T* y0, int m, const T* d, T* x, T* y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    x[i] = x0[i] + d[0];
    y[i] = y0[i] + d[1];
  }
}

template <typename T>
__global__ void k_coords_3dof(const T* x0, const T* y0, int m, T xc, T yc, const T* d, T* x, T* y) {
  const T cs = cos(d[2]), sn = sin(d[2]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const T xr = x0[i] - xc, yr = y0[i] - yc;
    x[i] = ((xc + d[0]) + xr * cs) - yr * sn;
    y[i] = ((yc + d[1]) + xr * sn) + yr * cs;
  }
}

template <typename T>
__global__ void k_vel_3dof(const T* x, const T* y, int m, T xc, T yc, const T* d, const T* v, T* vel) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    const T xr = (x[i] - xc) - d[0], yr = (y[i] - yc) - d[1];
    vel[2 * i] = v[0] - v[2] * yr;
    vel[2 * i + 1] = v[1] + v[2] * xr;
  }
}

// Sums in marker order (single thread; m is a few thousand at most).
template <typename T>
__global__ void k_force(const T* h, int m, int c, T* out) {
  const int cc = threadIdx.x;
  if (cc >= c) return;
  T acc = h[cc];
  for (int i = 1; i < m; ++i) acc = acc + h[i * c + cc];
  out[cc] = acc;
}

template <typename T>
__global__ void k_torque(const T* x, const T* y, int m, T xc, T yc, const T* d, const T* h, T* out) {
  if (threadIdx.x != 0) return;
  const T cx = xc + d[0], cy = yc + d[1];
  T acc = T(0);
  for (int i = 0; i < m; ++i) {
    const T t = (x[i] - cx) * h[2 * i + 1] - (y[i] - cy) * h[2 * i];
    acc = i == 0 ? t : acc + t;
  }
  out[0] = acc;
}


// Multi-direct forcing over a CSR that may already be built (csr_ready) in `workspace`
// by an earlier call with the same I (the fused fixed-body step reuses it every step).
int ib_mdf_run(int dtype, bool csr_ready, const void* grid_u, int c, int64_t n_grid, const void* W, const int32_t* I,
               int m, int s, const void* u_target, const void* ds, double ds_scalar, int n_iter, void* grid_force,
               void* marker_force, void* workspace, size_t workspace_bytes, void* stream) {
  VS_REQUIRE(grid_u && W && I && u_target && grid_force && marker_force && c > 0 && m > 0 && s > 0 && n_grid > 0,
             "vs_ib_mdf: bad arguments");
  VS_REQUIRE(n_iter >= 0, "vs_ib_mdf: n_iter must be >= 0");
  VS_REQUIRE(workspace && workspace_bytes >= ws_bytes(m, s), "vs_ib_mdf: workspace of %zu bytes needed",
             ws_bytes(m, s));
  VS_REQUIRE(n_grid < (1ll << 31), "vs_ib_mdf: grid too large for int32 indices");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    cudaStream_t st = as_stream(stream);
    const int64_t P = (int64_t)m * s;
    IbWorkspace w = carve(workspace, m, s);
    T* U = (T*)w.tail;
    T* Fstep = U + (int64_t)m * c;
    T* Ftot = Fstep + (int64_t)m * c;
    T* nodes = (T*)(w.tail + align256(sizeof(double) * 3 * (int64_t)m * 3));
    const int64_t n_nodes = P;
    if (!csr_ready) {
      int rc = build_csr(I, P, n_grid, w, st);
      if (rc) return rc;
      k_uid_minus_one<<<grid_for(P, 256), 256, 0, st>>>(w.uid, P);
      k_pair_uid<<<grid_for(P, 256), 256, 0, st>>>(w.sids, w.skeys, w.uid, P, w.pair_uid);
    }
    const unsigned gm = grid_for((int64_t)m * c, 128);
    // U = interp(grid_u); F_step = (U_t - U) 2ds; F_tot = F_step (mdf.py:38-48)
    k_mdf_marker<T><<<gm, 128, 0, st>>>(1, n_iter > 0, n_iter <= 1, (const T*)grid_u, n_grid, nodes, n_nodes, I,
                                        w.pair_uid, (const T*)W, m, s, c, (const T*)u_target, (const T*)ds,
                                        (T)ds_scalar, U, Fstep, Ftot, (T*)marker_force);
    // iterations 1..n_iter-1; the spread and interpolation after the last force step only
    // update a marker velocity the reference discards (mdf.py:57-64), so they are skipped
    for (int it = 0; it + 1 < n_iter; ++it) {
      // nodes = 0.5 * spread(F_step)   (mdf.py:50-51)
      k_segment_sum<T><<<grid_for(P, 256), 256, 0, st>>>(1, w.skeys, w.sids, w.head, w.uid, P, Fstep, (const T*)W, c,
                                                         s, nullptr, nullptr, n_grid, nodes, n_nodes, T(0.5));
      // U += interp(nodes); next F_step; F_tot += F_step
      k_mdf_marker<T><<<gm, 128, 0, st>>>(0, 1, it + 2 == n_iter, (const T*)grid_u, n_grid, nodes, n_nodes, I,
                                          w.pair_uid, (const T*)W, m, s, c, (const T*)u_target, (const T*)ds,
                                          (T)ds_scalar, U, Fstep, Ftot, (T*)marker_force);
    }
    // grid_force = spread(F_total, zeros)   (mdf.py:60-62)
    cudaError_t e = cudaMemsetAsync(grid_force, 0, sizeof(T) * c * n_grid, st);
    if (e != cudaSuccess) return cuda_status(e, "vs_ib_mdf memset");
    k_segment_sum<T><<<grid_for(P, 256), 256, 0, st>>>(0, w.skeys, w.sids, w.head, w.uid, P, Ftot, (const T*)W, c, s,
                                                       (const T*)grid_force, (T*)grid_force, n_grid, nullptr, 0,
                                                       T(1));
    VS_CHECK_LAUNCH("vs_ib_mdf");
    return VS_OK;
  });
}

}  // namespace vs

using namespace vs;

extern "C" {

int vs_ib_kernel(int kernel, int dtype, const void* r, void* out, int64_t n, void* stream) {
  VS_REQUIRE(r && out && n > 0, "vs_ib_kernel: bad arguments");
  VS_REQUIRE(kernel >= VS_KERNEL_PESKIN3 && kernel <= VS_KERNEL_COSINE4, "vs_ib_kernel: bad kernel %d", kernel);
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_ib_kernel<T><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(kernel, (const T*)r, (T*)out, n);
    VS_CHECK_LAUNCH("vs_ib_kernel");
    return VS_OK;
  });
}

int vs_ib_stencil_2d(int kernel, int radius, int dtype, const void* marker_x, const void* marker_y, int m, int ny,
                     void* W, int32_t* I, void* stream) {
  VS_REQUIRE(marker_x && marker_y && W && I && m > 0 && ny > 0, "vs_ib_stencil_2d: bad arguments");
  VS_REQUIRE(radius >= 1 && radius <= 4, "vs_ib_stencil_2d: radius %d out of 1..4", radius);
  VS_REQUIRE(kernel >= VS_KERNEL_PESKIN3 && kernel <= VS_KERNEL_COSINE4, "vs_ib_stencil_2d: bad kernel");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    const int64_t total = (int64_t)m * 4 * radius * radius;
    k_stencil_2d<T><<<grid_for(total, 256), 256, 0, as_stream(stream)>>>(kernel, radius, (const T*)marker_x,
                                                                        (const T*)marker_y, m, ny, (T*)W, I);
    VS_CHECK_LAUNCH("vs_ib_stencil_2d");
    return VS_OK;
  });
}

int vs_ib_stencil_3d(int kernel, int radius, int dtype, const void* coords, int m, int nx, int ny, int nz, void* W,
                     int32_t* I, void* stream) {
  VS_REQUIRE(coords && W && I && m > 0 && nx > 0 && ny > 0 && nz > 0, "vs_ib_stencil_3d: bad arguments");
  VS_REQUIRE(radius >= 1 && radius <= 4, "vs_ib_stencil_3d: radius %d out of 1..4", radius);
  VS_REQUIRE((int64_t)nx * ny * nz < (1ll << 31), "vs_ib_stencil_3d: grid too large for int32 indices");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    const int64_t total = (int64_t)m * 8 * radius * radius * radius;
    k_stencil_3d<T><<<grid_for(total, 256), 256, 0, as_stream(stream)>>>(kernel, radius, (const T*)coords, m, ny,
                                                                        nz, (T*)W, I);
    VS_CHECK_LAUNCH("vs_ib_stencil_3d");
    return VS_OK;
  });
}

int vs_ib_interpolate(int dtype, const void* grid, int c, int64_t n_grid, const void* W, const int32_t* I, int m,
                      int s, void* out, void* stream) {
  VS_REQUIRE(grid && W && I && out && c > 0 && m > 0 && s > 0 && n_grid > 0, "vs_ib_interpolate: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_interpolate<T><<<grid_for((int64_t)m * c, 128), 128, 0, as_stream(stream)>>>((const T*)grid, c, n_grid,
                                                                                  (const T*)W, I, m, s, (T*)out);
    VS_CHECK_LAUNCH("vs_ib_interpolate");
    return VS_OK;
  });
}

size_t vs_ib_workspace_bytes(int m, int s) {
  if (m <= 0 || s <= 0) return 0;
  return ws_bytes(m, s);
}

int vs_ib_spread(int dtype, const void* marker_values, const void* grid_in, void* grid_out, int c, int64_t n_grid,
                 const void* W, const int32_t* I, int m, int s, void* workspace, size_t workspace_bytes,
                 void* stream) {
  VS_REQUIRE(marker_values && grid_in && grid_out && W && I && c > 0 && m > 0 && s > 0 && n_grid > 0,
             "vs_ib_spread: bad arguments");
  VS_REQUIRE(workspace && workspace_bytes >= ws_bytes(m, s), "vs_ib_spread: workspace of %zu bytes needed",
             ws_bytes(m, s));
  VS_REQUIRE(n_grid < (1ll << 31), "vs_ib_spread: grid too large for int32 indices");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    cudaStream_t st = as_stream(stream);
    const int64_t P = (int64_t)m * s;
    IbWorkspace w = carve(workspace, m, s);
    if (grid_out != grid_in) {
      k_copy<T><<<grid_for((int64_t)c * n_grid, 256), 256, 0, st>>>((const T*)grid_in, (T*)grid_out,
                                                                    (int64_t)c * n_grid);
    }
    int rc = build_csr(I, P, n_grid, w, st);
    if (rc) return rc;
    k_segment_sum<T><<<grid_for(P, 256), 256, 0, st>>>(0, w.skeys, w.sids, w.head, w.uid, P, (const T*)marker_values,
                                                       (const T*)W, c, s, (const T*)grid_out, (T*)grid_out, n_grid,
                                                       nullptr, 0, T(1));
    VS_CHECK_LAUNCH("vs_ib_spread");
    return VS_OK;
  });
}

int vs_ib_mdf(int dtype, const void* grid_u, int c, int64_t n_grid, const void* W, const int32_t* I, int m, int s,
              const void* u_target, const void* ds, double ds_scalar, int n_iter, void* grid_force,
              void* marker_force, void* workspace, size_t workspace_bytes, void* stream) {
  return vs::ib_mdf_run(dtype, false, grid_u, c, n_grid, W, I, m, s, u_target, ds, ds_scalar, n_iter, grid_force,
                        marker_force, workspace, workspace_bytes, stream);
}

int vs_ib_status(unsigned* status_out, int reset) {
  unsigned v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_ib_status, sizeof(v));
  if (e != cudaSuccess) return cuda_status(e, "vs_ib_status");
  if (reset) {
    unsigned z = 0;
    e = cudaMemcpyToSymbol(g_ib_status, &z, sizeof(z));
    if (e != cudaSuccess) return cuda_status(e, "vs_ib_status reset");
  }
  if (status_out) *status_out = v;
  return VS_OK;
}

int vs_newmark(int dtype, int ndof, const void* a, const void* v, const void* d, const void* h, double m, double k,
               double c, const void* m_mat, const void* k_mat, const void* c_mat, double dt, double gamma,
               double beta, void* a_next, void* v_next, void* d_next, void* stream) {
  VS_REQUIRE(a && v && d && h && a_next && v_next && d_next, "vs_newmark: null argument");
  VS_REQUIRE(ndof >= 1 && ndof <= 8, "vs_newmark: ndof must be 1..8");
  const int matrix = m_mat != nullptr;
  VS_REQUIRE(!matrix || (k_mat && c_mat), "vs_newmark: matrix form needs m, k and c matrices");
  const double den = m + gamma * dt * c + beta * dt * dt * k;
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_newmark<T><<<1, 32, 0, as_stream(stream)>>>(ndof, matrix, (const T*)a, (const T*)v, (const T*)d, (const T*)h,
                                                  (const T*)m_mat, (const T*)k_mat, (const T*)c_mat, (T)c, (T)k,
                                                  (T)den, dt, gamma, beta, (T*)a_next, (T*)v_next, (T*)d_next);
    VS_CHECK_LAUNCH("vs_newmark");
    return VS_OK;
  });
}

int vs_markers_coords_2dof(int dtype, const void* x0, const void* y0, int m, const void* d, void* x, void* y,
                           void* stream) {
  VS_REQUIRE(x0 && y0 && d && x && y && m > 0, "vs_markers_coords_2dof: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_coords_2dof<T><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>((const T*)x0, (const T*)y0, m, (const T*)d,
                                                                      (T*)x, (T*)y);
    VS_CHECK_LAUNCH("vs_markers_coords_2dof");
    return VS_OK;
  });
}

int vs_markers_coords_3dof(int dtype, const void* x0, const void* y0, int m, double xc, double yc, const void* d,
                           void* x, void* y, void* stream) {
  VS_REQUIRE(x0 && y0 && d && x && y && m > 0, "vs_markers_coords_3dof: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_coords_3dof<T><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>((const T*)x0, (const T*)y0, m, (T)xc, (T)yc,
                                                                      (const T*)d, (T*)x, (T*)y);
    VS_CHECK_LAUNCH("vs_markers_coords_3dof");
    return VS_OK;
  });
}

int vs_markers_velocity_3dof(int dtype, const void* x, const void* y, int m, double xc, double yc, const void* d,
                             const void* v, void* vel, void* stream) {
  VS_REQUIRE(x && y && d && v && vel && m > 0, "vs_markers_velocity_3dof: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_vel_3dof<T><<<grid_for(m, 128), 128, 0, as_stream(stream)>>>((const T*)x, (const T*)y, m, (T)xc, (T)yc,
                                                                   (const T*)d, (const T*)v, (T*)vel);
    VS_CHECK_LAUNCH("vs_markers_velocity_3dof");
    return VS_OK;
  });
}

int vs_force_to_obj(int dtype, const void* h, int m, int c, void* out, void* stream) {
  VS_REQUIRE(h && out && m > 0 && c > 0 && c <= 32, "vs_force_to_obj: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_force<T><<<1, 32, 0, as_stream(stream)>>>((const T*)h, m, c, (T*)out);
    VS_CHECK_LAUNCH("vs_force_to_obj");
    return VS_OK;
  });
}

int vs_torque_to_obj(int dtype, const void* x, const void* y, int m, double xc, double yc, const void* d,
                     const void* h, void* out, void* stream) {
  VS_REQUIRE(x && y && d && h && out && m > 0, "vs_torque_to_obj: bad arguments");
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_torque<T><<<1, 32, 0, as_stream(stream)>>>((const T*)x, (const T*)y, m, (T)xc, (T)yc, (const T*)d,
                                                 (const T*)h, (T*)out);
    VS_CHECK_LAUNCH("vs_torque_to_obj");
    return VS_OK;
  });
}

}  // extern "C"

// ------------------------------------------------------------------ spread without allocation
// vs_ib_spread_noalloc serves callers that cannot allocate device memory while they run:
// a foreign runtime that owns every device allocation and hands out no scratch (an XLA
// custom call registered without a workspace), or a latency-critical loop that cannot
// afford a trip into the allocator.  Its scratch is one file-scope device array, set up
// once per device (and again after the device's context is replaced) and shared by every
// call on that device.
namespace vs {
namespace {

constexpr int64_t kNoAllocMaxPairs = 65536;              // m * s: 4096 markers of a 4x4 stencil
constexpr size_t kNoAllocScratchBytes = (size_t)4 << 20;  // 4 MiB
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};  // context id the address belongs to

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current context (never reused within a process), or 0
// when the driver offers none.  A device reset ends the primary context; the next one
// gets a new id, so an address cached under the old id is looked up again.
unsigned long long current_context_id() {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (PfnCtxGetCurrent)p;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (PfnCtxGetId)p;
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Address of this device's copy of g_noalloc_scratch.  The first call on a device (and the
// first call after the device's context was replaced, e.g. by cudaDeviceReset) looks it up,
// loading this module on that device if it is not loaded yet, and caches it.
int noalloc_scratch(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "vs_ib_spread_noalloc: cudaGetDevice");
  VS_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "vs_ib_spread_noalloc: device %d beyond %d", dev,
             kNoAllocMaxDevices);
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev] || g_noalloc_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "vs_ib_spread_noalloc: cudaGetSymbolAddress");
    if (!p) {
      set_error("vs_ib_spread_noalloc: no device address for the scratch array");
      return VS_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
    g_noalloc_ctx[dev] = ctx;
  }
  *out = g_noalloc_ptr[dev];
  return VS_OK;
}

// Scratch the spread itself touches: the seven pair arrays and the CUB sort/scan storage
// (carve(.., false) lays out exactly these).
size_t spread_scratch_bytes(int m, int s) {
  const int64_t P = (int64_t)m * s;
  return 7 * align256(sizeof(int32_t) * P) + align256(cub_sort_bytes(P));
}

}  // namespace
}  // namespace vs

extern "C" {

int vs_ib_spread_noalloc(int dtype, const void* marker_values, const void* grid_in, void* grid_out, int c,
                         int64_t n_grid, const void* W, const int32_t* I, int m, int s, void* stream) {
  VS_REQUIRE(marker_values && grid_in && grid_out && W && I && c > 0 && m > 0 && s > 0 && n_grid > 0,
             "vs_ib_spread_noalloc: bad arguments");
  VS_REQUIRE((int64_t)m * s <= kNoAllocMaxPairs,
             "vs_ib_spread_noalloc: %lld marker-stencil pairs exceed the fixed scratch limit of %lld; "
             "use vs_ib_spread with a caller workspace",
             (long long)m * s, (long long)kNoAllocMaxPairs);
  VS_REQUIRE(n_grid < (1ll << 31), "vs_ib_spread_noalloc: grid too large for int32 indices");
  VS_REQUIRE(dtype == VS_F32 || dtype == VS_F64, "vs_ib_spread_noalloc: bad dtype %d", dtype);
  void* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  const size_t need = spread_scratch_bytes(m, s);
  VS_REQUIRE(need <= kNoAllocScratchBytes, "vs_ib_spread_noalloc: %zu scratch bytes needed, %zu available", need,
             kNoAllocScratchBytes);
  // Every scratch word the spread reads is written earlier in the same call (keys and ids
  // by k_iota_keys, the sorted copies by the sort, heads and ids by k_heads and the scan),
  // so nothing has to be cleared first.
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    cudaStream_t st = as_stream(stream);
    const int64_t P = (int64_t)m * s;
    IbWorkspace w = carve(scratch, m, s, false);
    if (grid_out != grid_in) {
      k_copy<T><<<grid_for((int64_t)c * n_grid, 256), 256, 0, st>>>((const T*)grid_in, (T*)grid_out,
                                                                    (int64_t)c * n_grid);
    }
    int rc2 = build_csr(I, P, n_grid, w, st);
    if (rc2) return rc2;
    k_segment_sum<T><<<grid_for(P, 256), 256, 0, st>>>(0, w.skeys, w.sids, w.head, w.uid, P, (const T*)marker_values,
                                                       (const T*)W, c, s, (const T*)grid_out, (T*)grid_out, n_grid,
                                                       nullptr, 0, T(1));
    VS_CHECK_LAUNCH("vs_ib_spread_noalloc");
    return VS_OK;
  });
}

}  // extern "C"
