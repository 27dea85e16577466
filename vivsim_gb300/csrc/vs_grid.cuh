// Device side of the fused grid kernel: launch parameters and the per-node and per-block
// work of one time step (collide, force, push-stream), shared by the grid kernels of
// vs_step.cu.
#pragma once

#include "vs_boundary.cuh"
#include "vs_fast.cuh"

namespace vs {

// Bounds-checked build (nvcc -DVIVSIM_BOUNDS_CHECK, vivsim_gb300._build.build(checked=True)):
// every gather and scatter index of the grid kernels is tested against its array first; an
// index outside it sets VS_ERR_RANGE in the plan's status word (vs_lattice_status) and the
// access is skipped.  The default build compiles the tests out.
#ifdef VIVSIM_BOUNDS_CHECK
__device__ __forceinline__ bool in_range(int64_t i, int64_t lim, int* status) {
  if (i >= 0 && i < lim) return true;
  if (status) atomicMax(status, VS_ERR_RANGE);
  return false;
}
#define VS_IN_RANGE(i, lim, st) ::vs::in_range((int64_t)(i), (int64_t)(lim), (st))
#else
#define VS_IN_RANGE(i, lim, st) true
#endif

// device window descriptor (int[8]): origin, extent, sticky status
// META_PX/PY: lower corner of the body's last stencil bounding box (2-D moving bodies
// predict their next window from it)
// META_PX2/PY2: a second prediction slot; the cluster-form body reads one slot while the
// concurrent grid kernel reads the same slot for the box it skips, and writes the other
enum {
  META_OX = 0, META_OY, META_OZ, META_WX, META_WY, META_WZ, META_STATUS, META_PX, META_PY, META_PX2, META_PY2,
  META_N = 12
};

// ------------------------------------------------------------------ grid kernel
template <class L, typename T>
struct StepParams {
  // the fields every launch reads come first (a launch fetches only the lines it touches)
  const T* fin;
  T* fout;
  int nx, ny, nz, n;
  int chunks;                    // blocks along the contiguous axis (3-D)
  int gx;                        // blocks per launch row (the launch's grid.x)
  int nreg;                      // 0: the whole grid; else the union of reg[0..nreg)
  int skip_box;                  // nodes inside box[] are left to another launch
  int skip_walls;                // the x = 0 and x = nx-1 planes are left to another launch
  int mask_load;                 // apply the previous step's obstacle bounce-back on load
  int dyn_slot, dyn_ext[2];      // predicted window: slot and extent (with dyn_meta)
  int forcing;
  int has_g0;
  int n_lazy;                    // face boundaries of the previous step applied on load
  int n_pre;                     // faces whose pre-stream populations are kept (bounce-back)
  const uint8_t* mask;           // obstacle cells (one byte per node) or null
  const int* dyn_meta;           // non-null: the skipped box is the body's predicted window
  CollideParams<T> cp;
  T g0[3];
  T guo_scale;                   // 1 - omega / 2 (Guo-BGK)
  const T* gw;                   // IB force window (D, wx, wy, wz) or null
  const int* meta;               // window descriptor (device)
  int* status;                   // the plan's status word (bounds-checked build)
  int box[6];
  int reg[3][6];                 // regions x0, x1, y0, y1, z0, z1 (half-open)
  int rowstart[4];               // first launch row (x plane) of each region
  WallArgs<T> lazy[2];
  int pre_loc[VS_MAX_BC];
  T* pre_buf[VS_MAX_BC];
  T op[L::Q * L::Q];             // MRT collision operator
  T fop[L::Q * L::Q];            // MRT forcing operator
};

// Per-node features a grid launch may need, as a compile-time mask (FEAT): a launch
// compiled without a feature carries none of its code or registers.  The general form
// (kFeatGeneral) tests each one at run time from StepParams.
enum {
  kFeatWalls = 1,  // the previous step's face boundaries applied on load (lazy walls)
  kFeatSkip = 2,   // regions, the body's box or window and the wall planes left to other launches
  kFeatForce = 4,  // body force: uniform g and the IB force window
  kFeatMask = 8,   // the previous step's obstacle bounce-back applied on load
  kFeatPre = 16,   // pre-stream populations kept for bounce-back faces
  kFeatStream = 32,  // streaming loads and stores (evict-first in L2), so that a grid larger
                     // than L2 does not evict the body kernels' small working set
  kFeatGeneral = kFeatSkip | kFeatForce | kFeatMask | kFeatPre
};

// Per-node work of the grid kernels: (lazy face boundaries,) moments, equilibrium,
// collision, forcing, push streaming.  f holds the node's loaded populations.
// population load and store of the grid kernels: plain, or cache-streaming (kFeatStream)
template <int FEAT, typename T>
__device__ __forceinline__ T pop_load(const T* p) {
  if constexpr ((FEAT & kFeatStream) != 0) return __ldcs(p);
  else return __ldg(p);
}
template <int FEAT, typename T>
__device__ __forceinline__ void pop_store(T* p, T v) {
  if constexpr ((FEAT & kFeatStream) != 0) __stcs(p, v);
  else *p = v;
}

// gext: the node's IB force, given by the caller (the cluster-form body kernel holds its
// window's force in shared memory), in place of the lookup in the force window P.gw.
template <class L, typename T, int COLL, int FEAT>
__device__ __forceinline__ void step_node(const StepParams<L, T>& P, int x, int y, int z, int p, T* f,
                                          const T* gext = nullptr) {
  constexpr int Q = L::Q;
  const int syz = P.ny * P.nz;

  // the previous step's face boundaries, applied to the wall nodes as they are loaded
  // (all of them on the x faces, so they touch disjoint nodes and commute)
  if constexpr ((FEAT & kFeatWalls) != 0) for (int k = 0; k < P.n_lazy; ++k) {
    const WallArgs<T>& A = P.lazy[k];
    const int a = loc_axis(A.loc), sg = loc_sign(A.loc);
    const int coord = a == 0 ? x : (a == 1 ? y : z);
    const int nn[3] = {P.nx, P.ny, P.nz};
    if (coord != (sg > 0 ? 0 : nn[a] - 1)) continue;
    T nb[Q], out[Q];
    if (bc_needs_neighbor<L>(A.kind, A.mode)) {
      const int stride = a == 0 ? syz : (a == 1 ? P.nz : 1);
      const int pn = p + sg * stride;
#pragma unroll
      for (int i = 0; i < Q; ++i) nb[i] = VS_IN_RANGE(pn, P.n, P.status) ? pop_load<FEAT>(P.fin + (size_t)i * P.n + pn) : T(0);
    }
    bc_node<L, T>(A, 0, f, nb, nullptr, out);
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = out[i];
  }
  // the previous step's obstacle bounce-back (lbm/boundary/bb.py:98-110), which follows its
  // face boundaries: an obstacle cell's populations swap with their opposites
  if ((FEAT & kFeatMask) && P.mask_load && VS_IN_RANGE(p, P.n, P.status) && P.mask[p]) {
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      const int o = L::opp(i);
      if (o > i) {
        const T t = f[i];
        f[i] = f[o];
        f[o] = t;
      }
    }
  }

  T rho, u[3] = {T(0), T(0), T(0)};
  fast::macro<L>(f, rho, u);

  T g[3] = {T(0), T(0), T(0)};
  bool has_g = (FEAT & kFeatForce) && P.has_g0;
  if (has_g) {
#pragma unroll
    for (int d = 0; d < L::D; ++d) g[d] = P.g0[d];
  }
  if ((FEAT & kFeatForce) && gext) {
#pragma unroll
    for (int d = 0; d < L::D; ++d) g[d] = has_g ? g[d] + gext[d] : gext[d];
    has_g = true;
  } else if ((FEAT & kFeatForce) && P.gw) {
    const int wx = x - P.meta[META_OX], wy = y - P.meta[META_OY], wz = z - P.meta[META_OZ];
    const int ex = P.meta[META_WX], ey = P.meta[META_WY], ez = P.meta[META_WZ];
    if (wx >= 0 && wx < ex && wy >= 0 && wy < ey && wz >= 0 && wz < ez) {
      const int cells = ex * ey * ez;
      const int c = (wx * ey + wy) * ez + wz;
#pragma unroll
      for (int d = 0; d < L::D; ++d) {
        const T gc = VS_IN_RANGE(c, cells, P.status) ? P.gw[d * cells + c] : T(0);
        g[d] = has_g ? g[d] + gc : gc;
      }
      has_g = true;
    }
  }

  // Guo forcing uses the half-force corrected velocity in the equilibrium
  // (examples/2d/poiseuille_channel.py:103-105); EDM uses the plain one.
  T ue[3] = {u[0], u[1], u[2]};
  const bool guo = has_g && (P.forcing == VS_FORCE_GUO_BGK || P.forcing == VS_FORCE_GUO_MRT);
  if (guo) {
#pragma unroll
    for (int d = 0; d < L::D; ++d) ue[d] = u[d] + (g[d] * T(0.5)) / rho;
  }
  T feq[Q];
  fast::equilibrium<L>(rho, ue, feq);
  fast::collide<L, COLL>(f, feq, P.cp, P.op);

  if (has_g && P.forcing != VS_FORCE_NONE) {
    if (P.forcing == VS_FORCE_EDM) {
#pragma unroll
      for (int i = 0; i < Q; ++i) f[i] = f[i] + guo_i(L{}, i, g, u);
    } else if (P.forcing == VS_FORCE_GUO_BGK) {
#pragma unroll
      for (int i = 0; i < Q; ++i) f[i] = f[i] + guo_i(L{}, i, g, ue) * P.guo_scale;
    } else {
      T gl[Q];
#pragma unroll
      for (int i = 0; i < Q; ++i) gl[i] = guo_i(L{}, i, g, ue);
#pragma unroll
      for (int i = 0; i < Q; ++i) {
        T acc = P.fop[i * Q] * gl[0];
#pragma unroll
        for (int j = 1; j < Q; ++j) acc = acc + P.fop[i * Q + j] * gl[j];
        f[i] = f[i] + acc;
      }
    }
  }

  // keep the pre-stream populations of bounce-back faces (lbm/boundary/bb.py needs them)
  if constexpr ((FEAT & kFeatPre) != 0) for (int k = 0; k < P.n_pre; ++k) {
    const int loc = P.pre_loc[k];
    const int a = loc_axis(loc);
    const int coord = a == 0 ? x : (a == 1 ? y : z);
    const int nn[3] = {P.nx, P.ny, P.nz};
    if (coord != (loc_sign(loc) > 0 ? 0 : nn[a] - 1)) continue;
    const int b0 = a == 0 ? 1 : 0, b1 = a == 2 ? 1 : 2;
    const int cc[3] = {x, y, z};
    const int64_t nf = face_size(loc, nn);
    const int64_t j = (int64_t)cc[b0] * nn[b1] + cc[b1];
#pragma unroll
    for (int i = 0; i < Q; ++i)
      if (VS_IN_RANGE(j, nf, P.status)) P.pre_buf[k][i * nf + j] = f[i];
  }

  // push streaming with periodic wrap on every axis (lbm/basic.py:60-85):
  // destination = p + per-axis offsets, each offset wrapping at the domain edge
  const int dxp = x == P.nx - 1 ? -(P.nx - 1) * syz : syz;
  const int dxm = x == 0 ? (P.nx - 1) * syz : -syz;
  const int dyp = y == P.ny - 1 ? -(P.ny - 1) * P.nz : P.nz;
  const int dym = y == 0 ? (P.ny - 1) * P.nz : -P.nz;
  const int dzp = z == P.nz - 1 ? -(P.nz - 1) : 1;
  const int dzm = z == 0 ? P.nz - 1 : -1;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const int cx = L::c(i, 0), cy = L::c(i, 1), cz = L::c(i, 2);
    const int d = (cx > 0 ? dxp : (cx < 0 ? dxm : 0)) + (cy > 0 ? dyp : (cy < 0 ? dym : 0)) +
                  (cz > 0 ? dzp : (cz < 0 ? dzm : 0));
    if (VS_IN_RANGE(p + d, P.n, P.status)) pop_store<FEAT>(P.fout + (size_t)i * P.n + (p + d), f[i]);
  }
}

// One thread per node.  blockIdx.y = x; blockIdx.x = (y, chunk of the contiguous axis)
// in 3-D or the chunk of y in 2-D; threads run along the contiguous axis, so every load
// and store of a warp covers 32 consecutive addresses.  Wrap-around offsets of the push
// are per-block uniform except along the contiguous axis.
// With nreg > 0 the launch rows walk a list of regions instead of the whole grid.
// One block of the grid kernel: block (bx, by) of the launch geometry set up by
// enqueue_grid (bx: chunk along the contiguous axis [x (y, chunk) in 3-D], by: row).
// Nodes another launch updates: the body's box, the body's predicted window, the wall planes.
template <class L, typename T>
__device__ __forceinline__ bool skipped(const StepParams<L, T>& P, int x, int y, int z) {
  if (P.skip_box && x >= P.box[0] && x < P.box[1] && y >= P.box[2] && y < P.box[3] && z >= P.box[4] &&
      z < P.box[5])
    return true;
  if (P.dyn_meta) {
    const int bx = P.dyn_meta[P.dyn_slot ? META_PX2 : META_PX] - 1, by = P.dyn_meta[P.dyn_slot ? META_PY2 : META_PY] - 1;
    if (x >= bx && x < bx + P.dyn_ext[0] && y >= by && y < by + P.dyn_ext[1]) return true;
  }
  return P.skip_walls && (x == 0 || x == P.nx - 1);
}

// (tid, width): the thread's index in a group of `width` threads that works as one block of
// the launch geometry (the block itself in the grid kernels; a part of a CTA in the
// persistent run kernel).
template <class L, typename T, int COLL, int FEAT>
__device__ __forceinline__ void step_block_t(const StepParams<L, T>& P, int bx, int by, int tid, int width) {
  constexpr int Q = L::Q;
  int x, y, z;
  if (!(FEAT & kFeatSkip) || P.nreg == 0) {
    x = by;
    if constexpr (L::D == 2) {
      y = bx * width + tid;
      if (y >= P.ny) return;
      z = 0;
    } else {
      y = bx / P.chunks;
      z = (bx - y * P.chunks) * width + tid;
      if (z >= P.nz) return;
    }
  } else {
    const int r = by;
    const int g = (r >= P.rowstart[1]) + (r >= P.rowstart[2]);
    const int* R = P.reg[g];
    x = R[0] + (r - P.rowstart[g]);
    if constexpr (L::D == 2) {
      y = R[2] + bx * width + tid;
      if (y >= R[3]) return;
      z = 0;
    } else {
      const int cy = bx / P.chunks;
      y = R[2] + cy;
      z = R[4] + (bx - cy * P.chunks) * width + tid;
      if (y >= R[3] || z >= R[5]) return;
    }
  }
  if ((FEAT & kFeatSkip) && skipped(P, x, y, z)) return;

  const int p = (x * P.ny + y) * P.nz + z;
  T f[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) f[i] = VS_IN_RANGE(p, P.n, P.status) ? pop_load<FEAT>(P.fin + (size_t)i * P.n + p) : T(0);
  step_node<L, T, COLL, FEAT>(P, x, y, z, p, f);
}

template <class L, typename T, int COLL, int FEAT>
__device__ __forceinline__ void step_block(const StepParams<L, T>& P, int bx, int by) {
  step_block_t<L, T, COLL, FEAT>(P, bx, by, (int)threadIdx.x, (int)blockDim.x);
}

// A D2Q9 block of the whole grid with two nodes per thread, `width` apart along y: both
// nodes' populations are loaded before either is updated, which doubles the loads in flight
// per thread.  No regions.
template <typename T, int COLL, int FEAT>
__device__ __forceinline__ void step_block2_t(const StepParams<L9, T>& P, int bx, int by, int tid, int width) {
  const int x = by;
  const int y0 = bx * 2 * width + tid, y1 = y0 + width;
  const bool a = y0 < P.ny && !((FEAT & kFeatSkip) && skipped(P, x, y0, 0));
  const bool b = y1 < P.ny && !((FEAT & kFeatSkip) && skipped(P, x, y1, 0));
  const int p0 = x * P.ny + y0, p1 = x * P.ny + y1;
  T f0[9], f1[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    if (a) f0[i] = VS_IN_RANGE(p0, P.n, P.status) ? pop_load<FEAT>(P.fin + (size_t)i * P.n + p0) : T(0);
    if (b) f1[i] = VS_IN_RANGE(p1, P.n, P.status) ? pop_load<FEAT>(P.fin + (size_t)i * P.n + p1) : T(0);
  }
  if (a) step_node<L9, T, COLL, FEAT>(P, x, y0, 0, p0, f0);
  if (b) step_node<L9, T, COLL, FEAT>(P, x, y1, 0, p1, f1);
}

template <typename T, int COLL, int FEAT>
__device__ __forceinline__ void step_block2(const StepParams<L9, T>& P, int bx, int by) {
  step_block2_t<T, COLL, FEAT>(P, bx, by, (int)threadIdx.x, (int)blockDim.x);
}

// NPT nodes per thread, `width` apart along y, all NPT nodes' populations loaded before the
// first is updated (the loads in flight of NPT threads).  No regions.
template <typename T, int COLL, int FEAT, int NPT>
__device__ __forceinline__ void step_block_n_t(const StepParams<L9, T>& P, int bx, int by, int tid, int width) {
  const int x = by;
  bool on[NPT];
  int pp[NPT];
  T f[NPT][9];
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    const int y = (bx * NPT + k) * width + tid;
    on[k] = y < P.ny && !((FEAT & kFeatSkip) && skipped(P, x, y, 0));
    pp[k] = x * P.ny + y;
  }
#pragma unroll
  for (int i = 0; i < 9; ++i)
#pragma unroll
    for (int k = 0; k < NPT; ++k)
      if (on[k]) f[k][i] = VS_IN_RANGE(pp[k], P.n, P.status) ? pop_load<FEAT>(P.fin + (size_t)i * P.n + pp[k]) : T(0);
#pragma unroll
  for (int k = 0; k < NPT; ++k)
    if (on[k]) step_node<L9, T, COLL, FEAT>(P, x, (bx * NPT + k) * width + tid, 0, pp[k], f[k]);
}

// The main launch of a batch walks each case's nodes in memory order: chunk j of a
// case is nodes [j * blockDim.x, (j + 1) * blockDim.x) of its flattened grid, so a block is
// full whatever the case's row length (rows of 64 nodes would leave 3/4 of a 256-thread
// block idle) and a warp still reads 32 consecutive addresses.
template <class L, typename T, int COLL, int FEAT>
__device__ __forceinline__ void step_flat(const StepParams<L, T>& P, int chunk) {
  const int p = chunk * (int)blockDim.x + (int)threadIdx.x;
  if (p >= P.n) return;
  int x, y, z;
  if constexpr (L::D == 2) {
    x = p / P.ny;
    y = p - x * P.ny;
    z = 0;
  } else {
    const int syz = P.ny * P.nz;
    x = p / syz;
    const int r = p - x * syz;
    y = r / P.nz;
    z = r - y * P.nz;
  }
  if ((FEAT & kFeatSkip) && skipped(P, x, y, z)) return;
  T f[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i] = VS_IN_RANGE(p, P.n, P.status) ? __ldg(P.fin + (size_t)i * P.n + p) : T(0);
  step_node<L, T, COLL, FEAT>(P, x, y, z, p, f);
}

// step_flat with two nodes per thread, blockDim.x apart in memory order (chunk j of the
// case: nodes [2 j blockDim.x, 2 (j + 1) blockDim.x)); both nodes' populations are loaded
// before either is updated.
template <class L, typename T, int COLL, int FEAT>
__device__ __forceinline__ void step_flat2(const StepParams<L, T>& P, int chunk) {
  int p[2], x[2], y[2], z[2];
  bool on[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    p[k] = (2 * chunk + k) * (int)blockDim.x + (int)threadIdx.x;
    on[k] = p[k] < P.n;
    if constexpr (L::D == 2) {
      x[k] = p[k] / P.ny;
      y[k] = p[k] - x[k] * P.ny;
      z[k] = 0;
    } else {
      const int syz = P.ny * P.nz;
      x[k] = p[k] / syz;
      const int r = p[k] - x[k] * syz;
      y[k] = r / P.nz;
      z[k] = r - y[k] * P.nz;
    }
    on[k] = on[k] && !((FEAT & kFeatSkip) && skipped(P, x[k], y[k], z[k]));
  }
  T f[2][L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i)
#pragma unroll
    for (int k = 0; k < 2; ++k)
      if (on[k]) f[k][i] = VS_IN_RANGE(p[k], P.n, P.status) ? __ldg(P.fin + (size_t)i * P.n + p[k]) : T(0);
#pragma unroll
  for (int k = 0; k < 2; ++k)
    if (on[k]) step_node<L, T, COLL, FEAT>(P, x[k], y[k], z[k], p[k], f[k]);
}

}  // namespace vs
