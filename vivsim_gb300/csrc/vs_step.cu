// Fused IB-LBM time step (D2Q9 / D3Q19).
//
// One step of the reference's composed update loop
//   rho,u = get_macroscopic(f); feq = get_equilibrium(rho,u); f = collision(f,feq)
//   IB: markers -> stencil -> multi_direct_forcing -> Newmark;  f += forcing(g, u)
//   f = streaming(f); f = boundary_k(f) for each face boundary in order
// (examples/2d/vortex_induced_vibration.py:96-148, examples/2d/lid_driven_cavity.py:55-63,
//  examples/3d/flow_past_sphere.py:139-180) runs as
//   [body kernel]  markers, stencil, CSR, MDF, Newmark -> force window g (device)
//   [grid kernel]  per node: load f (1 read/population), moments, equilibrium, collision,
//                  forcing from g, push-stream to the neighbours (1 write/population)
//   [face kernels] the ordered boundary conditions on the streamed populations
// The grid kernel carries all of the HBM traffic; the other two touch O(surface) nodes.
#include <cooperative_groups.h>
#include <cuda.h>
#include <cudaTypedefs.h>

#include <climits>
#include <cstring>
#include <cmath>
#include <cstdlib>
#include <new>
#include <type_traits>
#include <algorithm>
#include <vector>

#include "vs_boundary.cuh"
#include "vs_dispatch.cuh"
#include "vs_fast.cuh"
#include "vs_grid.cuh"
#include "vs_ib.cuh"

namespace vs {

template <class L, typename T, int COLL, bool WALLS>
__global__ void __launch_bounds__(256) k_step(const __grid_constant__ StepParams<L, T> P) {
  step_block<L, T, COLL, WALLS ? (kFeatGeneral | kFeatWalls) : kFeatGeneral>(P, blockIdx.x, blockIdx.y);
}

// The grid launches that read no per-node feature beyond (FEAT = kFeatSkip) the tests for
// nodes another launch updates: the bulk of every HBM-bound step.  Compiled without the
// force window, the load-time boundaries, the obstacle mask and the pre-stream copies, they
// need fewer registers, and the launch shape below holds more loads in flight per SM.
// FastShape: threads per block, resident blocks per SM (a register cap) and nodes per
// thread (D2Q9: two nodes blockDim apart along y), chosen by timing the 8192^2 D2Q9 and
// 256 x 128 x 128 / 512 x 256 x 256 D3Q19 grids on GB300.
// Measured (fraction of the measured copy bandwidth at 72 / 152 B per node): D2Q9 KBC two
// nodes x 128 threads, 8 blocks 0.90; D2Q9 BGK and MRT 256 threads, 8 blocks 0.99 and 0.93;
// D3Q19 BGK and REG 128 threads, 10 blocks 0.96 and 0.95; D3Q19 KBC 64 threads, 16 blocks
// 0.80 (the general kernel: 0.69-0.83).
// MINB_SKIP: the D2Q9 launch beside a 2-D body (the skip tests compiled in) holds 6 blocks
// per SM: the VIV step (1024 x 512, KBC) replays at 13.3 us against 14.0 us with 8, its
// bulk launch alone taking the same 8.7 us either way.
template <class L, int COLL>
struct FastShape {
  static constexpr bool heavy3 = L::Q == 19 && (COLL == VS_COLLIDE_KBC || COLL == VS_COLLIDE_MRT);
  static constexpr int NPT = (L::Q == 9 && COLL == VS_COLLIDE_KBC) ? 2 : 1;
  static constexpr int TB = L::Q == 9 ? (NPT == 2 ? 128 : 256) : (heavy3 ? 64 : 128);
  static constexpr int MINB = L::Q == 9 ? 8 : (heavy3 ? 16 : 10);
  static constexpr int MINB_SKIP = L::Q == 9 ? 6 : MINB;
};

template <class L, typename T, int COLL, int FEAT>
__global__ void __launch_bounds__(FastShape<L, COLL>::TB,
                                  (FEAT & kFeatSkip) ? FastShape<L, COLL>::MINB_SKIP : FastShape<L, COLL>::MINB)
    k_step_fast(const __grid_constant__ StepParams<L, T> P) {
  if constexpr (FastShape<L, COLL>::NPT == 2) step_block2<T, COLL, FEAT>(P, blockIdx.x, blockIdx.y);
  else step_block<L, T, COLL, FEAT>(P, blockIdx.x, blockIdx.y);
}

// (6 blocks of 256 threads per SM by registers: at the default 48 registers the loads in
// flight were too few, 5 % slower on the 64-case sweep; 8 blocks spill)
// FEAT: kFeatGeneral, or kFeatSkip when no case of the batch has a uniform body force,
// pre-stream copies or an obstacle mask (the usual sweep).
template <class L, typename T, int COLL, int FEAT>
__global__ void __launch_bounds__(256, 6) k_step_batch_flat(const StepParams<L, T>* __restrict__ Ps,
                                                         const int2* __restrict__ blk) {
  const int2 cb = blk[blockIdx.x];
  step_flat<L, T, COLL, FEAT>(Ps[cb.x], cb.y);
}

// Two nodes per thread (the loads of two nodes in flight; 4 blocks of 256 threads per SM).
template <class L, typename T, int COLL, int FEAT>
__global__ void __launch_bounds__(256, 4) k_step_batch_flat2(const StepParams<L, T>* __restrict__ Ps,
                                                          const int2* __restrict__ blk) {
  const int2 cb = blk[blockIdx.x];
  step_flat2<L, T, COLL, FEAT>(Ps[cb.x], cb.y);
}

// Grid kernel over many independent lattices in one launch: block b works on lattice
// blk[b].x, as block blk[b].y of that lattice's own launch geometry (chunks x rows,
// row-major), with that lattice's parameters (the batch's region launch).
template <class L, typename T, int COLL, bool WALLS>
__global__ void __launch_bounds__(256) k_step_batch(const StepParams<L, T>* __restrict__ Ps,
                                                    const int2* __restrict__ blk) {
  const int2 cb = blk[blockIdx.x];
  const StepParams<L, T>& P = Ps[cb.x];  // read through L1 (staging it in shared memory cost registers)
  const int by = cb.y / P.gx;
  step_block<L, T, COLL, WALLS ? (kFeatGeneral | kFeatWalls) : kFeatGeneral>(P, cb.y - by * P.gx, by);
}


// ------------------------------------------------------------------ TMA-pipelined grid kernel
// Persistent variant of k_step for the bulk of the grid.  A tile is TB consecutive nodes of
// one row along the contiguous axis; CTA b processes tiles b, b + gridDim.x, ...  For every
// tile, lane i < Q of warp 0 copies population i's TB contiguous values into a stage of a
// shared-memory ring with cp.async.bulk (TMA); an mbarrier per stage counts the bytes.
// NS stages are in flight per CTA, so the bytes in flight no longer scale with the
// registers of a thread.  All waits are bounded: on a timeout the CTA records
// VS_ERR_TIMEOUT in *P.status, drains its copies (bounded) and exits.
namespace tma {

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// true once the barrier has completed the phase with this parity; bounded spin
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int limit) {
  const unsigned a = smem_addr(bar);
  for (int it = 0; it < limit; ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace tma

constexpr int kTmaStages = 4;
constexpr int kTmaWaitLimit = 1 << 22;   // try_wait suspends in hardware between polls
constexpr int kTmaDrainLimit = 1 << 24;  // second wait, for copies already issued, after a timeout

// A block whose wait gave up must not leave while a bulk copy it issued may still write
// its shared memory.  No copy is issued after a failed wait, so only copies already
// counted by the barrier can be outstanding: wait for them once more (bounded).  Returns
// the status to record: VS_ERR_TIMEOUT when they landed, VS_ERR_TIMEOUT_INFLIGHT when
// one still had not (it may land after the block has left).
__device__ __forceinline__ int tma_drain(uint64_t* bar, unsigned parity) {
  return tma::mbar_wait(bar, parity, kTmaDrainLimit) ? VS_ERR_TIMEOUT : VS_ERR_TIMEOUT_INFLIGHT;
}

// Self-test of the bounded waits: an mbarrier expects 16 bytes that no copy delivers (no
// copy is in flight), the wait gives up after `limit` polls and the kernel reports
// VS_ERR_TIMEOUT, as the grid and body kernels do when their staged copies never land.
__global__ void k_selftest_wait(int* status, int limit) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar, 1);
    tma::fence_init();
    tma::mbar_expect_tx(&bar, 16);
    *status = tma::mbar_wait(&bar, 0, limit) ? VS_OK : VS_ERR_TIMEOUT;
  }
}

template <class L, typename T, int COLL, int TB>
__global__ void __launch_bounds__(TB) k_step_tma(const __grid_constant__ StepParams<L, T> P, int tiles,
                                                 int tiles_per_row, int* status) {
  constexpr int Q = L::Q;
  constexpr unsigned STAGE_BYTES = Q * TB * sizeof(T);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* buf = (T*)smem_raw;                                       // [NS][Q][TB]
  uint64_t* full = (uint64_t*)(smem_raw + kTmaStages * STAGE_BYTES);
  const int tid = threadIdx.x;
  const int nl = L::D == 2 ? P.ny : P.nz;  // contiguous extent

  auto tile_base = [&](int t) -> long long {
    const int row = t / tiles_per_row, col = t - row * tiles_per_row;
    return (long long)row * nl + (long long)col * TB;
  };
  auto issue = [&](int stage, int t) {  // called by warp 0
    const int lane = tid & 31;
    if (lane == 0) tma::mbar_expect_tx(&full[stage], STAGE_BYTES);
    __syncwarp();
    const long long base = tile_base(t);
    for (int i = lane; i < Q; i += 32)
      tma::bulk_load(buf + ((size_t)stage * Q + i) * TB, P.fin + (size_t)i * P.n + base, TB * sizeof(T),
                     &full[stage]);
  };

  if (tid == 0) {
    for (int s2 = 0; s2 < kTmaStages; ++s2) tma::mbar_init(&full[s2], 1);
    tma::fence_init();
  }
  __syncthreads();
  if (tid < 32)
    for (int s2 = 0; s2 < kTmaStages; ++s2) {
      const int t = blockIdx.x + s2 * gridDim.x;
      if (t < tiles) issue(s2, t);
    }

  int k = 0;
  for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++k) {
    const int stage = k % kTmaStages;
    const unsigned parity = (unsigned)((k / kTmaStages) & 1);
    const bool ok = tma::mbar_wait(&full[stage], parity, kTmaWaitLimit);
    if (__syncthreads_or(!ok)) {
      // some copy never completed: no stage is refilled past this point; drain the stages
      // already issued (this one and the next kTmaStages - 1 tiles), report, leave
      if (tid == 0) {
        int st = VS_ERR_TIMEOUT;
        for (int j = 0; j < kTmaStages; ++j) {
          const int tj = t + j * gridDim.x;
          if (tj < tiles && tma_drain(&full[(k + j) % kTmaStages], (unsigned)(((k + j) / kTmaStages) & 1)) !=
                                VS_ERR_TIMEOUT)
            st = VS_ERR_TIMEOUT_INFLIGHT;
        }
        atomicMax(status, st);
      }
      return;
    }
    T f[Q];
    const T* sb = buf + (size_t)stage * Q * TB;
#pragma unroll
    for (int i = 0; i < Q; ++i) f[i] = sb[i * TB + tid];
    __syncthreads();  // the stage has been read by every thread: refill it
    if (tid < 32) {
      const int tn = t + kTmaStages * gridDim.x;
      if (tn < tiles) issue(stage, tn);
    }
    const long long base = tile_base(t);
    const int p = (int)base + tid;
    int x, y, z;
    if constexpr (L::D == 2) {
      x = (int)(base / P.ny);
      y = (int)(base - (long long)x * P.ny) + tid;
      z = 0;
    } else {
      const int row = (int)(base / P.nz);
      x = row / P.ny;
      y = row - x * P.ny;
      z = (int)(base - (long long)row * P.nz) + tid;
    }
    if (P.skip_box && x >= P.box[0] && x < P.box[1] && y >= P.box[2] && y < P.box[3] && z >= P.box[4] &&
        z < P.box[5])
      continue;
    if (P.skip_walls && (x == 0 || x == P.nx - 1)) continue;
    step_node<L, T, COLL, kFeatGeneral>(P, x, y, z, p, f);
  }
}

// ------------------------------------------------------------------ face kernels
template <typename T>
struct BcGroup {
  int count;
  int64_t nf[2];
  WallArgs<T> A[2];
};

template <class L, typename T>
__global__ void k_bc(const __grid_constant__ BcGroup<T> G, T* f) {
  const int g = blockIdx.y;
  if (g >= G.count) return;
  const WallArgs<T>& A = G.A[g];
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= G.nf[g]) return;
  const int64_t n = (int64_t)A.n[0] * A.n[1] * A.n[2];
  const int64_t pw = face_node(A.loc, A.n, j, 0);
  T w[L::Q], nb[L::Q], pre[L::Q], out[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) w[i] = f[i * n + pw];
  if (bc_needs_neighbor<L>(A.kind, A.mode)) {
    const int64_t pn = face_node(A.loc, A.n, j, 1);
#pragma unroll
    for (int i = 0; i < L::Q; ++i) nb[i] = f[i * n + pn];
  }
  if (A.kind == VS_BC_BB || A.kind == VS_BC_SPECULAR) {
#pragma unroll
    for (int i = 0; i < L::Q; ++i) pre[i] = A.f_pre[i * A.pre_stride + j];
  }
  bc_node<L, T>(A, j, w, nb, pre, out);
#pragma unroll
  for (int i = 0; i < L::Q; ++i) f[i * n + pw] = out[i];
}

// ------------------------------------------------------------------ body kernel (2-D)
template <typename T>
struct BodyParams {
  const T* fin;
  const T* X0;
  const T* Y0;
  const T* ds_arr;
  T* state;  // a[3], v[3], d[3], h[3]
  T* base;   // fluid-structure sub-iterations: the step's saved a[3], v[3], d[3] (else null)
  int fsi_first;  // with base: this pass saves the state it starts from into base
  T* gw;
  int* meta;
  T* force_hist;
  int nx, ny;
  int M, kernel, n_iter;
  int chain_k;       // chain kernel: markers share stencil nodes only within +-chain_k (cyclic)
  int pred_slot;     // prediction slot to read (the cluster form writes the other one)
  int cap_x, cap_y;  // window region: (cap_x + 2) x (cap_y + 2) cells from the predicted corner
  int row_len;       // staged row length (multiple of 16 bytes), the TMA box's inner extent
  int bulk;          // stage the region with one tensor-map TMA copy
  int box[4];        // the window must stay inside x0..x1, y0..y1 (half-open)
  int free_dof[3];
  int rot;           // free rotation about (cx, cy): DOF 2 is the angle
  T ds2_scalar;      // 2 * ds as the reference forms it: (T)ds * 2
  T k1, k2, c1, c2, dt, damp, stiff, den, area;
  T cx, cy;                                   // initial centre of the body
  T rot_damp, rot_stiff, rot_den, rot_added;  // rotational Newmark constants, added inertia
  CUtensorMap map;   // f as a (ny, nx, 9) tensor, box (row_len, cap_x + 2, 9)
};

constexpr int kBodyThreads = 512;

// Rigid 2-D body kinematics (vivsim/dyn.py:68-120): the markers translate with d
// (get_markers_coords_2dof) or, with the rotation free, also turn by d[2] about the initial
// centre (get_markers_coords_3dof) and move with get_markers_velocity_3dof.  Products and
// sums are rounded one at a time in the reference's order.
template <typename T>
struct Kin2 {
  T d0, d1, v0, v1, v2, cs, sn, cx, cy;
  int rot;
  __device__ __forceinline__ Kin2(const BodyParams<T>& B, const T* d, const T* v)
      : d0(d[0]), d1(d[1]), v0(v[0]), v1(v[1]), v2(v[2]), cs(T(1)), sn(T(0)), cx(B.cx), cy(B.cy), rot(B.rot) {
    if (rot) {
      cs = cos(d[2]);
      sn = sin(d[2]);
    }
  }
  // marker position
  __device__ __forceinline__ void xy(const BodyParams<T>& B, int m, T& x, T& y) const {
    if (!rot) {
      x = B.X0[m] + d0;
      y = B.Y0[m] + d1;
      return;
    }
    const T xr = sub_rn(B.X0[m], cx), yr = sub_rn(B.Y0[m], cy);
    x = sub_rn(add_rn(add_rn(cx, d0), mul_rn(xr, cs)), mul_rn(yr, sn));
    y = add_rn(add_rn(add_rn(cy, d1), mul_rn(xr, sn)), mul_rn(yr, cs));
  }
  // MDF target velocity of a marker at (x, y), component c
  __device__ __forceinline__ T target(T x, T y, int c) const {
    if (!rot) return c == 0 ? v0 : v1;
    if (c == 0) return sub_rn(v0, mul_rn(v2, sub_rn(sub_rn(y, cy), d1)));
    return add_rn(v1, mul_rn(v2, sub_rn(sub_rn(x, cx), d0)));
  }
  __device__ __forceinline__ T target(const BodyParams<T>& B, int m, int c) const {
    if (!rot) return c == 0 ? v0 : v1;
    T x, y;
    xy(B, m, x, y);
    return target(x, y, c);
  }
};

// Warp 0 ends the body step: the force h = sum_m(-F_total) in a fixed tree (dyn.py:126-136);
// with the rotation free, the torque sum_m(x_rel h_y - y_rel h_x) (dyn.py:139-154); added
// mass h += a A (vortex_induced_vibration.py:136) and added inertia; Newmark per free DOF
// (dyn.py:5-51).  Ft holds every marker's total MDF force; a, v, d the state this pass
// started from.  With fluid-structure sub-iterations (B.base) the added mass uses that
// latest a while Newmark restarts from the step's saved state, as the reference's
// `for _ in range(FSI_ITER)` loop does (examples/2d/vortex_induced_vibration.py:114-139).
template <typename T>
__device__ __forceinline__ void body2d_finish(const BodyParams<T>& B, const Kin2<T>& K, const T* Ft, int M,
                                              const T* a, const T* v, const T* d, T* hist) {
  const int tid = threadIdx.x;
  T h[3];
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    T acc = T(0);
    for (int m = tid; m < M; m += 32) acc = m == tid ? -Ft[2 * m + c] : acc + (-Ft[2 * m + c]);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc = acc + __shfl_down_sync(0xffffffffu, acc, o);
    h[c] = acc;
  }
  h[2] = T(0);
  if (K.rot) {
    const T ox = add_rn(K.cx, K.d0), oy = add_rn(K.cy, K.d1);
    T acc = T(0);
    for (int m = tid; m < M; m += 32) {
      T x, y;
      K.xy(B, m, x, y);
      const T t = sub_rn(mul_rn(sub_rn(x, ox), -Ft[2 * m + 1]), mul_rn(sub_rn(y, oy), -Ft[2 * m]));
      acc = m == tid ? t : acc + t;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc = acc + __shfl_down_sync(0xffffffffu, acc, o);
    h[2] = acc;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) h[c] = __shfl_sync(0xffffffffu, h[c], 0);
  if (tid < 3) {
    const int c = tid;
    if (c == 2 && !K.rot) {
      B.state[9 + 2] = T(0);
      if (hist) hist[2] = T(0);
      return;
    }
    // selects, not indexing by the thread: the state stays in registers
    const T ac = c == 0 ? a[0] : (c == 1 ? a[1] : a[2]);
    const T vc = c == 0 ? v[0] : (c == 1 ? v[1] : v[2]);
    const T dc = c == 0 ? d[0] : (c == 1 ? d[1] : d[2]);
    const T hc = c == 0 ? h[0] : (c == 1 ? h[1] : h[2]);
    const T hh = add_rn(hc, mul_rn(ac, c < 2 ? B.area : B.rot_added));
    T ab = ac, vb = vc, db = dc;  // Newmark's starting state
    if (B.base) {
      if (B.fsi_first) {
        B.base[c] = ac;
        B.base[3 + c] = vc;
        B.base[6 + c] = dc;
      } else {
        ab = B.base[c];
        vb = B.base[3 + c];
        db = B.base[6 + c];
      }
    }
    T an = ab, vn = vb, dn = db;
    if (B.free_dof[c]) {
      const T damp = c < 2 ? B.damp : B.rot_damp, stiff = c < 2 ? B.stiff : B.rot_stiff;
      const T den = c < 2 ? B.den : B.rot_den;
      const T v1 = add_rn(vb, mul_rn(B.k1, ab));
      const T v2 = add_rn(add_rn(db, mul_rn(B.dt, vb)), mul_rn(B.k2, ab));
      an = sub_rn(sub_rn(hh, mul_rn(damp, v1)), mul_rn(stiff, v2)) / den;
      vn = add_rn(mul_rn(B.c1, an), v1);
      dn = add_rn(mul_rn(B.c2, an), v2);
    }
    B.state[c] = an;
    B.state[3 + c] = vn;
    B.state[6 + c] = dn;
    B.state[9 + c] = hh;
    if (hist) hist[c] = hh;
  }
}

template <typename T>
__device__ __forceinline__ void body2d_finish(const BodyParams<T>& B, const Kin2<T>& K, const T* Ft, int M,
                                              const T* a, const T* v, const T* d) {
  body2d_finish<T>(B, K, Ft, M, a, v, d, B.force_hist);
}

// Block scan over the window cells: cnt[k] pairs per cell -> CSR.  Writes, per cell,
// the scatter cursor (first sorted position, into cnt[]) and the touched-node slot (or -1,
// into cslot[]); per touched slot j its cell tcell[j] and first position tstart[j]
// (tstart[NT] = total).  Returns the number of touched cells.
__device__ int block_csr_scan(int* cnt, int* cslot, int* tcell, int* tstart, int B, int* warp_sums) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int chunk = (B + nt - 1) / nt;
  const int lo = min(B, tid * chunk), hi = min(B, lo + chunk);
  int local = 0;  // pairs in the low half-word, touched cells in the high one
  for (int k = lo; k < hi; ++k) local += cnt[k] + (cnt[k] > 0 ? 65536 : 0);
  const int lane = tid & 31, wid = tid >> 5;
  int v = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) warp_sums[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (nt + 31) >> 5;
    int sum = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, sum, o);
      if (lane >= o) sum += t;
    }
    if (lane < nw) warp_sums[lane] = sum;
  }
  __syncthreads();
  int run = v - local + (wid > 0 ? warp_sums[wid - 1] : 0);
  for (int k = lo; k < hi; ++k) {
    const int c = cnt[k];
    const int pos = run & 0xffff, j = run >> 16;
    cnt[k] = pos;
    if (c > 0) {
      cslot[k] = j;
      tcell[j] = k;
      tstart[j] = pos;
    } else {
      cslot[k] = -1;
    }
    run += c + (c > 0 ? 65536 : 0);
  }
  const int total = warp_sums[((nt + 31) >> 5) - 1];
  if (tid == 0) tstart[total >> 16] = total & 0xffff;
  return total >> 16;
}

// interpolation of node values to the markers, LN lanes per (marker, component):
// lane l sums its contiguous share of the stencil in order, the shares are then
// combined in a fixed pattern, so the result is deterministic.
template <typename T, int S, int LN>
__device__ __forceinline__ T interp_group(const T* W, const int* slot, const T* nodes, int m) {
  const int sub = threadIdx.x & (LN - 1);
  constexpr int PER = S / LN;
  T acc = T(0);
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int s = sub * PER + j;
    const T t = mul_rn(W[m * S + s], nodes[slot[m * S + s]]);
    acc = j == 0 ? t : add_rn(acc, t);
  }
  if constexpr (LN > 1) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned mask = ((1u << LN) - 1u) << (lane & ~(unsigned)(LN - 1));
#pragma unroll
    for (int o = LN / 2; o >= 1; o >>= 1) acc = acc + __shfl_down_sync(mask, acc, o, LN);
  }
  return acc;
}

// One CTA advances one 2-D rigid body by one step: marker positions from the body
// displacement, stencil weights, a counting-sort CSR of (node, pair) in shared memory,
// interpolation of u from f at the touched nodes, the multi-direct-forcing iterations,
// the force window for the grid kernel, the total force and the Newmark update.
// Each touched node keeps its contributions in increasing (marker, stencil point) order,
// the order of the reference's scatter-add; no floating-point atomics are used.
//
// Latency layout: one global round trip up front (body state, last bounding-box corner,
// marker coordinates).  The window region is predicted from the last corner (one node of
// slack per side, the body moves less than a node per step), so stencil keys need no
// block-wide bounding-box reduction, and the region's populations are staged into shared
// memory by bulk copies (TMA) issued by warp 0 while the CSR is built.
// The last MDF iteration only adds its force step: its spread and interpolation feed a
// marker velocity that the reference computes and then discards (ib/mdf.py:57-64).
template <typename T, int R>
__global__ void __launch_bounds__(kBodyThreads) k_body2d(const __grid_constant__ BodyParams<T> B) {
  constexpr int WD = 2 * R, S = WD * WD;
  constexpr int LN = S >= 16 ? 4 : 1;
  constexpr int AL = 16 / sizeof(T);  // elements per 16 bytes
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int M = B.M, P = M * S;
  const int EX = B.cap_x + 2, EY = B.cap_y + 2, NB = EX * EY, RL = B.row_len;
  T* fwin = (T*)smem;             // staged populations [9][EX][RL]
  T* wx = fwin + 9 * EX * RL;     // per marker: 2R one-dimensional weights along x
  T* wy = wx + WD * M;            //                              ... along y
  T* W = wy + WD * M;
  T* U = W + P;
  T* Fs = U + 2 * M;
  T* Ft = Fs + 2 * M;
  T* nu = Ft + 2 * M;             // per touched node: u [2][NB]
  T* nv = nu + 2 * NB;            // per touched node: 0.5 spread(F_step) [2][NB]
  int* key = (int*)(nv + 2 * NB); // pair -> region cell
  int* slot = key + P;            // pair -> touched-node slot
  int* sorted = slot + P;         // pairs grouped by touched node, in pair order
  int* cnt = sorted + P;          // per cell: pair count, then scatter cursor
  int* cslot = cnt + NB;          // per cell: touched slot or -1
  int* tcell = cslot + NB;        // touched slot -> cell
  int* tstart = tcell + NB;       // touched slot -> first sorted position (+ end)
  int* fxy = tstart + NB + 1;     // per marker: floor(X), floor(Y)
  int* misc = fxy + 2 * M;        // [0..3] bbox, [4] out-of-region flag, [8..39] warp sums
  uint64_t* bar = (uint64_t*)(((uintptr_t)(misc + 40) + 7) & ~(uintptr_t)7);
  {
    // the layout must fit the dynamic shared memory this launch received
    unsigned have;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(have));
    if ((size_t)((const unsigned char*)(bar + 1) - smem) > have) {
      if (tid == 0) {
        B.meta[META_STATUS] = VS_ERR_INVALID_ARG;
        B.meta[META_WX] = 0; B.meta[META_WY] = 0; B.meta[META_WZ] = 0;
      }
      return;
    }
  }

  // one round trip: state, last corner, marker coordinates
  T a[3], v[3], d[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a[c] = B.state[c];
    v[c] = B.state[3 + c];
    d[c] = B.state[6 + c];
  }
  const Kin2<T> kin(B, d, v);
  const int ox = B.meta[META_PX] - 1, oy = B.meta[META_PY] - 1;  // region corner
  const int ya = oy >= 0 ? oy - oy % AL : 0;                     // 16-byte aligned row start
  const int64_t n = (int64_t)B.nx * B.ny;
  const bool region_ok = ox >= B.box[0] && oy >= B.box[2] && ox + EX <= B.box[1] && oy + EY <= B.box[3];
  const bool bulk = B.bulk && region_ok;
  if (tid == 0) {
    misc[0] = INT_MAX; misc[1] = INT_MIN; misc[2] = INT_MAX; misc[3] = INT_MIN; misc[4] = 0;
    if (bulk) {
      tma::mbar_init(bar, 1);
      tma::fence_init();
    }
  }
  if (bulk && tid == 0) {
    // the region [ya, ya + RL) x [ox, ox + EX) x all 9 populations in one tensor copy;
    // elements past the grid's edge arrive as zeros
    tma::mbar_expect_tx(bar, (unsigned)(9 * EX * RL * sizeof(T)));
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(tma::smem_addr(fwin)),
        "l"(&B.map), "r"(ya), "r"(ox), "r"(0), "r"(tma::smem_addr(bar))
        : "memory");
  }
  for (int k = tid; k < NB; k += nt) cnt[k] = 0;
  __syncthreads();
  // markers follow the body (dyn.py:68-81); the tensor-product stencil weight
  // kernel(sx - X) * kernel(sy - Y) (ib/stencil.py:44-47) is formed from the 2R one-dimensional
  // values per axis, one thread per (marker, axis, offset)
  for (int t = tid; t < M * 2 * WD; t += nt) {
    const int m = t / (2 * WD), r = t - m * (2 * WD), ax = r / WD, o = r - ax * WD;
    T px, py;
    kin.xy(B, m, px, py);
    const T xm = ax == 0 ? px : py;
    const int fx = ifloor(xm);
    (ax == 0 ? wx : wy)[m * WD + o] = delta(B.kernel, (T)(fx + o - R + 1) - xm);
    if (o == 0) {
      fxy[2 * m + ax] = fx;
      atomicMin(&misc[2 * ax], fx);
      atomicMax(&misc[2 * ax + 1], fx);
    }
  }
  __syncthreads();
  // stencil (ib/stencil.py:7-51): weights and region-local node keys; pairs per cell
  for (int p = tid; p < P; p += nt) {
    const int m = p / S, k = p - m * S, ix = k / WD, iy = k % WD;
    W[p] = wx[m * WD + ix] * wy[m * WD + iy];
    const int cx = fxy[2 * m] + ix - R + 1 - ox, cy = fxy[2 * m + 1] + iy - R + 1 - oy;
    if (cx < 0 || cx >= EX || cy < 0 || cy >= EY) {
      misc[4] = 1;
      key[p] = 0;
      continue;
    }
    const int kk = cx * EY + cy;
    key[p] = kk;
    atomicAdd(&cnt[kk], 1);
  }
  __syncthreads();
  if (misc[4] || !region_ok) {
    // the body moved a node or more in one step, or its region left the box
    // let the staged copy land before the block leaves (bounded; reported if it does not)
    if (tid == 0) {
      const bool landed = !bulk || tma::mbar_wait(bar, 0, kTmaWaitLimit) || tma_drain(bar, 0) == VS_ERR_TIMEOUT;
      B.meta[META_STATUS] = landed ? VS_ERR_RANGE : VS_ERR_TIMEOUT_INFLIGHT;
      B.meta[META_WX] = 0; B.meta[META_WY] = 0; B.meta[META_WZ] = 0;
    }
    return;
  }
  const int NT = block_csr_scan(cnt, cslot, tcell, tstart, NB, misc + 8);
  __syncthreads();
  for (int p = tid; p < P; p += nt) {
    const int kk = key[p];
    sorted[atomicAdd(&cnt[kk], 1)] = p;
    slot[p] = cslot[kk];
  }
  bool staged = true;
  if (bulk) staged = tma::mbar_wait(bar, 0, kTmaWaitLimit);
  if (__syncthreads_or(!staged)) {
    if (tid == 0) {
      B.meta[META_STATUS] = tma_drain(bar, 0);  // the copy is waited for once more before the block leaves
      B.meta[META_WX] = 0; B.meta[META_WY] = 0; B.meta[META_WZ] = 0;
    }
    return;
  }
  // order each node's pairs by pair id (= the reference's scatter order); u at the node
  for (int j = tid; j < NT; j += nt) {
    const int lo = tstart[j], hi = tstart[j + 1];
    for (int i = lo + 1; i < hi; ++i) {
      const int val = sorted[i];
      int q = i - 1;
      while (q >= lo && sorted[q] > val) {
        sorted[q + 1] = sorted[q];
        --q;
      }
      sorted[q + 1] = val;
    }
    const int k = tcell[j], cx = k / EY, cy = k - cx * EY;
    T fl[9];
    if (bulk) {
#pragma unroll
      for (int i = 0; i < 9; ++i) fl[i] = fwin[(i * EX + cx) * RL + (oy - ya) + cy];
    } else {
      const int64_t pn = (int64_t)(ox + cx) * B.ny + (oy + cy);
#pragma unroll
      for (int i = 0; i < 9; ++i) fl[i] = __ldg(B.fin + i * n + pn);
    }
    T r, uu[3];
    macro(L9{}, fl, r, uu);
    nu[j] = uu[0];
    nu[NB + j] = uu[1];
  }
  __syncthreads();
  // U = interpolate(u) and the first force step (ib/mdf.py:38-48); target = body velocity
  for (int t = tid; t < 2 * M * LN; t += nt) {
    const int q = t / LN, m = q >> 1, c = q & 1;
    const T acc = interp_group<T, S, LN>(W, slot, nu + c * NB, m);
    if ((t & (LN - 1)) == 0) {
      U[q] = acc;
      const T d2 = B.ds_arr ? B.ds_arr[m] * T(2) : B.ds2_scalar;
      const T fs = mul_rn(kin.target(B, m, c) - acc, d2);
      Fs[q] = fs;
      Ft[q] = B.n_iter > 0 ? fs : T(0);
    }
  }
  __syncthreads();
  for (int it = 0; it + 1 < B.n_iter; ++it) {
    // 0.5 * spread(F_step) at the touched nodes (ib/mdf.py:50-51)
    for (int j = tid; j < NT; j += nt) {
      const int lo = tstart[j], hi = tstart[j + 1];
      T a0 = T(0), a1 = T(0);
      for (int i = lo; i < hi; ++i) {
        const int p = sorted[i];
        const int m = p / S;
        const T w = W[p];
        const T t0 = mul_rn(Fs[2 * m], w), t1 = mul_rn(Fs[2 * m + 1], w);
        a0 = i == lo ? t0 : add_rn(a0, t0);
        a1 = i == lo ? t1 : add_rn(a1, t1);
      }
      nv[j] = a0 * T(0.5);
      nv[NB + j] = a1 * T(0.5);
    }
    __syncthreads();
    // U += interpolate(0.5 spread); next force step (ib/mdf.py:41-52)
    for (int t = tid; t < 2 * M * LN; t += nt) {
      const int q = t / LN, m = q >> 1, c = q & 1;
      const T acc = interp_group<T, S, LN>(W, slot, nv + c * NB, m);
      if ((t & (LN - 1)) == 0) {
        const T uq = U[q] + acc;
        U[q] = uq;
        const T d2 = B.ds_arr ? B.ds_arr[m] * T(2) : B.ds2_scalar;
        const T fs = mul_rn(kin.target(B, m, c) - uq, d2);
        Fs[q] = fs;
        Ft[q] = Ft[q] + fs;
      }
    }
    __syncthreads();
  }
  // g = spread(F_total) over the region (ib/mdf.py:60-62); zero where no marker reaches
  for (int k = tid; k < NB; k += nt) {
    const int j = cslot[k];
    T a0 = T(0), a1 = T(0);
    if (j >= 0) {
      const int lo = tstart[j], hi = tstart[j + 1];
      for (int i = lo; i < hi; ++i) {
        const int p = sorted[i];
        const int m = p / S;
        const T w = W[p];
        const T t0 = mul_rn(Ft[2 * m], w), t1 = mul_rn(Ft[2 * m + 1], w);
        a0 = i == lo ? t0 : add_rn(a0, t0);
        a1 = i == lo ? t1 : add_rn(a1, t1);
      }
    }
    B.gw[k] = a0;
    B.gw[NB + k] = a1;
  }
  if (tid == 0) {
    B.meta[META_OX] = ox; B.meta[META_OY] = oy; B.meta[META_OZ] = 0;
    B.meta[META_WX] = EX; B.meta[META_WY] = EY; B.meta[META_WZ] = 1;
    B.meta[META_PX] = misc[0] - R + 1;
    B.meta[META_PY] = misc[2] - R + 1;
    B.meta[META_PX2] = misc[0] - R + 1;
    B.meta[META_PY2] = misc[2] - R + 1;
  }
  // total force h = sum_m(-F_total) (dyn.py:126-136) by warp 0 in a fixed tree, added
  // mass h += a A (vortex_induced_vibration.py:136), Newmark update (dyn.py:5-51)
  if (tid < 32) body2d_finish<T>(B, kin, Ft, M, a, v, d);
}

// shared memory of k_body2d for M markers, radius R, region EX x EY, staged rows of RL
template <typename T>
static size_t body2d_smem(int M, int R, int EX, int EY, int RL) {
  const size_t S = 4 * R * R, P = M * S, NB = (size_t)EX * EY;
  return sizeof(T) * (9 * (size_t)EX * RL + (4 * (size_t)R + 6) * M + P + 4 * NB) +
         sizeof(int) * (3 * P + 4 * NB + 1 + 2 * (size_t)M + 40) + 16;
}

template <typename T>
static cudaError_t body2d_attr(int R, int smem) {
  switch (R) {
    case 1: return cudaFuncSetAttribute(k_body2d<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case 2: return cudaFuncSetAttribute(k_body2d<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    default: return cudaFuncSetAttribute(k_body2d<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  }
}

template <typename T>
static void body2d_launch(int R, size_t smem, cudaStream_t st, const BodyParams<T>& P) {
  switch (R) {
    case 1: k_body2d<T, 1><<<1, kBodyThreads, smem, st>>>(P); break;
    case 2: k_body2d<T, 2><<<1, kBodyThreads, smem, st>>>(P); break;
    default: k_body2d<T, 3><<<1, kBodyThreads, smem, st>>>(P); break;
  }
}

// ------------------------------------------------------------------ 2-D body kernel, chain form
// For most immersed boundaries the markers are ordered along a curve, and two markers
// whose stencils can share a node are at most K positions apart in that (cyclic) order.
// The markers of a rigid body only translate, so K is a property of the marker set that
// the plan computes once on the host (markers i, j can share a node under some
// translation iff |x_i - x_j| < 2R and |y_i - y_j| < 2R).  The node of pair (j, s) then
// receives contributions only from markers j-K..j+K; which of them reach it follows from
// their stencil corners by index arithmetic, and taking them in increasing marker index is
// the reference's scatter order (each marker reaches a node through at most one stencil
// point).  So every pair recomputes its own node's spread value: no sort, no per-node
// lists, one block-wide barrier per MDF iteration.  Results equal those of k_body2d.
__device__ __forceinline__ void chain_range(int j, int K, int M, int& a0, int& nA, int& b0, int& nc) {
  if (2 * K + 1 >= M) {
    a0 = 0; nA = M; b0 = 0; nc = M;
    return;
  }
  nc = 2 * K + 1;
  const int lo = j - K, hi = j + K;
  if (lo < 0) {         // {0..hi} then {lo+M..M-1}
    a0 = 0; nA = hi + 1; b0 = lo + M;
  } else if (hi >= M) { // {0..hi-M} then {lo..M-1}
    a0 = 0; nA = hi - M + 1; b0 = lo;
  } else {
    a0 = lo; nA = nc; b0 = 0;
  }
}

// sum over the contributors in `msk` of F[i] * W[i, s_i] for the node (nx, ny), both
// components, first term not added to zero (as the ordered segment sums do)
template <typename T, int WD>
__device__ __forceinline__ void chain_node_sum(unsigned msk, int a0, int nA, int b0, int nx, int ny, const int* fxy,
                                               const T* W, const T* F, T& s0, T& s1) {
  constexpr int S = WD * WD;
  bool first = true;
  s0 = T(0);
  s1 = T(0);
  while (msk) {
    const int b = __ffs(msk) - 1;
    msk &= msk - 1;
    const int i = b < nA ? a0 + b : b0 + (b - nA);
    const int k = (nx - fxy[2 * i]) * WD + (ny - fxy[2 * i + 1]);
    const T w = W[i * S + k];
    const T t0 = mul_rn(F[2 * i], w), t1 = mul_rn(F[2 * i + 1], w);
    s0 = first ? t0 : add_rn(s0, t0);
    s1 = first ? t1 : add_rn(s1, t1);
    first = false;
  }
}

template <typename T, int LN>
__device__ __forceinline__ T group_sum(T acc) {
  if constexpr (LN > 1) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned mask = ((1u << LN) - 1u) << (lane & ~(unsigned)(LN - 1));
#pragma unroll
    for (int o = LN / 2; o >= 1; o >>= 1) acc = acc + __shfl_down_sync(mask, acc, o, LN);
  }
  return acc;
}

template <typename T, int R>
__device__ __forceinline__ void body2d_chain(const BodyParams<T>& B) {
  constexpr int WD = 2 * R, S = WD * WD;
  constexpr int LN = S >= 16 ? 4 : 1;  // lanes per marker
  constexpr int PER = S / LN;          // stencil points per lane, contiguous
  constexpr int AL = 16 / sizeof(T);
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int M = B.M, P = M * S, K = B.chain_k;
  const int EX = B.cap_x + 2, EY = B.cap_y + 2, NB = EX * EY, RL = B.row_len;
  T* fwin = (T*)smem;          // staged populations [9][EX][RL]
  T* W = fwin + 9 * EX * RL;   // [P] stencil weights
  T* U = W + P;                // [2M] marker velocity
  T* Fa = U + 2 * M;           // [2M] force step, ping
  T* Fb = Fa + 2 * M;          // [2M] force step, pong
  T* Ft = Fb + 2 * M;          // [2M] total force
  int* fxy = (int*)(Ft + 2 * M);               // [2M] stencil corner (floor - R + 1)
  unsigned* cmask = (unsigned*)(fxy + 2 * M);  // [P] contributors of each pair's node
  int* misc = (int*)(cmask + P);               // [0..3] min/max floor x, y; [4] out-of-region
  uint64_t* bar = (uint64_t*)(((uintptr_t)(misc + 8) + 7) & ~(uintptr_t)7);
  {
    // the layout must fit the dynamic shared memory this launch received
    unsigned have;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(have));
    if ((size_t)((const unsigned char*)(bar + 1) - smem) > have) {
      if (tid == 0) {
        B.meta[META_STATUS] = VS_ERR_INVALID_ARG;
        B.meta[META_WX] = 0; B.meta[META_WY] = 0; B.meta[META_WZ] = 0;
      }
      return;
    }
  }

  T a[3], v[3], d[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a[c] = B.state[c];
    v[c] = B.state[3 + c];
    d[c] = B.state[6 + c];
  }
  const Kin2<T> kin(B, d, v);
  const int ox = B.meta[META_PX] - 1, oy = B.meta[META_PY] - 1;  // predicted region corner
  const int ya = oy >= 0 ? oy - oy % AL : 0;
  const int64_t n = (int64_t)B.nx * B.ny;
  const bool region_ok = ox >= B.box[0] && oy >= B.box[2] && ox + EX <= B.box[1] && oy + EY <= B.box[3];
  const bool bulk = B.bulk && region_ok;
  if (tid == 0) {
    misc[0] = INT_MAX; misc[1] = INT_MIN; misc[2] = INT_MAX; misc[3] = INT_MIN; misc[4] = 0;
    if (bulk) {
      tma::mbar_init(bar, 1);
      tma::fence_init();
      tma::mbar_expect_tx(bar, (unsigned)(9 * EX * RL * sizeof(T)));
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
          "%4}], [%5];\n" ::"r"(tma::smem_addr(fwin)),
          "l"(&B.map), "r"(ya), "r"(ox), "r"(0), "r"(tma::smem_addr(bar))
          : "memory");
    }
  }
  // the force window starts at zero; cells no marker reaches stay zero
  if (region_ok)
    for (int k = tid; k < 2 * NB; k += nt) B.gw[k] = T(0);
  __syncthreads();
  // markers follow the body (dyn.py:68-81); stencil weights kernel(sx - X) * kernel(sy - Y)
  // (ib/stencil.py:7-51), one thread per (marker, lane), PER stencil points each
  for (int t = tid; t < M * LN; t += nt) {
    const int m = t / LN, sub = t - m * LN;
    T xm, ym;
    kin.xy(B, m, xm, ym);
    const int fx = ifloor(xm), fy = ifloor(ym);
    if (sub == 0) {
      fxy[2 * m] = fx - R + 1;
      fxy[2 * m + 1] = fy - R + 1;
      atomicMin(&misc[0], fx); atomicMax(&misc[1], fx);
      atomicMin(&misc[2], fy); atomicMax(&misc[3], fy);
    }
    bool out = false;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int s = sub * PER + j, ix = s / WD, iy = s - ix * WD;
      W[m * S + s] = delta(B.kernel, (T)(fx + ix - R + 1) - xm) * delta(B.kernel, (T)(fy + iy - R + 1) - ym);
      const int cx = fx + ix - R + 1 - ox, cy = fy + iy - R + 1 - oy;
      out |= cx < 0 || cx >= EX || cy < 0 || cy >= EY;
    }
    if (out) misc[4] = 1;
  }
  __syncthreads();
  if (misc[4] || !region_ok) {
    // the body moved a node or more in one step, or its region left the box
    // let the staged copy land before the block leaves (bounded; reported if it does not)
    if (tid == 0) {
      const bool landed = !bulk || tma::mbar_wait(bar, 0, kTmaWaitLimit) || tma_drain(bar, 0) == VS_ERR_TIMEOUT;
      B.meta[META_STATUS] = landed ? VS_ERR_RANGE : VS_ERR_TIMEOUT_INFLIGHT;
      B.meta[META_WX] = 0; B.meta[META_WY] = 0; B.meta[META_WZ] = 0;
    }
    return;
  }
  bool staged = true;
  if (bulk) staged = tma::mbar_wait(bar, 0, kTmaWaitLimit);
  if (__syncthreads_or(!staged)) {
    if (tid == 0) {
      B.meta[META_STATUS] = tma_drain(bar, 0);  // the copy is waited for once more before the block leaves
      B.meta[META_WX] = 0; B.meta[META_WY] = 0; B.meta[META_WZ] = 0;
    }
    return;
  }
  // contributors of each pair's node; u there; U = interpolate(u) and the first force
  // step (ib/mdf.py:38-48) with the body velocity as target
  for (int t = tid; t < M * LN; t += nt) {
    const int m = t / LN, sub = t - m * LN;
    int a0, nA, b0, nc;
    chain_range(m, K, M, a0, nA, b0, nc);
    const int bx = fxy[2 * m], by = fxy[2 * m + 1];
    T acc0 = T(0), acc1 = T(0);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int s = sub * PER + j, ix = s / WD, iy = s - ix * WD;
      const int nx = bx + ix, ny = by + iy;
      unsigned msk = 0;
      for (int b = 0; b < nc; ++b) {
        const int i = b < nA ? a0 + b : b0 + (b - nA);
        const unsigned dx = (unsigned)(nx - fxy[2 * i]), dy = (unsigned)(ny - fxy[2 * i + 1]);
        if (dx < (unsigned)WD && dy < (unsigned)WD) msk |= 1u << b;
      }
      cmask[m * S + s] = msk;
      const int cx = nx - ox, cy = ny - oy;
      T fl[9];
      if (bulk) {
#pragma unroll
        for (int i = 0; i < 9; ++i) fl[i] = fwin[(i * EX + cx) * RL + (oy - ya) + cy];
      } else {
        const int64_t pn = (int64_t)nx * B.ny + ny;
#pragma unroll
        for (int i = 0; i < 9; ++i) fl[i] = __ldg(B.fin + i * n + pn);
      }
      T r, uu[3];
      macro(L9{}, fl, r, uu);
      const T w = W[m * S + s];
      const T t0 = mul_rn(w, uu[0]), t1 = mul_rn(w, uu[1]);
      acc0 = j == 0 ? t0 : add_rn(acc0, t0);
      acc1 = j == 0 ? t1 : add_rn(acc1, t1);
    }
    acc0 = group_sum<T, LN>(acc0);
    acc1 = group_sum<T, LN>(acc1);
    if (sub == 0) {
      const T d2 = B.ds_arr ? B.ds_arr[m] * T(2) : B.ds2_scalar;
      const T acc[2] = {acc0, acc1};
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        U[2 * m + c] = acc[c];
        const T fs = mul_rn(kin.target(B, m, c) - acc[c], d2);
        Fa[2 * m + c] = fs;
        Ft[2 * m + c] = B.n_iter > 0 ? fs : T(0);
      }
    }
  }
  __syncthreads();
  // MDF iterations (ib/mdf.py:41-52): U += interpolate(0.5 spread(F_step)); next force step
  T* Fcur = Fa;
  T* Fnext = Fb;
  for (int it = 0; it + 1 < B.n_iter; ++it) {
    for (int t = tid; t < M * LN; t += nt) {
      const int m = t / LN, sub = t - m * LN;
      int a0, nA, b0, nc;
      chain_range(m, K, M, a0, nA, b0, nc);
      const int bx = fxy[2 * m], by = fxy[2 * m + 1];
      T acc0 = T(0), acc1 = T(0);
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        const int s = sub * PER + j, ix = s / WD, iy = s - ix * WD;
        T n0, n1;
        chain_node_sum<T, WD>(cmask[m * S + s], a0, nA, b0, bx + ix, by + iy, fxy, W, Fcur, n0, n1);
        const T w = W[m * S + s];
        const T t0 = mul_rn(w, n0 * T(0.5)), t1 = mul_rn(w, n1 * T(0.5));
        acc0 = j == 0 ? t0 : add_rn(acc0, t0);
        acc1 = j == 0 ? t1 : add_rn(acc1, t1);
      }
      acc0 = group_sum<T, LN>(acc0);
      acc1 = group_sum<T, LN>(acc1);
      if (sub == 0) {
        const T d2 = B.ds_arr ? B.ds_arr[m] * T(2) : B.ds2_scalar;
        const T acc[2] = {acc0, acc1};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const T uq = U[2 * m + c] + acc[c];
          U[2 * m + c] = uq;
          const T fs = mul_rn(kin.target(B, m, c) - uq, d2);
          Fnext[2 * m + c] = fs;
          Ft[2 * m + c] = Ft[2 * m + c] + fs;
        }
      }
    }
    __syncthreads();
    T* tmp = Fcur;
    Fcur = Fnext;
    Fnext = tmp;
  }
  // g = spread(F_total) (ib/mdf.py:60-62): every pair writes its node's sum; pairs that
  // share a node compute the same value in the same order
  for (int t = tid; t < M * LN; t += nt) {
    const int m = t / LN, sub = t - m * LN;
    int a0, nA, b0, nc;
    chain_range(m, K, M, a0, nA, b0, nc);
    const int bx = fxy[2 * m], by = fxy[2 * m + 1];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int s = sub * PER + j, ix = s / WD, iy = s - ix * WD;
      T g0, g1;
      chain_node_sum<T, WD>(cmask[m * S + s], a0, nA, b0, bx + ix, by + iy, fxy, W, Ft, g0, g1);
      const int k = (bx + ix - ox) * EY + (by + iy - oy);
      B.gw[k] = g0;
      B.gw[NB + k] = g1;
    }
  }
  if (tid == 0) {
    B.meta[META_OX] = ox; B.meta[META_OY] = oy; B.meta[META_OZ] = 0;
    B.meta[META_WX] = EX; B.meta[META_WY] = EY; B.meta[META_WZ] = 1;
    B.meta[META_PX] = misc[0] - R + 1;
    B.meta[META_PY] = misc[2] - R + 1;
    B.meta[META_PX2] = misc[0] - R + 1;
    B.meta[META_PY2] = misc[2] - R + 1;
  }
  // total force h = sum_m(-F_total) (dyn.py:126-136) in a fixed tree by warp 0, added mass
  // h += a A (vortex_induced_vibration.py:136), Newmark update (dyn.py:5-51)
  if (tid < 32) body2d_finish<T>(B, kin, Ft, M, a, v, d);
}

template <typename T, int R>
__global__ void __launch_bounds__(kBodyThreads) k_body2d_chain(const __grid_constant__ BodyParams<T> B) {
  body2d_chain<T, R>(B);
}

// many bodies, one CTA each (each of its own lattice)
template <typename T, int R>
__global__ void __launch_bounds__(kBodyThreads) k_body2d_chain_batch(const BodyParams<T>* __restrict__ Bs) {
  body2d_chain<T, R>(Bs[blockIdx.x]);
}

// ------------------------------------------------------------------ 2-D body, cluster form
// The chain form spread over a thread-block cluster of CL CTAs (distributed shared memory),
// one stencil pair per thread, followed by the box update that waits for the body force.
// CTA r owns markers [r M / CL, (r+1) M / CL); it recomputes the positions of all markers
// and the weights of its own markers and their +-K neighbours, so only the per-iteration
// force steps travel between CTAs: each CTA writes its markers' values into every CTA's
// replica (st.shared::cluster) before a cluster barrier.  The sums use the chain form's
// order (4 stencil points per lane-group, then (0 + 2) + (1 + 3); the total force in
// warp 0's tree on the replicated totals), so the results equal the single-CTA kernels'.
// After the body, all CTAs of the cluster update the body's box and the lazy face planes
// (the work of the post-join box launch), so one time step is this kernel beside the
// grid kernel over the rest of the grid.
constexpr int kClusterPairs = 256;    // stencil pairs a CTA holds (one per thread)
constexpr int kClusterThreads = 384;  // launch bound; a plan uses enough threads for its window

// One time step of the body over the CTAs of the calling cluster (the body of
// k_body2d_cluster, also run by the persistent k_viv_run); hist: where h goes (or null).
template <typename T, int R, int COLL>
__device__ __forceinline__ void body2d_cluster_step(const BodyParams<T>& B, const StepParams<L9, T>& SP, T* hist) {
  namespace cg = cooperative_groups;
  constexpr int WD = 2 * R, S = WD * WD;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int CL = (int)cluster.num_blocks(), rank = (int)cluster.block_rank();
  const int M = B.M, K = B.chain_k;
  const int EX = B.cap_x + 2, EY = B.cap_y + 2, NB = EX * EY;
  const int m0 = (int)((int64_t)rank * M / CL), m1 = (int)((int64_t)(rank + 1) * M / CL);
  T* W = (T*)smem;              // [M S] (own markers and their neighbours filled)
  T* Fa = W + M * S;            // [2M] force step replica, ping
  T* Fb = Fa + 2 * M;           // [2M] pong
  T* Ft = Fb + 2 * M;           // [2M] total force replica
  T* U = Ft + 2 * M;            // [2M] own markers' velocity
  T* prod = U + 2 * M;          // [2 nt] interpolation products (generic radius)
  T* xs = prod + 2 * nt;        // [2M] marker positions X0 + d, Y0 + d
  // the IB force of this CTA's window nodes: node k belongs to CTA (k mod CL nt) / nt, at
  // slot (k mod CL nt) mod nt + nt (k / CL nt); x components, then y after GW entries
  const int GW = nt * ((EX * EY + CL * nt - 1) / (CL * nt));
  T* gl = xs + 2 * M;           // [2 GW]
  int* fxy = (int*)(gl + 2 * GW);    // [2M]
  unsigned* cm = (unsigned*)(fxy + 2 * M);  // [nt] contributor mask of the thread's pair
  int* flags = (int*)(cm + nt);      // [0] a pair of this CTA left the predicted region, [1..2] min corner
  // every CTA of the cluster must be running before any distributed shared memory access:
  // arrive now, wait just before the first remote store
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");

  T a[3], v[3], d[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a[c] = B.state[c];
    v[c] = B.state[3 + c];
    d[c] = B.state[6 + c];
  }
  const Kin2<T> kin(B, d, v);
  const int slot = B.pred_slot;
  const int ox = B.meta[slot ? META_PX2 : META_PX] - 1, oy = B.meta[slot ? META_PY2 : META_PY] - 1;
  const bool region_ok = ox >= B.box[0] && oy >= B.box[2] && ox + EX <= B.box[1] && oy + EY <= B.box[3];
  const int64_t n = (int64_t)SP.nx * SP.ny;
  // The populations of the thread's own pair's node (needed first) and of its first window
  // node (needed at the end) are both known now and f_in does not change during the step;
  // the pair's loads are issued first.
  const int kw = rank * nt + tid;
  const int own = m1 - m0;
  const int lp = tid, m = m0 + lp / S, s = lp - (lp / S) * S;
  const bool has_pair = lp < own * S;
  int nxp = 0, nyp = 0;
  bool in_region = true;
  T fl[9];
  if (has_pair) {
    const int ix = s / WD, iy = s - ix * WD;
    T px, py;
    kin.xy(B, m, px, py);
    nxp = ifloor(px) - R + 1 + ix;
    nyp = ifloor(py) - R + 1 + iy;
    const int cx = nxp - ox, cy = nyp - oy;
    in_region = cx >= 0 && cx < EX && cy >= 0 && cy < EY;
    if (in_region) {
      const int64_t pn = (int64_t)nxp * SP.ny + nyp;
#pragma unroll
      for (int i = 0; i < 9; ++i) fl[i] = __ldg(B.fin + i * n + pn);
    }
  }
  // prefetch of the window node, behind the pair's loads
  int wx = 0, wy = 0, wp = -1;
  T fw[9];
  if (kw < NB) {
    wx = ox + kw / EY;
    wy = oy + kw % EY;
    if (wx >= 0 && wx < SP.nx && wy >= 0 && wy < SP.ny && !(SP.skip_walls && (wx == 0 || wx == SP.nx - 1))) {
      wp = wx * SP.ny + wy;
#pragma unroll
      for (int i = 0; i < 9; ++i) fw[i] = __ldg(SP.fin + (size_t)i * n + wp);
    }
  }
  // all marker positions in one round trip (the own pair's above is the same load)
  for (int mm = tid; mm < M; mm += nt) {
    kin.xy(B, mm, xs[mm], xs[M + mm]);
  }
  if (tid == 0) {
    flags[0] = 0;
    flags[1] = INT_MAX;
    flags[2] = INT_MAX;
  }
  if (rank == 0 && tid == 0) {  // window descriptor for the force lookup (grid kernels read it after the body)
    B.meta[META_OX] = ox; B.meta[META_OY] = oy; B.meta[META_OZ] = 0;
    B.meta[META_WX] = EX; B.meta[META_WY] = EY; B.meta[META_WZ] = 1;
  }
  // the window force starts at zero (remote writes come after several cluster barriers)
  for (int i = tid; i < 2 * GW; i += nt) gl[i] = T(0);
  __syncthreads();
  // every marker's stencil corner (and their minimum, the next prediction); weights of the
  // own markers and their +-K neighbours
  const int Mw = ((M + 31) / 32) * 32;  // whole warps (nt is a multiple of 32): a warp-wide minimum
  for (int m2 = tid; m2 < Mw; m2 += nt) {
    int cx = INT_MAX, cy = INT_MAX;
    if (m2 < M) {
      cx = ifloor(xs[m2]) - R + 1;
      cy = ifloor(xs[M + m2]) - R + 1;
      fxy[2 * m2] = cx;
      fxy[2 * m2 + 1] = cy;
    }
    cx = __reduce_min_sync(0xffffffffu, cx);
    cy = __reduce_min_sync(0xffffffffu, cy);
    if ((tid & 31) == 0 && cx != INT_MAX) {
      atomicMin(&flags[1], cx);
      atomicMin(&flags[2], cy);
    }
  }
  if (has_pair && !in_region) atomicOr(&flags[0], 1);
  const int span = own + 2 * K < M ? own + 2 * K : M;
  for (int t = tid; t < span * S; t += nt) {
    const int k = t / S, s2 = t - k * S, ix = s2 / WD, iy = s2 - ix * WD;
    int mm = span == M ? k : m0 - K + k;
    mm = mm < 0 ? mm + M : (mm >= M ? mm - M : mm);
    const T xm = xs[mm], ym = xs[M + mm];
    const int fx = ifloor(xm), fy = ifloor(ym);
    W[mm * S + s2] = delta(B.kernel, (T)(fx + ix - R + 1) - xm) * delta(B.kernel, (T)(fy + iy - R + 1) - ym);
  }
  __syncthreads();
  // the thread's own pair: contributors, u at its node, U0 = interp(u), first force step
  int a0 = 0, nA = 0, b0 = 0, nc = 0;
  unsigned msk = 0;
  T uu[2] = {T(0), T(0)};
  if (has_pair) {
    chain_range(m, K, M, a0, nA, b0, nc);
    for (int b = 0; b < nc; ++b) {
      const int i = b < nA ? a0 + b : b0 + (b - nA);
      const unsigned dx = (unsigned)(nxp - fxy[2 * i]), dy = (unsigned)(nyp - fxy[2 * i + 1]);
      if (dx < (unsigned)WD && dy < (unsigned)WD) msk |= 1u << b;
    }
    if (in_region) {
      T r;
      macro(L9{}, fl, r, uu);
    }
  }
  cm[tid] = msk;
  auto interp = [&](T p0, T p1, T* acc) {
    // sum of the S products of one marker in the chain form's order
    if constexpr (S == 16) {
      const unsigned lane = threadIdx.x & 31, base = lane & ~15u;
      const unsigned gm = 0xffffu << base;
      T q[2] = {p0, p1};
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const T v1 = __shfl_down_sync(gm, q[c], 1, 16), v2 = __shfl_down_sync(gm, q[c], 2, 16),
                v3 = __shfl_down_sync(gm, q[c], 3, 16);
        const T Lq = add_rn(add_rn(add_rn(q[c], v1), v2), v3);  // lanes 4k: their 4 stencil points
        const T L1 = __shfl_down_sync(gm, Lq, 4, 16), L2 = __shfl_down_sync(gm, Lq, 8, 16),
                L3 = __shfl_down_sync(gm, Lq, 12, 16);
        acc[c] = add_rn(add_rn(Lq, L2), add_rn(L1, L3));
      }
    } else {
      prod[2 * tid] = p0;
      prod[2 * tid + 1] = p1;
      __syncthreads();
      if (has_pair && s == 0)
        for (int c = 0; c < 2; ++c) {
          T z = prod[2 * tid + c];
          for (int k = 1; k < S; ++k) z = add_rn(z, prod[2 * (tid + k) + c]);
          acc[c] = z;
        }
      __syncthreads();
    }
  };
  // the marker's two values (held by its lane s == 0) into every CTA's replica at dst:
  // with 16-lane groups, lane r of the group stores to CTA r
  auto publish = [&](T* dst, T v0, T v1, bool skip_self) {
    if constexpr (S == 16) {
      const unsigned lane = threadIdx.x & 31, base = lane & ~15u;
      const unsigned gm = 0xffffu << base;
      v0 = __shfl_sync(gm, v0, 0, 16);
      v1 = __shfl_sync(gm, v1, 0, 16);
      if (has_pair && s < CL && !(skip_self && s == rank)) {
        T* r = cluster.map_shared_rank(dst + 2 * m, s);
        r[0] = v0;
        r[1] = v1;
      }
    } else {
      if (has_pair && s == 0)
        for (int r = 0; r < CL; ++r)
          if (!(skip_self && r == rank)) {
            T* q = cluster.map_shared_rank(dst + 2 * m, r);
            q[0] = v0;
            q[1] = v1;
          }
    }
  };
  const T wself = has_pair ? W[m * S + s] : T(0);
  const T d2 = has_pair ? (B.ds_arr ? B.ds_arr[m] * T(2) : B.ds2_scalar) : T(0);
  asm volatile("barrier.cluster.wait.aligned;\n" ::: "memory");
  {
    T acc[2] = {T(0), T(0)}, fs[2] = {T(0), T(0)};
    interp(mul_rn(wself, uu[0]), mul_rn(wself, uu[1]), acc);
    if (has_pair && s == 0) {
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        U[2 * m + c] = acc[c];
        fs[c] = mul_rn(kin.target(B, m, c) - acc[c], d2);
        Ft[2 * m + c] = B.n_iter > 0 ? fs[c] : T(0);
      }
    }
    publish(Fa, fs[0], fs[1], false);
  }
  cluster.sync();
  int bad = 0;
  for (int r = 0; r < CL; ++r) bad |= *cluster.map_shared_rank(flags, r);
  const bool ok = region_ok && bad == 0;
  T* Fcur = Fa;
  T* Fnext = Fb;
  if (ok) {
    for (int it = 0; it + 1 < B.n_iter; ++it) {
      T n0 = T(0), n1 = T(0);
      if (has_pair) chain_node_sum<T, WD>(msk, a0, nA, b0, nxp, nyp, fxy, W, Fcur, n0, n1);
      T acc[2] = {T(0), T(0)}, fs[2] = {T(0), T(0)}, ft[2] = {T(0), T(0)};
      interp(mul_rn(wself, n0 * T(0.5)), mul_rn(wself, n1 * T(0.5)), acc);
      if (has_pair && s == 0) {
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const T uq = U[2 * m + c] + acc[c];
          U[2 * m + c] = uq;
          fs[c] = mul_rn(kin.target(B, m, c) - uq, d2);
          ft[c] = Ft[2 * m + c] + fs[c];
          Ft[2 * m + c] = ft[c];
        }
      }
      if (it + 2 < B.n_iter) publish(Fnext, fs[0], fs[1], false);
      else publish(Ft, ft[0], ft[1], true);  // the last iteration sends the totals
      cluster.sync();
      T* tmp = Fcur;
      Fcur = Fnext;
      Fnext = tmp;
    }
    if (B.n_iter <= 1) {  // no iteration carried the totals: send them now
      const T t0 = has_pair ? Ft[2 * m] : T(0), t1 = has_pair ? Ft[2 * m + 1] : T(0);
      publish(Ft, t0, t1, true);
      cluster.sync();
    }
    // g = spread(F_total): each pair writes its node's sum into the node's owner CTA
    if (has_pair) {
      T g0, g1;
      chain_node_sum<T, WD>(msk, a0, nA, b0, nxp, nyp, fxy, W, Ft, g0, g1);
      const int k = (nxp - ox) * EY + (nyp - oy);
      const int kr = k % (CL * nt);
      T* dst = cluster.map_shared_rank(gl, kr / nt);
      const int li = kr % nt + nt * (k / (CL * nt));
      dst[li] = g0;
      dst[GW + li] = g1;
    }
  } else if (rank == 0 && tid == 0) {
    B.meta[META_STATUS] = VS_ERR_RANGE;
    B.meta[META_WX] = 0; B.meta[META_WY] = 0; B.meta[META_WZ] = 0;
  }
  // the body force of every CTA (and the window descriptor) are in place
  cluster.sync();
  if (ok && rank == 0 && tid < 32) {
    // h = sum_m(-F_total) (and the torque) in warp 0's fixed tree, added mass, Newmark
    body2d_finish<T>(B, kin, Ft, M, a, v, d, hist);
    if (tid == 2) {
      B.meta[slot ? META_PX : META_PX2] = flags[1];  // the next step reads the other slot
      B.meta[slot ? META_PY : META_PY2] = flags[2];
    }
  }
  // the nodes of the predicted window, which the concurrent grid launch skips (the same
  // slot gives it the same window); lazy face planes are another launch's
  // (their force from shared memory; with the window out of its region no force, as the
  // emptied window descriptor gives the per-node lookup)
  if (wp >= 0) {
    const T gn[2] = {gl[tid], gl[GW + tid]};
    step_node<L9, T, COLL, kFeatGeneral>(SP, wx, wy, 0, wp, fw, ok ? gn : nullptr);
  }
  for (int k = kw + CL * nt, j = 1; k < NB; k += CL * nt, ++j) {
    const int x = ox + k / EY, y = oy + k % EY;
    if (x < 0 || x >= SP.nx || y < 0 || y >= SP.ny || (SP.skip_walls && (x == 0 || x == SP.nx - 1))) continue;
    const int p = x * SP.ny + y;
    T f[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) f[i] = __ldg(SP.fin + (size_t)i * SP.n + p);
    const T gn[2] = {gl[tid + nt * j], gl[GW + tid + nt * j]};
    step_node<L9, T, COLL, kFeatGeneral>(SP, x, y, 0, p, f, ok ? gn : nullptr);
  }
}

template <typename T, int R, int COLL>
__global__ void __launch_bounds__(kClusterThreads) k_body2d_cluster(const __grid_constant__ BodyParams<T> B,
                                                                   const __grid_constant__ StepParams<L9, T> SP) {
  body2d_cluster_step<T, R, COLL>(B, SP, B.force_hist);
}

template <typename T>
static size_t body2d_cluster_smem(int M, int R, int nt, int CL, int NB) {
  const size_t S = 4 * R * R;
  const size_t GW = (size_t)nt * ((NB + CL * nt - 1) / (CL * nt));
  return sizeof(T) * (M * S + 10 * (size_t)M + 2 * (size_t)nt + 2 * GW) +
         sizeof(int) * (2 * (size_t)M + (size_t)nt + 4) + 16;
}

template <typename T>
static size_t body2d_chain_smem(int M, int R, int EX, int RL) {
  const size_t S = 4 * R * R, P = M * S;
  return sizeof(T) * (9 * (size_t)EX * RL + P + 8 * (size_t)M) + sizeof(int) * (2 * (size_t)M + P + 8) + 16;
}

template <typename T>
static cudaError_t body2d_chain_attr(int R, int smem) {
  switch (R) {
    case 1: return cudaFuncSetAttribute(k_body2d_chain<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case 2: return cudaFuncSetAttribute(k_body2d_chain<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    default: return cudaFuncSetAttribute(k_body2d_chain<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  }
}

template <typename T>
static void body2d_chain_launch(int R, size_t smem, cudaStream_t st, const BodyParams<T>& P) {
  switch (R) {
    case 1: k_body2d_chain<T, 1><<<1, kBodyThreads, smem, st>>>(P); break;
    case 2: k_body2d_chain<T, 2><<<1, kBodyThreads, smem, st>>>(P); break;
    default: k_body2d_chain<T, 3><<<1, kBodyThreads, smem, st>>>(P); break;
  }
}

static bool getenv_flag(const char* name) {
  const char* v = getenv(name);
  return v && v[0] && !(v[0] == '0' && v[1] == 0);
}

// Chain width of a rigid 2-D marker set (coordinates in the plan precision): the largest
// cyclic index distance between two markers whose stencils can share a node under some
// translation, i.e. |dx| < 2R and |dy| < 2R (with a small margin for rounding).  A body that
// also turns can bring any pair closer than 2R sqrt(2) to that test's 45-degree corner, so
// there the distance decides.
static int chain_width(const double* x, const double* y, int M, int R, int rot) {
  const double lim = 2.0 * R + 1e-3, lim_r = 2.0 * R * sqrt(2.0) + 1e-3;
  int K = 0;
  for (int i = 0; i < M; ++i)
    for (int j = i + 1; j < M; ++j) {
      const double dx = x[i] - x[j], dy = y[i] - y[j];
      if (rot ? hypot(dx, dy) < lim_r : (fabs(dx) < lim && fabs(dy) < lim)) {
        const int dd = j - i, cyc = dd < M - dd ? dd : M - dd;
        K = cyc > K ? cyc : K;
      }
    }
  return K;
}

// ------------------------------------------------------------------ body kernels (3-D fixed)
// The stencil of a fixed body never moves, so its (node, pair) CSR is built once; each
// step then runs node-parallel and marker-parallel kernels over the compacted node list.

// The stencil weights and marker ids of the pairs in CSR (node) order: wsort[i] = W[sids[i]],
// msort[i] = sids[i] / S.
template <typename T>
__global__ void k_csr_gather(const int32_t* __restrict__ sids, const T* __restrict__ W, int S, int64_t P,
                             T* __restrict__ wsort, int32_t* __restrict__ msort) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P; i += (int64_t)gridDim.x * blockDim.x) {
    const int p = sids[i];
    wsort[i] = W[p];
    msort[i] = p / S;
  }
}

// How the body phases load node and marker values: kLoadRO through the read-only path (the
// per-phase kernels), kLoadL2 bypassing L1 (values written earlier in the same launch by
// other CTAs: the cooperative kernel), kLoadPlain with a generic load (shared memory:
// the cluster kernel).
enum { kLoadRO = 0, kLoadL2 = 1, kLoadPlain = 2 };
template <int MODE, typename T>
__device__ __forceinline__ T body_load(const T* p) {
  if constexpr (MODE == kLoadL2) return __ldcg(p);
  else if constexpr (MODE == kLoadPlain) return *p;
  else return __ldg(p);
}

// u at touched node k (vivsim/lbm3d/basic.py:90-106)
template <class L, typename T>
__device__ __forceinline__ void static_node_u(int k, const T* __restrict__ fin, int ny, int nz, int64_t n, int ox,
                                              int oy, int oz, int ey, int ez, const int32_t* __restrict__ node_cell,
                                              int U, T* __restrict__ nu) {
  const int cell = node_cell[k];
  const int wx = cell / (ey * ez), wy = (cell / ez) % ey, wz = cell % ez;
  const int64_t pn = ((int64_t)(ox + wx) * ny + (oy + wy)) * nz + (oz + wz);
  T fl[L::Q];
#pragma unroll
  for (int i = 0; i < L::Q; ++i) fl[i] = __ldg(fin + i * n + pn);
  T r, uu[3] = {T(0), T(0), T(0)};
  macro(L{}, fl, r, uu);
#pragma unroll
  for (int d = 0; d < 3; ++d) nu[d * U + k] = uu[d];
}

// Marker m, one warp: U (+)= sum_s W nodes[uid] per component, lanes over the stencil,
// shuffle-reduced in a fixed tree; then F_step = (v_body - U) 2 ds, F_total (ib/mdf.py:38-52).
template <int MODE, typename T>
__device__ __forceinline__ void static_marker(int m, int lane, int first, int use_step, const T* __restrict__ W,
                                              const int32_t* __restrict__ pair_uid, int S, const T* nodes, int U,
                                              const T* state, const T* __restrict__ ds, T ds_scalar, T* Ua, T* Fs,
                                              T* Ft) {
  T acc[3] = {T(0), T(0), T(0)};
  bool firstterm = true;
  for (int s = lane; s < S; s += 32) {
    const int64_t q = (int64_t)m * S + s;
    const T w = W[q];
    const int id = pair_uid[q];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T t = mul_rn(w, body_load<MODE>(nodes + c * U + id));
      acc[c] = firstterm ? t : add_rn(acc[c], t);
    }
    firstterm = false;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc[c] = acc[c] + __shfl_down_sync(0xffffffffu, acc[c], o);
  if (lane == 0) {
    const T d2 = (ds ? ds[m] : ds_scalar) * T(2);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t q = (int64_t)m * 3 + c;
      const T u = first ? acc[c] : Ua[q] + acc[c];
      Ua[q] = u;
      const T fs = mul_rn(state[3 + c] - u, d2);
      Fs[q] = fs;
      Ft[q] = first ? (use_step ? fs : T(0)) : Ft[q] + fs;
    }
  }
}

// Node k of the spread in pair order: sum_p F[m(p)][c] W[p] over the pairs of node k,
// wsort/msort[seg[k] .. seg[k+1]) (weights and marker ids in CSR order, so the loop's loads
// are independent of one another).
template <int MODE, typename T>
__device__ __forceinline__ void static_spread_node(int k, const int32_t* __restrict__ seg,
                                                   const int32_t* __restrict__ msort, const T* __restrict__ wsort,
                                                   const T* F, T a[3]) {
  const int lo = seg[k], hi = seg[k + 1];
  a[0] = a[1] = a[2] = T(0);
#pragma unroll 4
  for (int i = lo; i < hi; ++i) {
    const int m = msort[i];
    const T w = wsort[i];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T t = mul_rn(body_load<MODE>(F + m * 3 + c), w);
      a[c] = i == lo ? t : add_rn(a[c], t);
    }
  }
}

// h = sum_m(-F_total) by one block (256 threads) in a fixed tree (dyn.py:126-136)
template <int MODE, typename T>
__device__ __forceinline__ void static_total_force(const T* F, int M, T* state, T* force_hist) {
  __shared__ T red[3][256];
  const int tid = threadIdx.x;
  for (int c = 0; c < 3; ++c) {
    T acc = T(0);
    for (int m = tid; m < M; m += blockDim.x) {
      const T v = -body_load<MODE>(F + m * 3 + c);
      acc = m == tid ? v : acc + v;
    }
    red[c][tid] = acc;
  }
  __syncthreads();
  for (int o = blockDim.x / 2; o >= 1; o >>= 1) {
    if (tid < o)
      for (int c = 0; c < 3; ++c) red[c][tid] = red[c][tid] + red[c][tid + o];
    __syncthreads();
  }
  if (tid < 3) {
    state[9 + tid] = red[tid][0];
    if (force_hist) force_hist[tid] = red[tid][0];
  }
}

// u at the touched nodes
template <class L, typename T>
__global__ void k_static_node_u(const T* __restrict__ fin, int nx, int ny, int nz, const int* __restrict__ meta,
                                const int32_t* __restrict__ node_cell, int U, T* __restrict__ nu,
                                const int* __restrict__ Ud) {
  // U: the node-array stride; Ud (moving bodies): the number of touched nodes this step
  const int ey = meta[META_WY], ez = meta[META_WZ];
  const int ox = meta[META_OX], oy = meta[META_OY], oz = meta[META_OZ];
  const int64_t n = (int64_t)nx * ny * nz;
  const int nU = Ud ? *Ud : U;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nU; k += gridDim.x * blockDim.x)
    static_node_u<L, T>(k, fin, ny, nz, n, ox, oy, oz, ey, ez, node_cell, U, nu);
}

// One warp per marker
template <typename T>
__global__ void k_static_marker(int first, int use_step, const T* __restrict__ W, const int32_t* __restrict__ pair_uid,
                                int M, int S, const T* __restrict__ nodes, int U, const T* __restrict__ state,
                                const T* __restrict__ ds, T ds_scalar, T* __restrict__ Ua, T* __restrict__ Fs,
                                T* __restrict__ Ft) {
  const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (m >= M) return;
  static_marker<kLoadRO, T>(m, threadIdx.x & 31, first, use_step, W, pair_uid, S, nodes, U, state, ds, ds_scalar, Ua,
                          Fs, Ft);
}

// Node-parallel spread: out[c][k] = scale * sum F[m(p)][c] W[p].  With gw != null the sums
// land in the force window at node_cell[k] instead (scale 1), and block 0 then also forms
// the total force h = sum_m(-F_total).
template <typename T>
__global__ void k_static_spread(const int32_t* __restrict__ seg, const int32_t* __restrict__ msort,
                                const int32_t* __restrict__ node_cell, const T* __restrict__ wsort,
                                const T* __restrict__ F, int U, T scale, T* __restrict__ out, T* gw, int cells,
                                int M, T* state, T* force_hist, const int* __restrict__ Ud) {
  const int nU = Ud ? *Ud : U;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nU; k += gridDim.x * blockDim.x) {
    T a[3];
    static_spread_node<kLoadRO, T>(k, seg, msort, wsort, F, a);
    if (gw) {
      const int cell = node_cell[k];
#pragma unroll
      for (int c = 0; c < 3; ++c) gw[c * cells + cell] = a[c];
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) out[c * U + k] = a[c] * scale;
    }
  }
  if (!gw || blockIdx.x != 0) return;
  static_total_force<kLoadRO, T>(F, M, state, force_hist);
}

// ---- the whole 3-D body step in one launch
// The phases of the per-phase kernels above (node u, then per MDF iteration markers and a
// spread, then the force window and h) in one cooperative launch of G CTAs: CTA b owns the
// nodes [U b / G, U (b + 1) / G) and the markers [M b / G, M (b + 1) / G), and a grid
// barrier separates the phases.  The arithmetic and its order are the per-phase kernels',
// so the results are equal.  On a grid larger than L2 the launch runs beside the grid
// kernel with the HBM saturated; one launch replaces seven dependent ones, each of which
// would wait for SM slots and for its first loads behind the grid kernel's traffic.
constexpr int kBody3Threads = 256;
constexpr int kGridBarrierLimit = 1 << 22;  // polls of a grid barrier (about 0.3 s) before it gives up

template <typename T>
struct Body3Params {
  const T* fin;
  int nx, ny, nz;
  const int* meta;
  const int32_t* node_cell;
  int U;
  const int* Ud;
  const T* W;
  const int32_t* pair_uid;
  int M, S;
  const int32_t* seg;
  const int32_t* msort;
  const T* wsort;
  T* state;
  const T* ds;
  T ds_scalar;
  T* nu;
  T* nv;
  T* Ua;
  T* Fs;
  T* Ft;
  T* gw;
  int cells;
  T* force_hist;
  int n_iter;
  unsigned* bar;  // [0] arrivals, [1] generation, [2] abort flag, [3] CTAs done
  int* status;
};

// Grid barrier over the launch's CTAs (a cooperative launch: all of them are resident).
// Thread 0 arrives with a device-scope release and waits (bounded) for the generation to
// move on; the last CTA to arrive resets the count and publishes the next generation.
// After kGridBarrierLimit polls, or when another CTA gave up, the CTA records
// VS_ERR_TIMEOUT, sets the abort flag and the launch skips its remaining phases.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* status) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned gen;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(gen) : "l"(bar + 1) : "memory");
    unsigned abort_flag;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(abort_flag) : "l"(bar + 2) : "memory");
    if (abort_flag) {
      ok = 0;
    } else {
      __threadfence();
      const unsigned arrived = atomicAdd(bar, 1u);
      if (arrived == gridDim.x - 1) {
        atomicExch(bar, 0u);
        __threadfence();
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(bar + 1), "r"(gen + 1) : "memory");
      } else {
        int it = 0;
        for (;;) {
          unsigned g, ab;
          asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(bar + 1) : "memory");
          if (g != gen) break;
          asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(ab) : "l"(bar + 2) : "memory");
          if (ab || ++it > kGridBarrierLimit) {
            atomicExch(bar + 2, 1u);
            atomicMax(status, VS_ERR_TIMEOUT);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

template <class L, typename T>
__global__ void __launch_bounds__(kBody3Threads) k_body3d_fused(const __grid_constant__ Body3Params<T> B) {
  const int G = (int)gridDim.x, b = (int)blockIdx.x, tid = (int)threadIdx.x;
  const int nU = B.Ud ? *B.Ud : B.U;
  const int k0 = (int)((int64_t)nU * b / G), k1 = (int)((int64_t)nU * (b + 1) / G);
  const int m0 = (int)((int64_t)B.M * b / G), m1 = (int)((int64_t)B.M * (b + 1) / G);
  const int lane = tid & 31, warp = tid >> 5, nwarps = kBody3Threads / 32;
  // the static data of this CTA's markers and nodes into L2 while the node phase runs
  {
    const char* wb = (const char*)(B.W + (int64_t)m0 * B.S);
    const char* ub = (const char*)(B.pair_uid + (int64_t)m0 * B.S);
    const int64_t mbytes = (int64_t)(m1 - m0) * B.S * (int64_t)sizeof(T);
    const int64_t ubytes = (int64_t)(m1 - m0) * B.S * 4;
    for (int64_t o = (int64_t)tid * 128; o < mbytes; o += kBody3Threads * 128)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(wb + o));
    for (int64_t o = (int64_t)tid * 128; o < ubytes; o += kBody3Threads * 128)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(ub + o));
  }
  bool ok = true;
  {
    const int ey = B.meta[META_WY], ez = B.meta[META_WZ];
    const int ox = B.meta[META_OX], oy = B.meta[META_OY], oz = B.meta[META_OZ];
    const int64_t n = (int64_t)B.nx * B.ny * B.nz;
    for (int k = k0 + tid; k < k1; k += kBody3Threads)
      static_node_u<L, T>(k, B.fin, B.ny, B.nz, n, ox, oy, oz, ey, ez, B.node_cell, B.U, B.nu);
  }
  ok = grid_barrier(B.bar, B.status);
  for (int m = m0 + warp; ok && m < m1; m += nwarps)
    static_marker<kLoadL2, T>(m, lane, 1, B.n_iter > 0, B.W, B.pair_uid, B.S, B.nu, B.U, B.state, B.ds, B.ds_scalar, B.Ua,
                           B.Fs, B.Ft);
  for (int it = 0; ok && it + 1 < B.n_iter; ++it) {
    ok = grid_barrier(B.bar, B.status);
    if (!ok) break;
    for (int k = k0 + tid; k < k1; k += kBody3Threads) {
      T a[3];
      static_spread_node<kLoadL2, T>(k, B.seg, B.msort, B.wsort, B.Fs, a);
#pragma unroll
      for (int c = 0; c < 3; ++c) B.nv[c * B.U + k] = a[c] * T(0.5);
    }
    ok = grid_barrier(B.bar, B.status);
    if (!ok) break;
    for (int m = m0 + warp; m < m1; m += nwarps)
      static_marker<kLoadL2, T>(m, lane, 0, 1, B.W, B.pair_uid, B.S, B.nv, B.U, B.state, B.ds, B.ds_scalar, B.Ua, B.Fs,
                             B.Ft);
  }
  if (ok) ok = grid_barrier(B.bar, B.status);
  if (ok) {
    for (int k = k0 + tid; k < k1; k += kBody3Threads) {
      T a[3];
      static_spread_node<kLoadL2, T>(k, B.seg, B.msort, B.wsort, B.Ft, a);
      const int cell = B.node_cell[k];
#pragma unroll
      for (int c = 0; c < 3; ++c) B.gw[c * B.cells + cell] = a[c];
    }
    if (b == 0) static_total_force<kLoadL2, T>(B.Ft, B.M, B.state, B.force_hist);
  }
  // the last CTA out clears the arrival count and the abort flag for the next launch (the
  // generation only ever moves on, so it needs no reset)
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(B.bar + 3, 1u) == gridDim.x - 1) {
      atomicExch(B.bar, 0u);
      atomicExch(B.bar + 2, 0u);
      atomicExch(B.bar + 3, 0u);
    }
  }
}

// ---- many 2-D time steps in one persistent launch
// One cooperative launch of G CTAs in clusters of CL (the body's cluster size) advances
// n_steps time steps of a plan whose body takes the cluster form.  Cluster 0 runs the
// body's step (body2d_cluster_step: markers, stencil, MDF, Newmark, and the nodes of the
// predicted window); every other CTA works as groups of kRunGroup threads, each group
// updating whole tiles of the bulk grid launch's geometry (a row x and kRunGroup * NPT
// consecutive nodes along y, k_step_fast's node order) and, while the face boundaries are
// deferred to the next step's load, tiles of the two x-face planes.  A barrier over all
// CTAs ends every step.  Every node goes through the device functions of the per-step
// launches, so the populations equal vs_run's launch-per-step form bit for bit; what the
// persistent form removes is the launches, the fork and join of streams per step, and the
// body kernel's start-up behind the grid launch's traffic.
constexpr int kRunThreads = 384;
constexpr int kRunGroup = 128;
constexpr int kRunNodes = 4;  // nodes per thread of a grid tile (their loads in flight together)

template <typename T>
struct VivRunParams {
  BodyParams<T> B[2];           // [parity of the step]: populations read, prediction slot
  StepParams<L9, T> SPb[2][2];  // [parity][lazy_in]: the body's window nodes
  StepParams<L9, T> SPm[2][2];  // [parity][lazy_in]: tiles of the bulk launch
  StepParams<L9, T> SPw[2];     // [parity]: x-face plane tiles (lazy_in only)
  T* hist;                      // force history, 3 values per step, or null
  unsigned* bar;                // barrier words: arrivals, generation, abort, exits
  int* status;                  // the plan's status word
  int n_steps;
  int lazy;                     // face boundaries deferred to the next step's load
  int lazy_first;               // the run's first step already reads deferred boundaries
  int chunks_m, rows_m;         // bulk tiles: chunks along y, rows
  int chunks_w;                 // plane tiles per plane
};

// Barrier over every CTA of the run, agreed within each cluster.  After a cluster barrier,
// thread 0 of the cluster's rank-0 CTA adds one to word 0 (release; bit 31: abort) and polls
// it until it reaches (k + 1) x clusters for the k-th barrier of the launch, then acquires;
// it gives up after kGridBarrierLimit polls (abort bit, VS_ERR_TIMEOUT), as does every
// poller that sees the bit.  A second cluster barrier releases the cluster, whose CTAs all
// read rank 0's decision, so a cluster never splits over a timeout and its CTAs keep meeting
// at the same cluster barriers.  false: the run aborts.
__device__ __forceinline__ bool run_barrier(unsigned* bar, int* status, int k, int* ok_s) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  cluster.sync();
  if (cluster.block_rank() == 0 && threadIdx.x == 0) {
    const unsigned target = (unsigned)(k + 1) * (gridDim.x / cluster.num_blocks());
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
    unsigned v;
    int it = 0;
    for (;;) {
      asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
      if ((v & 0x7fffffffu) >= target || (v & 0x80000000u)) break;
      if (++it > kGridBarrierLimit) {
        atomicOr(bar, 0x80000000u);
        atomicMax(status, VS_ERR_TIMEOUT);
        v |= 0x80000000u;
        break;
      }
      __nanosleep(20);
    }
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    *ok_s = (v & 0x80000000u) ? 0 : 1;
  }
  cluster.sync();
  return *cluster.map_shared_rank(ok_s, 0) != 0;
}

template <typename T, int R, int COLL>
__global__ void __launch_bounds__(kRunThreads, 1) k_viv_run(const __grid_constant__ VivRunParams<T> P) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ int ok_s;
  const int CL = (int)cluster.num_blocks();
  const bool body = (int)blockIdx.x < CL;
  const int gpc = (int)blockDim.x / kRunGroup, gt = (int)threadIdx.x % kRunGroup;
  const int ng = ((int)gridDim.x - CL) * gpc, g0 = ((int)blockIdx.x - CL) * gpc + (int)threadIdx.x / kRunGroup;
  const int nm = P.chunks_m * P.rows_m;
  bool ok = true;
  for (int s = 0; s < P.n_steps && ok; ++s) {
    const int p = s & 1;
    const int lz = P.lazy && (s > 0 || P.lazy_first) ? 1 : 0;
    if (body) {
      body2d_cluster_step<T, R, COLL>(P.B[p], P.SPb[p][lz], P.hist ? P.hist + 3 * (int64_t)s : nullptr);
    } else {
      const int nt = nm + (lz ? 2 * P.chunks_w : 0);
      for (int t = g0; t < nt; t += ng) {
        if (t < nm) {
          const int by = t / P.chunks_m, bx = t - by * P.chunks_m;
          step_block_n_t<T, COLL, kFeatSkip, kRunNodes>(P.SPm[p][lz], bx, by, gt, kRunGroup);
        } else {
          const int u = t - nm, by = u / P.chunks_w, bx = u - by * P.chunks_w;
          step_block_t<L9, T, COLL, kFeatGeneral | kFeatWalls>(P.SPw[p], bx, by, gt, kRunGroup);
        }
      }
    }
    ok = run_barrier(P.bar, P.status, s, &ok_s);
  }
  // the last cluster out resets the arrival count (and the abort bit) for the next launch;
  // a CTA leaves only after its cluster has read rank 0's last decision
  cluster.sync();
  if (cluster.block_rank() == 0 && threadIdx.x == 0 && atomicAdd(P.bar + 1, 1u) == gridDim.x / (unsigned)CL - 1) {
    atomicExch(P.bar, 0u);
    atomicExch(P.bar + 1, 0u);
  }
}

// ---- the fixed 3-D body step in one thread-block cluster
// The phases of the per-phase kernels over a cluster of CL CTAs whose exchanges stay in
// distributed shared memory: CTA r holds the stencil weights and pair node keys of its
// markers [part[CL+1+r], part[CL+2+r]), and the CSR slice, weights, marker ids and node
// values of its nodes [part[r], part[r+1]) (split so that every CTA spreads about the same
// number of pairs).  A marker reads the nodes of its stencil from the CTAs that own them
// (key = owner << 16 | local index), and writes the force it spreads into every CTA's
// replica of the marker forces, so a spread reads only its own shared memory.  Hardware
// cluster barriers separate the phases.  Global memory is read once at the start (the
// populations at the touched nodes, the plan's static arrays) and written once at the end
// (the force window and h), so the phases do not queue behind the grid launch's traffic.
// The arithmetic and its order are the per-phase kernels': the results are equal.
constexpr int kBody3ClusterThreads = 1024;

template <typename T>
struct Body3ClusterParams {
  const T* fin;
  int nx, ny, nz;
  const int* meta;
  const int32_t* node_cell;
  const T* W;          // (M, S) stencil weights
  const int32_t* pkey; // (M, S) owner << 16 | index in the owner's node slice
  int M, S;
  const int32_t* seg;
  const int32_t* msort;
  const T* wsort;
  T* state;
  const T* ds;
  T ds_scalar;
  T* gw;
  int cells;
  T* force_hist;
  int n_iter;
  const int* part;     // node bounds [CL + 1], then marker bounds [CL + 1]
  int MK, NK, PK;      // per-CTA capacities: markers, nodes, node-side pairs
};

template <typename T>
__host__ __device__ inline size_t body3_cluster_smem(int M, int S, int MK, int NK, int PK) {
  const size_t nT = (size_t)MK * S + PK + 3 * (size_t)NK + 3 * (size_t)M + 6 * (size_t)MK + 3 * 256;
  const size_t nI = (size_t)MK * S + (NK + 1) + PK;
  return nT * sizeof(T) + nI * sizeof(int32_t);
}

template <class L, typename T>
__global__ void __launch_bounds__(kBody3ClusterThreads) k_body3d_cluster(const __grid_constant__ Body3ClusterParams<T> B) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem[];
  const int CL = (int)cluster.num_blocks(), r = (int)cluster.block_rank();
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const int M = B.M, S = B.S, MK = B.MK, NK = B.NK, PK = B.PK;
  T* Wm = (T*)smem;           // [MK S]
  T* wsl = Wm + MK * S;       // [PK]
  T* nodes = wsl + PK;        // [3 NK] u, then the spread force step, of this CTA's nodes
  T* Frep = nodes + 3 * NK;   // [3 M] the forces being spread, every marker
  T* Ua = Frep + 3 * M;       // [3 MK] this CTA's markers
  T* Ftl = Ua + 3 * MK;       // [3 MK]
  T* red = Ftl + 3 * MK;      // [3 256]
  int32_t* keym = (int32_t*)(red + 3 * 256);  // [MK S]
  int32_t* segl = keym + MK * S;              // [NK + 1]
  int32_t* msl = segl + NK + 1;               // [PK]
  const int n0 = B.part[r], n1 = B.part[r + 1];
  const int m0 = B.part[CL + 1 + r], m1 = B.part[CL + 2 + r];
  const int nn = n1 - n0, nm = m1 - m0;
  const int q0 = B.seg[n0], nq = B.seg[n1] - q0;
  // static slices
  for (int i = tid; i < nm * S; i += nt) {
    Wm[i] = B.W[(int64_t)m0 * S + i];
    keym[i] = B.pkey[(int64_t)m0 * S + i];
  }
  for (int i = tid; i <= nn; i += nt) segl[i] = B.seg[n0 + i] - q0;
  for (int i = tid; i < nq; i += nt) {
    msl[i] = B.msort[q0 + i];
    wsl[i] = B.wsort[q0 + i];
  }
  // u at this CTA's nodes (vivsim/lbm3d/basic.py:90-106)
  {
    const int ey = B.meta[META_WY], ez = B.meta[META_WZ];
    const int ox = B.meta[META_OX], oy = B.meta[META_OY], oz = B.meta[META_OZ];
    const int64_t n = (int64_t)B.nx * B.ny * B.nz;
    for (int k = tid; k < nn; k += nt) {
      const int cell = B.node_cell[n0 + k];
      const int wx = cell / (ey * ez), wy = (cell / ez) % ey, wz = cell % ez;
      const int64_t pn = ((int64_t)(ox + wx) * B.ny + (oy + wy)) * B.nz + (oz + wz);
      T fl[L::Q];
#pragma unroll
      for (int i = 0; i < L::Q; ++i) fl[i] = __ldg(B.fin + i * n + pn);
      T rr, uu[3] = {T(0), T(0), T(0)};
      macro(L{}, fl, rr, uu);
#pragma unroll
      for (int d = 0; d < 3; ++d) nodes[d * NK + k] = uu[d];
    }
  }
  cluster.sync();
  T v_body[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) v_body[c] = B.state[3 + c];
  const int n_marker_phases = B.n_iter > 1 ? B.n_iter : 1;
  for (int ph = 0; ph < n_marker_phases; ++ph) {
    const bool first = ph == 0, last = ph + 1 == n_marker_phases;
    const int use_step = first ? (B.n_iter > 0) : 1;
    // markers: interpolate the node values (ib/stencil.py:54-78), force step and total
    // (ib/mdf.py:38-52), in k_static_marker's order
    for (int ml = warp; ml < nm; ml += nwarps) {
      const int m = m0 + ml;
      T acc[3] = {T(0), T(0), T(0)};
      bool firstterm = true;
      for (int s = lane; s < S; s += 32) {
        const T w = Wm[ml * S + s];
        const int key = keym[ml * S + s];
        const T* rn = cluster.map_shared_rank(nodes, key >> 16);
        const int li = key & 0xffff;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const T t = mul_rn(w, rn[c * NK + li]);
          acc[c] = firstterm ? t : add_rn(acc[c], t);
        }
        firstterm = false;
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) acc[c] = acc[c] + __shfl_down_sync(0xffffffffu, acc[c], o);
      T out[3];
      if (lane == 0) {
        const T d2 = (B.ds ? B.ds[m] : B.ds_scalar) * T(2);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const T u = first ? acc[c] : Ua[ml * 3 + c] + acc[c];
          Ua[ml * 3 + c] = u;
          const T fs = mul_rn(v_body[c] - u, d2);
          const T ft = first ? (use_step ? fs : T(0)) : Ftl[ml * 3 + c] + fs;
          Ftl[ml * 3 + c] = ft;
          out[c] = last ? ft : fs;  // the spread that follows: a force step, or the totals
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) out[c] = __shfl_sync(0xffffffffu, out[c], 0);
      // into every CTA's replica: lane j writes component j % 3 to CTA j / 3
      for (int j = lane; j < 3 * CL; j += 32) {
        T* dst = cluster.map_shared_rank(Frep, j / 3);
        const int c = j % 3;
        dst[m * 3 + c] = c == 0 ? out[0] : (c == 1 ? out[1] : out[2]);
      }
    }
    cluster.sync();
    if (last) break;
    // spread of the force step to this CTA's nodes (k_static_spread's order), times 0.5
    for (int k = tid; k < nn; k += nt) {
      T a[3];
      static_spread_node<kLoadPlain, T>(k, segl, msl, wsl, Frep, a);
#pragma unroll
      for (int c = 0; c < 3; ++c) nodes[c * NK + k] = a[c] * T(0.5);
    }
    cluster.sync();
  }
  // the totals into the force window, and h = sum_m(-F_total) (dyn.py:126-136)
  for (int k = tid; k < nn; k += nt) {
    T a[3];
    static_spread_node<kLoadPlain, T>(k, segl, msl, wsl, Frep, a);
    const int cell = B.node_cell[n0 + k];
#pragma unroll
    for (int c = 0; c < 3; ++c) B.gw[c * B.cells + cell] = a[c];
  }
  if (r == 0) {
    // static_total_force's order over 256 threads
    for (int c = 0; c < 3 && tid < 256; ++c) {
      T acc = T(0);
      for (int m = tid; m < M; m += 256) {
        const T v = -Frep[m * 3 + c];
        acc = m == tid ? v : acc + v;
      }
      red[c * 256 + tid] = acc;
    }
    __syncthreads();
    for (int o = 128; o >= 1; o >>= 1) {
      if (tid < o)
        for (int c = 0; c < 3; ++c) red[c * 256 + tid] = red[c * 256 + tid] + red[c * 256 + tid + o];
      __syncthreads();
    }
    if (tid < 3) {
      B.state[9 + tid] = red[tid * 256];
      if (B.force_hist) B.force_hist[tid] = red[tid * 256];
    }
  }
}

// moving 3-D body (examples/3d/oscillating_cylinder.py:228-283): markers X0 + d, window
// origin floor(min X) - R + 1 (rounded as the markers are), weights and window-cell keys of
// every (marker, stencil point) pair, from coordinates relative to the window
// (ib3d/stencil.py:7-59).  The window must stay inside the body's box (else VS_ERR_RANGE).
template <typename T>
__global__ void k_mov3_stencil(const T* __restrict__ X0, const T* __restrict__ state, double lo0, double lo1,
                               double lo2, int R, int kernel, int c0, int c1, int c2, int bx0, int bx1, int by0,
                               int by1, int bz0, int bz1, int* meta, T* __restrict__ W, int32_t* __restrict__ keys,
                               int M) {
  const T d0 = state[6], d1 = state[7], d2 = state[8];
  const int o0 = ifloor((T)lo0 + d0) - R + 1, o1 = ifloor((T)lo1 + d1) - R + 1, o2 = ifloor((T)lo2 + d2) - R + 1;
  const bool inside = o0 >= bx0 && o0 + c0 <= bx1 && o1 >= by0 && o1 + c1 <= by1 && o2 >= bz0 && o2 + c2 <= bz1;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    meta[META_OX] = o0; meta[META_OY] = o1; meta[META_OZ] = o2;
    meta[META_WX] = inside ? c0 : 0; meta[META_WY] = c1; meta[META_WZ] = c2;
    if (!inside) meta[META_STATUS] = VS_ERR_RANGE;
  }
  const int w = 2 * R, s = w * w * w;
  const int64_t total = (int64_t)M * s;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int mk = (int)(p / s), k = (int)(p % s);
    const int ox = k / (w * w) - R + 1, oy = (k / w) % w - R + 1, oz = k % w - R + 1;
    const T x = (X0[3 * mk] + d0) - (T)o0, y = (X0[3 * mk + 1] + d1) - (T)o1, z = (X0[3 * mk + 2] + d2) - (T)o2;
    const int sx = ifloor(x) + ox, sy = ifloor(y) + oy, sz = ifloor(z) + oz;
    W[p] = (delta(kernel, (T)sx - x) * delta(kernel, (T)sy - y)) * delta(kernel, (T)sz - z);
    const bool ok = inside && sx >= 0 && sx < c0 && sy >= 0 && sy < c1 && sz >= 0 && sz < c2;
    keys[p] = ok ? (sx * c1 + sy) * c2 + sz : -1;  // out-of-window pairs are dropped (and flagged)
    if (!ok && inside) meta[META_STATUS] = VS_ERR_RANGE;
  }
}

// touched-node count of this step's CSR (uid is 0-based), and the end of the last segment
__global__ void k_csr_count(const int32_t* __restrict__ uid, int64_t P, int* U, int32_t* seg) {
  const int u = uid[P - 1] + 1;
  *U = u;
  seg[u] = (int32_t)P;
}

// added mass h += a A (vortex_induced_vibration.py:136) and the Newmark update (dyn.py:5-51)
// of the free DOFs; h (without the added mass) comes from the spread kernel's reduction
template <typename T>
__global__ void k_body_newmark(T* state, int f0, int f1, int f2, T k1, T k2, T c1, T c2, T dt, T damp, T stiff,
                               T den, T area, T* force_hist) {
  const int c = threadIdx.x;
  if (c >= 3) return;
  const int fr = c == 0 ? f0 : (c == 1 ? f1 : f2);
  const T ac = state[c], vc = state[3 + c], dc = state[6 + c];
  const T hh = add_rn(state[9 + c], mul_rn(ac, area));
  T an = ac, vn = vc, dn = dc;
  if (fr) {
    const T v1 = add_rn(vc, mul_rn(k1, ac));
    const T v2 = add_rn(add_rn(dc, mul_rn(dt, vc)), mul_rn(k2, ac));
    an = sub_rn(sub_rn(hh, mul_rn(damp, v1)), mul_rn(stiff, v2)) / den;
    vn = add_rn(mul_rn(c1, an), v1);
    dn = add_rn(mul_rn(c2, an), v2);
  }
  state[c] = an;
  state[3 + c] = vn;
  state[6 + c] = dn;
  state[9 + c] = hh;
  if (force_hist) force_hist[c] = hh;
}

__global__ void k_compact_csr(const int32_t* __restrict__ skeys, const int32_t* __restrict__ head,
                              const int32_t* __restrict__ uid, int64_t P, int32_t* __restrict__ node_cell,
                              int32_t* __restrict__ seg) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x)
    if (head[p]) {
      node_cell[uid[p]] = skeys[p];
      seg[uid[p]] = (int32_t)p;
    }
}

// obstacle bounce-back in place (the last step of a run: its output must be complete)
template <class L, typename T>
__global__ void k_mask_bb(T* f, const uint8_t* __restrict__ mask, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    if (!mask[p]) continue;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      const int o = L::opp(i);
      if (o > i) {
        const T t = f[i * n + p];
        f[i * n + p] = f[o * n + p];
        f[o * n + p] = t;
      }
    }
  }
}

// body state from a device copy; a 2-D body's window prediction restarts from the new
// displacement (floor of the smallest marker coordinate, as vs_body_set_state does)
template <typename T>
__global__ void k_set_state(T* state, const T* src, int* meta, double lo0, double lo1, int R,
                            const __grid_constant__ BodyParams<T> B) {
  const int i = threadIdx.x;
  if (i < 12) state[i] = src[i];
  if (meta && i < 2) {
    int c;
    if (B.rot) {  // smallest stencil corner of the turned markers, as the body kernel finds it
      T d[3], v[3] = {T(0), T(0), T(0)};
      for (int k = 0; k < 3; ++k) d[k] = src[6 + k];
      const Kin2<T> kin(B, d, v);
      int lo = INT_MAX;
      for (int m = 0; m < B.M; ++m) {
        T x, y;
        kin.xy(B, m, x, y);
        const int f = ifloor(i == 0 ? x : y);
        lo = f < lo ? f : lo;
      }
      c = lo - R + 1;
    } else {
      c = (int)floor((i == 0 ? (T)lo0 : (T)lo1) + src[6 + i]) - R + 1;
    }
    meta[META_PX + i] = c;
    meta[META_PX2 + i] = c;
  }
}

// NaN/Inf watchdog: any non-finite value sets the status word (first error kept)
template <typename T>
__global__ void k_check_finite(const T* __restrict__ f, int64_t n, int* status) {
  bool bad = false;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(f[p]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(status, 0, VS_ERR_NONFINITE);
}

template <typename T>
__global__ void k_fill(T* p, T v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

}  // namespace vs

using namespace vs;

// ====================================================================== plans
struct vs_lattice_plan {
  vs_lattice_cfg cfg;
  int dim;
  int64_t n;
  void* pre_buf[VS_MAX_BC];  // bounce-back face buffers
  void* cbc_buf[VS_MAX_BC];  // characteristic walls: rho_next, u_next (1 + dim face arrays)
  int bc_group[VS_MAX_BC];   // group id of each boundary op
  int n_groups;
  int lazy_ok;               // all boundaries in one launch group and none needs pre-stream data
  int* d_status;             // device status word of the grid kernels (VS_ERR_TIMEOUT)
  int tma_tb;                // tile width of the TMA grid kernel, 0 when it does not apply
  int bb_load;               // set per step: the input still lacks the obstacle bounce-back
  int tma_grid;              // persistent CTAs of the TMA grid kernel
  int run_form;              // VS_RUN_STEPS or VS_RUN_PERSISTENT (vs_lattice_set_run_form)
  int stream_pop;            // one population buffer is larger than L2: a grid launch beside
                             // body kernels streams it (evict-first) past their working set
  // graph cache
  cudaGraphExec_t graph;
  const void* g_fa;
  const void* g_fb;
  const void* g_hist;
  const void* g_body;
  int g_steps;
  cudaStream_t g_stream;
};

struct vs_body_plan {
  vs_body_cfg cfg;
  int dim, M, S, C;
  int cap[3];
  void* d_X0;     // (M) x, (M) y [, (M) z]  or (M,3) coords for 3-D
  void* d_ds;     // (M) or null
  void* d_state;  // 12 values
  void* d_base;   // fluid-structure sub-iterations: the step's saved state (9 values) or null
  int fsi;        // fluid-structure passes per step (>= 1)
  void* d_gw;     // window force (C, cells)
  int* d_meta;
  // 3-D fixed body: stencil and its compacted CSR (built once)
  void* d_W;
  int32_t* d_I;
  void* d_ws;       // CSR workspace (holds the sorted pair ids and pair -> node ids)
  size_t ws_bytes;
  int32_t* sids;    // views into d_ws
  int32_t* pair_uid;
  int32_t* d_node_cell;
  int32_t* d_seg;
  int prio;         // priority of the side-stream launches (the device's highest)
  unsigned* d_bar;  // grid barrier words of the fused 3-D body kernel
  int c3;           // CTAs of the 3-D body cluster kernel (0: not used)
  size_t c3_smem;
  int c3_cap[3];    // per-CTA markers, nodes, node-side pairs
  int* d_c3part;    // node bounds [c3 + 1], marker bounds [c3 + 1]
  int32_t* d_pkey;  // (M, S): owner CTA << 16 | index in its node slice
  int fused3;       // CTAs of the fused 3-D body kernel (0: the per-phase kernels)
  void* d_wsort;    // stencil weights of the pairs in CSR order
  int32_t* d_msort; // marker ids of the pairs in CSR order
  int U;            // touched nodes
  void* d_nu;       // 3 x U node velocity
  void* d_nv;       // 3 x U node force step
  void* d_mk;       // U, F_step, F_total: 3 x (3 M)
  size_t smem;
  int row_len, bulk;  // 2-D body kernel: staged row length, bulk staging on/off
  int chain, chain_k; // 2-D body kernel: chain form and its width
  int cluster, cl_size;  // 2-D body kernel: cluster form (with the box update) and its CTAs
  int cl_threads;        // threads per CTA of the cluster form
  int parity;            // cluster form: prediction slot of the next step
  size_t cl_smem;
  int run_ctas;          // CTAs of the persistent run (k_viv_run), 0 where it does not apply
  size_t run_smem;
  CUtensorMap maps[2]; // tensor maps of the last two population buffers seen
  const void* map_ptr[2];
  int map_next;
  double nm[13];  // k1, k2, c1, c2, dt, damping, stiffness, den, area; rotation: damping, stiffness, den, added inertia
  int rot;        // 2-D body with a free rotation (DOF 2 is the angle about the initial centre)
  int box[6];    // region the body's window never leaves (half-open x0,x1,y0,y1,z0,z1)
  double lo_t[2];  // 2-D: smallest marker x and y, rounded to the plan precision
  double lo_t3;    // 3-D: smallest marker z, rounded
  int* d_U;        // moving 3-D body: touched nodes of the current step (device)
  cudaStream_t side;
  cudaEvent_t ev_fork, ev_join;
  cudaStream_t side2;    // cluster form: the lazy face planes, beside the grid launch
  cudaEvent_t ev_join2;
};

static size_t dsize(int dtype) { return dtype == VS_F64 ? 8 : 4; }

// the marker geometry k_set_state needs (turning 2-D bodies)
template <typename T>
static BodyParams<T> kin_params(const vs_body_plan* b) {
  BodyParams<T> P{};
  P.X0 = (const T*)b->d_X0;
  P.Y0 = (const T*)b->d_X0 + b->M;
  P.M = b->M;
  P.rot = b->rot;
  P.cx = (T)b->cfg.center_x;
  P.cy = (T)b->cfg.center_y;
  return P;
}

static void free_lattice(vs_lattice_plan* p) {
  if (!p) return;
  for (int k = 0; k < VS_MAX_BC; ++k)
    if (p->pre_buf[k]) cudaFree(p->pre_buf[k]);
  for (int k = 0; k < VS_MAX_BC; ++k)
    if (p->cbc_buf[k]) cudaFree(p->cbc_buf[k]);
  if (p->graph) cudaGraphExecDestroy(p->graph);
  if (p->d_status) cudaFree(p->d_status);
  delete p;
}

static void free_body(vs_body_plan* b) {
  if (!b) return;
  void* ptrs[] = {b->d_X0, b->d_ds, b->d_state, b->d_base, b->d_gw, b->d_meta, b->d_W, b->d_I, b->d_ws,
                  b->d_node_cell, b->d_seg, b->d_nu, b->d_nv, b->d_mk, b->d_U, b->d_wsort, b->d_msort, b->d_bar, b->d_c3part, b->d_pkey};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_join) cudaEventDestroy(b->ev_join);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->ev_join2) cudaEventDestroy(b->ev_join2);
  if (b->side2) cudaStreamDestroy(b->side2);
  delete b;
}

template <typename T>
static WallArgs<T> wall_args_from_bc(const vs_bc& bc, const vs_lattice_plan* L, int k) {
  WallArgs<T> A{};
  A.kind = bc.kind;
  A.mode = bc.mode;
  A.loc = bc.loc;
  A.n[0] = L->cfg.nx;
  A.n[1] = L->cfg.ny;
  A.n[2] = L->cfg.nz;
  double rho = bc.rho, u3[3] = {bc.ux, bc.uy, bc.uz};
  if (bc.mode == VS_WALL_CHARACTERISTIC) {  // wall data per node, written by k_cbc_face this step
    const int64_t nf = face_size(bc.loc, A.n);
    const T* buf = (const T*)L->cbc_buf[k];
    A.mode = VS_WALL_GIVEN;
    A.rho_arr = buf;
    for (int d = 0; d < L->dim; ++d) A.u_arr[d] = buf + (1 + d) * nf;
    const double zero[3] = {0.0, 0.0, 0.0};
    wall_args_scalars(A, 1.0, zero, L->dim);
    A.un_scalar = 0;
    A.all_scalar = 0;
    return A;
  }
  if (bc.mode == VS_WALL_FORCE_CORRECTED) {
    const double g3[3] = {bc.gx, bc.gy, bc.gz};
    for (int d = 0; d < 3; ++d) u3[d] = u3[d] - (g3[d] * 0.5) / rho;
  }
  A.un_scalar = bc.mode != VS_WALL_PRESSURE;
  A.all_scalar = bc.mode == VS_WALL_GIVEN || bc.mode == VS_WALL_FORCE_CORRECTED;
  wall_args_scalars(A, rho, u3, L->dim);
  A.f_pre = (const T*)L->pre_buf[k];
  A.pre_stride = face_size(bc.loc, A.n);
  A.pre_face = 1;
  return A;
}

// Characteristic walls: rho_next and u_next of every face node from the step's INPUT
// populations (the moments a composed step takes with get_macroscopic before colliding) at
// the wall and the next two planes, into the plan's face buffer; the face epilogue then
// imposes them with the boundary's scheme.  A masked node whose obstacle bounce-back is
// still pending (applied on load) is swapped first, as the grid kernel does.
template <class L, typename T>
__global__ void k_cbc_face(const T* __restrict__ f, int nx, int ny, int nz, int loc, const uint8_t* mask,
                           int mask_load, T* __restrict__ buf) {
  const int nn[3] = {nx, ny, nz};
  const int64_t n = (int64_t)nx * ny * nz;
  const int64_t nf = face_size(loc, nn);
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= nf) return;
  const int a = loc_axis(loc), sg = loc_sign(loc);
  T r[3], un[3], u0[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int64_t p = face_node(loc, nn, j, k);
    const bool swap = mask_load && mask && mask[p];
    T fl[L::Q], rr, uu[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int i = 0; i < L::Q; ++i) fl[i] = f[(int64_t)(swap ? L::opp(i) : i) * n + p];
    macro(L{}, fl, rr, uu);
    r[k] = rr;
    un[k] = uu[a];
    if (k == 0)
#pragma unroll
      for (int d = 0; d < 3; ++d) u0[d] = uu[d];
  }
  T rn, vn;
  cbc_values<T>(sg, cbc_cs<T>(L::D), r[0], r[1], r[2], un[0], un[1], un[2], rn, vn);
  buf[j] = rn;
#pragma unroll
  for (int d = 0; d < L::D; ++d) buf[(1 + d) * nf + j] = d == a ? vn : u0[d];
}

static int enqueue_cbc(const vs_lattice_plan* LP, const void* fin, cudaStream_t st) {
  const vs_lattice_cfg& c = LP->cfg;
  for (int k = 0; k < c.n_bc; ++k) {
    if (c.bc[k].mode != VS_WALL_CHARACTERISTIC) continue;
    const int nn[3] = {c.nx, c.ny, c.nz};
    const int64_t nf = face_size(c.bc[k].loc, nn);
    int rc = dispatch(c.q, c.dtype, [&](auto l, auto t) -> int {
      using LL = decltype(l);
      using T = typename decltype(t)::type;
      k_cbc_face<LL, T><<<grid_for(nf, 128), 128, 0, st>>>((const T*)fin, c.nx, c.ny, c.nz, c.bc[k].loc,
                                                           c.obstacle_mask, LP->bb_load, (T*)LP->cbc_buf[k]);
      VS_CHECK_LAUNCH("vs_step characteristic wall");
      return VS_OK;
    });
    if (rc) return rc;
  }
  return VS_OK;
}

static int enqueue_bcs(const vs_lattice_plan* L, void* f, cudaStream_t st) {
  const vs_lattice_cfg& c = L->cfg;
  return dispatch(c.q, c.dtype, [&](auto l, auto t) -> int {
    using LL = decltype(l);
    using T = typename decltype(t)::type;
    int k = 0;
    while (k < c.n_bc) {
      BcGroup<T> G{};
      const int gid = L->bc_group[k];
      int64_t nfmax = 0;
      while (k < c.n_bc && L->bc_group[k] == gid && G.count < 2) {
        G.A[G.count] = wall_args_from_bc<T>(c.bc[k], L, k);
        G.nf[G.count] = face_size(c.bc[k].loc, G.A[G.count].n);
        nfmax = G.nf[G.count] > nfmax ? G.nf[G.count] : nfmax;
        ++G.count;
        ++k;
      }
      dim3 grid(grid_for(nfmax, 128), G.count);
      k_bc<LL, T><<<grid, 128, 0, st>>>(G, (T*)f);
      VS_CHECK_LAUNCH("vs_step face kernel");
    }
    return VS_OK;
  });
}

template <class L, typename T>
static StepParams<L, T> make_step_params(const vs_lattice_plan* LP, const vs_body_plan* B, const void* fin,
                                         void* fout) {
  const vs_lattice_cfg& c = LP->cfg;
  StepParams<L, T> P{};
  P.fin = (const T*)fin;
  P.fout = (T*)fout;
  P.nx = c.nx;
  P.ny = c.ny;
  P.nz = c.nz;
  P.n = (int)LP->n;
  P.cp.omega = (T)c.omega;
  P.cp.one_m_omega = (T)(1.0 - c.omega);
  P.cp.inv_omega = (T)(1.0 / c.omega);
  P.cp.one_m_inv = (T)(1.0 - 1.0 / c.omega);
  P.cp.mrt = nullptr;
  P.forcing = c.forcing;
  P.has_g0 = (c.g_uniform[0] != 0.0 || c.g_uniform[1] != 0.0 || c.g_uniform[2] != 0.0) && c.forcing != VS_FORCE_NONE;
  for (int d = 0; d < 3; ++d) P.g0[d] = (T)c.g_uniform[d];
  P.guo_scale = (T)(1.0 - 0.5 * c.omega);
  P.gw = B ? (const T*)B->d_gw : nullptr;
  P.meta = B ? B->d_meta : nullptr;
  P.status = LP->d_status;
  P.mask = c.obstacle_mask;
  P.mask_load = c.obstacle_mask && LP->bb_load ? 1 : 0;
  P.n_pre = 0;
  for (int k = 0; k < c.n_bc; ++k) {
    if (c.bc[k].kind == VS_BC_BB || c.bc[k].kind == VS_BC_SPECULAR) {
      P.pre_loc[P.n_pre] = c.bc[k].loc;
      P.pre_buf[P.n_pre] = (T*)LP->pre_buf[k];
      ++P.n_pre;
    }
  }
  for (int i = 0; i < L::Q * L::Q; ++i) {
    P.op[i] = (T)c.mrt_op[i];
    P.fop[i] = (T)c.mrt_fop[i];
  }
  return P;
}


// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// Tensor map of population buffer f (viewed as (ny, nx, 9)) with the body's region box.
static const CUtensorMap* body_map(vs_body_plan* b, const vs_lattice_plan* L, const void* f) {
  for (int k = 0; k < 2; ++k)
    if (b->map_ptr[k] == f) return &b->maps[k];
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_tiled();
  if (!enc) return nullptr;
  const int ts = L->cfg.dtype == VS_F64 ? 8 : 4;
  const cuuint64_t dims[3] = {(cuuint64_t)L->cfg.ny, (cuuint64_t)L->cfg.nx, 9};
  const cuuint64_t strides[2] = {(cuuint64_t)L->cfg.ny * ts, (cuuint64_t)L->n * ts};
  const cuuint32_t box[3] = {(cuuint32_t)b->row_len, (cuuint32_t)(b->cap[0] + 2), 9};
  const cuuint32_t estr[3] = {1, 1, 1};
  const int k = b->map_next;
  CUresult r = enc(&b->maps[k], ts == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                   const_cast<void*>(f), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return nullptr;
  b->map_ptr[k] = f;
  b->map_next = 1 - k;
  return &b->maps[k];
}

// Parameters of the 2-D body kernel for one step reading populations fin.  allow_bulk: the
// window may be staged by a tensor-map TMA copy (the map travels in the parameters).
template <typename T>
static BodyParams<T> body_params2d(vs_body_plan* B, const vs_lattice_plan* LP, const void* fin, void* force_hist,
                                   bool allow_bulk) {
  BodyParams<T> P{};
  P.fin = (const T*)fin;
  P.nx = LP->cfg.nx;
  P.ny = LP->cfg.ny;
  P.X0 = (const T*)B->d_X0;
  P.Y0 = (const T*)B->d_X0 + B->M;
  P.ds_arr = (const T*)B->d_ds;
  P.ds2_scalar = (T)B->cfg.ds_scalar * T(2);
  P.M = B->M;
  P.kernel = B->cfg.kernel;
  P.n_iter = B->cfg.n_iter;
  P.cap_x = B->cap[0];
  P.cap_y = B->cap[1];
  // without staging the kernel's shared memory holds no window rows (its size is
  // computed for row_len 0 then)
  P.row_len = allow_bulk ? B->row_len : 0;
  P.bulk = 0;
  if (allow_bulk && B->bulk && ((uintptr_t)fin % 16) == 0) {
    const CUtensorMap* m = body_map(B, LP, fin);
    if (m) {
      P.map = *m;
      P.bulk = 1;
    }
  }
  for (int q = 0; q < 4; ++q) P.box[q] = B->box[q];
  P.state = (T*)B->d_state;
  P.base = B->fsi > 1 ? (T*)B->d_base : nullptr;
  P.fsi_first = 1;
  P.gw = (T*)B->d_gw;
  P.meta = B->d_meta;
  P.force_hist = (T*)force_hist;
  for (int c = 0; c < 3; ++c) P.free_dof[c] = B->cfg.free_dof[c];
  P.k1 = (T)B->nm[0]; P.k2 = (T)B->nm[1]; P.c1 = (T)B->nm[2]; P.c2 = (T)B->nm[3]; P.dt = (T)B->nm[4];
  P.damp = (T)B->nm[5]; P.stiff = (T)B->nm[6]; P.den = (T)B->nm[7]; P.area = (T)B->nm[8];
  P.rot = B->rot;
  P.cx = (T)B->cfg.center_x;
  P.cy = (T)B->cfg.center_y;
  P.rot_damp = (T)B->nm[9]; P.rot_stiff = (T)B->nm[10]; P.rot_den = (T)B->nm[11]; P.rot_added = (T)B->nm[12];
  P.chain_k = B->chain_k;
  return P;
}

static int enqueue_body(vs_body_plan* B, const vs_lattice_plan* LP, const void* fin, void* force_hist,
                        cudaStream_t st) {
  const int dtype = B->cfg.dtype;
  if (B->dim == 2) {
    return dispatch_t(dtype, [&](auto t) -> int {
      using T = typename decltype(t)::type;
      BodyParams<T> P = body_params2d<T>(B, LP, fin, force_hist, true);
      // one pass per fluid-structure sub-iteration; the last one leaves the force window,
      // the body force and the state of the step
      for (int it = 0; it < B->fsi; ++it) {
        P.fsi_first = it == 0;
        if (B->chain) body2d_chain_launch<T>(B->cfg.radius, B->smem, st, P);
        else body2d_launch<T>(B->cfg.radius, B->smem, st, P);
        VS_CHECK_LAUNCH("vs_step body kernel");
      }
      return VS_OK;
    });
  }
  // 3-D fixed body: static stencil and CSR; node- and marker-parallel kernels
  return dispatch(LP->cfg.q, dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    const int U = B->U, M = B->M, S = B->S;
    const int cells = B->cap[0] * B->cap[1] * B->cap[2];
    if (B->cfg.moving) {
      // markers follow the body; the window follows its stencil box; the (node, pair) CSR
      // is rebuilt for this step
      const int64_t P = (int64_t)M * S;
      cudaError_t e = cudaMemsetAsync(B->d_gw, 0, sizeof(T) * 3 * cells, st);
      if (e != cudaSuccess) return cuda_status(e, "vs_step body window");
      k_mov3_stencil<T><<<grid_for(P, 256), 256, 0, st>>>(
          (const T*)B->d_X0, (const T*)B->d_state, B->lo_t[0], B->lo_t[1], B->lo_t3, B->cfg.radius, B->cfg.kernel,
          B->cap[0], B->cap[1], B->cap[2], B->box[0], B->box[1], B->box[2], B->box[3], B->box[4], B->box[5],
          B->d_meta, (T*)B->d_W, B->d_I, M);
      IbCsrView v{};
      int rc = ib_build_csr(B->d_I, P, cells, B->d_ws, M, S, &v, st);
      if (rc) return rc;
      k_csr_count<<<1, 1, 0, st>>>(v.uid, P, B->d_U, B->d_seg);
      k_compact_csr<<<grid_for(P, 256), 256, 0, st>>>(v.skeys, v.head, v.uid, P, B->d_node_cell, B->d_seg);
      k_csr_gather<T><<<grid_for(P, 256), 256, 0, st>>>(v.sids, (const T*)B->d_W, S, P, (T*)B->d_wsort, B->d_msort);
    }
    T* Ua = (T*)B->d_mk;
    T* Fs = Ua + 3 * M;
    T* Ft = Fs + 3 * M;
    const T ds2 = (T)B->cfg.ds_scalar;
    if (B->c3 > 0 && !B->cfg.moving) {  // one cluster launch for the whole body step
      Body3ClusterParams<T> cp{};
      cp.fin = (const T*)fin;
      cp.nx = LP->cfg.nx;
      cp.ny = LP->cfg.ny;
      cp.nz = LP->cfg.nz;
      cp.meta = B->d_meta;
      cp.node_cell = B->d_node_cell;
      cp.W = (const T*)B->d_W;
      cp.pkey = B->d_pkey;
      cp.M = M;
      cp.S = S;
      cp.seg = B->d_seg;
      cp.msort = B->d_msort;
      cp.wsort = (const T*)B->d_wsort;
      cp.state = (T*)B->d_state;
      cp.ds = (const T*)B->d_ds;
      cp.ds_scalar = ds2;
      cp.gw = (T*)B->d_gw;
      cp.cells = cells;
      cp.force_hist = (T*)force_hist;
      cp.n_iter = B->cfg.n_iter;
      cp.part = B->d_c3part;
      cp.MK = B->c3_cap[0];
      cp.NK = B->c3_cap[1];
      cp.PK = B->c3_cap[2];
      cudaLaunchConfig_t lc = {};
      lc.gridDim = dim3((unsigned)B->c3);
      lc.blockDim = dim3(kBody3ClusterThreads);
      lc.dynamicSmemBytes = B->c3_smem;
      lc.stream = st;
      cudaLaunchAttribute at[2];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)B->c3;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      at[1].id = cudaLaunchAttributePriority;
      at[1].val.priority = B->prio;
      lc.attrs = at;
      lc.numAttrs = 2;
      cudaError_t e = cudaLaunchKernelEx(&lc, k_body3d_cluster<L19, T>, cp);
      if (e != cudaSuccess) return cuda_status(e, "vs_step 3-D body cluster kernel");
    } else if (B->fused3 > 0) {  // one cooperative launch for the whole body step
      Body3Params<T> bp{};
      bp.fin = (const T*)fin;
      bp.nx = LP->cfg.nx;
      bp.ny = LP->cfg.ny;
      bp.nz = LP->cfg.nz;
      bp.meta = B->d_meta;
      bp.node_cell = B->d_node_cell;
      bp.U = U;
      bp.Ud = B->d_U;
      bp.W = (const T*)B->d_W;
      bp.pair_uid = B->pair_uid;
      bp.M = M;
      bp.S = S;
      bp.seg = B->d_seg;
      bp.msort = B->d_msort;
      bp.wsort = (const T*)B->d_wsort;
      bp.state = (T*)B->d_state;
      bp.ds = (const T*)B->d_ds;
      bp.ds_scalar = ds2;
      bp.nu = (T*)B->d_nu;
      bp.nv = (T*)B->d_nv;
      bp.Ua = Ua;
      bp.Fs = Fs;
      bp.Ft = Ft;
      bp.gw = (T*)B->d_gw;
      bp.cells = cells;
      bp.force_hist = B->cfg.moving ? nullptr : (T*)force_hist;
      bp.n_iter = B->cfg.n_iter;
      bp.bar = B->d_bar;
      bp.status = LP->d_status;
      cudaLaunchConfig_t lc = {};
      lc.gridDim = dim3((unsigned)B->fused3);
      lc.blockDim = dim3(kBody3Threads);
      lc.stream = st;
      cudaLaunchAttribute at[2];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      at[1].id = cudaLaunchAttributePriority;
      at[1].val.priority = B->prio;
      lc.attrs = at;
      lc.numAttrs = 2;
      cudaError_t e = cudaLaunchKernelEx(&lc, k_body3d_fused<L19, T>, bp);  // 3-D bodies live on D3Q19 lattices
      if (e != cudaSuccess) return cuda_status(e, "vs_step 3-D body kernel");
    } else {
    const unsigned gn = grid_for(B->cfg.moving ? (int64_t)M * S : U, 128), gm = grid_for((int64_t)M * 32, 128);
    k_static_node_u<L, T><<<gn, 128, 0, st>>>((const T*)fin, LP->cfg.nx, LP->cfg.ny, LP->cfg.nz, B->d_meta,
                                               B->d_node_cell, U, (T*)B->d_nu, B->d_U);
    k_static_marker<T><<<gm, 128, 0, st>>>(1, B->cfg.n_iter > 0, (const T*)B->d_W, B->pair_uid, M, S,
                                           (const T*)B->d_nu, U, (const T*)B->d_state, (const T*)B->d_ds, ds2, Ua, Fs,
                                           Ft);
    for (int it = 0; it + 1 < B->cfg.n_iter; ++it) {
      k_static_spread<T><<<gn, 128, 0, st>>>(B->d_seg, B->d_msort, B->d_node_cell, (const T*)B->d_wsort, Fs, U,
                                             T(0.5), (T*)B->d_nv, nullptr, cells, M, nullptr, nullptr, B->d_U);
      k_static_marker<T><<<gm, 128, 0, st>>>(0, 1, (const T*)B->d_W, B->pair_uid, M, S, (const T*)B->d_nv, U,
                                             (const T*)B->d_state, (const T*)B->d_ds, ds2, Ua, Fs, Ft);
    }
    k_static_spread<T><<<gn, 256, 0, st>>>(B->d_seg, B->d_msort, B->d_node_cell, (const T*)B->d_wsort, Ft, U, T(1),
                                           nullptr, (T*)B->d_gw, cells, M, (T*)B->d_state,
                                           B->cfg.moving ? nullptr : (T*)force_hist, B->d_U);
    }
    if (B->cfg.moving) {  // added mass and Newmark on the free DOFs
      k_body_newmark<T><<<1, 32, 0, st>>>((T*)B->d_state, B->cfg.free_dof[0], B->cfg.free_dof[1], B->cfg.free_dof[2],
                                          (T)B->nm[0], (T)B->nm[1], (T)B->nm[2], (T)B->nm[3], (T)B->nm[4],
                                          (T)B->nm[5], (T)B->nm[6], (T)B->nm[7], (T)B->nm[8], (T*)force_hist);
    }
    VS_CHECK_LAUNCH("vs_step 3-D body kernels");
    return VS_OK;
  });
}


template <class L, typename T, int COLL, int TB>
static size_t tma_smem() {
  return (size_t)kTmaStages * L::Q * TB * sizeof(T) + kTmaStages * sizeof(uint64_t);
}

// Persistent CTAs for the TMA kernel: resident CTAs per SM x SMs (set once per plan).
template <class L, typename T, int COLL, int TB>
static int tma_configure(int* grid_out) {
  const size_t smem = tma_smem<L, T, COLL, TB>();
  cudaError_t e = cudaFuncSetAttribute(k_step_tma<L, T, COLL, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "tma attribute");
  int per_sm = 0, dev = 0, sms = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_tma<L, T, COLL, TB>, TB, smem);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_status(e, "tma occupancy");
  *grid_out = (per_sm > 0 ? per_sm : 1) * sms;
  return VS_OK;
}

template <class L, typename T, int COLL, int TB>
static int tma_launch(vs_lattice_plan* LP, const StepParams<L, T>& P, cudaStream_t st) {
  if (LP->tma_grid == 0) {
    int rc = tma_configure<L, T, COLL, TB>(&LP->tma_grid);
    if (rc) return rc;
  }
  const int nl = L::D == 2 ? P.ny : P.nz;
  const int tiles_per_row = nl / TB;
  const int tiles = (int)(P.n / TB);
  const int grid = tiles < LP->tma_grid ? tiles : LP->tma_grid;
  k_step_tma<L, T, COLL, TB><<<grid, TB, tma_smem<L, T, COLL, TB>(), st>>>(P, tiles, tiles_per_row, LP->d_status);
  return VS_OK;
}

template <class L, typename T, int COLL>
static int tma_dispatch(vs_lattice_plan* LP, const StepParams<L, T>& P, cudaStream_t st) {
  if constexpr (L::Q == 9) {
    if (LP->tma_tb == 256) return tma_launch<L, T, COLL, 256>(LP, P, st);
  }
  return tma_launch<L, T, COLL, 128>(LP, P, st);
}

// mode 0: every node.
// mode 1: every node except the body's box and, with lazy_walls, the x = 0 / nx-1 planes
//         (nodes outside the box read no force window).
// mode 2: the body's box and, with lazy_walls, the x = 0 / nx-1 planes, whose populations
//         first get the previous step's face boundaries.
// mode 3: only the x = 0 / nx-1 planes, with the previous step's face boundaries on load.
// mode 4: every node except the body's predicted window (read on the device from
//         prediction slot `slot`) and, with lazy_walls, the x = 0 / nx-1 planes.
// Fills the grid-kernel parameters and launch geometry; false when there is no node to do.
// tb_force > 0 fixes the threads per block (the batched launches use one block size).
template <class L, typename T>
static bool grid_setup(const vs_lattice_plan* LP, const vs_body_plan* B, const void* fin, void* fout, int mode,
                       bool lazy_walls, int tb_force, StepParams<L, T>& P, dim3& grid, int& tb, int slot = 0) {
  const vs_lattice_cfg& c = LP->cfg;
  P = make_step_params<L, T>(LP, B, fin, fout);
  P.nreg = 0;
  P.skip_box = mode == 1 && B;
  P.skip_walls = (mode == 1 || mode == 4) && lazy_walls;
  for (int q = 0; q < 6; ++q) P.box[q] = B ? B->box[q] : 0;
  P.n_lazy = 0;
  if (mode == 4 && B) {
    P.dyn_meta = B->d_meta;
    P.dyn_slot = slot;
    P.dyn_ext[0] = B->cap[0] + 2;
    P.dyn_ext[1] = B->cap[1] + 2;
  }
  if (mode == 1 || mode == 3 || mode == 4) {  // outside the box no node reads the force window
    P.gw = nullptr;
    P.meta = nullptr;
  }
  int rows = c.nx, ext_last = L::D == 2 ? c.ny : c.nz, ext_mid = c.ny;
  if (mode == 2 || mode == 3) {
    int nr = 0;
    auto add = [&](const int* R) {
      for (int q = 0; q < 6; ++q) P.reg[nr][q] = R[q];
      ++nr;
    };
    if (B && mode == 2) add(B->box);
    if (lazy_walls) {
      int w0[6] = {0, 1, 0, c.ny, 0, c.nz}, w1[6] = {c.nx - 1, c.nx, 0, c.ny, 0, c.nz};
      if (!B || mode == 3 || B->box[0] > 0) add(w0);
      if (!B || mode == 3 || B->box[1] < c.nx) add(w1);
      for (int k = 0; k < c.n_bc && k < 2; ++k) P.lazy[P.n_lazy++] = wall_args_from_bc<T>(c.bc[k], LP, k);
    }
    P.nreg = nr;
    rows = 0;
    ext_last = 0;
    ext_mid = 0;
    for (int g = 0; g < nr; ++g) {
      P.rowstart[g] = rows;
      rows += P.reg[g][1] - P.reg[g][0];
      const int el = L::D == 2 ? P.reg[g][3] - P.reg[g][2] : P.reg[g][5] - P.reg[g][4];
      ext_last = el > ext_last ? el : ext_last;
      ext_mid = P.reg[g][3] - P.reg[g][2] > ext_mid ? P.reg[g][3] - P.reg[g][2] : ext_mid;
    }
    for (int g = nr; g < 4; ++g) P.rowstart[g] = 1 << 30;
    if (nr == 0) return false;
  }
  // threads along the contiguous axis (y in 2-D, z in 3-D)
  tb = tb_force > 0 ? tb_force : (ext_last >= 256 ? 256 : (ext_last >= 128 ? 128 : ((ext_last + 31) / 32) * 32));
  P.chunks = (ext_last + tb - 1) / tb;
  grid = dim3(L::D == 2 ? P.chunks : P.chunks * ext_mid, rows);
  P.gx = (int)grid.x;
  return true;
}

// A launch with a priority attribute (kept by graph capture as the node's priority); prio 0
// launches plainly, with the stream's priority.
template <typename... KArgs, typename... Args>
static void launch_prio(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, int prio, Args... args) {
  if (prio == 0) {
    k<<<grid, block, 0, st>>>(args...);
    return;
  }
  cudaLaunchConfig_t lc = {};
  lc.gridDim = grid;
  lc.blockDim = block;
  lc.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio;
  lc.attrs = at;
  lc.numAttrs = 1;
  cudaLaunchKernelEx(&lc, k, args...);
}

// Launch geometry of k_step_fast: NPT nodes per thread along the contiguous axis, whole grid.
// (false: the contiguous extent is shorter than one block's nodes; the general kernel runs)
// stream: the launch runs beside body kernels on a grid larger than L2 (kFeatStream).
template <class L, int COLL>
static bool launch_fast(StepParams<L, float> P, bool skip, bool stream, cudaStream_t st) {
  using S = FastShape<L, COLL>;
  const int ext = L::D == 2 ? P.ny : P.nz;
  if (ext < S::TB * S::NPT) return false;
  P.chunks = (ext + S::TB * S::NPT - 1) / (S::TB * S::NPT);
  const dim3 grid(L::D == 2 ? P.chunks : P.chunks * P.ny, P.nx);
  P.gx = (int)grid.x;
  if (skip && stream) k_step_fast<L, float, COLL, kFeatSkip | kFeatStream><<<grid, S::TB, 0, st>>>(P);
  else if (skip) k_step_fast<L, float, COLL, kFeatSkip><<<grid, S::TB, 0, st>>>(P);
  else k_step_fast<L, float, COLL, 0><<<grid, S::TB, 0, st>>>(P);
  return true;
}

static int enqueue_grid(const vs_lattice_plan* LP, const vs_body_plan* B, const void* fin, void* fout,
                        cudaStream_t st, int mode = 0, bool lazy_walls = false, int slot = 0) {
  const vs_lattice_cfg& c = LP->cfg;
  int rc = dispatch(c.q, c.dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    StepParams<L, T> P;
    dim3 grid;
    int tb = 0;
    if (!grid_setup<L, T>(LP, B, fin, fout, mode, lazy_walls, 0, P, grid, tb, slot)) return VS_OK;
    const bool walls = (mode == 2 || mode == 3) && lazy_walls;
    const bool aligned = ((uintptr_t)fin % 16) == 0;
    if ((mode == 0 || mode == 1) && LP->tma_tb > 0 && aligned) {
      vs_lattice_plan* mp = const_cast<vs_lattice_plan*>(LP);
      int trc;
      switch (c.collision) {
        case VS_COLLIDE_BGK: trc = tma_dispatch<L, T, VS_COLLIDE_BGK>(mp, P, st); break;
        case VS_COLLIDE_KBC: trc = tma_dispatch<L, T, VS_COLLIDE_KBC>(mp, P, st); break;
        case VS_COLLIDE_REG: trc = tma_dispatch<L, T, VS_COLLIDE_REG>(mp, P, st); break;
        default: trc = tma_dispatch<L, T, VS_COLLIDE_MRT>(mp, P, st); break;
      }
      if (trc) return trc;
      VS_CHECK_LAUNCH("vs_step grid kernel (TMA)");
      return VS_OK;
    }
    if constexpr (std::is_same<T, float>::value) {
      // the bulk launches of a step: specialised kernel when no per-node feature is needed
      const bool bulk = (mode == 0 || mode == 1 || mode == 4) && !walls && P.nreg == 0 && !P.gw && !P.has_g0 &&
                        !P.mask_load && P.n_pre == 0;
      if (bulk) {
        const bool skip = P.skip_box || P.dyn_meta || P.skip_walls;
        const bool stream = B && LP->stream_pop && !getenv_flag("VIVSIM_GB300_NO_STREAM");
        bool done;
        switch (c.collision) {
          case VS_COLLIDE_BGK: done = launch_fast<L, VS_COLLIDE_BGK>(P, skip, stream, st); break;
          case VS_COLLIDE_KBC: done = launch_fast<L, VS_COLLIDE_KBC>(P, skip, stream, st); break;
          case VS_COLLIDE_REG: done = launch_fast<L, VS_COLLIDE_REG>(P, skip, stream, st); break;
          default: done = launch_fast<L, VS_COLLIDE_MRT>(P, skip, stream, st); break;
        }
        if (done) {
          VS_CHECK_LAUNCH("vs_step grid kernel");
          return VS_OK;
        }
      }
    }
    // the box and face-plane launches beside the grid launch carry the side streams' priority
    const int prio = B && (mode == 2 || mode == 3) ? B->prio : 0;
#define VS_LAUNCH_STEP(K)                                                              \
  (walls ? launch_prio(k_step<L, T, K, true>, grid, tb, st, prio, P) : launch_prio(k_step<L, T, K, false>, grid, tb, st, prio, P))
    switch (c.collision) {
      case VS_COLLIDE_BGK: VS_LAUNCH_STEP(VS_COLLIDE_BGK); break;
      case VS_COLLIDE_KBC: VS_LAUNCH_STEP(VS_COLLIDE_KBC); break;
      case VS_COLLIDE_REG: VS_LAUNCH_STEP(VS_COLLIDE_REG); break;
      default: VS_LAUNCH_STEP(VS_COLLIDE_MRT); break;
    }
#undef VS_LAUNCH_STEP
    VS_CHECK_LAUNCH("vs_step grid kernel");
    return VS_OK;
  });
  return rc;
}

// With a body, the body kernel(s) run on the plan's side stream while the grid kernel
// updates every node outside the body's box; after the join a small grid launch updates
// the box with the new force window.  Each (node, direction) destination of the push is
// written by exactly one source node, so the two grid launches never write the same word.
// lazy_in: fin holds the previous step's populations before its face boundaries (they
// are applied on load); bc_out: run the face kernels on fout (else the next step will).
// Cluster form: the body kernel also updates the box and the lazy face planes, so the
// step is that one launch beside the grid launch over the rest of the grid.
template <typename T, int R, int COLL>
static cudaError_t launch_cluster_t(vs_body_plan* B, const BodyParams<T>& P, const StepParams<L9, T>& SP,
                                    cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)B->cl_size);
  cfg.blockDim = dim3((unsigned)B->cl_threads);
  cfg.dynamicSmemBytes = B->cl_smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)B->cl_size;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributePriority;
  attr[1].val.priority = B->prio;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, k_body2d_cluster<T, R, COLL>, P, SP);
}

template <typename T, int R>
static cudaError_t cluster_attr_t(int coll, int smem) {
  switch (coll) {
    case VS_COLLIDE_BGK:
      return cudaFuncSetAttribute(k_body2d_cluster<T, R, VS_COLLIDE_BGK>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case VS_COLLIDE_KBC:
      return cudaFuncSetAttribute(k_body2d_cluster<T, R, VS_COLLIDE_KBC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    case VS_COLLIDE_REG:
      return cudaFuncSetAttribute(k_body2d_cluster<T, R, VS_COLLIDE_REG>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    default:
      return cudaFuncSetAttribute(k_body2d_cluster<T, R, VS_COLLIDE_MRT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  }
}

static cudaError_t cluster_attr(int dtype, int R, int coll, int smem) {
  if (dtype == VS_F64)
    return R == 1 ? cluster_attr_t<double, 1>(coll, smem)
                  : (R == 2 ? cluster_attr_t<double, 2>(coll, smem) : cluster_attr_t<double, 3>(coll, smem));
  return R == 1 ? cluster_attr_t<float, 1>(coll, smem)
                : (R == 2 ? cluster_attr_t<float, 2>(coll, smem) : cluster_attr_t<float, 3>(coll, smem));
}

static int enqueue_cluster_body(vs_body_plan* B, const vs_lattice_plan* LP, const void* fin, void* fout,
                                void* force_hist, bool lazy_in, cudaStream_t st) {
  return dispatch_t(B->cfg.dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    BodyParams<T> P = body_params2d<T>(B, LP, fin, force_hist, false);
    P.pred_slot = B->parity;
    StepParams<L9, T> SP;
    dim3 grid;
    int tb = 0;
    grid_setup<L9, T>(LP, B, fin, fout, 2, false, 0, SP, grid, tb);  // the force window and the node physics
    SP.nreg = 0;
    SP.skip_walls = lazy_in ? 1 : 0;
    cudaError_t e;
    auto go = [&](auto rt) {
      constexpr int R = decltype(rt)::value;
      switch (LP->cfg.collision) {
        case VS_COLLIDE_BGK: return launch_cluster_t<T, R, VS_COLLIDE_BGK>(B, P, SP, st);
        case VS_COLLIDE_KBC: return launch_cluster_t<T, R, VS_COLLIDE_KBC>(B, P, SP, st);
        case VS_COLLIDE_REG: return launch_cluster_t<T, R, VS_COLLIDE_REG>(B, P, SP, st);
        default: return launch_cluster_t<T, R, VS_COLLIDE_MRT>(B, P, SP, st);
      }
    };
    switch (B->cfg.radius) {
      case 1: e = go(std::integral_constant<int, 1>{}); break;
      case 2: e = go(std::integral_constant<int, 2>{}); break;
      default: e = go(std::integral_constant<int, 3>{}); break;
    }
    if (e != cudaSuccess) return cuda_status(e, "vs_step cluster body kernel");
    return VS_OK;
  });
}

static int enqueue_step(const vs_lattice_plan* LP, vs_body_plan* B, const void* fin, void* fout, void* force_hist,
                        cudaStream_t st, bool lazy_in = false, bool bc_out = true, bool bb_in = false,
                        bool bb_out = true) {
  int rc;
  const_cast<vs_lattice_plan*>(LP)->bb_load = bb_in ? 1 : 0;  // read by make_step_params below
  rc = enqueue_cbc(LP, fin, st);
  if (rc) return rc;
  if (B && B->cluster) {
    cudaError_t e = cudaEventRecord(B->ev_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(B->side, B->ev_fork, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_step fork");
    rc = enqueue_cluster_body(B, LP, fin, fout, force_hist, lazy_in, B->side);
    if (rc) return rc;
    if (lazy_in) {  // the face planes on a third stream, beside the grid launch
      e = cudaStreamWaitEvent(B->side2, B->ev_fork, 0);
      if (e != cudaSuccess) return cuda_status(e, "vs_step fork");
      rc = enqueue_grid(LP, B, fin, fout, B->side2, 3, true);
      if (rc) return rc;
      e = cudaEventRecord(B->ev_join2, B->side2);
      if (e != cudaSuccess) return cuda_status(e, "vs_step join");
    }
    rc = enqueue_grid(LP, B, fin, fout, st, 4, lazy_in, B->parity);
    if (rc) return rc;
    e = cudaEventRecord(B->ev_join, B->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, B->ev_join, 0);
    if (e == cudaSuccess && lazy_in) e = cudaStreamWaitEvent(st, B->ev_join2, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_step join");
    B->parity ^= 1;
  } else if (B) {
    // side stream: body kernels, then the box's nodes (they need the new force window);
    // third stream: the lazy face planes; main stream: every other node.  The three
    // launches read f_in only and write disjoint words of f_out, so they run side by side
    // and the step takes max(grid, body + box, planes).
    cudaError_t e = cudaEventRecord(B->ev_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(B->side, B->ev_fork, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_step fork");
    rc = enqueue_body(B, LP, fin, force_hist, B->side);
    if (rc) return rc;
    rc = enqueue_grid(LP, B, fin, fout, B->side, 2, false);
    if (rc) return rc;
    if (lazy_in) {
      e = cudaStreamWaitEvent(B->side2, B->ev_fork, 0);
      if (e != cudaSuccess) return cuda_status(e, "vs_step fork");
      rc = enqueue_grid(LP, B, fin, fout, B->side2, 3, true);
      if (rc) return rc;
      e = cudaEventRecord(B->ev_join2, B->side2);
      if (e != cudaSuccess) return cuda_status(e, "vs_step join");
    }
    rc = enqueue_grid(LP, B, fin, fout, st, 1, lazy_in);
    if (rc) return rc;
    e = cudaEventRecord(B->ev_join, B->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, B->ev_join, 0);
    if (e == cudaSuccess && lazy_in) e = cudaStreamWaitEvent(st, B->ev_join2, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_step join");
  } else {
    rc = enqueue_grid(LP, B, fin, fout, st, 0, lazy_in);
  }
  if (rc) return rc;
  if (bc_out) {
    rc = enqueue_bcs(LP, fout, st);
    if (rc) return rc;
  }
  if (!bb_out || !LP->cfg.obstacle_mask) return VS_OK;
  return dispatch(LP->cfg.q, LP->cfg.dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    k_mask_bb<L, T><<<grid_for(LP->n, 256), 256, 0, st>>>((T*)fout, LP->cfg.obstacle_mask, LP->n);
    VS_CHECK_LAUNCH("vs_step obstacle bounce-back");
    return VS_OK;
  });
}

// Boundaries can be deferred to the next step's load when they all sit on one axis and
// the body's box (whose nodes the body kernel reads) touches none of their walls.
static bool lazy_boundaries(const vs_lattice_plan* LP, const vs_body_plan* B) {
  if (!LP->lazy_ok || LP->cfg.n_bc == 0 || !B) return false;
  for (int k = 0; k < LP->cfg.n_bc; ++k)
    if (loc_axis(LP->cfg.bc[k].loc) != 0) return false;
  const int nn[3] = {LP->cfg.nx, LP->cfg.ny, LP->cfg.nz};
  for (int k = 0; k < LP->cfg.n_bc; ++k) {
    const int a = loc_axis(LP->cfg.bc[k].loc);
    const int wall = loc_sign(LP->cfg.bc[k].loc) > 0 ? 0 : nn[a] - 1;
    if (wall >= B->box[2 * a] && wall < B->box[2 * a + 1]) return false;
  }
  return true;
}

// ---- host side of the persistent run (k_viv_run)
static_assert(sizeof(VivRunParams<float>) <= 32000, "k_viv_run parameters exceed the launch parameter space");

template <int COLL>
static cudaError_t viv_run_launch_t(const vs_body_plan* B, const VivRunParams<float>& P, cudaStream_t st) {
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)B->run_ctas);
  lc.blockDim = dim3(kRunThreads);
  lc.dynamicSmemBytes = B->run_smem;
  lc.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)B->cl_size;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeCooperative;
  at[1].val.cooperative = 1;
  lc.attrs = at;
  lc.numAttrs = 2;
  return cudaLaunchKernelEx(&lc, k_viv_run<float, 2, COLL>, P);
}

// CTAs of the persistent run: as many whole clusters of the body's size as are resident at
// once (at least two: the body's and one of grid tiles), 0 where the device has no
// cooperative cluster launch.
template <int COLL>
static cudaError_t viv_run_setup_t(vs_body_plan* B, int& ctas) {
  ctas = 0;
  auto kern = k_viv_run<float, 2, COLL>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)B->run_smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3((unsigned)B->cl_size);
  lc.blockDim = dim3(kRunThreads);
  lc.dynamicSmemBytes = B->run_smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)B->cl_size;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  lc.attrs = at;
  lc.numAttrs = 1;
  int ncl = 0;
  e = cudaOccupancyMaxActiveClusters(&ncl, kern, &lc);
  if (e != cudaSuccess) return e;
  if (ncl >= 2) ctas = ncl * B->cl_size;
  return cudaSuccess;
}

static cudaError_t viv_run_setup(vs_body_plan* B, int coll, int& ctas) {
  switch (coll) {
    case VS_COLLIDE_BGK: return viv_run_setup_t<VS_COLLIDE_BGK>(B, ctas);
    case VS_COLLIDE_KBC: return viv_run_setup_t<VS_COLLIDE_KBC>(B, ctas);
    case VS_COLLIDE_REG: return viv_run_setup_t<VS_COLLIDE_REG>(B, ctas);
    default: return viv_run_setup_t<VS_COLLIDE_MRT>(B, ctas);
  }
}

// The persistent run applies to float 2-D plans whose body takes the cluster form with a
// 4 x 4 stencil, whose face boundaries are deferred to the next step's load (or absent),
// and whose bulk nodes need no per-node feature (no uniform force, obstacle mask,
// characteristic wall or pre-stream faces).  It is selected per plan with
// vs_lattice_set_run_form (or for every plan with VIVSIM_GB300_RUN_FORM=persistent); the
// default is the launch-per-step form, which measured faster on the benchmark VIV case
// (14.0 against 17.1 us per step).
static bool viv_run_applies(const vs_lattice_plan* LP, const vs_body_plan* B, bool lazy) {
  const char* form = getenv("VIVSIM_GB300_RUN_FORM");
  if (LP->run_form != VS_RUN_PERSISTENT && (!form || strcmp(form, "persistent") != 0)) return false;
  if (!B || !B->cluster || B->run_ctas <= 0 || B->dim != 2) return false;
  const vs_lattice_cfg& c = LP->cfg;
  if (c.dtype != VS_F32 || c.q != 9 || B->cfg.radius != 2 || c.obstacle_mask) return false;
  if (!lazy && c.n_bc > 0) return false;
  for (int k = 0; k < c.n_bc; ++k)
    if (c.bc[k].mode == VS_WALL_CHARACTERISTIC) return false;
  for (int q = 0; q < 3; ++q)
    if (c.g_uniform[q] != 0.0) return false;
  for (int k = 0; k < c.n_bc; ++k)
    if (c.bc[k].kind == VS_BC_BB || c.bc[k].kind == VS_BC_SPECULAR) return false;
  return true;
}

// n time steps from global step s0 of a run (step s reads f_a when s is even), in one launch.
static int viv_run_chunk(const vs_lattice_plan* LP, vs_body_plan* B, void* f_a, void* f_b, int s0, int n, bool lazy,
                         void* force_hist, cudaStream_t st) {
  VivRunParams<float>* P = new (std::nothrow) VivRunParams<float>();
  if (!P) {
    set_error("vs_run: out of host memory");
    return VS_ERR_INVALID_ARG;
  }
  const vs_lattice_cfg& c = LP->cfg;
  const int parity0 = B->parity;  // prediction slot of step s0
  for (int p = 0; p < 2; ++p) {
    void* fin = p == 0 ? f_a : f_b;
    void* fout = p == 0 ? f_b : f_a;
    const int slot = parity0 ^ ((p ^ s0) & 1);
    P->B[p] = body_params2d<float>(B, LP, fin, nullptr, false);
    P->B[p].pred_slot = slot;
    for (int lz = 0; lz < 2; ++lz) {
      dim3 grid;
      int tb = 0;
      StepParams<L9, float> SP;
      grid_setup<L9, float>(LP, B, fin, fout, 2, false, 0, SP, grid, tb);
      SP.nreg = 0;
      SP.skip_walls = lz;
      P->SPb[p][lz] = SP;
      grid_setup<L9, float>(LP, B, fin, fout, 4, lz != 0, 0, SP, grid, tb, slot);
      P->SPm[p][lz] = SP;
    }
    if (lazy) {
      dim3 grid;
      int tb = 0;
      StepParams<L9, float> SP;
      grid_setup<L9, float>(LP, B, fin, fout, 3, true, 0, SP, grid, tb);
      SP.chunks = (c.ny + kRunGroup - 1) / kRunGroup;
      SP.gx = SP.chunks;
      P->SPw[p] = SP;
    }
  }
  const int npt = kRunNodes;
  P->hist = force_hist ? (float*)force_hist + 3 * (int64_t)s0 : nullptr;
  P->bar = B->d_bar;
  P->status = LP->d_status;
  P->n_steps = n;
  P->lazy = lazy ? 1 : 0;
  P->lazy_first = s0 > 0 ? 1 : 0;
  P->chunks_m = (c.ny + kRunGroup * npt - 1) / (kRunGroup * npt);
  P->rows_m = c.nx;
  P->chunks_w = (c.ny + kRunGroup - 1) / kRunGroup;
  // the kernel numbers its steps from 0: swap the buffers when the chunk starts on an odd step
  if (s0 & 1) {
    std::swap(P->B[0], P->B[1]);
    std::swap(P->SPb[0], P->SPb[1]);
    std::swap(P->SPm[0], P->SPm[1]);
    std::swap(P->SPw[0], P->SPw[1]);
  }
  cudaError_t e;
  switch (c.collision) {
    case VS_COLLIDE_BGK: e = viv_run_launch_t<VS_COLLIDE_BGK>(B, *P, st); break;
    case VS_COLLIDE_KBC: e = viv_run_launch_t<VS_COLLIDE_KBC>(B, *P, st); break;
    case VS_COLLIDE_REG: e = viv_run_launch_t<VS_COLLIDE_REG>(B, *P, st); break;
    default: e = viv_run_launch_t<VS_COLLIDE_MRT>(B, *P, st); break;
  }
  delete P;
  if (e != cudaSuccess) return cuda_status(e, "vs_run persistent launch");
  B->parity = parity0 ^ (n & 1);
  return VS_OK;
}

// The cluster form of a fixed 3-D body step: the largest cluster of up to 16 CTAs (8
// where the device allows no larger one) whose per-CTA shared memory fits, with the nodes
// split by pair count.  VIVSIM_GB300_BODY3D_CLUSTER: another largest size, 0 for none.
template <typename T>
static int body3_cluster_setup(vs_body_plan* b) {
  b->c3 = 0;
  int maxcl = 16;
  if (const char* v = getenv("VIVSIM_GB300_BODY3D_CLUSTER")) maxcl = atoi(v);
  int dev = 0, cl_ok = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&cl_ok, cudaDevAttrClusterLaunch, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (!cl_ok || maxcl < 1) return VS_OK;
  const int M = b->M, S = b->S, U = b->U;
  const int64_t P = (int64_t)M * S;
  std::vector<int32_t> seg(U + 1), uid(P);
  cudaError_t e = cudaMemcpy(seg.data(), b->d_seg, sizeof(int32_t) * (U + 1), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(uid.data(), b->pair_uid, sizeof(int32_t) * P, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e, "vs_body_plan_create cluster layout");
  auto kern = k_body3d_cluster<L19, T>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return cuda_status(e, "vs_body_plan_create cluster attributes");
  for (int CL = 16; CL >= 1; CL /= 2) {
    if (CL > maxcl || CL > M || CL > U) continue;
    std::vector<int> part(2 * (CL + 1));
    part[0] = 0;
    for (int r = 1; r < CL; ++r) {
      const int64_t target = P * r / CL;
      int k = (int)(std::lower_bound(seg.begin(), seg.end(), (int32_t)target) - seg.begin());
      k = k < part[r - 1] ? part[r - 1] : (k > U ? U : k);
      part[r] = k;
    }
    part[CL] = U;
    for (int r = 0; r <= CL; ++r) part[CL + 1 + r] = (int)((int64_t)M * r / CL);
    int MK = 0, NK = 0, PK = 0;
    for (int r = 0; r < CL; ++r) {
      MK = std::max(MK, part[CL + 2 + r] - part[CL + 1 + r]);
      NK = std::max(NK, part[r + 1] - part[r]);
      PK = std::max(PK, seg[part[r + 1]] - seg[part[r]]);
    }
    if (NK > 65535 || NK < 1) continue;
    const size_t smem = body3_cluster_smem<T>(M, S, MK, NK, PK);
    if ((int64_t)smem > optin) continue;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)CL);
    lc.blockDim = dim3(kBody3ClusterThreads);
    lc.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)CL;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &lc) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      continue;
    }
    std::vector<int32_t> key(P);
    for (int64_t p = 0; p < P; ++p) {
      const int u = uid[p];
      const int owner = (int)(std::upper_bound(part.begin(), part.begin() + CL + 1, u) - part.begin()) - 1;
      key[p] = (owner << 16) | (u - part[owner]);
    }
    if ((e = cudaMalloc((void**)&b->d_pkey, sizeof(int32_t) * P)) != cudaSuccess ||
        (e = cudaMalloc((void**)&b->d_c3part, sizeof(int) * part.size())) != cudaSuccess ||
        (e = cudaMemcpy(b->d_pkey, key.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_c3part, part.data(), sizeof(int) * part.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
      return cuda_status(e, "vs_body_plan_create cluster layout");
    b->c3 = CL;
    b->c3_smem = smem;
    b->c3_cap[0] = MK;
    b->c3_cap[1] = NK;
    b->c3_cap[2] = PK;
    return VS_OK;
  }
  return VS_OK;
}

extern "C" {

int vs_lattice_plan_create(const vs_lattice_cfg* cfg, vs_lattice_plan** out) {
  VS_REQUIRE(cfg && out, "vs_lattice_plan_create: null argument");
  VS_REQUIRE(cfg->q == 9 || cfg->q == 19, "q must be 9 or 19");
  VS_REQUIRE(cfg->dtype == VS_F32 || cfg->dtype == VS_F64, "bad dtype");
  const int nz = cfg->q == 9 ? 1 : cfg->nz;
  VS_REQUIRE(cfg->nx >= 4 && cfg->ny >= 4 && (cfg->q == 9 ? cfg->nz == 1 : cfg->nz >= 4),
             "grid %d x %d x %d too small (>= 4 per axis; nz = 1 for D2Q9)", cfg->nx, cfg->ny, cfg->nz);
  const int64_t n = (int64_t)cfg->nx * cfg->ny * nz;
  VS_REQUIRE(n < (1ll << 31), "grid of %lld nodes too large for 32-bit node indices", (long long)n);
  VS_REQUIRE(cfg->nx <= 65535 && (cfg->q == 9 || (int64_t)cfg->ny * ((nz + 127) / 128) < (1ll << 31)),
             "grid extent too large for the launch geometry");
  VS_REQUIRE(cfg->collision >= VS_COLLIDE_BGK && cfg->collision <= VS_COLLIDE_REG, "bad collision %d",
             cfg->collision);
  VS_REQUIRE(cfg->forcing >= VS_FORCE_NONE && cfg->forcing <= VS_FORCE_GUO_MRT, "bad forcing %d", cfg->forcing);
  VS_REQUIRE(cfg->n_bc >= 0 && cfg->n_bc <= VS_MAX_BC, "n_bc must be 0..%d", VS_MAX_BC);
  VS_REQUIRE(cfg->variant >= VS_GRID_AUTO && cfg->variant <= VS_GRID_TMA, "bad grid kernel variant %d", cfg->variant);
  const int dim = cfg->q == 9 ? 2 : 3;
  for (int k = 0; k < cfg->n_bc; ++k) {
    const vs_bc& b = cfg->bc[k];
    VS_REQUIRE(b.loc >= 0 && b.loc < 2 * dim, "boundary %d: loc %d invalid", k, b.loc);
    VS_REQUIRE(b.kind >= VS_BC_NEE && b.kind <= VS_BC_SPECULAR, "boundary %d: bad kind", k);
    VS_REQUIRE(b.mode >= VS_WALL_GIVEN && b.mode <= VS_WALL_CHARACTERISTIC, "boundary %d: bad mode", k);
    VS_REQUIRE(b.mode != VS_WALL_CHARACTERISTIC || b.kind == VS_BC_NEE || b.kind == VS_BC_NEBB || b.kind == VS_BC_EQ,
               "boundary %d: a characteristic wall is imposed by NEE, NEBB or equilibrium", k);
    VS_REQUIRE(!((b.kind == VS_BC_BB || b.kind == VS_BC_SPECULAR) && b.mode != VS_WALL_GIVEN),
               "boundary %d: bounce-back takes no wall mode", k);
  }
  vs_lattice_plan* p = new (std::nothrow) vs_lattice_plan();
  if (!p) {
    set_error("out of host memory");
    return VS_ERR_INVALID_ARG;
  }
  p->cfg = *cfg;
  p->cfg.nz = nz;
  p->dim = dim;
  p->n = n;
  const int nn[3] = {cfg->nx, cfg->ny, nz};
  for (int k = 0; k < cfg->n_bc; ++k) {
    const vs_bc& b = cfg->bc[k];
    if (b.mode == VS_WALL_CHARACTERISTIC) {
      cudaError_t e = cudaMalloc(&p->cbc_buf[k], dsize(cfg->dtype) * (1 + dim) * face_size(b.loc, nn));
      if (e != cudaSuccess) {
        free_lattice(p);
        return cuda_status(e, "vs_lattice_plan_create");
      }
    }
    if (b.kind == VS_BC_BB || b.kind == VS_BC_SPECULAR) {
      cudaError_t e = cudaMalloc(&p->pre_buf[k], dsize(cfg->dtype) * cfg->q * face_size(b.loc, nn));
      if (e != cudaSuccess) {
        free_lattice(p);
        return cuda_status(e, "vs_lattice_plan_create");
      }
    }
  }
  // Consecutive boundaries on the two opposite faces of one axis touch disjoint nodes
  // (wall + neighbour planes at 0,1 and N-1,N-2 with N >= 4): launch them together.
  int gid = 0, gsize = 0;
  for (int k = 0; k < cfg->n_bc; ++k) {
    if (k > 0) {
      const vs_bc& a = cfg->bc[k - 1];
      const vs_bc& b = cfg->bc[k];
      const bool pair = gsize == 1 && loc_axis(a.loc) == loc_axis(b.loc) && a.loc != b.loc &&
                        nn[loc_axis(a.loc)] >= 4;
      if (!pair) {
        ++gid;
        gsize = 0;
      }
    }
    p->bc_group[k] = gid;
    ++gsize;
  }
  p->n_groups = cfg->n_bc ? gid + 1 : 0;
  {
    const int nl = cfg->q == 9 ? cfg->ny : nz;
    p->tma_tb = cfg->variant != VS_GRID_TMA ? 0 : ((cfg->q == 9 && nl % 256 == 0) ? 256 : (nl % 128 == 0 ? 128 : 0));
    int dev = 0, l2 = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    p->stream_pop = l2 > 0 && (double)cfg->q * (double)p->n * (cfg->dtype == VS_F64 ? 8.0 : 4.0) > (double)l2;
    cudaError_t e = cudaMalloc(&p->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(int));
    if (e != cudaSuccess) {
      free_lattice(p);
      return cuda_status(e, "vs_lattice_plan_create status");
    }
  }
  p->lazy_ok = p->n_groups == 1;
  for (int k = 0; k < cfg->n_bc; ++k)
    if (cfg->bc[k].kind == VS_BC_BB || cfg->bc[k].kind == VS_BC_SPECULAR ||
        cfg->bc[k].mode == VS_WALL_CHARACTERISTIC)
      p->lazy_ok = 0;
  *out = p;
  return VS_OK;
}

int vs_lattice_set_run_form(vs_lattice_plan* plan, int form) {
  VS_REQUIRE(plan, "vs_lattice_set_run_form: null plan");
  VS_REQUIRE(form == VS_RUN_STEPS || form == VS_RUN_PERSISTENT,
             "vs_lattice_set_run_form: form must be VS_RUN_STEPS or VS_RUN_PERSISTENT");
  plan->run_form = form;
  return VS_OK;
}

int vs_lattice_status(const vs_lattice_plan* plan, int reset, void* stream) {
  VS_REQUIRE(plan, "vs_lattice_status: null plan");
  int v = 0;
  cudaStream_t st = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(&v, plan->d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && reset && v) e = cudaMemset(plan->d_status, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_status(e, "vs_lattice_status");
  if (v == VS_ERR_NONFINITE) set_error("the watchdog found a NaN or Inf population");
  else if (v == VS_ERR_RANGE) set_error("a grid kernel met an index outside its array (bounds-checked build)");
  else if (v == VS_ERR_TIMEOUT_INFLIGHT)
    set_error("a grid kernel gave up waiting for its bulk copies and one had still not landed when it left");
  else if (v) set_error("a grid kernel gave up waiting for its bulk copies (device status %d)", v);
  return v;
}

int vs_selftest_bounded_wait(int limit, int* status_dev, void* stream) {
  VS_REQUIRE(status_dev && limit > 0 && limit <= (1 << 20), "vs_selftest_bounded_wait: bad arguments");
  k_selftest_wait<<<1, 32, 0, as_stream(stream)>>>(status_dev, limit);
  VS_CHECK_LAUNCH("vs_selftest_bounded_wait");
  return VS_OK;
}

int vs_check_finite(int dtype, const void* f, int64_t n, int* status_dev, void* stream) {
  VS_REQUIRE(f && status_dev && n >= 0, "vs_check_finite: bad arguments");
  if (n == 0) return VS_OK;
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    const int64_t blocks = (n + 255) / 256;
    k_check_finite<T><<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, as_stream(stream)>>>((const T*)f, n,
                                                                                                status_dev);
    VS_CHECK_LAUNCH("vs_check_finite");
    return VS_OK;
  });
}

int vs_lattice_plan_destroy(vs_lattice_plan* plan) {
  free_lattice(plan);
  return VS_OK;
}

int vs_body_plan_create(const vs_body_cfg* cfg, const vs_lattice_plan* lattice, vs_body_plan** out) {
  VS_REQUIRE(cfg && lattice && out, "vs_body_plan_create: null argument");
  VS_REQUIRE(cfg->dim == lattice->dim, "body dim %d does not match the lattice", cfg->dim);
  VS_REQUIRE(cfg->dtype == lattice->cfg.dtype, "body dtype does not match the lattice");
  VS_REQUIRE(cfg->n_markers > 0 && cfg->x0_host && cfg->y0_host && (cfg->dim == 2 || cfg->z0_host),
             "vs_body_plan_create: marker coordinates required");
  VS_REQUIRE(cfg->radius >= 1 && cfg->radius <= 3, "stencil radius must be 1..3");
  VS_REQUIRE(cfg->kernel >= VS_KERNEL_PESKIN3 && cfg->kernel <= VS_KERNEL_COSINE4, "bad kernel");
  VS_REQUIRE(cfg->n_iter >= 0 && cfg->n_iter <= 64, "n_iter must be 0..64");
  VS_REQUIRE(!(cfg->dim == 2 && cfg->free_dof[2]) || (cfg->moving && cfg->inertia > 0),
             "a free rotation needs a moving body with a positive moment of inertia");
  VS_REQUIRE(lattice->cfg.forcing == VS_FORCE_EDM || lattice->cfg.forcing == VS_FORCE_GUO_BGK ||
                 lattice->cfg.forcing == VS_FORCE_GUO_MRT,
             "an immersed body needs a forcing scheme on the lattice (EDM or Guo)");
  VS_REQUIRE(cfg->fsi_iter >= 0 && cfg->fsi_iter <= 64, "fsi_iter must be 0..64");
  VS_REQUIRE(cfg->fsi_iter <= 1 || (cfg->dim == 2 && cfg->moving),
             "fluid-structure sub-iterations need a moving 2-D body");
  vs_body_plan* b = new (std::nothrow) vs_body_plan();
  if (!b) {
    set_error("out of host memory");
    return VS_ERR_INVALID_ARG;
  }
  b->cfg = *cfg;
  b->cfg.x0_host = b->cfg.y0_host = b->cfg.z0_host = b->cfg.ds_host = nullptr;
  b->dim = cfg->dim;
  b->M = cfg->n_markers;
  const int w = 2 * cfg->radius;
  b->S = cfg->dim == 2 ? w * w : w * w * w;
  b->C = cfg->dim;
  const size_t ts = dsize(cfg->dtype);
  const int M = b->M;
  auto fail = [&](cudaError_t e) {
    free_body(b);
    return cuda_status(e, "vs_body_plan_create");
  };
  // host marker data in the plan precision
  std::vector<unsigned char> hx(ts * M * 3);
  auto put = [&](int idx, double v) {
    if (ts == 8) ((double*)hx.data())[idx] = v;
    else ((float*)hx.data())[idx] = (float)v;
  };
  // extents of the marker cloud (for the window capacity)
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  const double* src[3] = {cfg->x0_host, cfg->y0_host, cfg->z0_host};
  for (int m = 0; m < M; ++m)
    for (int d = 0; d < cfg->dim; ++d) {
      const double v = src[d][m];
      lo[d] = v < lo[d] ? v : lo[d];
      hi[d] = v > hi[d] ? v : hi[d];
      if (cfg->dim == 2) put(d * M + m, v);
      else put(m * 3 + d, v);
    }
  b->rot = cfg->dim == 2 && cfg->free_dof[2] ? 1 : 0;
  double rmax = 0.0;
  if (b->rot) {
    // a turning body sweeps the disc about its centre: window and box cover every angle
    for (int m = 0; m < M; ++m) {
      const double r = hypot(cfg->x0_host[m] - cfg->center_x, cfg->y0_host[m] - cfg->center_y);
      rmax = r > rmax ? r : rmax;
    }
    lo[0] = cfg->center_x - rmax; hi[0] = cfg->center_x + rmax;
    lo[1] = cfg->center_y - rmax; hi[1] = cfg->center_y + rmax;
  }
  for (int d = 0; d < cfg->dim; ++d) b->cap[d] = (int)(floor(hi[d]) - floor(lo[d])) + w + 2;
  for (int d = 0; d < 2; ++d) b->lo_t[d] = ts == 8 ? lo[d] : (double)(float)lo[d];
  b->lo_t3 = cfg->dim == 3 ? (ts == 8 ? lo[2] : (double)(float)lo[2]) : 0.0;
  if (cfg->dim == 2) b->cap[2] = 1;
  {
    // region the window can reach: the initial stencil box, widened along free DOFs by the
    // margin (default: one body extent) and by 2 nodes along every axis, clipped to the grid
    const int nn[3] = {lattice->cfg.nx, lattice->cfg.ny, lattice->cfg.nz};
    for (int d = 0; d < 3; ++d) {
      if (d >= cfg->dim) {
        b->box[2 * d] = 0;
        b->box[2 * d + 1] = nn[d];
        continue;
      }
      const int lo_n = (int)floor(lo[d]) - cfg->radius + 1, hi_n = (int)floor(hi[d]) + cfg->radius + 1;
      // a fixed 3-D body's force window is exactly its stencil box; a 2-D body's predicted
      // window reaches one node below and three above the stencil box
      int margin = cfg->dim == 3 && !cfg->moving ? 0 : 4;
      if (cfg->moving && cfg->free_dof[d])
        margin += cfg->window_margin > 0 ? cfg->window_margin : (hi_n - lo_n);
      b->box[2 * d] = lo_n - margin < 0 ? 0 : lo_n - margin;
      b->box[2 * d + 1] = hi_n + margin > nn[d] ? nn[d] : hi_n + margin;
    }
  }
  {
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    b->prio = prio_hi;
    cudaError_t es = cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, prio_hi);
    if (es == cudaSuccess) es = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (es == cudaSuccess) es = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
    if (es == cudaSuccess) es = cudaStreamCreateWithPriority(&b->side2, cudaStreamNonBlocking, prio_hi);
    if (es == cudaSuccess) es = cudaEventCreateWithFlags(&b->ev_join2, cudaEventDisableTiming);
    if (es != cudaSuccess) {
      free_body(b);
      return cuda_status(es, "vs_body_plan_create stream");
    }
  }
  cudaError_t e;
  if ((e = cudaMalloc(&b->d_X0, ts * M * 3)) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpy(b->d_X0, hx.data(), ts * M * 3, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
  if (cfg->ds_host) {
    std::vector<unsigned char> hd(ts * M);
    for (int m = 0; m < M; ++m) {
      if (ts == 8) ((double*)hd.data())[m] = cfg->ds_host[m];
      else ((float*)hd.data())[m] = (float)cfg->ds_host[m];
    }
    if ((e = cudaMalloc(&b->d_ds, ts * M)) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpy(b->d_ds, hd.data(), ts * M, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
  }
  if ((e = cudaMalloc(&b->d_state, ts * 12)) != cudaSuccess) return fail(e);
  b->fsi = cfg->fsi_iter > 1 ? cfg->fsi_iter : 1;
  if (b->fsi > 1 && (e = cudaMalloc(&b->d_base, ts * 9)) != cudaSuccess) return fail(e);
  {
    double st[12] = {0};
    for (int c = 0; c < 3; ++c) {
      st[c] = cfg->a0[c];
      st[3 + c] = cfg->v0[c];
      st[6 + c] = cfg->d0[c];
    }
    const int rc = vs_body_set_state(b, st, nullptr);
    if (rc) {
      free_body(b);
      return rc;
    }
  }
  // force window: a 2-D body writes its predicted region, (cap + 2) nodes per axis
  const int64_t cells = cfg->dim == 2 ? (int64_t)(b->cap[0] + 2) * (b->cap[1] + 2)
                                      : (int64_t)b->cap[0] * b->cap[1] * b->cap[2];
  if ((e = cudaMalloc(&b->d_gw, ts * b->C * cells)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&b->d_meta, sizeof(int) * META_N)) != cudaSuccess) return fail(e);
  {
    int meta[META_N] = {0, 0, 0, 0, 0, 0, 0, 0};
    if ((e = cudaMemcpy(b->d_meta, meta, sizeof(meta), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
  }
  // Newmark scalars formed in double as the reference's Python floats (dyn.py:31-49)
  const double dt = 1.0, gamma = 0.5, beta = 0.25;
  b->nm[0] = dt * (1 - gamma);
  b->nm[1] = dt * dt * (0.5 - beta);
  b->nm[2] = gamma * dt;
  b->nm[3] = beta * dt * dt;
  b->nm[4] = dt;
  b->nm[5] = cfg->damping;
  b->nm[6] = cfg->stiffness;
  b->nm[7] = cfg->mass + b->nm[2] * cfg->damping + b->nm[3] * cfg->stiffness;
  b->nm[8] = cfg->added_mass_area;
  b->nm[9] = cfg->rot_damping;
  b->nm[10] = cfg->rot_stiffness;
  b->nm[11] = cfg->inertia + b->nm[2] * cfg->rot_damping + b->nm[3] * cfg->rot_stiffness;
  b->nm[12] = cfg->added_inertia;
  if (cfg->dim == 2) {
    const int EX = b->cap[0] + 2, EY = b->cap[1] + 2;
    if ((int64_t)M * b->S >= 65536 || (int64_t)EX * EY >= 65536) {
      free_body(b);
      set_error("2-D body with %d markers (%d x %d window) exceeds the single-CTA body kernel", M, EX, EY);
      return VS_ERR_UNSUPPORTED;
    }
    const int al = (int)(16 / ts);
    b->row_len = ((EY + al - 1 + al - 1) / al) * al;  // region row plus alignment slack
    b->bulk = lattice->cfg.ny % al == 0 && b->row_len <= 256 && EX <= 256;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    {
      // chain form when the marker order bounds node sharing (markers rounded to the plan precision)
      std::vector<double> xr(M), yr(M);
      for (int m = 0; m < M; ++m) {
        xr[m] = ts == 8 ? cfg->x0_host[m] : (double)(float)cfg->x0_host[m];
        yr[m] = ts == 8 ? cfg->y0_host[m] : (double)(float)cfg->y0_host[m];
      }
      b->chain_k = chain_width(xr.data(), yr.data(), M, cfg->radius, b->rot);
      b->chain = (M <= 32 || 2 * b->chain_k + 1 <= 31) && !getenv_flag("VIVSIM_GB300_BODY_CSR");
    }
    auto smem_of = [&](int rl) {
      if (b->chain)
        return ts == 8 ? body2d_chain_smem<double>(M, cfg->radius, EX, rl) : body2d_chain_smem<float>(M, cfg->radius, EX, rl);
      return ts == 8 ? body2d_smem<double>(M, cfg->radius, EX, EY, rl) : body2d_smem<float>(M, cfg->radius, EX, EY, rl);
    };
    b->smem = smem_of(b->bulk ? b->row_len : 0);
    if ((int64_t)b->smem > optin && b->bulk) {  // fall back to direct loads without staging
      b->bulk = 0;
      b->smem = smem_of(0);
    }
    if ((int64_t)b->smem > optin) {
      free_body(b);
      set_error("body of %d markers needs %zu bytes of shared memory (> %d available)", M, b->smem, optin);
      return VS_ERR_UNSUPPORTED;
    }
    if (!b->bulk) b->row_len = 0;
    {
      // last bounding-box corner before the first step
      int meta0[META_N] = {0};
      meta0[META_PX] = (int)floor(lo[0] + cfg->d0[0]) - cfg->radius + 1;
      meta0[META_PY] = (int)floor(lo[1] + cfg->d0[1]) - cfg->radius + 1;
      meta0[META_PX2] = meta0[META_PX];
      meta0[META_PY2] = meta0[META_PY];
      if ((e = cudaMemcpy(b->d_meta, meta0, sizeof(meta0), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
      if (b->rot) {  // a turning body: the corner of its markers at the initial angle
        if (ts == 8)
          k_set_state<double><<<1, 32>>>((double*)b->d_state, (const double*)b->d_state, b->d_meta, 0.0, 0.0,
                                         cfg->radius, kin_params<double>(b));
        else
          k_set_state<float><<<1, 32>>>((float*)b->d_state, (const float*)b->d_state, b->d_meta, 0.0, 0.0,
                                        cfg->radius, kin_params<float>(b));
        if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
      }
    }
    // the limit is a property of the kernel function, shared by every plan: raise it to the
    // device maximum once rather than to this plan's size (a smaller later plan would
    // otherwise invalidate the launches of a larger one)
    if (b->chain)
      e = ts == 8 ? body2d_chain_attr<double>(cfg->radius, optin) : body2d_chain_attr<float>(cfg->radius, optin);
    else
      e = ts == 8 ? body2d_attr<double>(cfg->radius, optin) : body2d_attr<float>(cfg->radius, optin);
    if (e != cudaSuccess) return fail(e);
    // cluster form: one pair per thread over up to 8 CTAs, each holding a contiguous share
    // of the markers (ceil(M / CL) markers' pairs per CTA)
    b->cluster = 0;
    if (b->chain && b->fsi == 1 && !getenv_flag("VIVSIM_GB300_BODY_SINGLE")) {
      int cl_ok = 0;
      cudaDeviceGetAttribute(&cl_ok, cudaDevAttrClusterLaunch, dev);
      int c = 1;
      while (c <= 8 && ((M + c - 1) / c) * b->S > kClusterPairs) ++c;
      // threads: the CTA's pairs, and enough for one window node each
      const int NB = (b->cap[0] + 2) * (b->cap[1] + 2);
      int th = ((M + c - 1) / c) * b->S;
      th = th > (NB + c - 1) / c ? th : (NB + c - 1) / c;
      th = ((th + 31) / 32) * 32;
      th = th < kClusterThreads ? th : kClusterThreads;
      if (cl_ok && c <= 8 && c <= M) {
        b->cl_size = c;
        b->cl_threads = th;
        b->cl_smem = ts == 8 ? body2d_cluster_smem<double>(M, cfg->radius, th, c, NB)
                             : body2d_cluster_smem<float>(M, cfg->radius, th, c, NB);
        if ((int64_t)b->cl_smem <= optin) {
          e = cluster_attr(cfg->dtype, cfg->radius, lattice->cfg.collision, optin);
          if (e != cudaSuccess) return fail(e);
          b->cluster = 1;
        }
      }
    }
    // the persistent run (float, 4 x 4 stencils): its size, and its barrier words
    b->run_ctas = 0;
    if (b->cluster && ts == 4 && cfg->radius == 2) {
      int coop = 0;
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
      b->run_smem = body2d_cluster_smem<float>(M, 2, kRunThreads, b->cl_size, (b->cap[0] + 2) * (b->cap[1] + 2));
      int ctas = 0;
      if (coop && (int64_t)b->run_smem <= optin && viv_run_setup(b, lattice->cfg.collision, ctas) != cudaSuccess) {
        cudaGetLastError();
        ctas = 0;
      }
      if (ctas > 0) {
        if ((e = cudaMalloc((void**)&b->d_bar, 4 * sizeof(unsigned))) != cudaSuccess) return fail(e);
        if ((e = cudaMemset(b->d_bar, 0, 4 * sizeof(unsigned))) != cudaSuccess) return fail(e);
        b->run_ctas = ctas;
      }
    }
  } else if (cfg->moving) {
    // moving 3-D body: the window follows the stencil box (one node of slack per axis for
    // the floor of a moving coordinate); CSR rebuilt every step inside the workspace
    const int nn[3] = {lattice->cfg.nx, lattice->cfg.ny, lattice->cfg.nz};
    for (int d = 0; d < 3; ++d) {
      b->cap[d] = (int)(floor(hi[d]) - floor(lo[d])) + w + 1;
      if (b->box[2 * d + 1] - b->box[2 * d] < b->cap[d] || b->box[2 * d] < 0 || b->box[2 * d + 1] > nn[d]) {
        free_body(b);
        set_error("moving body window does not fit the grid along axis %d", d);
        return VS_ERR_RANGE;
      }
    }
    const int64_t wcells = (int64_t)b->cap[0] * b->cap[1] * b->cap[2];
    const int64_t P = (int64_t)M * b->S;
    VS_REQUIRE(P < (1ll << 31) && wcells < (1ll << 31), "moving body too large");
    b->U = (int)P;  // node arrays are sized for every pair touching a distinct node
    e = cudaFree(b->d_gw);
    b->d_gw = nullptr;
    if (e != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_gw, ts * 3 * wcells)) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(b->d_gw, 0, ts * 3 * wcells)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_W, ts * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_I, sizeof(int32_t) * P)) != cudaSuccess) return fail(e);
    b->ws_bytes = vs_ib_workspace_bytes(M, b->S);
    if ((e = cudaMalloc(&b->d_ws, b->ws_bytes)) != cudaSuccess) return fail(e);
    {
      // the CSR views are fixed offsets into the workspace: fill them once from a dry build
      // of an all-dropped key set (every key -1)
      if ((e = cudaMemset(b->d_I, 0xff, sizeof(int32_t) * P)) != cudaSuccess) return fail(e);
      IbCsrView v{};
      int rc = ib_build_csr(b->d_I, P, wcells, b->d_ws, M, b->S, &v, nullptr);
      if (rc) {
        free_body(b);
        return rc;
      }
      unsigned st0 = 0;
      vs_ib_status(&st0, 1);  // the dry build's dropped keys are not an error
      b->sids = v.sids;
      b->pair_uid = v.pair_uid;
    }
    if ((e = cudaMalloc(&b->d_node_cell, sizeof(int32_t) * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_seg, sizeof(int32_t) * (P + 1))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_wsort, ts * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&b->d_msort, sizeof(int32_t) * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&b->d_U, sizeof(int))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_nu, ts * 3 * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_nv, ts * 3 * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_mk, ts * 9 * M)) != cudaSuccess) return fail(e);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
  } else {
    // fixed 3-D body: stencil once over a fixed window around the markers
    const int nn[3] = {lattice->cfg.nx, lattice->cfg.ny, lattice->cfg.nz};
    int org[3];
    for (int d = 0; d < 3; ++d) {
      org[d] = (int)floor(lo[d]) - cfg->radius + 1;
      b->cap[d] = (int)(floor(hi[d]) - floor(lo[d])) + w;
      if (org[d] < 0 || org[d] + b->cap[d] > nn[d]) {
        free_body(b);
        set_error("body stencil leaves the grid along axis %d", d);
        return VS_ERR_RANGE;
      }
    }
    int meta[META_N] = {org[0], org[1], org[2], b->cap[0], b->cap[1], b->cap[2], 0, 0};
    for (int d = 0; d < 3; ++d) {
      b->box[2 * d] = org[d];
      b->box[2 * d + 1] = org[d] + b->cap[d];
    }
    if ((e = cudaMemcpy(b->d_meta, meta, sizeof(meta), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
    const int64_t wcells = (int64_t)b->cap[0] * b->cap[1] * b->cap[2];
    const int64_t P = (int64_t)M * b->S;
    // window-relative marker coordinates
    std::vector<unsigned char> hr(ts * M * 3);
    for (int m = 0; m < M; ++m)
      for (int d = 0; d < 3; ++d) {
        const double v = src[d][m] - org[d];
        if (ts == 8) ((double*)hr.data())[m * 3 + d] = v;
        else ((float*)hr.data())[m * 3 + d] = (float)((float)src[d][m] - (float)org[d]);
      }
    void* d_rel = nullptr;
    if ((e = cudaMalloc(&d_rel, ts * M * 3)) != cudaSuccess) return fail(e);
    cudaMemcpy(d_rel, hr.data(), ts * M * 3, cudaMemcpyHostToDevice);
    if ((e = cudaMalloc(&b->d_W, ts * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_I, sizeof(int32_t) * P)) != cudaSuccess) return fail(e);
    int rc = vs_ib_stencil_3d(cfg->kernel, cfg->radius, cfg->dtype, d_rel, M, b->cap[0], b->cap[1], b->cap[2],
                              b->d_W, b->d_I, nullptr);
    cudaFree(d_rel);
    if (rc) {
      free_body(b);
      return rc;
    }
    e = cudaFree(b->d_gw);
    b->d_gw = nullptr;
    if (e != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_gw, ts * 3 * wcells)) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(b->d_gw, 0, ts * 3 * wcells)) != cudaSuccess) return fail(e);
    b->ws_bytes = vs_ib_workspace_bytes(M, b->S);
    if ((e = cudaMalloc(&b->d_ws, b->ws_bytes)) != cudaSuccess) return fail(e);
    IbCsrView v{};
    rc = ib_build_csr(b->d_I, P, wcells, b->d_ws, M, b->S, &v, nullptr);
    if (rc) {
      free_body(b);
      return rc;
    }
    int32_t last_uid = 0;
    if ((e = cudaMemcpy(&last_uid, v.uid + (P - 1), sizeof(int32_t), cudaMemcpyDeviceToHost)) != cudaSuccess)
      return fail(e);
    b->U = last_uid + 1;
    b->sids = v.sids;
    b->pair_uid = v.pair_uid;
    if ((e = cudaMalloc(&b->d_node_cell, sizeof(int32_t) * b->U)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_seg, sizeof(int32_t) * (b->U + 1))) != cudaSuccess) return fail(e);
    k_compact_csr<<<grid_for(P, 256), 256>>>(v.skeys, v.head, v.uid, P, b->d_node_cell, b->d_seg);
    if ((e = cudaMalloc(&b->d_wsort, ts * P)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&b->d_msort, sizeof(int32_t) * P)) != cudaSuccess) return fail(e);
    if (ts == 8)
      k_csr_gather<double><<<grid_for(P, 256), 256>>>(v.sids, (const double*)b->d_W, b->S, P, (double*)b->d_wsort,
                                                      b->d_msort);
    else
      k_csr_gather<float><<<grid_for(P, 256), 256>>>(v.sids, (const float*)b->d_W, b->S, P, (float*)b->d_wsort,
                                                     b->d_msort);
    const int32_t endP = (int32_t)P;
    if ((e = cudaMemcpy(b->d_seg + b->U, &endP, sizeof(int32_t), cudaMemcpyHostToDevice)) != cudaSuccess)
      return fail(e);
    if ((e = cudaMalloc(&b->d_nu, ts * 3 * b->U)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_nv, ts * 3 * b->U)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc(&b->d_mk, ts * 9 * M)) != cudaSuccess) return fail(e);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
  }
  if (b->dim == 3 && !cfg->moving) {
    int rc3 = ts == 8 ? body3_cluster_setup<double>(b) : body3_cluster_setup<float>(b);
    if (rc3) {
      free_body(b);
      return rc3;
    }
  }
  if (b->dim == 3) {
    // the fused 3-D body kernel: one CTA per SM by default (VIVSIM_GB300_BODY3D_CTAS: another
    // count, 0 for the per-phase kernels), at most what can be resident at once
    int dev = 0, coop = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = ts == 8 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_body3d_fused<L19, double>, kBody3Threads, 0)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_body3d_fused<L19, float>, kBody3Threads, 0);
    if (e != cudaSuccess) return fail(e);
    int G = sms;
    if (const char* v = getenv("VIVSIM_GB300_BODY3D_CTAS")) G = atoi(v);
    if (G > per_sm * sms) G = per_sm * sms;
    b->fused3 = coop && G > 0 ? G : 0;
    if (b->fused3) {
      if ((e = cudaMalloc((void**)&b->d_bar, 4 * sizeof(unsigned))) != cudaSuccess) return fail(e);
      if ((e = cudaMemset(b->d_bar, 0, 4 * sizeof(unsigned))) != cudaSuccess) return fail(e);
    }
  }
  *out = b;
  return VS_OK;
}

int vs_body_plan_destroy(vs_body_plan* plan) {
  free_body(plan);
  return VS_OK;
}

int vs_body_set_state(vs_body_plan* plan, const double* state_host, void* stream) {
  VS_REQUIRE(plan && state_host, "vs_body_set_state: null argument");
  const size_t ts = dsize(plan->cfg.dtype);
  unsigned char buf[12 * 8];
  for (int i = 0; i < 12; ++i) {
    if (ts == 8) ((double*)buf)[i] = state_host[i];
    else ((float*)buf)[i] = (float)state_host[i];
  }
  cudaStream_t st = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(plan->d_state, buf, ts * 12, cudaMemcpyHostToDevice, st);
  int corner[2];
  if (plan->rot && plan->d_meta && e == cudaSuccess) {
    // a turning body: the corner of its turned markers, found on the device
    const int rc = dispatch_t(plan->cfg.dtype, [&](auto t) -> int {
      using T = typename decltype(t)::type;
      k_set_state<T><<<1, 32, 0, st>>>((T*)plan->d_state, (const T*)plan->d_state, plan->d_meta, 0.0, 0.0,
                                        plan->cfg.radius, kin_params<T>(plan));
      VS_CHECK_LAUNCH("vs_body_set_state");
      return VS_OK;
    });
    if (rc) return rc;
  } else if (plan->dim == 2 && plan->d_meta) {
    // the 2-D body kernel predicts its window from the last stencil corner: restart that
    // prediction from the new displacement (floor of the smallest marker coordinate)
    for (int d = 0; d < 2; ++d) {
      const double x = ts == 8 ? plan->lo_t[d] + state_host[6 + d] : (double)((float)plan->lo_t[d] + (float)state_host[6 + d]);
      corner[d] = (int)floor(x) - plan->cfg.radius + 1;
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(plan->d_meta + META_PX, corner, sizeof(corner), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(plan->d_meta + META_PX2, corner, sizeof(corner), cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_status(e, "vs_body_set_state");
}

int vs_body_set_state_device(vs_body_plan* plan, const void* state, void* stream) {
  VS_REQUIRE(plan && state, "vs_body_set_state_device: null argument");
  return dispatch_t(plan->cfg.dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_set_state<T><<<1, 32, 0, as_stream(stream)>>>((T*)plan->d_state, (const T*)state,
                                                    plan->dim == 2 ? plan->d_meta : nullptr, plan->lo_t[0],
                                                    plan->lo_t[1], plan->cfg.radius, kin_params<T>(plan));
    VS_CHECK_LAUNCH("vs_body_set_state_device");
    return VS_OK;
  });
}

int vs_body_state_device(const vs_body_plan* plan, void** state) {
  VS_REQUIRE(plan && state, "vs_body_state_device: null argument");
  *state = plan->d_state;
  return VS_OK;
}

int vs_body_get_state(const vs_body_plan* plan, double* state_host, void* stream) {
  VS_REQUIRE(plan && state_host, "vs_body_get_state: null argument");
  const size_t ts = dsize(plan->cfg.dtype);
  unsigned char buf[12 * 8];
  int meta[META_N];
  cudaStream_t st = as_stream(stream);
  cudaError_t e = cudaMemcpyAsync(buf, plan->d_state, ts * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(meta, plan->d_meta, sizeof(meta), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "vs_body_get_state");
  for (int i = 0; i < 12; ++i) state_host[i] = ts == 8 ? ((double*)buf)[i] : (double)((float*)buf)[i];
  if (meta[META_STATUS] != 0) {
    if (meta[META_STATUS] == VS_ERR_RANGE) set_error("immersed body left its window or the grid (stencil out of range)");
    else if (meta[META_STATUS] == VS_ERR_TIMEOUT_INFLIGHT)
      set_error("a body kernel gave up waiting for its bulk copy, which had still not landed when it left");
    else set_error("a body kernel gave up waiting for its bulk copy (device status %d)", meta[META_STATUS]);
    return meta[META_STATUS];
  }
  return VS_OK;
}

int vs_step(const vs_lattice_plan* lattice, vs_body_plan* body, const void* f_in, void* f_out, void* force_hist,
            void* stream) {
  VS_REQUIRE(lattice && f_in && f_out && f_in != f_out, "vs_step: f_in and f_out must be distinct device buffers");
  return enqueue_step(lattice, body, f_in, f_out, force_hist, as_stream(stream));
}

int vs_step_grid_only(const vs_lattice_plan* lattice, const vs_body_plan* body, const void* f_in, void* f_out,
                      void* stream) {
  VS_REQUIRE(lattice && f_in && f_out && f_in != f_out, "vs_step_grid_only: bad arguments");
  return enqueue_grid(lattice, body, f_in, f_out, as_stream(stream));
}

int vs_run(const vs_lattice_plan* lattice, vs_body_plan* body, void* f_a, void* f_b, int n_steps, void* force_hist,
           void* stream) {
  VS_REQUIRE(lattice && f_a && f_b && f_a != f_b && n_steps >= 0, "vs_run: bad arguments");
  const size_t hs = 3 * dsize(lattice->cfg.dtype);
  const bool lazy = lazy_boundaries(lattice, body);
  if (n_steps > 1 && viv_run_applies(lattice, body, lazy)) {
    // persistent form: one launch per watchdog interval (or for the whole run)
    const int K = lattice->cfg.watchdog_every;
    for (int s0 = 0; s0 < n_steps;) {
      // (at most 2^20 steps per launch: the barrier's arrival count stays below 2^31)
      const int n = std::min(K > 0 ? std::min(K - s0 % K, n_steps - s0) : n_steps - s0, 1 << 20);
      int rc = viv_run_chunk(lattice, body, f_a, f_b, s0, n, lazy, force_hist, as_stream(stream));
      if (rc) return rc;
      s0 += n;
      void* last = ((s0 - 1) % 2 == 0) ? f_b : f_a;  // the output of step s0 - 1
      if (s0 == n_steps && lazy) {
        rc = enqueue_bcs(lattice, last, as_stream(stream));
        if (rc) return rc;
      }
      if (K > 0 && (s0 % K == 0 || s0 == n_steps)) {
        rc = vs_check_finite(lattice->cfg.dtype, last, lattice->n * lattice->cfg.q, lattice->d_status, stream);
        if (rc) return rc;
      }
    }
    return VS_OK;
  }
  for (int s = 0; s < n_steps; ++s) {
    void* src = (s % 2 == 0) ? f_a : f_b;
    void* dst = (s % 2 == 0) ? f_b : f_a;
    void* hist = force_hist ? (void*)((char*)force_hist + hs * s) : nullptr;
    // obstacle bounce-back: deferred to the next step's load, applied at the end of the run
    int rc = enqueue_step(lattice, body, src, dst, hist, as_stream(stream), lazy && s > 0, !lazy || s == n_steps - 1,
                          s > 0, s == n_steps - 1);
    if (rc) return rc;
    const int K = lattice->cfg.watchdog_every;
    if (K > 0 && ((s + 1) % K == 0 || s == n_steps - 1)) {
      rc = vs_check_finite(lattice->cfg.dtype, dst, lattice->n * lattice->cfg.q, lattice->d_status, stream);
      if (rc) return rc;
    }
  }
  return VS_OK;
}

int vs_run_persistent(const vs_lattice_plan* lattice, const vs_body_plan* body, int n_steps) {
  if (!lattice || n_steps < 2) return 0;
  return viv_run_applies(lattice, body, lazy_boundaries(lattice, body)) ? 1 : 0;
}

int vs_run_graph(vs_lattice_plan* lattice, vs_body_plan* body, void* f_a, void* f_b, int n_steps, void* force_hist,
                 void* stream) {
  VS_REQUIRE(lattice && f_a && f_b && f_a != f_b && n_steps > 0, "vs_run_graph: bad arguments");
  cudaStream_t st = as_stream(stream);
  VS_REQUIRE(st != nullptr, "vs_run_graph: needs a non-default stream (stream capture)");
  // the persistent form is already one launch per run: no graph to capture
  if (n_steps > 1 && viv_run_applies(lattice, body, lazy_boundaries(lattice, body)))
    return vs_run(lattice, body, f_a, f_b, n_steps, force_hist, stream);
  const bool hit = lattice->graph && lattice->g_fa == f_a && lattice->g_fb == f_b && lattice->g_steps == n_steps &&
                   lattice->g_hist == force_hist && lattice->g_body == body && lattice->g_stream == st;
  if (!hit) {
    if (lattice->graph) {
      cudaGraphExecDestroy(lattice->graph);
      lattice->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_status(e, "vs_run_graph capture");
    int rc = vs_run(lattice, body, f_a, f_b, n_steps, force_hist, stream);
    e = cudaStreamEndCapture(st, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_status(e, "vs_run_graph end capture");
    // side-stream launches keep their priority in the replayed graph
    e = cudaGraphInstantiateWithFlags(&lattice->graph, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_status(e, "vs_run_graph instantiate");
    lattice->g_fa = f_a;
    lattice->g_fb = f_b;
    lattice->g_steps = n_steps;
    lattice->g_hist = force_hist;
    lattice->g_body = body;
    lattice->g_stream = st;
  }
  return cuda_status(cudaGraphLaunch(lattice->graph, st), "vs_run_graph launch");
}

}  // extern "C"

// ------------------------------------------------------------------ many cases per launch
// A batch advances many independent cases (each a lattice plan with an optional body plan)
// in lock step: per time step ONE body launch (one CTA per body, chain form), ONE grid
// launch over the nodes of every case outside its body's box (a flattened block list:
// block b works on case blk[b].x as block blk[b].y of that case's own geometry), and ONE
// launch over every box (+ lazy walls) after the join.  Per-case parameters sit in device
// arrays, built once for a pair of population buffer sets.  The middle time steps can be
// replayed from a CUDA graph of `steps_per_graph` steps.
struct vs_batch_plan {
  int n = 0;
  std::vector<vs_lattice_plan*> L;
  std::vector<vs_body_plan*> B;
  std::vector<int> lazy;        // per case: face boundaries deferred to the next step's load
  std::vector<int> chain_bodies, other_bodies;  // case indices
  int q = 0, dtype = 0, collision = 0, radius = 0;
  int tb = 128;                 // threads per block of the grid launches
  int npt = 1;                  // nodes per thread of the main launch (1 or 2)
  int built_npt = 0;
  int spg = 64;                 // default steps per graph
  size_t body_smem = 0;
  std::vector<const void*> fa, fb;  // buffers the device parameters were built for
  int built_tb = 0;
  void* d_main[2][2] = {};      // [parity][first step] StepParams per case
  void* d_reg[2][2] = {};       // [parity][first step] StepParams per chain-body case
  int2* d_blk_main = nullptr;
  int2* d_blk_reg[2] = {};
  int n_blk_main = 0, n_blk_reg[2] = {0, 0};
  int main_skip_only = 0;       // the main launch needs no per-node feature but the skip tests
  void* d_body[2] = {};         // [parity] BodyParams per chain body
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaGraphExec_t graph = nullptr;
  int g_steps = 0;
  cudaStream_t g_stream = nullptr;
};

namespace vs {

static void batch_free_params(vs_batch_plan* bp) {
  for (int p = 0; p < 2; ++p) {
    for (int f = 0; f < 2; ++f) {
      if (bp->d_main[p][f]) cudaFree(bp->d_main[p][f]);
      if (bp->d_reg[p][f]) cudaFree(bp->d_reg[p][f]);
      bp->d_main[p][f] = bp->d_reg[p][f] = nullptr;
    }
    if (bp->d_body[p]) cudaFree(bp->d_body[p]);
    bp->d_body[p] = nullptr;
    if (bp->d_blk_reg[p]) cudaFree(bp->d_blk_reg[p]);
    bp->d_blk_reg[p] = nullptr;
  }
  if (bp->d_blk_main) cudaFree(bp->d_blk_main);
  bp->d_blk_main = nullptr;
  if (bp->graph) cudaGraphExecDestroy(bp->graph);
  bp->graph = nullptr;
  bp->fa.clear();
  bp->fb.clear();
}

template <typename V>
static cudaError_t upload(void** dst, const std::vector<V>& v) {
  if (v.empty()) return cudaSuccess;
  cudaError_t e = cudaMalloc(dst, sizeof(V) * v.size());
  if (e == cudaSuccess) e = cudaMemcpy(*dst, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice);
  return e;
}

template <class L, typename T>
static int batch_build(vs_batch_plan* bp, void* const* fa, void* const* fb) {
  batch_free_params(bp);
  std::vector<StepParams<L, T>> main[2][2], reg[2][2];
  std::vector<int2> bm, br[2];
  std::vector<BodyParams<T>> body[2];
  bool skip_only = true;
  for (int p = 0; p < 2; ++p)
    for (int first = 0; first < 2; ++first) {
      for (int k = 0; k < bp->n; ++k) {
        const void* fin = p == 0 ? fa[k] : fb[k];
        void* fout = p == 0 ? fb[k] : fa[k];
        const bool lazy_in = !first && bp->lazy[k];
        StepParams<L, T> P;
        dim3 g;
        int tb = 0;
        const bool chain_body = bp->B[k] && bp->B[k]->dim == 2 && bp->B[k]->chain;
        if (bp->B[k] && !chain_body) {
          // a body outside the batched form runs its own kernels; its whole grid then
          // goes after the join (it reads the force window)
          if (grid_setup<L, T>(bp->L[k], bp->B[k], fin, fout, 0, false, bp->tb, P, g, tb)) {
            const int idx = (int)reg[p][first].size();
            reg[p][first].push_back(P);
            if (p == 0)
              for (int j = 0; j < (int)(g.x * g.y); ++j) br[first].push_back(make_int2(idx, j));
          }
          continue;
        }
        const vs_body_plan* Bk = bp->B[k];
        if (grid_setup<L, T>(bp->L[k], Bk, fin, fout, Bk ? 1 : 0, lazy_in, bp->tb, P, g, tb)) {
          const int idx = (int)main[p][first].size();
          main[p][first].push_back(P);
          skip_only = skip_only && !P.gw && !P.has_g0 && !P.mask_load && P.n_pre == 0 && P.n_lazy == 0;
          if (p == 0 && first == 1) {  // flat chunks of the case's nodes (k_step_batch_flat)
            const int64_t per = (int64_t)bp->tb * bp->npt;
            const int nch = (int)((bp->L[k]->n + per - 1) / per);
            for (int j = 0; j < nch; ++j) bm.push_back(make_int2(idx, j));
          }
        }
        if (!chain_body) continue;
        if (grid_setup<L, T>(bp->L[k], Bk, fin, fout, 2, lazy_in, bp->tb, P, g, tb)) {
          const int idx = (int)reg[p][first].size();
          reg[p][first].push_back(P);
          if (p == 0)
            for (int j = 0; j < (int)(g.x * g.y); ++j) br[first].push_back(make_int2(idx, j));
        }
        if (first == 0) body[p].push_back(body_params2d<T>(bp->B[k], bp->L[k], fin, nullptr, false));
      }
    }
  cudaError_t e = cudaSuccess;
  for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
    for (int f = 0; f < 2 && e == cudaSuccess; ++f) {
      e = upload(&bp->d_main[p][f], main[p][f]);
      if (e == cudaSuccess) e = upload(&bp->d_reg[p][f], reg[p][f]);
    }
    if (e == cudaSuccess) e = upload(&bp->d_body[p], body[p]);
    if (e == cudaSuccess) e = upload((void**)&bp->d_blk_reg[p], br[p]);
    bp->n_blk_reg[p] = (int)br[p].size();
  }
  if (e == cudaSuccess) e = upload((void**)&bp->d_blk_main, bm);
  bp->n_blk_main = (int)bm.size();
  bp->main_skip_only = skip_only ? 1 : 0;
  if (e != cudaSuccess) {
    batch_free_params(bp);
    return cuda_status(e, "vs_batch_run parameters");
  }
  bp->fa.assign(fa, fa + bp->n);
  bp->fb.assign(fb, fb + bp->n);
  bp->built_tb = bp->tb;
  bp->built_npt = bp->npt;
  return VS_OK;
}

template <class L, typename T, int COLL>
static int batch_step_t(vs_batch_plan* bp, int s, int n_steps, void* const* fa, void* const* fb, cudaStream_t st) {
  const int p = s & 1, first = s == 0 ? 1 : 0;
  const int nb = (int)bp->chain_bodies.size();
  const bool fork = nb > 0 || !bp->other_bodies.empty();
  cudaError_t e = cudaSuccess;
  if (fork) {
    e = cudaEventRecord(bp->ev_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(bp->side, bp->ev_fork, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_batch fork");
    if (nb > 0) {
      const BodyParams<T>* bpar = (const BodyParams<T>*)bp->d_body[p];
      switch (bp->radius) {
        case 1: k_body2d_chain_batch<T, 1><<<nb, kBodyThreads, bp->body_smem, bp->side>>>(bpar); break;
        case 2: k_body2d_chain_batch<T, 2><<<nb, kBodyThreads, bp->body_smem, bp->side>>>(bpar); break;
        default: k_body2d_chain_batch<T, 3><<<nb, kBodyThreads, bp->body_smem, bp->side>>>(bpar); break;
      }
    }
    // bodies outside the batched form: their own kernel(s), full grid in the main launch
    for (int k : bp->other_bodies) {
      const int rc = enqueue_body(bp->B[k], bp->L[k], p == 0 ? fa[k] : fb[k], nullptr, bp->side);
      if (rc) return rc;
    }
  }
  if (bp->n_blk_main > 0) {
    const StepParams<L, T>* mp = (const StepParams<L, T>*)bp->d_main[p][first];
    if (bp->npt == 2) {
      if (bp->main_skip_only)
        k_step_batch_flat2<L, T, COLL, kFeatSkip><<<bp->n_blk_main, bp->tb, 0, st>>>(mp, bp->d_blk_main);
      else
        k_step_batch_flat2<L, T, COLL, kFeatGeneral><<<bp->n_blk_main, bp->tb, 0, st>>>(mp, bp->d_blk_main);
    } else if (bp->main_skip_only) {
      k_step_batch_flat<L, T, COLL, kFeatSkip><<<bp->n_blk_main, bp->tb, 0, st>>>(mp, bp->d_blk_main);
    } else {
      k_step_batch_flat<L, T, COLL, kFeatGeneral><<<bp->n_blk_main, bp->tb, 0, st>>>(mp, bp->d_blk_main);
    }
  }
  if (fork) {
    e = cudaEventRecord(bp->ev_join, bp->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, bp->ev_join, 0);
    if (e != cudaSuccess) return cuda_status(e, "vs_batch join");
  }
  if (bp->n_blk_reg[first] > 0)
    k_step_batch<L, T, COLL, true><<<bp->n_blk_reg[first], bp->tb, 0, st>>>(
        (const StepParams<L, T>*)bp->d_reg[p][first], bp->d_blk_reg[first]);
  VS_CHECK_LAUNCH("vs_batch step");
  for (int k = 0; k < bp->n; ++k) {
    if (bp->lazy[k] && s != n_steps - 1) continue;
    const int rc = enqueue_bcs(bp->L[k], p == 0 ? fb[k] : fa[k], st);
    if (rc) return rc;
  }
  return VS_OK;
}

static int batch_step(vs_batch_plan* bp, int s, int n_steps, void* const* fa, void* const* fb, cudaStream_t st) {
  return dispatch(bp->q, bp->dtype, [&](auto l, auto t) -> int {
    using L = decltype(l);
    using T = typename decltype(t)::type;
    switch (bp->collision) {
      case VS_COLLIDE_BGK: return batch_step_t<L, T, VS_COLLIDE_BGK>(bp, s, n_steps, fa, fb, st);
      case VS_COLLIDE_KBC: return batch_step_t<L, T, VS_COLLIDE_KBC>(bp, s, n_steps, fa, fb, st);
      case VS_COLLIDE_REG: return batch_step_t<L, T, VS_COLLIDE_REG>(bp, s, n_steps, fa, fb, st);
      default: return batch_step_t<L, T, VS_COLLIDE_MRT>(bp, s, n_steps, fa, fb, st);
    }
  });
}

static void batch_destroy(vs_batch_plan* bp) {
  batch_free_params(bp);
  if (bp->ev_fork) cudaEventDestroy(bp->ev_fork);
  if (bp->ev_join) cudaEventDestroy(bp->ev_join);
  if (bp->side) cudaStreamDestroy(bp->side);
  delete bp;
}

}  // namespace vs

extern "C" {

int vs_batch_plan_create(vs_lattice_plan* const* lattices, vs_body_plan* const* bodies, int n_cases,
                         vs_batch_plan** out) {
  VS_REQUIRE(lattices && out && n_cases > 0, "vs_batch_plan_create: bad arguments");
  vs_batch_plan* bp = new (std::nothrow) vs_batch_plan();
  if (!bp) {
    set_error("out of host memory");
    return VS_ERR_INVALID_ARG;
  }
  auto fail = [&](int rc) {
    batch_destroy(bp);
    return rc;
  };
  bp->n = n_cases;
  for (int k = 0; k < n_cases; ++k) {
    vs_lattice_plan* Lk = lattices[k];
    vs_body_plan* Bk = bodies ? bodies[k] : nullptr;
    if (!Lk) {
      set_error("vs_batch_plan_create: case %d has no lattice plan", k);
      return fail(VS_ERR_INVALID_ARG);
    }
    if (Lk->cfg.obstacle_mask) {
      set_error("vs_batch_plan_create: case %d has an obstacle mask (not supported in a batch)", k);
      return fail(VS_ERR_UNSUPPORTED);
    }
    for (int b = 0; b < Lk->cfg.n_bc; ++b)
      if (Lk->cfg.bc[b].mode == VS_WALL_CHARACTERISTIC) {
        set_error("vs_batch_plan_create: case %d has a characteristic wall (not supported in a batch)", k);
        return fail(VS_ERR_UNSUPPORTED);
      }
    if (k == 0) {
      bp->q = Lk->cfg.q;
      bp->dtype = Lk->cfg.dtype;
      bp->collision = Lk->cfg.collision;
    } else if (Lk->cfg.q != bp->q || Lk->cfg.dtype != bp->dtype || Lk->cfg.collision != bp->collision) {
      set_error("vs_batch_plan_create: case %d differs in lattice, dtype or collision from case 0", k);
      return fail(VS_ERR_UNSUPPORTED);
    }
    bp->L.push_back(Lk);
    bp->B.push_back(Bk);
    // one pass per step in the batched body launch; bodies with sub-iterations run their own
    const bool batched_body = Bk && Bk->dim == 2 && Bk->chain && Bk->fsi == 1;
    bp->lazy.push_back(batched_body && lazy_boundaries(Lk, Bk) ? 1 : 0);
    if (batched_body) {
      if (bp->chain_bodies.empty()) bp->radius = Bk->cfg.radius;
      if (Bk->cfg.radius != bp->radius) {
        set_error("vs_batch_plan_create: bodies with different stencil radii");
        return fail(VS_ERR_UNSUPPORTED);
      }
      bp->chain_bodies.push_back(k);
      const size_t sm = bp->dtype == VS_F64 ? body2d_chain_smem<double>(Bk->M, Bk->cfg.radius, Bk->cap[0] + 2, 0)
                                            : body2d_chain_smem<float>(Bk->M, Bk->cfg.radius, Bk->cap[0] + 2, 0);
      bp->body_smem = sm > bp->body_smem ? sm : bp->body_smem;
    } else if (Bk) {
      bp->other_bodies.push_back(k);
    }
  }
  for (size_t i = 0; i < bp->B.size(); ++i)
    for (size_t j = i + 1; j < bp->B.size(); ++j)
      if ((bp->B[i] && bp->B[i] == bp->B[j]) || bp->L[i] == bp->L[j]) {
        set_error("vs_batch_plan_create: cases %zu and %zu share a plan", i, j);
        return fail(VS_ERR_INVALID_ARG);
      }
  if (!bp->chain_bodies.empty()) {
    cudaError_t e = bp->dtype == VS_F64 ? cudaSuccess : cudaSuccess;
    auto attr = [&](auto fn) {
      int dev = 0, optin = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      if ((int64_t)bp->body_smem > optin) return cudaErrorInvalidValue;
      return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    };
    if (bp->dtype == VS_F64)
      e = bp->radius == 1 ? attr(k_body2d_chain_batch<double, 1>)
                          : (bp->radius == 2 ? attr(k_body2d_chain_batch<double, 2>) : attr(k_body2d_chain_batch<double, 3>));
    else
      e = bp->radius == 1 ? attr(k_body2d_chain_batch<float, 1>)
                          : (bp->radius == 2 ? attr(k_body2d_chain_batch<float, 2>) : attr(k_body2d_chain_batch<float, 3>));
    if (e != cudaSuccess) return fail(cuda_status(e, "vs_batch_plan_create body kernel"));
  }
  if (!bp->chain_bodies.empty() || !bp->other_bodies.empty()) {
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    cudaError_t e = cudaStreamCreateWithPriority(&bp->side, cudaStreamNonBlocking, prio_hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bp->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bp->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(cuda_status(e, "vs_batch_plan_create stream"));
  }
  *out = bp;
  return VS_OK;
}

int vs_batch_plan_destroy(vs_batch_plan* plan) {
  if (plan) batch_destroy(plan);
  return VS_OK;
}

int vs_batch_set_launch(vs_batch_plan* plan, int threads_per_block, int steps_per_graph) {
  VS_REQUIRE(plan, "vs_batch_set_launch: null plan");
  VS_REQUIRE(threads_per_block == 32 || threads_per_block == 64 || threads_per_block == 128 ||
                 threads_per_block == 256,
             "vs_batch_set_launch: threads_per_block must be 32, 64, 128 or 256");
  VS_REQUIRE(steps_per_graph >= 0, "vs_batch_set_launch: steps_per_graph must be >= 0");
  plan->tb = threads_per_block;
  plan->spg = steps_per_graph;
  return VS_OK;
}

int vs_batch_set_nodes_per_thread(vs_batch_plan* plan, int nodes_per_thread) {
  VS_REQUIRE(plan, "vs_batch_set_nodes_per_thread: null plan");
  VS_REQUIRE(nodes_per_thread == 1 || nodes_per_thread == 2, "vs_batch_set_nodes_per_thread: 1 or 2");
  plan->npt = nodes_per_thread;
  return VS_OK;
}

int vs_batch_run(vs_batch_plan* plan, void* const* f_a, void* const* f_b, int n_steps, void* stream) {
  VS_REQUIRE(plan && f_a && f_b && n_steps >= 0, "vs_batch_run: bad arguments");
  for (int k = 0; k < plan->n; ++k)
    VS_REQUIRE(f_a[k] && f_b[k] && f_a[k] != f_b[k], "vs_batch_run: case %d needs two distinct buffers", k);
  if (n_steps == 0) return VS_OK;
  cudaStream_t st = as_stream(stream);
  // The batched chain form reads its window prediction from slot 0 (and writes both slots):
  // after a single-case run of the cluster form the current prediction may sit in slot 1
  for (int k : plan->chain_bodies) {
    vs_body_plan* Bk = plan->B[k];
    if (Bk->parity) {
      cudaError_t e = cudaMemcpyAsync(Bk->d_meta + META_PX, Bk->d_meta + META_PX2, 2 * sizeof(int),
                                      cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return cuda_status(e, "vs_batch_run prediction slot");
      Bk->parity = 0;
    }
  }
  bool same = plan->built_tb == plan->tb && plan->built_npt == plan->npt && (int)plan->fa.size() == plan->n;
  for (int k = 0; same && k < plan->n; ++k) same = plan->fa[k] == f_a[k] && plan->fb[k] == f_b[k];
  if (!same) {
    const int rc = dispatch(plan->q, plan->dtype, [&](auto l, auto t) -> int {
      return batch_build<decltype(l), typename decltype(t)::type>(plan, f_a, f_b);
    });
    if (rc) return rc;
  }
  // first step, then whole graphs of G middle steps (G even: every replay starts on an odd
  // step, so one graph serves all), then the remaining steps one by one
  const int G = (plan->spg / 2) * 2;
  int s = 0;
  int rc = batch_step(plan, s++, n_steps, f_a, f_b, st);
  if (rc) return rc;
  if (G > 0 && st != nullptr && n_steps - 1 - s >= G) {
    if (!plan->graph || plan->g_steps != G || plan->g_stream != st) {
      if (plan->graph) cudaGraphExecDestroy(plan->graph);
      plan->graph = nullptr;
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return cuda_status(e, "vs_batch_run capture");
      int crc = VS_OK;
      for (int j = 0; j < G && crc == VS_OK; ++j) crc = batch_step(plan, 1 + j, 1 << 30, f_a, f_b, st);
      e = cudaStreamEndCapture(st, &g);
      if (crc) {
        if (g) cudaGraphDestroy(g);
        return crc;
      }
      if (e != cudaSuccess) return cuda_status(e, "vs_batch_run end capture");
      e = cudaGraphInstantiateWithFlags(&plan->graph, g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_status(e, "vs_batch_run instantiate");
      plan->g_steps = G;
      plan->g_stream = st;
    }
    while (n_steps - 1 - s >= G) {
      cudaError_t e = cudaGraphLaunch(plan->graph, st);
      if (e != cudaSuccess) return cuda_status(e, "vs_batch_run graph launch");
      s += G;
    }
  }
  for (; s < n_steps; ++s) {
    rc = batch_step(plan, s, n_steps, f_a, f_b, st);
    if (rc) return rc;
  }
  return VS_OK;
}

}  // extern "C"
