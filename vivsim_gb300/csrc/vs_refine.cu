// Grid-refinement transfers of vivsim/multigrid.py between D2Q9 blocks of neighbouring
// levels (factor 2).  Both run after streaming and rewrite one line of the destination
// block in place: the three populations that cross the interface, nothing else.
//
// Shapes follow the reference's array semantics.  Along the interface the fine block's
// even nodes (0::2, length ceil(m/2)) and odd nodes (1::2, length floor(m/2)) are combined
// with NumPy/JAX broadcasting, so a length-1 operand stretches; any other mismatch is the
// reference's shape error and is rejected here.  The host resolves the broadcast into
// three lengths and the kernels index with them.
#include "vs_dispatch.cuh"

namespace vs {
namespace refine {

// LEFT/RIGHT/UP/DOWN direction triples of D2Q9 (vivsim/lbm/lattice.py:58-61)
__constant__ int kDirs[4][3] = {{3, 7, 6}, {1, 5, 8}, {2, 5, 6}, {4, 7, 8}};

struct Face {
  int dir;           // VS_REFINE_*
  int row0, row1;    // fine rows summed first and second (fine_to_coarse)
  int line;          // destination line (normal index)
  int src_line;      // source line (coarse_to_fine)
  int len_a, len_b;  // even / odd fine lengths along the interface
  int len_v;         // broadcast length of the combined value
  int n_out;         // nodes written per population
};

// node (normal index r, tangential index t) of a (9, nx, ny) block; x is the normal for
// LEFT/RIGHT, y for UP/DOWN
__device__ __forceinline__ int64_t at(int dir, int r, int t, int nx, int ny) {
  return dir <= VS_REFINE_RIGHT ? (int64_t)r * ny + t : (int64_t)t * ny + r;
}

// fine_to_coarse, multigrid.py:58-95: coarse[d, line, j] = 0.25 * (((F[r0, even] + F[r0, odd])
// + F[r1, even]) + F[r1, odd]), the reference's summation order
template <typename T>
__global__ void k_fine_to_coarse(const T* __restrict__ ff, int nxf, int nyf, T* __restrict__ fc, int nxc, int nyc,
                                 Face F) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (j >= F.n_out) return;
  const int d = kDirs[F.dir][k];
  const int v = F.len_v == 1 ? 0 : j;
  const int ea = 2 * (F.len_a == 1 ? 0 : v);
  const int ob = 2 * (F.len_b == 1 ? 0 : v) + 1;
  const int64_t nf = (int64_t)nxf * nyf;
  const T* src = ff + d * nf;
  T s = src[at(F.dir, F.row0, ea, nxf, nyf)] + src[at(F.dir, F.row0, ob, nxf, nyf)];
  s = s + src[at(F.dir, F.row1, ea, nxf, nyf)];
  s = s + src[at(F.dir, F.row1, ob, nxf, nyf)];
  fc[d * (int64_t)nxc * nyc + at(F.dir, F.line, j, nxc, nyc)] = T(0.25) * s;
}

// coarse_to_fine, multigrid.py:97-128: fine[d, line, i] = coarse[d, src_line, i / 2]
// (i even and odd), index 0 when the coarse line has length 1
template <typename T>
__global__ void k_coarse_to_fine(const T* __restrict__ fc, int nxc, int nyc, T* __restrict__ ff, int nxf, int nyf,
                                 Face F) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i >= F.n_out) return;
  const int d = kDirs[F.dir][k];
  const int c = F.len_v == 1 ? 0 : i / 2;
  ff[d * (int64_t)nxf * nyf + at(F.dir, F.line, i, nxf, nyf)] =
      fc[d * (int64_t)nxc * nyc + at(F.dir, F.src_line, c, nxc, nyc)];
}

// NumPy broadcast of two lengths, -1 when they do not broadcast
static int bcast(int a, int b) {
  if (a == b) return a;
  if (a == 1) return b;
  if (b == 1) return a;
  return -1;
}

static const char* kDirNames = "'left', 'right', 'up', 'down'";

}  // namespace refine
}  // namespace vs

using namespace vs;
using namespace vs::refine;

extern "C" {

int vs_fine_to_coarse(int dtype, const void* f_fine, int nxf, int nyf, void* f_coarse, int nxc, int nyc, int dir,
                      void* stream) {
  VS_REQUIRE(f_fine && f_coarse, "fine_to_coarse: null argument");
  VS_REQUIRE(dir >= VS_REFINE_LEFT && dir <= VS_REFINE_DOWN, "fine_to_coarse: dir must be one of %s", kDirNames);
  VS_REQUIRE(nxf >= 1 && nyf >= 1 && nxc >= 1 && nyc >= 1, "fine_to_coarse: empty block");
  const bool horiz = dir <= VS_REFINE_RIGHT;
  const int nf_normal = horiz ? nxf : nyf, m = horiz ? nyf : nxf;
  const int nc_normal = horiz ? nxc : nyc, c = horiz ? nyc : nxc;
  VS_REQUIRE(nf_normal >= 2, "fine_to_coarse: the fine block needs 2 nodes across the interface");
  Face F{};
  F.dir = dir;
  const bool low = dir == VS_REFINE_LEFT || dir == VS_REFINE_DOWN;  // fine rows 0, 1 (else -1, -2)
  F.row0 = low ? 0 : nf_normal - 1;
  F.row1 = low ? 1 : nf_normal - 2;
  // left / down write the coarse block's last line, right / up its first
  F.line = (dir == VS_REFINE_LEFT || dir == VS_REFINE_DOWN) ? nc_normal - 1 : 0;
  F.len_a = (m + 1) / 2;
  F.len_b = m / 2;
  F.len_v = bcast(F.len_a, F.len_b);
  VS_REQUIRE(F.len_v >= 0 && (F.len_v == c || F.len_v == 1),
             "fine_to_coarse: fine extent %d along the interface does not match coarse extent %d", m, c);
  F.n_out = c;
  const dim3 grid((c + 127) / 128, 3);
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_fine_to_coarse<T><<<grid, 128, 0, as_stream(stream)>>>((const T*)f_fine, nxf, nyf, (T*)f_coarse, nxc, nyc, F);
    VS_CHECK_LAUNCH("vs_fine_to_coarse");
    return VS_OK;
  });
}

int vs_coarse_to_fine(int dtype, const void* f_coarse, int nxc, int nyc, void* f_fine, int nxf, int nyf, int dir,
                      void* stream) {
  VS_REQUIRE(f_coarse && f_fine, "coarse_to_fine: null argument");
  VS_REQUIRE(dir >= VS_REFINE_LEFT && dir <= VS_REFINE_DOWN, "coarse_to_fine: dir must be one of %s", kDirNames);
  VS_REQUIRE(nxf >= 1 && nyf >= 1 && nxc >= 1 && nyc >= 1, "coarse_to_fine: empty block");
  const bool horiz = dir <= VS_REFINE_RIGHT;
  const int nf_normal = horiz ? nxf : nyf, m = horiz ? nyf : nxf;
  const int nc_normal = horiz ? nxc : nyc, c = horiz ? nyc : nxc;
  const int len_a = (m + 1) / 2, len_b = m / 2;
  VS_REQUIRE((c == len_a || c == 1) && (c == len_b || c == 1),
             "coarse_to_fine: coarse extent %d along the interface does not match fine extent %d", c, m);
  Face F{};
  F.dir = dir;
  // left / down write the fine block's last line from the coarse block's first; right / up
  // the fine block's first line from the coarse block's last
  const bool low = dir == VS_REFINE_LEFT || dir == VS_REFINE_DOWN;
  F.line = low ? nf_normal - 1 : 0;
  F.src_line = low ? 0 : nc_normal - 1;
  F.len_v = c;
  F.n_out = m;
  const dim3 grid((m + 127) / 128, 3);
  return dispatch_t(dtype, [&](auto t) -> int {
    using T = typename decltype(t)::type;
    k_coarse_to_fine<T><<<grid, 128, 0, as_stream(stream)>>>((const T*)f_coarse, nxc, nyc, (T*)f_fine, nxf, nyf, F);
    VS_CHECK_LAUNCH("vs_coarse_to_fine");
    return VS_OK;
  });
}

}  // extern "C"
