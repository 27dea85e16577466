// XLA FFI handlers over libvivsim_gb300: every per-operator entry point, their vector-
// Jacobian products and the fused multi-step run, as custom calls that a jax.jit-compiled
// update step calls through jax.ffi.ffi_call.
//
// Built by vivsim_gb300/jax_ffi.py where jaxlib is installed (its FFI headers come from
// jax.ffi.include_dir()).  Each handler reads the operand shapes and dtype, calls one C
// entry point on XLA's CUDA stream and turns a non-zero status into an FFI error carrying
// vs_last_error().  Shapes are the reference's: f (Q, NX, NY[, NZ]), rho (NX, NY[, NZ]),
// u (D, NX, NY[, NZ]), marker arrays (M, C), stencils W / I (M, S).  Scalars travel as
// attributes; matrices of the MRT operators as f64 array attributes (row-major Q x Q).
// Scratch (spread, MDF, the second population buffer of the fused run) comes from XLA's
// scratch allocator, so the handlers allocate nothing themselves.
#include <cuda_runtime_api.h>

#include <cstdint>
#include <cstring>
#include <optional>

#include "vivsim_gb300.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

using Buf = ffi::AnyBuffer;
using Out = ffi::Result<ffi::AnyBuffer>;
using Stream = cudaStream_t;

ffi::Error status(int rc) {
  if (rc == VS_OK) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInternal, vs_last_error());
}

ffi::Error bad(const char* msg) { return ffi::Error(ffi::ErrorCode::kInvalidArgument, msg); }

bool dtype_of(const Buf& b, int* dt) {
  if (b.element_type() == ffi::F32) *dt = VS_F32;
  else if (b.element_type() == ffi::F64) *dt = VS_F64;
  else return false;
  return true;
}

// populations (Q, NX, NY[, NZ]): q, grid extents (nz = 1 in 2-D) and the node count
bool grid_of(const Buf& f, int* q, int n3[3], int64_t* n) {
  const auto d = f.dimensions();
  if (d.size() != 3 && d.size() != 4) return false;
  *q = (int)d[0];
  if (!((*q == 9 && d.size() == 3) || (*q == 19 && d.size() == 4))) return false;
  n3[0] = (int)d[1];
  n3[1] = (int)d[2];
  n3[2] = d.size() == 4 ? (int)d[3] : 1;
  *n = (int64_t)n3[0] * n3[1] * n3[2];
  return true;
}

// a field (C, N...) on the grid: c and the node count
bool field_of(const Buf& g, int* c, int64_t* n) {
  const auto d = g.dimensions();
  if (d.size() < 2) return false;
  *c = (int)d[0];
  *n = 1;
  for (size_t k = 1; k < d.size(); ++k) *n *= d[k];
  return true;
}

// a (M, S) stencil
bool stencil_of(const Buf& W, const Buf& I, int* m, int* s) {
  const auto dw = W.dimensions(), di = I.dimensions();
  if (dw.size() != 2 || di.size() != 2 || dw[0] != di[0] || dw[1] != di[1]) return false;
  if (I.element_type() != ffi::S32) return false;
  *m = (int)dw[0];
  *s = (int)dw[1];
  return true;
}

int q_of_velocity(const Buf& u) { return u.dimensions()[0] == 2 ? 9 : 19; }

bool op_ok(ffi::Span<const double> op, int q) { return (int64_t)op.size() == (int64_t)q * q; }

// ------------------------------------------------------------------------ LBM ops

// streaming(f) — lbm/basic.py:60-85, lbm3d/basic.py:52-87
ffi::Error Streaming(Stream st, Buf f, Out out) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("streaming: f must be (9, NX, NY) or (19, NX, NY, NZ)");
  return status(vs_streaming(q, dt, f.untyped_data(), out->untyped_data(), n3[0], n3[1], n3[2], st));
}

// rho, u = get_macroscopic(f) — lbm/basic.py:88-111, lbm3d/basic.py:90-106
ffi::Error Macroscopic(Stream st, Buf f, Out rho, Out u) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("get_macroscopic: bad populations");
  return status(vs_get_macroscopic(q, dt, f.untyped_data(), rho->untyped_data(), u->untyped_data(), n, st));
}

// feq = get_equilibrium(rho, u) — lbm/basic.py:114-135, lbm3d/basic.py:109-130
ffi::Error Equilibrium(Stream st, Buf rho, Buf u, Out feq) {
  int dt;
  if (!dtype_of(rho, &dt)) return bad("get_equilibrium: rho must be float32 or float64");
  return status(vs_get_equilibrium(q_of_velocity(u), dt, rho.untyped_data(), u.untyped_data(), feq->untyped_data(),
                                   (int64_t)rho.element_count(), st));
}

// collision_bgk / collision_kbc / collision_reg (f, feq, omega); kind = VS_COLLIDE_*
ffi::Error Collision(Stream st, Buf f, Buf feq, Out out, int32_t kind, double omega) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("collision: bad populations");
  return status(vs_collision(q, dt, kind, f.untyped_data(), feq.untyped_data(), omega, out->untyped_data(), n, st));
}

// collision_mrt(f, feq, op) — lbm/collision/mrt.py:66-88, lbm3d/collision/mrt.py:88-98
ffi::Error CollisionMrt(Stream st, Buf f, Buf feq, Out out, ffi::Span<const double> op) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("collision_mrt: bad populations");
  if (!op_ok(op, q)) return bad("collision_mrt: op must hold q*q values");
  return status(vs_collision_mrt(q, dt, f.untyped_data(), feq.untyped_data(), op.begin(), out->untyped_data(), n, st));
}

// get_guo_forcing_term(g, u) — lbm/forcing/guo.py:6-35, lbm3d/forcing/guo.py:13-38
ffi::Error GuoForcingTerm(Stream st, Buf g, Buf u, Out out) {
  int c, dt;
  int64_t n;
  if (!field_of(u, &c, &n) || !dtype_of(u, &dt)) return bad("get_guo_forcing_term: bad velocity");
  return status(vs_guo_forcing_term(q_of_velocity(u), dt, g.untyped_data(), u.untyped_data(), out->untyped_data(), n,
                                    st));
}

// forcing_edm / forcing_guo_bgk (f, g, u[, omega]); kind = VS_FORCE_EDM / VS_FORCE_GUO_BGK
ffi::Error Forcing(Stream st, Buf f, Buf g, Buf u, Out out, int32_t kind, double omega) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("forcing: bad populations");
  return status(vs_forcing(q, dt, kind, f.untyped_data(), g.untyped_data(), u.untyped_data(), omega,
                           out->untyped_data(), n, st));
}

// forcing_guo_mrt(f, g, u, op) — lbm/forcing/guo.py:83-107, lbm3d/forcing/guo.py:71-87
ffi::Error ForcingGuoMrt(Stream st, Buf f, Buf g, Buf u, Out out, ffi::Span<const double> op) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("forcing_guo_mrt: bad populations");
  if (!op_ok(op, q)) return bad("forcing_guo_mrt: op must hold q*q values");
  return status(vs_forcing_guo_mrt(q, dt, f.untyped_data(), g.untyped_data(), u.untyped_data(), op.begin(),
                                   out->untyped_data(), n, st));
}

// get_velocity_correction(g, rho) — lbm/basic.py:175-194
ffi::Error VelocityCorrection(Stream st, Buf g, Buf rho, Out out) {
  int dt;
  if (!dtype_of(rho, &dt)) return bad("get_velocity_correction: bad rho");
  return status(vs_velocity_correction(q_of_velocity(g), dt, g.untyped_data(), rho.untyped_data(),
                                       out->untyped_data(), (int64_t)rho.element_count(), st));
}

// boundary_* with scalar wall values (the sources cited at vs_boundary).  f_before_stream
// is read only by bounce-back and specular reflection (pass f_in otherwise).
ffi::Error Boundary(Stream st, Buf f_in, Buf f_before, Out out, int32_t kind, int32_t mode, int32_t loc, double rho,
                    double ux, double uy, double uz, double gx, double gy, double gz) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f_in, &q, n3, &n) || !dtype_of(f_in, &dt)) return bad("boundary: bad populations");
  vs_wall w{};
  w.rho = rho;
  w.ux = ux;
  w.uy = uy;
  w.uz = uz;
  w.gx = gx;
  w.gy = gy;
  w.gz = gz;
  return status(vs_boundary(q, dt, kind, mode, loc, f_in.untyped_data(), out->untyped_data(),
                            f_before.untyped_data(), n3[0], n3[1], n3[2], &w, st));
}

// boundary_* with per-node wall arrays (the face's shape; rho, ux, uy, uz)
ffi::Error BoundaryArrays(Stream st, Buf f_in, Buf f_before, Buf rho_a, Buf ux_a, Buf uy_a, Buf uz_a, Out out,
                          int32_t kind, int32_t mode, int32_t loc, int32_t which) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f_in, &q, n3, &n) || !dtype_of(f_in, &dt)) return bad("boundary: bad populations");
  vs_wall w{};
  // which: bit 0 rho, bit 1 ux, bit 2 uy, bit 3 uz given per node
  w.rho_arr = (which & 1) ? rho_a.untyped_data() : nullptr;
  w.ux_arr = (which & 2) ? ux_a.untyped_data() : nullptr;
  w.uy_arr = (which & 4) ? uy_a.untyped_data() : nullptr;
  w.uz_arr = (which & 8) ? uz_a.untyped_data() : nullptr;
  return status(vs_boundary(q, dt, kind, mode, loc, f_in.untyped_data(), out->untyped_data(),
                            f_before.untyped_data(), n3[0], n3[1], n3[2], &w, st));
}

// obstacle_bounce_back(f, mask) — lbm/boundary/bb.py:98-110, lbm3d/boundary/bb.py:56-59
ffi::Error ObstacleBounceBack(Stream st, Buf f, Buf mask, Out out) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("obstacle_bounce_back: bad populations");
  if (mask.element_type() != ffi::PRED && mask.element_type() != ffi::U8 && mask.element_type() != ffi::S8)
    return bad("obstacle_bounce_back: mask must be bool or 8-bit");
  return status(vs_obstacle_bounce_back(q, dt, f.untyped_data(), out->untyped_data(),
                                        (const uint8_t*)mask.untyped_data(), n, st));
}

// boundary_characteristic(rho, u, loc) — lbm/boundary/cbc.py:14-53, lbm3d/boundary/cbc.py:16-51
ffi::Error Characteristic(Stream st, Buf rho, Buf u, Out rho_next, Out u_next, int32_t loc) {
  int dt;
  if (!dtype_of(rho, &dt)) return bad("boundary_characteristic: bad rho");
  const auto d = rho.dimensions();
  const int nx = (int)d[0], ny = (int)d[1], nz = d.size() == 3 ? (int)d[2] : 1;
  return status(vs_boundary_characteristic(q_of_velocity(u), dt, loc, rho.untyped_data(), u.untyped_data(), nx, ny,
                                           nz, rho_next->untyped_data(), u_next->untyped_data(), st));
}

// -------------------------------------------------------------------------- IB ops

// kernel_peskin_3pt / _4pt / kernel_cosine_4pt — ib/kernels.py:4-61
ffi::Error IbKernel(Stream st, Buf r, Out out, int32_t kernel) {
  int dt;
  if (!dtype_of(r, &dt)) return bad("ib kernel: bad input");
  return status(vs_ib_kernel(kernel, dt, r.untyped_data(), out->untyped_data(), (int64_t)r.element_count(), st));
}

// get_ib_stencil(x, y, ny, kernel, radius) — ib/stencil.py:7-51
ffi::Error IbStencil2d(Stream st, Buf x, Buf y, Out W, Out I, int32_t kernel, int32_t radius, int32_t ny) {
  int dt;
  if (!dtype_of(x, &dt)) return bad("get_ib_stencil: bad coordinates");
  return status(vs_ib_stencil_2d(kernel, radius, dt, x.untyped_data(), y.untyped_data(), (int)x.element_count(), ny,
                                 W->untyped_data(), (int32_t*)I->untyped_data(), st));
}

// ib3d.get_ib_stencil(coords (M, 3), shape, kernel, radius) — ib3d/stencil.py:7-59
ffi::Error IbStencil3d(Stream st, Buf coords, Out W, Out I, int32_t kernel, int32_t radius, int32_t nx, int32_t ny,
                       int32_t nz) {
  int dt;
  if (!dtype_of(coords, &dt)) return bad("get_ib_stencil: bad coordinates");
  return status(vs_ib_stencil_3d(kernel, radius, dt, coords.untyped_data(), (int)coords.dimensions()[0], nx, ny, nz,
                                 W->untyped_data(), (int32_t*)I->untyped_data(), st));
}

// interpolate(grid (C, N...), W, I) -> (M, C) — ib/stencil.py:54-78
ffi::Error Interpolate(Stream st, Buf grid, Buf W, Buf I, Out out) {
  int c, m, s, dt;
  int64_t n;
  if (!field_of(grid, &c, &n) || !dtype_of(grid, &dt) || !stencil_of(W, I, &m, &s)) return bad("interpolate: bad operands");
  return status(vs_ib_interpolate(dt, grid.untyped_data(), c, n, W.untyped_data(), (const int32_t*)I.untyped_data(),
                                  m, s, out->untyped_data(), st));
}

// spread(values (M, C), grid (C, N...), W, I) — ib/stencil.py:81-110 (deterministic)
ffi::Error Spread(Stream st, ffi::ScratchAllocator scratch, Buf values, Buf grid, Buf W, Buf I, Out out) {
  int c, m, s, dt;
  int64_t n;
  if (!field_of(grid, &c, &n) || !dtype_of(grid, &dt) || !stencil_of(W, I, &m, &s)) return bad("spread: bad operands");
  const size_t ws = vs_ib_workspace_bytes(m, s);
  std::optional<void*> mem = scratch.Allocate(ws, 256);
  if (!mem.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "spread: no scratch");
  return status(vs_ib_spread(dt, values.untyped_data(), grid.untyped_data(), out->untyped_data(), c, n,
                             W.untyped_data(), (const int32_t*)I.untyped_data(), m, s, *mem, ws, st));
}

// multi_direct_forcing(u, W, I, u_target, ds, n_iter) — ib/mdf.py:10-64; ds (M,) or a
// scalar attribute (per_marker_ds = 0)
ffi::Error Mdf(Stream st, ffi::ScratchAllocator scratch, Buf u, Buf W, Buf I, Buf target, Buf ds, Out g, Out mf,
               int32_t n_iter, int32_t per_marker_ds, double ds_scalar) {
  int c, m, s, dt;
  int64_t n;
  if (!field_of(u, &c, &n) || !dtype_of(u, &dt) || !stencil_of(W, I, &m, &s)) return bad("multi_direct_forcing: bad operands");
  const size_t ws = vs_ib_workspace_bytes(m, s);
  std::optional<void*> mem = scratch.Allocate(ws, 256);
  if (!mem.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "multi_direct_forcing: no scratch");
  return status(vs_ib_mdf(dt, u.untyped_data(), c, n, W.untyped_data(), (const int32_t*)I.untyped_data(), m, s,
                          target.untyped_data(), per_marker_ds ? ds.untyped_data() : nullptr, ds_scalar, n_iter,
                          g->untyped_data(), mf->untyped_data(), *mem, ws, st));
}

// ----------------------------------------------------------------------- dynamics

// newmark(a, v, d, h, m, k, c) scalar branch — dyn.py:42-45
ffi::Error Newmark(Stream st, Buf a, Buf v, Buf d, Buf h, Out an, Out vn, Out dn, double m, double k, double c,
                   double dt_, double gamma, double beta) {
  int dt;
  if (!dtype_of(a, &dt)) return bad("newmark: bad state");
  return status(vs_newmark(dt, (int)a.element_count(), a.untyped_data(), v.untyped_data(), d.untyped_data(),
                           h.untyped_data(), m, k, c, nullptr, nullptr, nullptr, dt_, gamma, beta, an->untyped_data(),
                           vn->untyped_data(), dn->untyped_data(), st));
}

// newmark matrix branch (M, K, C as ndof x ndof device matrices) — dyn.py:36-41
ffi::Error NewmarkMatrix(Stream st, Buf a, Buf v, Buf d, Buf h, Buf Mm, Buf Km, Buf Cm, Out an, Out vn, Out dn,
                         double dt_, double gamma, double beta) {
  int dt;
  if (!dtype_of(a, &dt)) return bad("newmark: bad state");
  return status(vs_newmark(dt, (int)a.element_count(), a.untyped_data(), v.untyped_data(), d.untyped_data(),
                           h.untyped_data(), 0.0, 0.0, 0.0, Mm.untyped_data(), Km.untyped_data(), Cm.untyped_data(),
                           dt_, gamma, beta, an->untyped_data(), vn->untyped_data(), dn->untyped_data(), st));
}

// get_force_to_obj(h (M, C)) — dyn.py:126-136
ffi::Error ForceToObj(Stream st, Buf h, Out out) {
  int dt;
  if (!dtype_of(h, &dt)) return bad("get_force_to_obj: bad forces");
  const auto dd = h.dimensions();
  return status(vs_force_to_obj(dt, h.untyped_data(), (int)dd[0], (int)dd[1], out->untyped_data(), st));
}

// ----------------------------------------------------------------------- fused run

// n_steps fused steps of a lattice plan (and body plan) created by the library; f is
// donated (input_output_aliases {0: 0}); the other ping-pong buffer is scratch.
ffi::Error Run(Stream st, ffi::ScratchAllocator scratch, Buf f, Out out, Out hist, int64_t lattice, int64_t body,
               int32_t n_steps) {
  if (!lattice) return bad("run: no lattice plan");
  if (n_steps < 0) return bad("run: negative step count");
  const size_t bytes = f.size_bytes();
  void* fa = out->untyped_data();
  if (fa != f.untyped_data()) {
    cudaError_t e = cudaMemcpyAsync(fa, f.untyped_data(), bytes, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return ffi::Error(ffi::ErrorCode::kInternal, cudaGetErrorString(e));
  }
  std::optional<void*> fb = scratch.Allocate(bytes, 256);
  if (!fb.has_value()) return ffi::Error(ffi::ErrorCode::kResourceExhausted, "run: no scratch");
  int rc = vs_run((const vs_lattice_plan*)(intptr_t)lattice, (vs_body_plan*)(intptr_t)body, fa, *fb, n_steps,
                  hist->element_count() ? hist->untyped_data() : nullptr, st);
  if (rc) return status(rc);
  if (n_steps % 2) {
    cudaError_t e = cudaMemcpyAsync(fa, *fb, bytes, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return ffi::Error(ffi::ErrorCode::kInternal, cudaGetErrorString(e));
  }
  return ffi::Error::Success();
}

// -------------------------------------------------------------------- VJP handlers

ffi::Error StreamingVjp(Stream st, Buf g_out, Out g_in) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(g_out, &q, n3, &n) || !dtype_of(g_out, &dt)) return bad("streaming_vjp: bad cotangent");
  return status(vs_streaming_vjp(q, dt, g_out.untyped_data(), g_in->untyped_data(), n3[0], n3[1], n3[2], st));
}

ffi::Error MacroscopicVjp(Stream st, Buf f, Buf g_rho, Buf g_u, Out g_f) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("get_macroscopic_vjp: bad populations");
  return status(vs_macroscopic_vjp(q, dt, f.untyped_data(), g_rho.untyped_data(), g_u.untyped_data(),
                                   g_f->untyped_data(), n, st));
}

ffi::Error EquilibriumVjp(Stream st, Buf rho, Buf u, Buf g_feq, Out g_rho, Out g_u) {
  int dt;
  if (!dtype_of(rho, &dt)) return bad("get_equilibrium_vjp: bad rho");
  return status(vs_equilibrium_vjp(q_of_velocity(u), dt, rho.untyped_data(), u.untyped_data(), g_feq.untyped_data(),
                                   g_rho->untyped_data(), g_u->untyped_data(), (int64_t)rho.element_count(), st));
}

// g_omega_node: one share per node; their sum is the cotangent of omega
ffi::Error CollisionVjp(Stream st, Buf f, Buf feq, Buf g_out, Out g_f, Out g_feq, Out g_omega_node, int32_t kind,
                        double omega) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("collision_vjp: bad populations");
  return status(vs_collision_vjp(q, dt, kind, f.untyped_data(), feq.untyped_data(), omega, g_out.untyped_data(),
                                 g_f->untyped_data(), g_feq->untyped_data(), g_omega_node->untyped_data(), n, st));
}

ffi::Error CollisionMrtVjp(Stream st, Buf f, Buf feq, Buf g_out, Out g_f, Out g_feq, Out g_op,
                           ffi::Span<const double> op) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("collision_mrt_vjp: bad populations");
  if (!op_ok(op, q)) return bad("collision_mrt_vjp: op must hold q*q values");
  if (g_op->element_type() != ffi::F64) return bad("collision_mrt_vjp: g_op is float64");
  return status(vs_collision_mrt_vjp(q, dt, f.untyped_data(), feq.untyped_data(), op.begin(), g_out.untyped_data(),
                                     g_f->untyped_data(), g_feq->untyped_data(), (double*)g_op->untyped_data(), n,
                                     st));
}

// g_scale_node: per node g_out . guo (the Guo-BGK omega cotangent is -1/2 of its sum)
ffi::Error ForcingVjp(Stream st, Buf g, Buf u, Buf g_out, Out g_g, Out g_u, Out g_scale_node, int32_t kind,
                      double omega) {
  int c, dt;
  int64_t n;
  if (!field_of(u, &c, &n) || !dtype_of(u, &dt)) return bad("forcing_vjp: bad velocity");
  return status(vs_forcing_vjp(q_of_velocity(u), dt, kind, g.untyped_data(), u.untyped_data(), omega,
                               g_out.untyped_data(), nullptr, g_g->untyped_data(), g_u->untyped_data(),
                               g_scale_node->untyped_data(), n, st));
}

// g_wall_node: 4 shares per face node (rho, ux, uy, uz wall values)
ffi::Error BoundaryVjp(Stream st, Buf f_in, Buf f_before, Buf g_out, Out g_in, Out g_before, Out g_wall_node,
                       int32_t kind, int32_t mode, int32_t loc, double rho, double ux, double uy, double uz) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f_in, &q, n3, &n) || !dtype_of(f_in, &dt)) return bad("boundary_vjp: bad populations");
  return status(vs_boundary_vjp(q, dt, kind, mode, loc, f_in.untyped_data(), f_before.untyped_data(),
                                g_out.untyped_data(), g_in->untyped_data(), g_before->untyped_data(),
                                g_wall_node->untyped_data(), n3[0], n3[1], n3[2], rho, ux, uy, uz, st));
}

// out[m, s] = sum_c A[m, c] grid[c, I[m, s]] (the stencil weights' cotangent)
ffi::Error IbPairDot(Stream st, Buf A, Buf grid, Buf I, Out out) {
  int c, dt;
  int64_t n;
  if (!field_of(grid, &c, &n) || !dtype_of(grid, &dt)) return bad("ib_pair_dot: bad field");
  const auto di = I.dimensions();
  if (di.size() != 2) return bad("ib_pair_dot: I must be (M, S)");
  return status(vs_ib_pair_dot(dt, A.untyped_data(), grid.untyped_data(), c, n, (const int32_t*)I.untyped_data(),
                               (int)di[0], (int)di[1], out->untyped_data(), st));
}

ffi::Error IbStencilVjp2d(Stream st, Buf x, Buf y, Buf g_W, Out g_x, Out g_y, int32_t kernel, int32_t radius) {
  int dt;
  if (!dtype_of(x, &dt)) return bad("get_ib_stencil_vjp: bad coordinates");
  return status(vs_ib_stencil_vjp(kernel, radius, dt, 2, x.untyped_data(), y.untyped_data(), nullptr,
                                  g_W.untyped_data(), g_x->untyped_data(), g_y->untyped_data(), nullptr,
                                  (int)x.element_count(), st));
}

ffi::Error IbStencilVjp3d(Stream st, Buf x, Buf y, Buf z, Buf g_W, Out g_x, Out g_y, Out g_z, int32_t kernel,
                          int32_t radius) {
  int dt;
  if (!dtype_of(x, &dt)) return bad("get_ib_stencil_vjp: bad coordinates");
  return status(vs_ib_stencil_vjp(kernel, radius, dt, 3, x.untyped_data(), y.untyped_data(), z.untyped_data(),
                                  g_W.untyped_data(), g_x->untyped_data(), g_y->untyped_data(), g_z->untyped_data(),
                                  (int)x.element_count(), st));
}

// scalar-branch Newmark VJP; g_mkc: cotangents of m, k, c
ffi::Error NewmarkVjp(Stream st, Buf a, Buf v, Buf d, Buf h, Buf ga_n, Buf gv_n, Buf gd_n, Out g_a, Out g_v, Out g_d,
                      Out g_h, Out g_mkc, double m, double k, double c, double dt_, double gamma, double beta) {
  int dt;
  if (!dtype_of(a, &dt)) return bad("newmark_vjp: bad state");
  return status(vs_newmark_vjp(dt, (int)a.element_count(), a.untyped_data(), v.untyped_data(), d.untyped_data(),
                               h.untyped_data(), m, k, c, nullptr, nullptr, nullptr, dt_, gamma, beta,
                               ga_n.untyped_data(), gv_n.untyped_data(), gd_n.untyped_data(), g_a->untyped_data(),
                               g_v->untyped_data(), g_d->untyped_data(), g_h->untyped_data(), g_mkc->untyped_data(),
                               nullptr, st));
}

}  // namespace

#define VS_CTX ffi::Ffi::Bind().Ctx<ffi::PlatformStream<cudaStream_t>>()
#define VS_CTX_SCRATCH VS_CTX.Ctx<ffi::ScratchAllocator>()

XLA_FFI_DEFINE_HANDLER_SYMBOL(VsStreaming, Streaming, VS_CTX.Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsMacroscopic, Macroscopic, VS_CTX.Arg<Buf>().Ret<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsEquilibrium, Equilibrium, VS_CTX.Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsCollision, Collision,
                              VS_CTX.Arg<Buf>().Arg<Buf>().Ret<Buf>().Attr<int32_t>("kind").Attr<double>("omega"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsCollisionMrt, CollisionMrt,
                              VS_CTX.Arg<Buf>().Arg<Buf>().Ret<Buf>().Attr<ffi::Span<const double>>("op"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsGuoForcingTerm, GuoForcingTerm, VS_CTX.Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsForcing, Forcing,
                              VS_CTX.Arg<Buf>().Arg<Buf>().Arg<Buf>().Ret<Buf>().Attr<int32_t>("kind").Attr<double>(
                                  "omega"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsForcingGuoMrt, ForcingGuoMrt,
                              VS_CTX.Arg<Buf>().Arg<Buf>().Arg<Buf>().Ret<Buf>().Attr<ffi::Span<const double>>("op"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsVelocityCorrection, VelocityCorrection, VS_CTX.Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsBoundary, Boundary,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kind")
                                  .Attr<int32_t>("mode")
                                  .Attr<int32_t>("loc")
                                  .Attr<double>("rho")
                                  .Attr<double>("ux")
                                  .Attr<double>("uy")
                                  .Attr<double>("uz")
                                  .Attr<double>("gx")
                                  .Attr<double>("gy")
                                  .Attr<double>("gz"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsBoundaryArrays, BoundaryArrays,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kind")
                                  .Attr<int32_t>("mode")
                                  .Attr<int32_t>("loc")
                                  .Attr<int32_t>("which"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsObstacleBounceBack, ObstacleBounceBack, VS_CTX.Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsCharacteristic, Characteristic,
                              VS_CTX.Arg<Buf>().Arg<Buf>().Ret<Buf>().Ret<Buf>().Attr<int32_t>("loc"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsIbKernel, IbKernel, VS_CTX.Arg<Buf>().Ret<Buf>().Attr<int32_t>("kernel"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsIbStencil2d, IbStencil2d,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kernel")
                                  .Attr<int32_t>("radius")
                                  .Attr<int32_t>("ny"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsIbStencil3d, IbStencil3d,
                              VS_CTX.Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kernel")
                                  .Attr<int32_t>("radius")
                                  .Attr<int32_t>("nx")
                                  .Attr<int32_t>("ny")
                                  .Attr<int32_t>("nz"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsInterpolate, Interpolate, VS_CTX.Arg<Buf>().Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsSpread, Spread, VS_CTX_SCRATCH.Arg<Buf>().Arg<Buf>().Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsMdf, Mdf,
                              VS_CTX_SCRATCH.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("n_iter")
                                  .Attr<int32_t>("per_marker_ds")
                                  .Attr<double>("ds"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsNewmark, Newmark,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<double>("m")
                                  .Attr<double>("k")
                                  .Attr<double>("c")
                                  .Attr<double>("dt")
                                  .Attr<double>("gamma")
                                  .Attr<double>("beta"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsNewmarkMatrix, NewmarkMatrix,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<double>("dt")
                                  .Attr<double>("gamma")
                                  .Attr<double>("beta"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsForceToObj, ForceToObj, VS_CTX.Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsRun, Run,
                              VS_CTX_SCRATCH.Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int64_t>("lattice")
                                  .Attr<int64_t>("body")
                                  .Attr<int32_t>("n_steps"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsStreamingVjp, StreamingVjp, VS_CTX.Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsMacroscopicVjp, MacroscopicVjp, VS_CTX.Arg<Buf>().Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsEquilibriumVjp, EquilibriumVjp,
                              VS_CTX.Arg<Buf>().Arg<Buf>().Arg<Buf>().Ret<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsCollisionVjp, CollisionVjp,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kind")
                                  .Attr<double>("omega"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsCollisionMrtVjp, CollisionMrtVjp,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<ffi::Span<const double>>("op"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsForcingVjp, ForcingVjp,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kind")
                                  .Attr<double>("omega"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsBoundaryVjp, BoundaryVjp,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kind")
                                  .Attr<int32_t>("mode")
                                  .Attr<int32_t>("loc")
                                  .Attr<double>("rho")
                                  .Attr<double>("ux")
                                  .Attr<double>("uy")
                                  .Attr<double>("uz"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsIbPairDot, IbPairDot, VS_CTX.Arg<Buf>().Arg<Buf>().Arg<Buf>().Ret<Buf>());
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsIbStencilVjp2d, IbStencilVjp2d,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kernel")
                                  .Attr<int32_t>("radius"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsIbStencilVjp3d, IbStencilVjp3d,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<int32_t>("kernel")
                                  .Attr<int32_t>("radius"));
XLA_FFI_DEFINE_HANDLER_SYMBOL(VsNewmarkVjp, NewmarkVjp,
                              VS_CTX.Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Arg<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Ret<Buf>()
                                  .Attr<double>("m")
                                  .Attr<double>("k")
                                  .Attr<double>("c")
                                  .Attr<double>("dt")
                                  .Attr<double>("gamma")
                                  .Attr<double>("beta"));
