// XLA FFI handlers over libvivsim_gb300: the per-operator entry points as custom calls
// that a jax.jit-compiled update step calls through jax.ffi.ffi_call.
//
// Built by vivsim_gb300/jax_ffi.py only where jaxlib is installed (its FFI headers come from
// jax.ffi.include_dir()).  Each handler reads the operand shapes and dtype, calls one C
// entry point on XLA's CUDA stream and turns a non-zero status into an FFI error carrying
// vs_last_error().  Shapes are the reference's: f (Q, NX, NY[, NZ]), rho (NX, NY[, NZ]),
// u (D, NX, NY[, NZ]).
#include <cuda_runtime_api.h>

#include <cstdint>

#include "vivsim_gb300.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status(int rc) {
  if (rc == VS_OK) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInternal, vs_last_error());
}

bool dtype_of(const ffi::AnyBuffer& b, int* dt) {
  if (b.element_type() == ffi::F32) *dt = VS_F32;
  else if (b.element_type() == ffi::F64) *dt = VS_F64;
  else return false;
  return true;
}

ffi::Error bad(const char* msg) { return ffi::Error(ffi::ErrorCode::kInvalidArgument, msg); }

// populations (Q, NX, NY[, NZ]): q, grid extents (nz = 1 in 2-D) and the node count
bool grid_of(const ffi::AnyBuffer& f, int* q, int n3[3], int64_t* n) {
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

// streaming(f) — lbm/basic.py:60-85, lbm3d/basic.py:52-87
ffi::Error Streaming(cudaStream_t st, ffi::AnyBuffer f, ffi::Result<ffi::AnyBuffer> out) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("streaming: f must be (9, NX, NY) or (19, NX, NY, NZ)");
  return status(vs_streaming(q, dt, f.untyped_data(), out->untyped_data(), n3[0], n3[1], n3[2], st));
}

// rho, u = get_macroscopic(f) — lbm/basic.py:88-111, lbm3d/basic.py:90-106
ffi::Error Macroscopic(cudaStream_t st, ffi::AnyBuffer f, ffi::Result<ffi::AnyBuffer> rho,
                       ffi::Result<ffi::AnyBuffer> u) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("get_macroscopic: bad populations");
  return status(vs_get_macroscopic(q, dt, f.untyped_data(), rho->untyped_data(), u->untyped_data(), n, st));
}

// feq = get_equilibrium(rho, u) — lbm/basic.py:114-135, lbm3d/basic.py:109-130
ffi::Error Equilibrium(cudaStream_t st, ffi::AnyBuffer rho, ffi::AnyBuffer u, ffi::Result<ffi::AnyBuffer> feq) {
  int dt;
  if (!dtype_of(rho, &dt)) return bad("get_equilibrium: rho must be float32 or float64");
  const int q = u.dimensions()[0] == 2 ? 9 : 19;
  return status(vs_get_equilibrium(q, dt, rho.untyped_data(), u.untyped_data(), feq->untyped_data(),
                                   (int64_t)rho.element_count(), st));
}

// collision_bgk / collision_kbc / collision_reg (f, feq, omega); kind = VS_COLLIDE_*
ffi::Error Collision(cudaStream_t st, ffi::AnyBuffer f, ffi::AnyBuffer feq, ffi::Result<ffi::AnyBuffer> out,
                     int32_t kind, double omega) {
  int q, n3[3], dt;
  int64_t n;
  if (!grid_of(f, &q, n3, &n) || !dtype_of(f, &dt)) return bad("collision: bad populations");
  return status(vs_collision(q, dt, kind, f.untyped_data(), feq.untyped_data(), omega, out->untyped_data(), n, st));
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(VsStreaming, Streaming,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::AnyBuffer>()
                                  .Ret<ffi::AnyBuffer>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(VsMacroscopic, Macroscopic,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::AnyBuffer>()
                                  .Ret<ffi::AnyBuffer>()
                                  .Ret<ffi::AnyBuffer>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(VsEquilibrium, Equilibrium,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::AnyBuffer>()
                                  .Arg<ffi::AnyBuffer>()
                                  .Ret<ffi::AnyBuffer>());

XLA_FFI_DEFINE_HANDLER_SYMBOL(VsCollision, Collision,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::AnyBuffer>()
                                  .Arg<ffi::AnyBuffer>()
                                  .Ret<ffi::AnyBuffer>()
                                  .Attr<int32_t>("kind")
                                  .Attr<double>("omega"));
