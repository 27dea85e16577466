/*
 * vivsim_gb300 — C ABI of the GB300 (sm_103a) IB-LBM kernels.
 *
 * Each entry point replaces one pure function of the reference library haimingz/vivsim
 * (cited as path:line inside that project) or a composed step of it.  Conventions:
 *
 *   - every function returns an int status (VS_OK = 0); the message of the last failure
 *     on the calling thread is available from vs_last_error();
 *   - all array arguments are DEVICE pointers unless named *_host; the caller owns them;
 *   - arrays are C-order, structure of arrays: populations f[q][x][y] (D2Q9) and
 *     f[q][x][y][z] (D3Q19), velocities u[d][...], marker arrays [marker][component];
 *   - dtype selects float (VS_F32) or double (VS_F64) for every floating array of a call;
 *   - `stream` is a cudaStream_t (0 = legacy default stream); work is enqueued, not
 *     synchronised, exactly like a JAX/XLA custom call or a PyTorch op;
 *   - unless stated otherwise `out` may not alias an input.
 */
#ifndef VIVSIM_GB300_H
#define VIVSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ constants */
enum {
  VS_OK = 0,
  VS_ERR_INVALID_ARG = 1, /* bad shape, enum, pointer or size                      */
  VS_ERR_CUDA = 2,        /* a CUDA runtime call failed                            */
  VS_ERR_UNSUPPORTED = 3, /* valid request this build does not implement           */
  VS_ERR_RANGE = 4,       /* a stencil index / window fell outside its grid        */
  VS_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up                    */
  VS_ERR_NONFINITE = 6,   /* the NaN/Inf watchdog saw a non-finite population      */
  VS_ERR_TIMEOUT_INFLIGHT = 7 /* a wait gave up and a bulk copy it waited for had not
                               * landed by the end of a second bounded wait: the copy may
                               * write shared memory after its block left, so device state
                               * is not to be trusted (start a new context)              */
};
enum { VS_F32 = 0, VS_F64 = 1 };
enum { VS_COLLIDE_BGK = 0, VS_COLLIDE_KBC = 1, VS_COLLIDE_MRT = 2, VS_COLLIDE_REG = 3 };
enum { VS_FORCE_NONE = 0, VS_FORCE_EDM = 1, VS_FORCE_GUO_BGK = 2, VS_FORCE_GUO_MRT = 3 };
/* face locations; D2Q9 uses the first four (left/right: x = 0 / NX-1, bottom/top: y = 0 / NY-1) */
enum { VS_LEFT = 0, VS_RIGHT = 1, VS_BOTTOM = 2, VS_TOP = 3, VS_BACK = 4, VS_FRONT = 5 };
/* boundary schemes */
enum { VS_BC_NEE = 0, VS_BC_NEBB = 1, VS_BC_EQ = 2, VS_BC_BB = 3, VS_BC_SPECULAR = 4 };
/* how the wall state is completed (lbm/boundary/_helpers.py:175-239 wrappers) */
enum {
  VS_WALL_GIVEN = 0,          /* rho_wall and u_wall given                          */
  VS_WALL_VELOCITY = 1,       /* u_wall given, rho_wall recovered (wrap_velocity)    */
  VS_WALL_PRESSURE = 2,       /* rho_wall given, u_wall recovered (wrap_pressure)    */
  VS_WALL_FORCE_CORRECTED = 3, /* u_wall shifted by -g/(2 rho) (wrap_force_corrected) */
  VS_WALL_CHARACTERISTIC = 4   /* fused step only: rho_wall and u_wall per face node from
                                  boundary_characteristic (lbm/boundary/cbc.py:14-53,
                                  lbm3d/boundary/cbc.py:16-51) of the step's input moments
                                  at the wall and the next two planes; kind NEE, NEBB or EQ
                                  then imposes them after streaming (a non-reflective
                                  outflow) */
};
/* 1-D discrete delta kernels, vivsim/ib/kernels.py */
enum { VS_KERNEL_PESKIN3 = 0, VS_KERNEL_PESKIN4 = 1, VS_KERNEL_COSINE4 = 2 };

const char* vs_last_error(void);
const char* vs_status_string(int status);
int vs_version(void);

/* ===================================================================== LBM ops ===
 * q = 9 (D2Q9, vivsim/lbm) or 19 (D3Q19, vivsim/lbm3d); n = number of nodes.      */

/* periodic streaming — lbm/basic.py:60-85, lbm3d/basic.py:52-87 (nz = 1 for D2Q9) */
int vs_streaming(int q, int dtype, const void* f, void* out, int nx, int ny, int nz, void* stream);
/* rho, u = get_macroscopic(f) — lbm/basic.py:88-111, lbm3d/basic.py:90-106 */
int vs_get_macroscopic(int q, int dtype, const void* f, void* rho, void* u, int64_t n, void* stream);
/* feq = get_equilibrium(rho, u) — lbm/basic.py:114-135, lbm3d/basic.py:109-130 */
int vs_get_equilibrium(int q, int dtype, const void* rho, const void* u, void* feq, int64_t n, void* stream);
/* collision_bgk / collision_kbc / collision_reg (f, feq, omega)
 *   lbm/basic.py:138-156, lbm/collision/kbc.py:10-60, lbm/collision/reg.py:4-49,
 *   lbm3d/basic.py:133-146, lbm3d/collision/kbc.py:8-42, lbm3d/collision/reg.py:44-62 */
int vs_collision(int q, int dtype, int kind, const void* f, const void* feq, double omega, void* out,
                 int64_t n, void* stream);
/* collision_mrt(f, feq, op) with a q*q row-major host operator — lbm/collision/mrt.py:66-88,
 * lbm3d/collision/mrt.py:88-98 */
int vs_collision_mrt(int q, int dtype, const void* f, const void* feq, const double* op_host, void* out,
                     int64_t n, void* stream);
/* get_guo_forcing_term(g, u) — lbm/forcing/guo.py:6-35, lbm3d/forcing/guo.py:13-38 */
int vs_guo_forcing_term(int q, int dtype, const void* g, const void* u, void* out, int64_t n, void* stream);
/* forcing_edm / forcing_guo_bgk: out = f + scale * guo(g, u) with scale 1 (edm.py:4-31)
 * or 1 - omega/2 (guo.py:38-59); pass kind = VS_FORCE_EDM or VS_FORCE_GUO_BGK */
int vs_forcing(int q, int dtype, int kind, const void* f, const void* g, const void* u, double omega, void* out,
               int64_t n, void* stream);
/* forcing_guo_mrt(f, g, u, op) — lbm/forcing/guo.py:83-107, lbm3d/forcing/guo.py:71-87 */
int vs_forcing_guo_mrt(int q, int dtype, const void* f, const void* g, const void* u, const double* op_host,
                       void* out, int64_t n, void* stream);
/* get_velocity_correction(g, rho) = g * 0.5 / rho, g of shape (d, n) — lbm/basic.py:175-194 */
int vs_velocity_correction(int q, int dtype, const void* g, const void* rho, void* out, int64_t n, void* stream);

/* Wall data for one boundary call.  Scalars are used where the matching device array
 * pointer is NULL; arrays have the face's shape (N for D2Q9, the 2-D face for D3Q19). */
typedef struct vs_wall {
  double rho, ux, uy, uz, gx, gy, gz;
  const void* rho_arr;
  const void* ux_arr;
  const void* uy_arr;
  const void* uz_arr;
} vs_wall;

/* boundary_{nee,nebb,equilibrium,bounce_back,specular_reflection} and their velocity /
 * pressure / force-corrected wrappers: f_out = f_in with the face at `loc` rewritten.
 *   lbm/boundary/{nee.py:19-65, nebb.py:20-62, eq.py:25-61, bb.py:15-95, _helpers.py:50-239}
 *   lbm3d/boundary/{nee.py:13-37, nebb.py:13-37, eq.py:13-31, bb.py:8-53, _helpers.py:9-133}
 * f_before_stream is required for VS_BC_BB / VS_BC_SPECULAR, ignored otherwise.
 * f_out may equal f_in (in-place update of the face only). */
int vs_boundary(int q, int dtype, int kind, int mode, int loc, const void* f_in, void* f_out,
                const void* f_before_stream, int nx, int ny, int nz, const vs_wall* wall, void* stream);
/* obstacle_bounce_back(f, mask), mask one byte per node — lbm/boundary/bb.py:98-110, lbm3d/boundary/bb.py:56-59 */
int vs_obstacle_bounce_back(int q, int dtype, const void* f_in, void* f_out, const uint8_t* mask, int64_t n,
                            void* stream);
/* boundary_characteristic(rho, u, loc) -> rho_next (face), u_next (d, face)
 *   lbm/boundary/cbc.py:14-53, lbm3d/boundary/cbc.py:16-51 */
int vs_boundary_characteristic(int q, int dtype, int loc, const void* rho, const void* u, int nx, int ny, int nz,
                               void* rho_next, void* u_next, void* stream);

/* ====================================================================== IB ops === */

/* kernel_peskin_3pt / kernel_peskin_4pt / kernel_cosine_4pt — ib/kernels.py:4-61 */
int vs_ib_kernel(int kernel, int dtype, const void* r, void* out, int64_t n, void* stream);
/* get_ib_stencil(marker_x, marker_y, ny, kernel, radius) -> W (m, (2r)^2), I int32 — ib/stencil.py:7-51 */
int vs_ib_stencil_2d(int kernel, int radius, int dtype, const void* marker_x, const void* marker_y, int m,
                     int ny, void* W, int32_t* I, void* stream);
/* ib3d.get_ib_stencil(coords (m,3), (nx,ny,nz), kernel, radius) -> W (m, (2r)^3), I — ib3d/stencil.py:7-59 */
int vs_ib_stencil_3d(int kernel, int radius, int dtype, const void* coords, int m, int nx, int ny, int nz,
                     void* W, int32_t* I, void* stream);
/* interpolate(grid (c, n_grid), W (m,s), I (m,s)) -> (m, c) — ib/stencil.py:54-78 */
int vs_ib_interpolate(int dtype, const void* grid, int c, int64_t n_grid, const void* W, const int32_t* I, int m,
                      int s, void* out, void* stream);
/* Scratch bytes for vs_ib_spread / vs_ib_mdf with m markers of s stencil points. */
size_t vs_ib_workspace_bytes(int m, int s);
/* spread(marker_values (m,c), grid_in (c,n_grid), W, I) -> grid_out — ib/stencil.py:81-110.
 * Deterministic: contributions to a node are summed in (marker, stencil point) order,
 * the order of the reference's scatter-add; no floating-point atomics.  grid_out may
 * equal grid_in. */
int vs_ib_spread(int dtype, const void* marker_values, const void* grid_in, void* grid_out, int c, int64_t n_grid,
                 const void* W, const int32_t* I, int m, int s, void* workspace, size_t workspace_bytes,
                 void* stream);
/* multi_direct_forcing(grid_u, W, I, u_target, ds, n_iter) -> (grid_force (c,n_grid),
 * marker_force (m,c)) — ib/mdf.py:10-64.  ds is per marker (m,) when ds != NULL, else
 * the scalar ds_scalar. */
int vs_ib_mdf(int dtype, const void* grid_u, int c, int64_t n_grid, const void* W, const int32_t* I, int m, int s,
              const void* u_target, const void* ds, double ds_scalar, int n_iter, void* grid_force,
              void* marker_force, void* workspace, size_t workspace_bytes, void* stream);

/* spread() like vs_ib_spread, for callers that cannot allocate device memory while they
 * run: a host runtime that owns every device allocation and hands its custom calls no
 * scratch (an XLA FFI handler registered without a workspace, an engine with its own
 * pool), or a real-time loop that may not enter the allocator.  No counterpart in the
 * reference: vivsim's spread is a JAX scatter-add whose scratch XLA provides.  Scratch is
 * a fixed 4 MiB device array of the library, one per device, held until the process
 * exits; the first call on each device looks its address up (make that call before any
 * stream capture), and so does the first call after the device's context was replaced
 * (cudaDeviceReset); nothing is allocated.  Limit: m * s <= 65536 marker-stencil pairs
 * (4096 markers of a 4x4 stencil), else VS_ERR_INVALID_ARG.  All calls on a device share
 * the scratch, so calls that may overlap on the device (different streams, several host
 * threads) race: issue them in order on one stream.  Results equal vs_ib_spread's. */
int vs_ib_spread_noalloc(int dtype, const void* marker_values, const void* grid_in, void* grid_out, int c,
                         int64_t n_grid, const void* W, const int32_t* I, int m, int s, void* stream);

/* Read (and optionally clear) the IB status word: bit 0 is set when a stencil index fell
 * outside [0, n_grid) in an IB call (that contribution is dropped / read as zero).
 * Synchronous with respect to the device. */
int vs_ib_status(unsigned* status_out, int reset);

/* ===================================================================== dynamics ===
 * newmark(a, v, d, h, m, k, c, dt, gamma, beta) — dyn.py:5-51.  a, v, d, h are device
 * arrays of ndof.  Scalar branch (dyn.py:42-45): m, k, c are the host scalars and every
 * DOF advances independently; matrix branch (dyn.py:36-41) when m_mat != NULL: ndof x
 * ndof row-major device matrices, solved by Gaussian elimination with partial pivoting.
 * Outputs may alias inputs. */
int vs_newmark(int dtype, int ndof, const void* a, const void* v, const void* d, const void* h, double m, double k,
               double c, const void* m_mat, const void* k_mat, const void* c_mat, double dt, double gamma,
               double beta, void* a_next, void* v_next, void* d_next, void* stream);
/* get_markers_coords_2dof / _3dof, get_markers_velocity_3dof, get_force_to_obj,
 * get_torque_to_obj — dyn.py:68-154.  x0,y0,x,y are (m,); d, v device (2|3,); h (m,2). */
int vs_markers_coords_2dof(int dtype, const void* x0, const void* y0, int m, const void* d, void* x, void* y,
                           void* stream);
int vs_markers_coords_3dof(int dtype, const void* x0, const void* y0, int m, double xc, double yc, const void* d,
                           void* x, void* y, void* stream);
int vs_markers_velocity_3dof(int dtype, const void* x, const void* y, int m, double xc, double yc, const void* d,
                             const void* v, void* vel, void* stream);
int vs_force_to_obj(int dtype, const void* h, int m, int c, void* out, void* stream);
int vs_torque_to_obj(int dtype, const void* x, const void* y, int m, double xc, double yc, const void* d,
                     const void* h, void* out, void* stream);

/* ================================================================ fused step ===
 * One IB-LBM time step of the reference's composed update loop
 * (examples/2d/vortex_induced_vibration.py:96-148, examples/2d/lid_driven_cavity.py:55-63,
 * examples/3d/flow_past_sphere.py:139-180): moments, equilibrium, collision, forcing,
 * periodic streaming and the ordered face boundaries in ONE grid pass (push streaming,
 * one read and one write per population) plus a small ordered face epilogue.       */

typedef struct vs_bc {
  int kind; /* VS_BC_* */
  int mode; /* VS_WALL_* */
  int loc;  /* VS_LEFT ... */
  double rho, ux, uy, uz, gx, gy, gz;
} vs_bc;

#define VS_MAX_BC 8
/* grid kernel variants: one thread per node reading populations straight from global
 * memory, or a persistent kernel staging row tiles through shared memory with bulk
 * (TMA) copies; AUTO picks the plain kernel */
enum { VS_GRID_AUTO = 0, VS_GRID_PLAIN = 1, VS_GRID_TMA = 2 };
typedef struct vs_lattice_cfg {
  int q;         /* 9 or 19 */
  int dtype;     /* VS_F32 / VS_F64 */
  int nx, ny, nz;/* nz = 1 for D2Q9 */
  int collision; /* VS_COLLIDE_* */
  double omega;
  double mrt_op[19 * 19];  /* q*q collision operator when collision == VS_COLLIDE_MRT */
  int forcing;             /* VS_FORCE_* applied to g_uniform + IB force window       */
  double g_uniform[3];     /* body-force density added at every node                */
  double mrt_fop[19 * 19]; /* q*q forcing operator when forcing == VS_FORCE_GUO_MRT   */
  int n_bc;                /* boundaries applied in this order after streaming      */
  vs_bc bc[VS_MAX_BC];
  int variant;             /* grid kernel: VS_GRID_AUTO, VS_GRID_PLAIN or VS_GRID_TMA */
  const uint8_t* obstacle_mask; /* device, one byte per node or NULL: obstacle_bounce_back after
                                    the face boundaries (lbm/boundary/bb.py:98-110); the plan
                                    keeps the pointer, the caller keeps the memory alive */
  int watchdog_every;      /* > 0: vs_run / vs_run_graph scan the populations for NaN/Inf after
                              every watchdog_every-th step and after the last one; a hit sets
                              the plan's status word to VS_ERR_NONFINITE (vs_lattice_status) */
} vs_lattice_cfg;

typedef struct vs_lattice_plan vs_lattice_plan;
int vs_lattice_plan_create(const vs_lattice_cfg* cfg, vs_lattice_plan** out);
int vs_lattice_plan_destroy(vs_lattice_plan* plan);
/* Device status of the plan's grid kernels: VS_OK, VS_ERR_TIMEOUT when a bounded wait
 * for a bulk copy gave up (that launch left its nodes unwritten; the late copies landed
 * before the block left), VS_ERR_TIMEOUT_INFLIGHT when a late copy had still not landed
 * after a second bounded wait, or VS_ERR_NONFINITE when the watchdog found a NaN/Inf
 * population.  Synchronises the stream; reset != 0 clears it. */
int vs_lattice_status(const vs_lattice_plan* plan, int reset, void* stream);
/* Run form of vs_run for this plan: VS_RUN_STEPS (default: launches per time step) or
 * VS_RUN_PERSISTENT (one cooperative launch per run where vs_run_persistent says it
 * applies; elsewhere the per-step launches).  Both give the same bits.  No CUDA call.  No
 * counterpart in the reference (its loop is XLA's). */
#define VS_RUN_STEPS 0
#define VS_RUN_PERSISTENT 1
int vs_lattice_set_run_form(vs_lattice_plan* plan, int form);
/* NaN/Inf scan of n values: sets *status_dev (a device int) to VS_ERR_NONFINITE when one is
 * not finite and leaves it unchanged otherwise.  Asynchronous.  The reference has no
 * counterpart (a JAX run would carry the NaN on); this is the fused run's watchdog. */
int vs_check_finite(int dtype, const void* f, int64_t n, int* status_dev, void* stream);
/* Failure-detection self-test (no counterpart in the reference): one bounded mbarrier wait
 * on bytes that never arrive (limit polls, at most 2^20); *status_dev receives
 * VS_ERR_TIMEOUT and the context stays usable.  Asynchronous. */
int vs_selftest_bounded_wait(int limit, int* status_dev, void* stream);

/* Immersed body advanced by the IB step (dyn.py + ib/mdf.py).  Markers follow a rigid
 * translation d (get_markers_coords_2dof); DOFs with free[k] = 0 stay at zero.  In 2-D,
 * free_dof[2] = 1 adds a rotation by the angle d[2] about (center_x, center_y): markers
 * from get_markers_coords_3dof, MDF target velocities from get_markers_velocity_3dof, the
 * torque from get_torque_to_obj (dyn.py:84-154), h[2] = torque + a[2] * added_inertia and
 * Newmark with (inertia, rot_stiffness, rot_damping). */
typedef struct vs_body_cfg {
  int dim;        /* 2 or 3, must match the lattice                                    */
  int dtype;
  int n_markers;
  const double* x0_host; /* (n_markers,) initial marker coordinates                    */
  const double* y0_host;
  const double* z0_host; /* NULL in 2-D                                                */
  const double* ds_host; /* (n_markers,) or NULL to use ds_scalar                      */
  double ds_scalar;
  int kernel;            /* VS_KERNEL_*                                                */
  int radius;            /* stencil half-width (2 for the 4-point kernels)             */
  int n_iter;            /* MDF iterations                                             */
  int moving;            /* 0: stencil built once (fixed body), 1: rebuilt every step  */
  int free_dof[3];       /* Newmark-integrated DOFs: x, y, z (3-D) or x, y, angle (2-D)  */
  double mass, stiffness, damping, added_mass_area; /* h += a * area, vortex_induced_vibration.py:136 */
  double d0[3], v0[3], a0[3];                       /* initial body state                 */
  int window_margin;     /* extra nodes around the marker stencils reserved for motion */
  double center_x, center_y;                 /* 2-D rotation: initial centre of the body  */
  double inertia, rot_stiffness, rot_damping, added_inertia;
  int fsi_iter;          /* 2-D moving body: fluid-structure sub-iterations per step (0 or 1:
                          * one pass).  Each pass places the markers with the latest state,
                          * redoes stencil, MDF and force, and restarts Newmark from the
                          * step's saved state (examples/2d/vortex_induced_vibration.py:114-139) */
} vs_body_cfg;

typedef struct vs_body_plan vs_body_plan;
/* A 2-D body whose markers share stencil nodes only with neighbours a few positions away in
 * marker order (a curve of markers; checked once from the rigid marker set) uses the chain
 * form of the body kernel; others use the general form (an in-shared-memory sort).  Both
 * give the same results; VIVSIM_GB300_BODY_CSR=1 in the environment at plan creation
 * selects the general form.  The chain form runs over a cluster of up to 8 CTAs that also
 * update the body's box (VIVSIM_GB300_BODY_SINGLE=1: one CTA and a separate box launch). */
int vs_body_plan_create(const vs_body_cfg* cfg, const vs_lattice_plan* lattice, vs_body_plan** out);
int vs_body_plan_destroy(vs_body_plan* plan);
/* Copy the body state out: (a, v, d, h) as 4 x 3 doubles (device state, synchronises the stream). */
int vs_body_get_state(const vs_body_plan* plan, double* state_host, void* stream);
int vs_body_set_state(vs_body_plan* plan, const double* state_host, void* stream);
/* Device address of the body state (a[3], v[3], d[3], h[3] in the plan dtype), for
 * callers that copy or read it on the device between steps. */
int vs_body_state_device(const vs_body_plan* plan, void** state);
/* vs_body_set_state from a device copy of the 12 values, enqueued on the stream (no host
 * synchronisation; capturable into a CUDA graph). */
int vs_body_set_state_device(vs_body_plan* plan, const void* state, void* stream);

/* One step: f_out = step(f_in).  body may be NULL.  force_hist, when not NULL, receives
 * the body force h (3 values of the plan dtype) of this step.  f_out must not alias f_in. */
int vs_step(const vs_lattice_plan* lattice, vs_body_plan* body, const void* f_in, void* f_out, void* force_hist,
            void* stream);
/* n_steps steps ping-ponging between f_a (input) and f_b; the result ends in f_a when
 * n_steps is even, else in f_b.  force_hist (n_steps x 3) may be NULL.  The loop of the
 * reference's examples (examples/2d/vortex_induced_vibration.py:151-157, a lax.scan over
 * update_step).  With the run form VS_RUN_PERSISTENT (vs_lattice_set_run_form, or the
 * environment variable VIVSIM_GB300_RUN_FORM=persistent for every plan), a
 * float 2-D plan whose body takes the cluster form (4 x 4 stencil, face boundaries that
 * can wait for the next step's load) runs all n_steps in one persistent cooperative launch
 * (the body's thread-block cluster beside groups of grid tiles, a barrier per step; one
 * launch per watchdog interval); its populations equal the launch-per-step form's bit for
 * bit. */
int vs_run(const vs_lattice_plan* lattice, vs_body_plan* body, void* f_a, void* f_b, int n_steps,
           void* force_hist, void* stream);
/* 1 when vs_run(lattice, body, ..., n_steps, ...) takes the persistent form, else 0 (no
 * CUDA call).  No counterpart in the reference (its loop is XLA's). */
int vs_run_persistent(const vs_lattice_plan* lattice, const vs_body_plan* body, int n_steps);
/* As vs_run, but the n_steps launches are captured once into a CUDA graph owned by the
 * lattice plan (re-captured when the arguments change) and replayed.  A run that takes
 * the persistent form is already one launch: vs_run_graph then runs vs_run. */
int vs_run_graph(vs_lattice_plan* lattice, vs_body_plan* body, void* f_a, void* f_b, int n_steps,
                 void* force_hist, void* stream);

/* Profiling entry point: launches only the grid kernel of vs_step (collide, force from the
 * body's current window, push-stream), without the body and face kernels, so that the
 * dominant kernel can be timed on its own. */
int vs_step_grid_only(const vs_lattice_plan* lattice, const vs_body_plan* body, const void* f_in, void* f_out,
                      void* stream);

/* ================================================================ many cases ===
 * A batch advances many independent cases (one lattice plan each, with an optional body
 * plan) in lock step: every time step is one body launch (one CTA per 2-D body of the
 * chain form), one grid launch over the nodes of all cases outside their bodies' boxes,
 * and one launch over all boxes after the join, instead of three launches per case.
 * The reference runs such sweeps as separate jitted loops (one per case); this has no
 * single counterpart there.  Results equal vs_run of each case on its own.
 * All cases share q, dtype and collision model; other bodies (3-D, general form) run
 * their own kernels inside the batch.  The plans must stay alive while the batch is used. */
typedef struct vs_batch_plan vs_batch_plan;
int vs_batch_plan_create(vs_lattice_plan* const* lattices, vs_body_plan* const* bodies, int n_cases,
                         vs_batch_plan** out);
int vs_batch_plan_destroy(vs_batch_plan* plan);
/* Launch shape: threads per block of the grid launches (32, 64, 128, 256) and the number
 * of middle time steps captured per CUDA graph (0: no graph; rounded down to even). */
int vs_batch_set_launch(vs_batch_plan* plan, int threads_per_block, int steps_per_graph);
/* Nodes per thread of the main grid launch (1 or 2: two nodes' loads in flight per thread).
 * Results do not depend on it.  No counterpart in the reference (the batch is this
 * library's). */
int vs_batch_set_nodes_per_thread(vs_batch_plan* plan, int nodes_per_thread);
/* n_steps steps of every case; case k ping-pongs between f_a[k] (input) and f_b[k] as in
 * vs_run.  Device parameter tables are built on the first call for a set of buffers (a
 * synchronous upload); graphs need a non-default stream (else steps are launched one by
 * one). */
int vs_batch_run(vs_batch_plan* plan, void* const* f_a, void* const* f_b, int n_steps, void* stream);

/* ============================================================== diagnostics ===
 * vivsim/post.py on the device.  Derivatives as jnp.gradient: central differences
 * inside, one-sided at the two ends of each axis (no periodic wrap).  The velocity is
 * read from u (d, nx, ny[, nz]) or, when u is NULL, computed from the populations f
 * (get_macroscopic), which saves the separate moments pass. */
enum {
  VS_POST_VELOCITY_MAGNITUDE = 0,    /* post.py:6-14    (n)            */
  VS_POST_VELOCITY_GRADIENT = 1,     /* post.py:17-29   (d, d, n)      */
  VS_POST_VORTICITY = 2,             /* post.py:32-54   (1 | 3, n)     */
  VS_POST_VORTICITY_MAGNITUDE = 3,   /* post.py:57-68   (n)            */
  VS_POST_DIVERGENCE = 4,            /* post.py:72-83   (n)            */
  VS_POST_STRAIN_RATE = 5,           /* post.py:86-95   (d, d, n)      */
  VS_POST_STRAIN_RATE_MAGNITUDE = 6, /* post.py:98-107  (n)            */
  VS_POST_KINETIC_ENERGY = 7,        /* post.py:110-118 (n)            */
  VS_POST_ENSTROPHY = 8,             /* post.py:144-155 (n)            */
  VS_POST_Q_CRITERION = 9,           /* post.py:172-186 (n)            */
  VS_POST_MEAN_KINETIC_ENERGY = 10,  /* post.py:121-129: sum into *sum_dev */
  VS_POST_MEAN_ENSTROPHY = 11        /* post.py:158-167: sum into *sum_dev */
};
/* One field of the list above into out; for the two means, the sum over the nodes lands
 * in the device double *sum_dev (divide by the node count for the mean). */
int vs_post(int q, int dtype, int what, const void* u, const void* f, int nx, int ny, int nz, void* out,
            double* sum_dev, void* stream);
/* pressure(rho, cs2) = rho * cs2 — post.py:132-141 */
int vs_post_pressure(int dtype, const void* rho, int64_t n, double cs2, void* out, void* stream);
/* Components of a vs_post field (leading dimension of out). */
int vs_post_components(int q, int what);

/* ========================================================== grid refinement ===
 * Transfers between D2Q9 blocks of neighbouring refinement levels (factor 2), called after
 * streaming — vivsim/multigrid.py.  Both update the destination in place: only the three
 * populations of the direction cross the interface line; the reference returns the
 * updated array.  Shapes along the interface follow the reference's broadcasting (fine
 * extent 2 x coarse extent, or a length-1 operand); anything else is VS_ERR_INVALID_ARG,
 * where the reference raises its shape error.  init_grid, get_omega and coord_to_indices
 * (multigrid.py:21-55, 131-170) are host arithmetic in vivsim_gb300.multigrid. */
enum { VS_REFINE_LEFT = 0, VS_REFINE_RIGHT = 1, VS_REFINE_UP = 2, VS_REFINE_DOWN = 3 };
/* fine_to_coarse(f_fine, f_coarse, dir) — multigrid.py:58-95: the coarse block's buffer line
 * (last x line for left, first for right, first y line for up, last for down) gets the
 * 2 x 2 average of the fine populations that move in dir */
int vs_fine_to_coarse(int dtype, const void* f_fine, int nxf, int nyf, void* f_coarse, int nxc, int nyc, int dir,
                      void* stream);
/* coarse_to_fine(f_coarse, f_fine, dir) — multigrid.py:97-128: each coarse population of
 * the interface line onto the even and the odd fine node it covers */
int vs_coarse_to_fine(int dtype, const void* f_coarse, int nxc, int nyc, void* f_fine, int nxf, int nyf, int dir,
                      void* stream);

/* ================================================================== adjoint ===
 * Gradients of a 2-D cylinder VIV objective by a hand-written discrete adjoint of the
 * fused step: D2Q9 (BGK, KBC, regularised or MRT collision), exact-difference forcing, MDF immersed boundary, a 1-DOF
 * transverse spring (Newmark), equilibrium inflow ux = U0 at x = 0, pressure NEE
 * outflow at x = nx-1, periodic y (examples/2d/vortex_induced_vibration.py:96-148 with
 * BGK).  The reference obtains such gradients with jax.grad through its jitted loop; this
 * has no single counterpart there.  Objective: J = mean over steps [obj_start, n_steps)
 * of the x force on the body.  Parameters: U0 (inflow, initial state feq(1, (U0, 0)),
 * and omega = 1 / (3 U0 D / Re + 0.5)), the spring stiffness, and the radial offsets of
 * the markers (marker m at angle 2 pi m / n_markers, radius D/2 + offsets[m]; ds =
 * pi D / n_markers).  Populations are checkpointed every checkpoint_every steps and
 * each segment is recomputed before its reverse sweep. */
typedef struct vs_adjoint_cfg {
  int dtype;
  int nx, ny;
  double U0, D, Re, rho_out;
  int n_markers;
  double cx, cy;
  const double* offsets_host; /* (n_markers,) */
  int kernel, radius, n_iter;
  double mass, stiffness, damping, added_mass_area;
  int n_steps, checkpoint_every, obj_start;
  int collision;         /* VS_COLLIDE_BGK (default 0), _KBC, _REG or _MRT              */
  double mrt_op[81];     /* MRT: the 9 x 9 operator at this omega, and its derivative     */
  double mrt_dop[81];    /*      with respect to omega (row-major)                        */
} vs_adjoint_cfg;
typedef struct vs_adjoint_plan vs_adjoint_plan;
int vs_adjoint_plan_create(const vs_adjoint_cfg* cfg, vs_adjoint_plan** out);
int vs_adjoint_plan_destroy(vs_adjoint_plan* plan);
/* Forward run from rest; J_out receives the objective.  keep_checkpoints != 0 stores
 * what vs_adjoint_backward needs. */
int vs_adjoint_forward(vs_adjoint_plan* plan, int keep_checkpoints, double* J_out, void* stream);
/* Reverse sweep: seed * dJ/dU0, dJ/dstiffness and dJ/doffsets (n_markers). */
int vs_adjoint_backward(vs_adjoint_plan* plan, double seed, double* grad_U0, double* grad_K, double* grad_offsets,
                        void* stream);

/* ==================================================== vector-Jacobian products ===
 * Reverse-mode building blocks of the per-operator functions, so that a caller can
 * differentiate an update step it composes itself (the reference differentiates its
 * jitted loop with jax.grad; a composed torch step differentiates through these).
 * Each takes the forward inputs it needs and the cotangent g_out of the result and writes
 * the cotangents of the inputs.  Node-local Jacobians are exact: forward-mode dual numbers
 * through the same formulas as the forward kernels.  *_node outputs hold one value per
 * node (or face node) whose sum is the cotangent of a scalar parameter: reduce them with
 * vs_sum_ordered, which sums in a fixed order (deterministic).  Asynchronous. */
/* streaming (lbm/basic.py:60-85, lbm3d/basic.py:52-87): g_in_i(x) = g_out_i(x + c_i) */
int vs_streaming_vjp(int q, int dtype, const void* g_out, void* g_in, int nx, int ny, int nz, void* stream);
/* get_macroscopic (lbm/basic.py:88-111, lbm3d/basic.py:90-106): g_f from g_rho (n,) and
 * g_u (d, n); either may be NULL (zero) */
int vs_macroscopic_vjp(int q, int dtype, const void* f, const void* g_rho, const void* g_u, void* g_f, int64_t n,
                       void* stream);
/* get_equilibrium (lbm/basic.py:114-135, lbm3d/basic.py:109-130): g_rho, g_u from g_feq */
int vs_equilibrium_vjp(int q, int dtype, const void* rho, const void* u, const void* g_feq, void* g_rho, void* g_u,
                       int64_t n, void* stream);
/* collision_bgk / _kbc / _reg (lbm/basic.py:138-156, lbm/collision/kbc.py:10-60,
 * reg.py:4-49; lbm3d/basic.py:133-146, lbm3d/collision/kbc.py:8-42, reg.py:44-62):
 * g_f, g_feq, and per node the share of g_omega (g_omega_node may be NULL) */
int vs_collision_vjp(int q, int dtype, int kind, const void* f, const void* feq, double omega, const void* g_out,
                     void* g_f, void* g_feq, void* g_omega_node, int64_t n, void* stream);
/* collision_mrt (lbm/collision/mrt.py:66-88, lbm3d/collision/mrt.py:83-98): g_f, g_feq and,
 * when g_op != NULL, the cotangent of the q x q operator (device doubles, row-major) */
int vs_collision_mrt_vjp(int q, int dtype, const void* f, const void* feq, const double* op_host, const void* g_out,
                         void* g_f, void* g_feq, double* g_op, int64_t n, void* stream);
/* forcing_edm / forcing_guo_bgk (lbm/forcing/edm.py:4-31, guo.py:38-59; 3-D edm.py:6-26,
 * guo.py:41-55): g_f (may be NULL), g_g, g_u and per node g_out . guo, whose sum times
 * -1/2 is the Guo-BGK cotangent of omega (g_scale_node may be NULL) */
int vs_forcing_vjp(int q, int dtype, int kind, const void* g, const void* u, double omega, const void* g_out,
                   void* g_f, void* g_g, void* g_u, void* g_scale_node, int64_t n, void* stream);
/* forcing_guo_mrt (lbm/forcing/guo.py:62-107, lbm3d/forcing/guo.py:58-87): g_f, g_g, g_u
 * and, when g_op != NULL (needs guo_scratch of q x n values), the operator's cotangent */
int vs_forcing_guo_mrt_vjp(int q, int dtype, const void* g, const void* u, const double* op_host, const void* g_out,
                           void* g_f, void* g_g, void* g_u, void* guo_scratch, double* g_op, int64_t n, void* stream);
/* boundary_nee / _nebb / _equilibrium / _bounce_back / _specular_reflection and their
 * velocity / pressure forms (the sources cited at vs_boundary), scalar wall values:
 * g_in (and g_before_stream for bounce-back) from g_out; g_wall_node (4 per face node,
 * may be NULL): shares of the cotangents of rho_wall, ux_wall, uy_wall, uz_wall.  A
 * force-corrected wall is the given wall with the corrected velocity. */
int vs_boundary_vjp(int q, int dtype, int kind, int mode, int loc, const void* f_in, const void* f_before_stream,
                    const void* g_out, void* g_in, void* g_before_stream, void* g_wall_node, int nx, int ny, int nz,
                    double rho_wall, double ux_wall, double uy_wall, double uz_wall, void* stream);
/* out[m, s] = sum_c A[m, c] grid[c, I[m, s]]: the stencil weights' cotangent of
 * interpolate (A = g_U, grid = the interpolated field) and of spread (A = the spread
 * values, grid = g_out) (ib/stencil.py:54-110).  The field cotangents are the other
 * operation: interpolate^T = spread, spread^T = interpolate. */
int vs_ib_pair_dot(int dtype, const void* A, const void* grid, int c, int64_t n_grid, const int32_t* I, int m, int s,
                   void* out, void* stream);
/* get_ib_stencil (ib/stencil.py:7-51, ib3d/stencil.py:7-59): marker-coordinate
 * cotangents from g_W (m, s); z and g_z NULL in 2-D */
int vs_ib_stencil_vjp(int kernel, int radius, int dtype, int dim, const void* x, const void* y, const void* z,
                      const void* g_W, void* g_x, void* g_y, void* g_z, int m, void* stream);
/* newmark (dyn.py:5-51): g_a, g_v, g_d, g_h (ndof each) from the next state's cotangents
 * (any may be NULL = zero); scalar branch: g_mkc[3] = cotangents of m, k, c; matrix
 * branch: g_mats = g_M, g_K, g_C (3 ndof x ndof, row-major) */
int vs_newmark_vjp(int dtype, int ndof, const void* a, const void* v, const void* d, const void* h, double m, double k,
                   double c, const void* m_mat, const void* k_mat, const void* c_mat, double dt, double gamma,
                   double beta, const void* g_a_next, const void* g_v_next, const void* g_d_next, void* g_a,
                   void* g_v, void* g_d, void* g_h, void* g_mkc, void* g_mats, void* stream);
/* Deterministic sum of n values x[0], x[stride], ... into *out (a device double);
 * scratch: 256 device doubles.  No counterpart in the reference (XLA reduces there). */
int vs_sum_ordered(int dtype, const void* x, int64_t n, int64_t stride, double* scratch, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VIVSIM_GB300_H */
