/*
 * gbfluids: C ABI of the GB300 (sm_103a) single-phase finite-volume
 * right-hand side of JAX-Fluids.
 *
 * Every entry point takes plain device pointers, a case descriptor and a CUDA
 * stream (passed as void*, may be NULL for the legacy stream).  Nothing here
 * allocates device memory unless its comment says so, nothing synchronises
 * the device unless its comment says so, and no call traps: failures are
 * returned as negative status codes (gbf_status_string names them).
 *
 * Buffer layouts are the reference's (src/jaxfluids, paths below relative to
 * it):
 *   - halo buffers   double[5][Nx+2nh][Ny+2nh][Nz+2nh], C order, an inactive
 *                    axis (N = 1) has extent 1 and no halo
 *                    (initialization/helper_functions.py:49,
 *                    domain/domain_information.py:202-206);
 *   - interior       double[5][Nx][Ny][Nz] (rhs, solvers/space_solver.py:135-141);
 *   - primitives     (rho, u, v, w, p), conservatives (rho, rho u, rho v,
 *                    rho w, E) (equation_information.py:95-105).
 */
#ifndef GBFLUIDS_H
#define GBFLUIDS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBF_ABI_VERSION 6

/* status codes */
#define GBF_OK 0
#define GBF_ERR_INVALID_ARGUMENT -1
#define GBF_ERR_UNSUPPORTED -2
#define GBF_ERR_CUDA -3
#define GBF_ERR_SIZE -4
#define GBF_ERR_ALIGNMENT -5

/* reconstruction_stencil (stencils/__init__.py registry) */
#define GBF_RECON_WENO5Z 0
#define GBF_RECON_MINMOD 1
#define GBF_RECON_MINMOD_AD 2
#define GBF_RECON_WENO5JS 3   /* weno/weno5_js.py */
#define GBF_RECON_WENO3JS 4   /* weno/weno3_js.py */
#define GBF_RECON_WENO3Z 5    /* weno/weno3_z.py */
#define GBF_RECON_TENO5 6     /* teno/teno5.py */

/* reconstruction_variable (solvers/__init__.py:5-12) */
#define GBF_RECVAR_PRIMITIVE 0
#define GBF_RECVAR_CHAR_PRIMITIVE 1
#define GBF_RECVAR_CONSERVATIVE 2       /* high_order_godunov.py:282-296 (WENO5-Z) */
#define GBF_RECVAR_CHAR_CONSERVATIVE 3  /* high_order_godunov.py:404-416 (WENO5-Z) */

/* frozen_state (input/numerical_setup/read_conservatives.py:162-166) */
#define GBF_FROZEN_ARITHMETIC 0
#define GBF_FROZEN_ROE 1

/* riemann_solver (solvers/riemann_solvers/__init__.py:16) */
#define GBF_RIEMANN_HLLC 0
#define GBF_RIEMANN_RUSANOV 1
#define GBF_RIEMANN_HLL 2     /* riemann_solvers/HLL.py */
/* riemann_solvers/LaxFriedrichs.py: Rusanov's flux with one dissipation speed
 * per axis, the maximum of |u| + c over every reconstructed face state of the
 * axis (reduced by an extra reconstruction pass into the workspace of the
 * call) */
#define GBF_RIEMANN_LAXFRIEDRICHS 3

/* signal_speed (solvers/riemann_solvers/__init__.py:27) */
#define GBF_SIGNAL_EINFELDT 0
#define GBF_SIGNAL_DAVIS 1
#define GBF_SIGNAL_ARITHMETIC 2
#define GBF_SIGNAL_RUSANOV 3
#define GBF_SIGNAL_TORO 4

/* boundary types (halos/outer/boundary_condition.py:539-604,
 * halos/outer/material.py:140-210): WALL mirrors the interior with
 * u_halo = 2 u_wall - u (:473-531), DIRICHLET sets the given primitives
 * (:732-798), NEUMANN adds sign * dx * gradient to the boundary cell
 * (:825-866; sign +1 at west/south/bottom, -1 at east/north/top).  Values
 * come from gbf_case.bc_value, or per boundary cell from
 * gbf_case.bc_field_values (callables of the boundary coordinates).
 * GBF_BC_MIXED marks a face of several types (bounding_domain masks,
 * material.py:252-266): gbf_case.bc_field_types gives the type of each
 * boundary cell, and the edges of such a face take the mean rule
 * (boundary_condition.py:128-177, "ANY").  Values varying in time are not
 * supported. */
#define GBF_BC_PERIODIC 0
#define GBF_BC_ZEROGRADIENT 1
#define GBF_BC_SYMMETRY 2
#define GBF_BC_WALL 3
#define GBF_BC_DIRICHLET 4
#define GBF_BC_NEUMANN 5
#define GBF_BC_MIXED 6

/* dissipative-flux stencils (stencils/reconstruction/central/central_{2,4}.py,
 * stencils/derivative/deriv_{center,face}_{2,4}.py) */
#define GBF_CENTRAL4 0
#define GBF_CENTRAL2 1

/* face order of gbf_case.bc */
#define GBF_FACE_WEST 0
#define GBF_FACE_EAST 1
#define GBF_FACE_SOUTH 2
#define GBF_FACE_NORTH 3
#define GBF_FACE_BOTTOM 4
#define GBF_FACE_TOP 5

/* gbf_case.flags */
#define GBF_FLAG_VISCOUS 1u
#define GBF_FLAG_HEAT 2u
#define GBF_FLAG_VISCOUS_HEAT_PRODUCTION 4u
/* active_physics.is_convective_flux = false: the face flux starts at zero and
   carries only the dissipative fluxes (space_solver.py:512-529); needs
   GBF_FLAG_VISCOUS or GBF_FLAG_HEAT */
#define GBF_FLAG_NO_CONVECTIVE 8u
/* conservatives.positivity.is_interpolation_limiter: reconstructed face
   states with density < 1e-12 or pressure < 1e-10 fall back to the cell
   beside the face (limiter_interpolation.py:82-210, precision.py:54) for
   density and pressure, or for every primitive with GBF_FLAG_LIMIT_VELOCITY
   (positivity.limit_velocity) */
#define GBF_FLAG_INTERPOLATION_LIMITER 16u
#define GBF_FLAG_LIMIT_VELOCITY 32u
/* active_physics.is_volume_force: gravity (gbf_case.gravity, forcings.gravity)
   adds rho g to the momentum and g . (rho u) to the energy right-hand side
   after the flux divergence (space_solver.py:377-384,
   source_term_solver.py:165-186) */
#define GBF_FLAG_GRAVITY 64u

/* Case descriptor: the numerical_setup / case_setup keys the path reads. */
typedef struct gbf_case {
  int32_t n[3];          /* interior cells per axis; 1 marks an inactive axis */
  int32_t nh;            /* halo cells of the halo buffers (conservatives.halo_cells) */
  int32_t recon;         /* GBF_RECON_* */
  int32_t recon_var;     /* GBF_RECVAR_* */
  int32_t frozen_state;  /* GBF_FROZEN_* */
  int32_t riemann;       /* GBF_RIEMANN_* */
  int32_t signal_speed;  /* GBF_SIGNAL_* */
  int32_t bc[6];         /* GBF_BC_* per face, GBF_FACE_* order */
  uint32_t flags;        /* GBF_FLAG_* */
  double dx[3];          /* cell size per axis ((hi - lo) / n, homogenous.py:13) */
  double gamma;          /* specific_heat_ratio */
  double R;              /* specific_gas_constant */
  double mu;             /* constant dynamic viscosity (CUSTOM) */
  double bulk_mu;        /* bulk viscosity */
  double kappa;          /* thermal conductivity */
  double cfl;            /* time_integration.CFL */
  double fixed_dt;       /* time_integration.fixed_timestep, 0 = CFL time step */
  double eps;            /* precision epsilon (jnp.finfo(float64).eps) */
  double stencil_eps;    /* spatial stencil epsilon (1e-30) */
  double bc_value[6][5]; /* per face, GBF_FACE_* order: WALL [1..3] = wall velocity
                            (u, v, w); DIRICHLET [0..4] = (rho, u, v, w, p);
                            NEUMANN [0..4] = normal derivatives of (rho, u, v, w, p) */
  int32_t dissipative_stencil[3]; /* dissipative_fluxes.{reconstruction_stencil,
                            derivative_stencil_center, derivative_stencil_face}: GBF_CENTRAL4 or
                            GBF_CENTRAL2 (read_conservatives.py:374-445) */
  int32_t reserved;
  /* Boundary values along a face, device memory, NULL where the face uses
     bc_value: per face nt = the product of the interior extents of its two
     other axes (axis order, the later one fastest); bc_field_values[f] holds
     5 x nt doubles, variable-major, laid out as bc_value (WALL velocity in
     1..3), the callables' values at the boundary cells' centres;
     bc_field_types[f] (only with bc[f] = GBF_BC_MIXED, required there) holds
     nt GBF_BC_* types other than PERIODIC and MIXED.  Read by every launch;
     they must stay valid and unchanged while work of this case runs. */
  const double* bc_field_values[6];
  const int8_t* bc_field_types[6];
  double gravity[3];     /* forcings.gravity, with GBF_FLAG_GRAVITY */
} gbf_case;

/* Launch shape of the tile kernels; all-zero picks the built-in defaults.  For
 * the face kernels (the right-hand side and the fused stages) t gives the
 * faces per tile (default 16 along the face axis and 2 x 16 or 32 across it,
 * 16 x 8 on small cases); for the adjoint's tile kernels and the batched
 * stages the cells per tile (2-D 15x32, 3-D 7x8x8, 1-D 256).  The staged
 * stencil cells must fit 227 KB of shared memory (GBF_ERR_INVALID_ARGUMENT
 * otherwise). */
typedef struct gbf_tile {
  int32_t t[3];          /* cells per tile along each axis (1 on inactive axes) */
  int32_t threads;       /* threads per CTA (multiple of 32, 32..256) */
} gbf_tile;

/* GBF_ABI_VERSION the library was built with: a binding compares it with the
 * gbf_case layout it mirrors before the first call.  No reference counterpart. */
int gbf_abi_version(void);
/* Status returned by the most recent int-returning entry point called on this
 * host thread (GBF_OK before any call).  No reference counterpart: the
 * reference raises Python exceptions instead of returning codes. */
int gbf_last_status(void);
const char* gbf_status_string(int status);

/* Checks a descriptor without device work; returns GBF_OK or the reason it
 * cannot run (GBF_ERR_UNSUPPORTED for a setup the CUDA path does not build).
 * Takes the place of the setup readers' checks for this path
 * (input/numerical_setup/read_conservatives.py, halo count :361-365;
 * input/input_manager.py:116 sanity_check), which raise instead. */
int gbf_case_check(const gbf_case* c);

/*
 * Right-hand side of the conservative variables from a halo-filled primitive
 * buffer.  Replaces SpaceSolver.compute_rhs (solvers/space_solver.py:151-453,
 * per axis compute_rhs_xi :456-674) for the single-phase GODUNOV path:
 * reconstruct -> Riemann flux -> (1/dx)(F[i-1/2] - F[i+1/2]) summed over
 * the active axes in x, y, z order.  prims: halo buffer, read as it is (its
 * halos are the caller's); rhs: interior buffer.  The face fluxes of every
 * axis (N + 1 per line, as the reference's face arrays) go through a device
 * buffer of gbf_rhs_workspace_bytes(c) bytes, allocated for the call with
 * cudaMallocAsync on `stream` and released on it (gbf_rhs_ws takes it from
 * the caller instead).
 */
int gbf_rhs(const gbf_case* c, const double* prims, double* rhs, const gbf_tile* tile, void* stream);

/* As gbf_rhs with the halo-buffer conservatives `cons` beside the primitives
 * (SpaceSolver.compute_rhs, solvers/space_solver.py:151-453, receives both):
 * required by the CONSERVATIVE and CHAR-CONSERVATIVE reconstructions
 * (high_order_godunov.py:282-296, :404-416), which reconstruct the conservatives
 * (gbf_rhs returns GBF_ERR_INVALID_ARGUMENT for them); read by no other case. */
int gbf_rhs_cons(const gbf_case* c, const double* prims, const double* cons, double* rhs, const gbf_tile* tile,
                 void* stream);

/* As gbf_rhs_cons (cons may be null for the reconstructions that do not read
 * it) with a caller workspace of gbf_rhs_workspace_bytes(c) bytes of device
 * memory, 8-byte aligned: the face fluxes (5 doubles per face of every active
 * axis, N + 1 faces per line) and the Lax-Friedrichs axis speeds, so the call
 * allocates nothing and evaluations on concurrent streams, each with its own
 * workspace, share no state.  0 bytes for an invalid case. */
size_t gbf_rhs_workspace_bytes(const gbf_case* c);
int gbf_rhs_ws(const gbf_case* c, const double* prims, const double* cons, double* rhs, const gbf_tile* tile,
               void* workspace, void* stream);

/*
 * Face halos (and, for viscous cases, edge halos) of the primitive buffer and,
 * when cons != NULL, the conservatives of the halo cells recomputed from the
 * halo primitives.  Replaces HaloManager.perform_halo_update_material
 * (halos/halo_manager.py:146-234, halos/outer/material.py:94-287).
 */
int gbf_halo_fill(const gbf_case* c, double* prims, double* cons, void* stream);

/* SpaceSolver.compute_rhs volume forces (space_solver.py:377-384): with
 * GBF_FLAG_GRAVITY, rhs[1:5] (interior [5][N]) += the gravity forces of the
 * halo-buffer conservatives `cons`; nothing without the flag. */
int gbf_volume_force(const gbf_case* c, const double* cons, double* rhs, void* stream);

/* Primitive <-> conservative conversion over `count` cells of SoA buffers with
 * a variable stride of `count` (equation_manager.py:44-171). */
int gbf_prims_from_cons(const gbf_case* c, const double* cons, double* prims, int64_t count, void* stream);
int gbf_cons_from_prims(const gbf_case* c, const double* prims, double* cons, int64_t count, void* stream);

/*
 * One TVD-RK3 stage update of a halo buffer (RK3.py:31-62,
 * time_integrator.py:108-226): stage 0: U += dt rhs;
 * stage s>0: U = a_s U + b_s U0 (whole buffer), then U += (dt m_s) rhs
 * (interior).  dt is read from the device scalar *dt.
 */
int gbf_stage_integrate(const gbf_case* c, double* cons, const double* cons0, const double* rhs,
                        const double* dt, int stage, void* stream);

/*
 * CFL time step of a halo-filled primitive buffer
 * (time_integration/time_step_size.py:15-157), written to the device scalar
 * *dt_out.  Uses a device scratch of gbf_dt_workspace_bytes() bytes.
 */
size_t gbf_dt_workspace_bytes(void);
int gbf_dt(const gbf_case* c, const double* prims, double* dt_out, void* workspace, void* stream);

/*
 * Fused TVD-RK3 steps on interior conservatives (the hot path).  Replaces the
 * step loop of SimulationManager (do_runge_kutta_stages,
 * simulation_manager.py:536-1077, with compute_time_step_size,
 * time_integration/time_step_size.py:15-157, for the next step).
 * cons: double[5][Nx][Ny][Nz], advanced in place by `steps` steps.  Each
 * stage runs one face kernel per active axis (every face flux of the grid
 * once, from the stage primitives, boundary conditions applied by index
 * remapping) and one cell kernel (divergence, RK combination, the primitives
 * of the new state; in the last stage the next CFL time step's reductions).
 * prims: the interior primitives of cons (double[5][Nx][Ny][Nz]) for the first
 * stage of this call, as the reference's first stage reads the primitives the
 * state was initialised from (initialization/material_fields_initializer.py:
 * 148-210); NULL derives them from cons.  dt_state: device double[4] = {dt, t,
 * max_a, max_b} (dt of the next step, simulation time, reduction slots);
 * initialise with gbf_rk3_init (prims as for gbf_rk3_advance: the initial
 * time step from the initial primitives, time_control_initializer.py:34-70).
 * workspace: gbf_rk3_workspace_bytes(c) bytes of device memory (the stage
 * states U^1 and U^2 first, then two primitive buffers, the face fluxes of a
 * stage and the Lax-Friedrichs speed slots).  No host synchronisation;
 * graph-capturable.
 */
size_t gbf_rk3_workspace_bytes(const gbf_case* c);
int gbf_rk3_init(const gbf_case* c, const double* cons, const double* prims, double* dt_state, double t0,
                 void* stream);
int gbf_rk3_advance(const gbf_case* c, double* cons, const double* prims, double* dt_state, void* workspace,
                    int steps, const gbf_tile* tile, void* stream);

/*
 * One fused TVD-RK3 stage, for callers that drive the stage loop themselves
 * (SimulationManager.do_runge_kutta_stages, simulation_manager.py:770-1042,
 * one iteration: RHS of the stage state and TimeIntegrator.integrate, RK3.py:31-62).
 * stage 0: out = U^n + dt L(U^n) with cons_k == cons_n == U^n;
 * stage 1: out = 3/4 U^n + 1/4 U^1 + 1/4 dt L(U^1);
 * stage 2: out = 1/3 U^n + 2/3 U^2 + 2/3 dt L(U^2), then the next time step of
 * out is reduced into dt_state and the time advanced (three calls equal one
 * step of gbf_rk3_advance with prims NULL, bitwise).  out must not alias
 * cons_k; at stage 2 it may alias cons_n.  dt from dt_state[0] on the device.
 * workspace: gbf_rk3_workspace_bytes(c) bytes (the stage primitives and face
 * fluxes are kept there).
 */
int gbf_rk3_stage(const gbf_case* c, int stage, const double* cons_k, const double* cons_n, double* out,
                  double* dt_state, void* workspace, const gbf_tile* tile, void* stream);

/*
 * Numerical health of an interior conservative state [5][N]: counts[0] cells
 * with a non-finite value, counts[1] cells with rho <= 0, counts[2] cells with
 * p <= 0 (device uint64[3], overwritten; no host synchronisation).  The
 * reference propagates NaN silently at run time; this is the positive-count
 * warning channel of this library (a host reads counts when it wants to).
 */
int gbf_state_check(const gbf_case* c, const double* cons, uint64_t* counts, void* stream);

/*
 * Solver handle: the fused path with its workspace and time-step state owned
 * by the library (allocated on the current device by gbf_create, freed by
 * gbf_destroy).  No reference counterpart as a C object: it plays the part of
 * the SimulationManager instance (simulation_manager.py:94-138) for C callers.
 * gbf_solver_time copies {dt, t} to host memory and synchronises the stream.
 */
typedef struct gbf_solver gbf_solver;
int gbf_create(const gbf_case* c, const gbf_tile* tile, gbf_solver** out);
int gbf_destroy(gbf_solver* s);
int gbf_solver_init(gbf_solver* s, const double* cons, double t0, void* stream);
int gbf_solver_advance(gbf_solver* s, double* cons, int steps, void* stream);
int gbf_solver_time(gbf_solver* s, double* dt_t, void* stream);

/*
 * Adjoint (reverse mode) of the fused path, replacing jax.grad through
 * SimulationManager._feed_forward with a fixed time step
 * (feed_forward/feed_forward.py:231-524, simulation_manager.py:1296-1412).
 * Follows jax.grad's conventions at non-smooth points (|x|' = +1 at 0, half
 * of the cotangent to each argument of a max/min tie, zero derivative of
 * sign, where() passes the selected branch; the Lax-Friedrichs speed's
 * cotangent to the face states attaining the maximum, shared as jnp.max and
 * jnp.maximum share it).  Every reconstruction (PRIMITIVE WENO5-Z, WENO5-JS,
 * TENO5, WENO3-JS, WENO3-Z, MINMOD, MINMOD-AD; CHAR-PRIMITIVE, CONSERVATIVE
 * and CHAR-CONSERVATIVE with WENO5-Z and either frozen state), HLLC and HLL
 * with every signal-speed estimate, Rusanov, Lax-Friedrichs, the interpolation
 * limiter, gravity, and the CENTRAL4 / CENTRAL2 viscous and heat fluxes
 * (source_term_solver.py:188-350): every setup the forward accepts.
 *
 * gbf_rhs_vjp: out = J(U)^T w with J = d rhs / d U at the interior state
 *   `cons`; w, out interior [5][N].  workspace: gbf_vjp_workspace_bytes(c)
 *   (at least 5 N doubles; dissipative, conservative and Lax-Friedrichs
 *   cases more).
 * gbf_rk3_step_vjp: lam_out = (d U^{n+1} / d U^n)^T lam for one TVD-RK3 step
 *   from U^n = `cons` with the device time step *dt (stage states recomputed).
 *   workspace: gbf_vjp_workspace_bytes(c).  lam_out must not alias lam.
 */
size_t gbf_vjp_workspace_bytes(const gbf_case* c);  /* 0: invalid case */
int gbf_rhs_vjp(const gbf_case* c, const double* cons, const double* w, double* out, void* workspace,
                const gbf_tile* tile, void* stream);
int gbf_rk3_step_vjp(const gbf_case* c, const double* cons, const double* dt, const double* lam,
                     double* lam_out, void* workspace, const gbf_tile* tile, void* stream);
/* As gbf_rk3_step_vjp with the stage states U1, U2 of the step given by the
 * caller (kept from the forward run) instead of recomputed. */
int gbf_rk3_step_vjp_stages(const gbf_case* c, const double* cons, const double* u1, const double* u2,
                            const double* dt, const double* lam, double* lam_out, void* workspace,
                            const gbf_tile* tile, void* stream);
/* Reverse of one gbf_rk3_stage, U_out = a U_k + b U^n + c dt L(U_k) (stage 0:
 * a = 1, b = 0, c = 1; stage 1: 1/4, 3/4, 1/4; stage 2: 2/3, 1/3, 2/3):
 * lam_k = a lam + c dt J(U_k)^T lam; lam_n += b lam (stages 1 and 2; at stage 0,
 * where U_k is U^n, the caller adds lam_k to its U^n cotangent).  workspace:
 * gbf_vjp_workspace_bytes(c). */
int gbf_rk3_stage_vjp(const gbf_case* c, int stage, const double* cons_k, const double* dt, const double* lam,
                      double* lam_k, double* lam_n, void* workspace, const gbf_tile* tile, void* stream);

/*
 * Batched fused TVD-RK3 of many independent cases of uneven size sharing one
 * scheme (the reference batches equal-size cases with jax.vmap over
 * SimulationManager._feed_forward, simulation_manager.py:1248-1294; here each
 * case keeps its own size and its own CFL time step).
 *
 * Host-prepared device tables: `cases` (one gbf_batch_case per case) and
 * `worklist` (int32 pairs {case, tile index within the case} for every tile of
 * every case, tiles of shape `tile`).  States are packed per case: case c
 * occupies doubles [offset, offset + 5 n_c) of `cons`, variable-major with
 * stride n_c = cells of c.  `dt_states`: double[4 ncases] = per case {dt, t,
 * reduction slots}.  `workspace`: two stage buffers and two primitive
 * buffers of the packed size and the face fluxes of three axes
 * (gbf_batch_workspace_bytes).  Each stage is the single-case fused stage over
 * the work list: one face-kernel launch per active axis and one epilogue
 * launch, each of `ctas` CTAs (0 = 2 per SM) looping over the work list; one
 * more launch per step updates every case's dt.  A batched case advances
 * bitwise like the same case through gbf_rk3_advance.  No host
 * synchronisation; graph-capturable.
 * `scheme` supplies everything but the sizes (n, dx are taken per case): any
 * inviscid PRIMITIVE or CHAR-PRIMITIVE scheme but Lax-Friedrichs, without the
 * limiter, gravity or boundary value fields (GBF_ERR_UNSUPPORTED otherwise).
 */
typedef struct gbf_batch_case {
  int32_t n[3];          /* interior cells per axis */
  int32_t tiles[3];      /* tiles per axis for the batch tile shape */
  int64_t offset;        /* first double of the case in the packed buffers */
  double dx[3];          /* cell sizes */
} gbf_batch_case;

/* Host-side case table and work list of a batch (no device work): cells and
 * dx are 3 per case; cases receives n, tiles (for the tile shape; 1 on axes no
 * case uses), offset (packed in the given order) and dx; worklist receives
 * (case, tile) pairs, largest cases first.  *nitems and *total_doubles are set
 * even when worklist is NULL or capacity (pairs) is too small, which returns
 * GBF_ERR_SIZE: call once to size the list. */
int gbf_batch_worklist(const int32_t* cells, const double* dx, int ncases, const gbf_tile* tile,
                       gbf_batch_case* cases, int32_t* worklist, int64_t capacity, int64_t* nitems,
                       int64_t* total_doubles);
size_t gbf_batch_workspace_bytes(int64_t total_doubles);
int gbf_batch_init(const gbf_case* scheme, const gbf_batch_case* cases, int ncases,
                   const int32_t* worklist, int ntiles, const gbf_tile* tile, const double* cons,
                   double* dt_states, double t0, void* stream);
int gbf_batch_advance(const gbf_case* scheme, const gbf_batch_case* cases, int ncases,
                      const int32_t* worklist, int ntiles, const gbf_tile* tile, int ctas,
                      double* cons, double* dt_states, void* workspace, int64_t total_doubles,
                      int steps, void* stream);

/*
 * Allocation-free gbf_rk3_advance.  It has no counterpart in the reference.
 * For callers that can neither pass a workspace nor let the library call
 * cudaMalloc: an XLA custom call, whose device memory must come from XLA's
 * allocator (which reserves most of the GPU up front); host code with a fixed
 * device-memory budget; loops that must not stall on cudaFree, which
 * synchronises the device.  The workspace of gbf_rk3_advance lives in a fixed
 * GBF_NOALLOC_SCRATCH_BYTES (32 MiB) device array inside the library (held by
 * every GPU that loads it until the process exits), so only cases with
 * gbf_rk3_workspace_bytes(c) <= GBF_NOALLOC_SCRATCH_BYTES run (about 120 000
 * interior cells in 3-D); larger cases return GBF_ERR_SIZE before any CUDA
 * call.  Same arguments and results as gbf_rk3_advance with prims NULL and
 * without the workspace; cons and dt_state are the caller's (initialise
 * dt_state with gbf_rk3_init).  The first call on each device looks up the
 * array's device address with that device current and caches it per device
 * index; make that first call before any stream capture, and do not call it
 * again on a device after cudaDeviceReset there (the cached address is stale).
 * All calls share the one array: calls whose work overlaps on the GPU (other
 * streams, other threads) race on it.
 */
#define GBF_NOALLOC_SCRATCH_BYTES 33554432
int gbf_rk3_advance_noalloc(const gbf_case* c, double* cons, double* dt_state, int steps,
                            const gbf_tile* tile, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBFLUIDS_H */
