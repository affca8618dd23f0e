// C ABI of the GB300 single-phase right-hand side (declarations and reference
// citations in include/gbfluids.h).  Every entry point validates its inputs,
// enqueues work on the caller's stream and returns a status code; none of
// them traps, synchronises or allocates device memory.
#include <math.h>
#include <stdint.h>

#include "gbf_kernels.cuh"

namespace gbf {

int make_case_info(const gbf_case* c, CaseInfo* ci) {
  if (!c || !ci) return GBF_ERR_INVALID_ARGUMENT;
  ci->active_mask = 0;
  ci->cells = 1;
  ci->halo_cells = 1;
  ci->nh = c->nh;
  double mdx = INFINITY;
  for (int a = 0; a < 3; ++a) {
    if (c->n[a] < 1) return GBF_ERR_SIZE;
    ci->n[a] = c->n[a];
    const bool act = c->n[a] > 1;
    if (act) {
      ci->active_mask |= 1 << a;
      if (!(c->dx[a] > 0.0)) return GBF_ERR_INVALID_ARGUMENT;
      mdx = fmin(mdx, c->dx[a]);
    }
    ci->hs[a] = act ? c->n[a] + 2 * c->nh : 1;
    ci->cells *= c->n[a];
    ci->halo_cells *= ci->hs[a];
  }
  if (ci->active_mask == 0) return GBF_ERR_SIZE;
  if (ci->cells > (1LL << 31) - 1) return GBF_ERR_SIZE;
  ci->min_dx = mdx;
  ci->fp.gamma = c->gamma;
  ci->fp.gm1 = c->gamma - 1.0;
  ci->fp.stencil_eps = c->stencil_eps;
  ci->fp.eps = c->eps;
  ci->fp.signal_speed = c->signal_speed;
  ci->fp.frozen_state = c->frozen_state;
  return GBF_OK;
}

static int check_case(const gbf_case* c, CaseInfo* ci) {
  int st = make_case_info(c, ci);
  if (st != GBF_OK) return st;
  if (c->recon < GBF_RECON_WENO5Z || c->recon > GBF_RECON_TENO5) return GBF_ERR_UNSUPPORTED;
  if (c->recon_var < GBF_RECVAR_PRIMITIVE || c->recon_var > GBF_RECVAR_CHAR_CONSERVATIVE)
    return GBF_ERR_UNSUPPORTED;
  // the characteristic and conservative reconstructions are built with WENO5-Z
  if (c->recon_var != GBF_RECVAR_PRIMITIVE && c->recon != GBF_RECON_WENO5Z) return GBF_ERR_UNSUPPORTED;
  if ((c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE || c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE) &&
      c->frozen_state != GBF_FROZEN_ARITHMETIC && c->frozen_state != GBF_FROZEN_ROE)
    return GBF_ERR_UNSUPPORTED;
  if (c->riemann < GBF_RIEMANN_HLLC || c->riemann > GBF_RIEMANN_LAXFRIEDRICHS) return GBF_ERR_UNSUPPORTED;
  if (c->signal_speed < GBF_SIGNAL_EINFELDT || c->signal_speed > GBF_SIGNAL_TORO)
    return GBF_ERR_UNSUPPORTED;
  if (c->flags & ~(GBF_FLAG_VISCOUS | GBF_FLAG_HEAT | GBF_FLAG_VISCOUS_HEAT_PRODUCTION | GBF_FLAG_NO_CONVECTIVE |
                   GBF_FLAG_INTERPOLATION_LIMITER | GBF_FLAG_LIMIT_VELOCITY | GBF_FLAG_GRAVITY))
    return GBF_ERR_INVALID_ARGUMENT;
  if ((c->flags & GBF_FLAG_LIMIT_VELOCITY) && !(c->flags & GBF_FLAG_INTERPOLATION_LIMITER))
    return GBF_ERR_INVALID_ARGUMENT;
  if ((c->flags & GBF_FLAG_NO_CONVECTIVE) && !(c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)))
    return GBF_ERR_INVALID_ARGUMENT;  // nothing to compute
  if (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) {
    // dissipative fluxes beside any convective scheme; the tangential
    // stencils read edge halos (global_prim's edge rule)
    for (int k = 0; k < 3; ++k)
      if (c->dissipative_stencil[k] != GBF_CENTRAL4 && c->dissipative_stencil[k] != GBF_CENTRAL2)
        return GBF_ERR_UNSUPPORTED;
    // centre derivatives on a ring of the reconstruction's halo width
    // (source_term_solver.py:63-71): CENTRAL4 needs 2 cells, CENTRAL2 1
    auto halos = [](int st) { return st == GBF_CENTRAL4 ? 2 : 1; };
    const int need = (c->flags & GBF_FLAG_VISCOUS)
                         ? halos(c->dissipative_stencil[0]) + halos(c->dissipative_stencil[1])
                         : 2;
    if (c->nh < need) return GBF_ERR_INVALID_ARGUMENT;
    if (!(c->mu >= 0.0) || !(c->kappa >= 0.0) || !(c->R > 0.0)) return GBF_ERR_INVALID_ARGUMENT;
  }
  if (!(c->gamma > 1.0)) return GBF_ERR_INVALID_ARGUMENT;
  const int R = recon_radius(c->recon);
  if (c->nh < R) return GBF_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; ++a) {
    if (c->n[a] > 1) {
      if (c->n[a] < c->nh) return GBF_ERR_SIZE;  // halo retrieve slices need nh interior cells
      for (int s = 0; s < 2; ++s) {
        const int f = 2 * a + s;
        const int b = c->bc[f];
        if (b < GBF_BC_PERIODIC || b > GBF_BC_MIXED) return GBF_ERR_UNSUPPORTED;
        // per-cell types exactly on MIXED faces; no value fields on PERIODIC
        // faces; values 8-byte aligned
        if ((b == GBF_BC_MIXED) != (c->bc_field_types[f] != nullptr)) return GBF_ERR_INVALID_ARGUMENT;
        if (b == GBF_BC_PERIODIC && c->bc_field_values[f]) return GBF_ERR_INVALID_ARGUMENT;
        if ((uintptr_t)c->bc_field_values[f] & 7u) return GBF_ERR_ALIGNMENT;
      }
      if ((c->bc[2 * a] == GBF_BC_PERIODIC) != (c->bc[2 * a + 1] == GBF_BC_PERIODIC))
        return GBF_ERR_INVALID_ARGUMENT;
    }
  }
  if (!(c->cfl > 0.0) && !(c->fixed_dt > 0.0)) return GBF_ERR_INVALID_ARGUMENT;
  return GBF_OK;
}

namespace {
thread_local int g_last_status = GBF_OK;
}  // namespace

int record_status(int status) {
  g_last_status = status;
  return status;
}

}  // namespace gbf

namespace gbf {

bool aligned8(const void* p) { return ((uintptr_t)p & 7u) == 0; }

// The fused steps on a workspace of gbf_rk3_workspace_bytes(c) bytes (shared
// with the allocation-free entry point, gbf_noalloc.cu).  prims: the
// primitives of cons for the first stage, or null (derived from cons).
int rk3_advance_on(const gbf_case* c, double* cons, const double* prims, double* dt_state, double* workspace,
                   int steps, const gbf_tile* tile, cudaStream_t s) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (!cons || !dt_state || !workspace || steps < 0) return GBF_ERR_INVALID_ARGUMENT;
  if (!aligned8(cons) || !aligned8(workspace) || !aligned8(dt_state) || !aligned8(prims)) return GBF_ERR_ALIGNMENT;
  SweepParams p;
  int threads;
  size_t smem;
  st = make_sweep_params(c, ci, tile, &p, &threads, &smem);
  if (st != GBF_OK) return st;
  double* A = workspace;
  double* B = A + 5 * ci.cells;
  double* W[2] = {B + 5 * ci.cells, B + 10 * ci.cells};
  FaceBuffers fb;
  stage_face_buffers(c, ci, B + 15 * ci.cells, &fb);
  unsigned long long* red = (unsigned long long*)(dt_state + 2);
  p.dt_state = dt_state;
  if (steps == 0) return GBF_OK;
  // the primitives of U^n: the caller's, or derived once per call (every
  // stage after that writes the primitives of its new state)
  const double* Pn = prims;
  int wn = -1;  // index of the W buffer holding Pn (-1: the caller's)
  if (!Pn) {
    if ((st = launch_convert(c, cons, W[0], ci.cells, 1, s)) != GBF_OK) return st;
    Pn = W[0];
    wn = 0;
  }
  for (int step = 0; step < steps; ++step) {
    const int w1 = (wn == 1) ? 0 : 1, w2 = 1 - w1;
    // U1 = U^n + dt L(U^n)
    p.stage = 0; p.cons = cons; p.cons0 = cons; p.out = A; p.prims = Pn; p.reduce_dt = 0;
    if ((st = launch_rk3_stage(c, ci, tile, p, fb, W[w1], s)) != GBF_OK) return st;
    // U2 = 3/4 U^n + 1/4 U1 + 1/4 dt L(U1)
    p.stage = 1; p.cons = A; p.out = B; p.prims = W[w1];
    if ((st = launch_rk3_stage(c, ci, tile, p, fb, W[w2], s)) != GBF_OK) return st;
    // U^{n+1} = 1/3 U^n + 2/3 U2 + 2/3 dt L(U2), written over U^n (read pointwise)
    p.stage = 2; p.cons = B; p.out = cons; p.prims = W[w2]; p.reduce_dt = 1;
    if ((st = launch_rk3_stage(c, ci, tile, p, fb, W[w1], s)) != GBF_OK) return st;
    if ((st = launch_dt_finalize(c, ci, red, dt_state, dt_state + 1, 1, s)) != GBF_OK) return st;
    Pn = W[w1];
    wn = w1;
  }
  return GBF_OK;
}

}  // namespace gbf

using namespace gbf;

extern "C" {

int gbf_last_status(void) { return g_last_status; }


int gbf_abi_version(void) { return GBF_ABI_VERSION; }

const char* gbf_status_string(int status) {
  switch (status) {
    case GBF_OK: return "ok";
    case GBF_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GBF_ERR_UNSUPPORTED: return "unsupported setup";
    case GBF_ERR_CUDA: return "CUDA launch error";
    case GBF_ERR_SIZE: return "invalid or unsupported size";
    case GBF_ERR_ALIGNMENT: return "misaligned pointer";
    default: return "unknown status";
  }
}

static int gbf_case_check_impl(const gbf_case* c) {
  CaseInfo ci;
  return check_case(c, &ci);
}

int gbf_case_check(const gbf_case* c) {
  return record_status(gbf_case_check_impl(c));
}


// The drop-in right-hand side: the face kernels on the caller's halo buffers
// (cons read by the conservative reconstructions only: required there,
// ignored elsewhere) and a divergence epilogue.  ws: the face buffers and the
// Lax-Friedrichs speed slots (rhs_face_doubles); null: allocated for the call
// from the device's stream-ordered pool and released on the same stream.
static int rhs_common(const gbf_case* c, const double* prims, const double* cons, bool cons_given, double* rhs,
                      const gbf_tile* tile, double* ws, void* stream) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (!prims || !rhs || (cons_given && !cons)) return GBF_ERR_INVALID_ARGUMENT;
  if (!aligned8(prims) || !aligned8(rhs) || (cons && !aligned8(cons))) return GBF_ERR_ALIGNMENT;
  SweepParams p;
  int threads;
  size_t smem;
  st = make_sweep_params(c, ci, tile, &p, &threads, &smem);
  if (st != GBF_OK) return st;
  p.prims_halo = prims;
  p.cons_halo = cons;
  p.out = rhs;
  cudaStream_t s = (cudaStream_t)stream;
  if (ws) return launch_rhs_faces(c, ci, tile, p, ws, s);
  void* tmp = nullptr;
  if (cudaMallocAsync(&tmp, (size_t)rhs_face_doubles(ci) * sizeof(double), s) != cudaSuccess) return GBF_ERR_CUDA;
  st = launch_rhs_faces(c, ci, tile, p, static_cast<double*>(tmp), s);
  if (cudaFreeAsync(tmp, s) != cudaSuccess && st == GBF_OK) st = GBF_ERR_CUDA;
  return st;
}

int gbf_rhs(const gbf_case* c, const double* prims, double* rhs, const gbf_tile* tile, void* stream) {
  return record_status(rhs_common(c, prims, nullptr, false, rhs, tile, nullptr, stream));
}

int gbf_rhs_cons(const gbf_case* c, const double* prims, const double* cons, double* rhs, const gbf_tile* tile,
                 void* stream) {
  return record_status(rhs_common(c, prims, cons, true, rhs, tile, nullptr, stream));
}

size_t gbf_rhs_workspace_bytes(const gbf_case* c) {
  CaseInfo ci;
  if (check_case(c, &ci) != GBF_OK) return 0;
  return (size_t)rhs_face_doubles(ci) * sizeof(double);
}

static int gbf_rhs_ws_impl(const gbf_case* c, const double* prims, const double* cons, double* rhs,
                           const gbf_tile* tile, void* workspace, void* stream) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (!workspace) return GBF_ERR_INVALID_ARGUMENT;
  if (!aligned8(workspace)) return GBF_ERR_ALIGNMENT;
  return rhs_common(c, prims, cons, false, rhs, tile, static_cast<double*>(workspace), stream);
}

int gbf_rhs_ws(const gbf_case* c, const double* prims, const double* cons, double* rhs, const gbf_tile* tile,
               void* workspace, void* stream) {
  return record_status(gbf_rhs_ws_impl(c, prims, cons, rhs, tile, workspace, stream));
}

static int gbf_volume_force_impl(const gbf_case* c, const double* cons, double* rhs, void* stream) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (!cons || !rhs) return GBF_ERR_INVALID_ARGUMENT;
  if (!aligned8(cons) || !aligned8(rhs)) return GBF_ERR_ALIGNMENT;
  if (!(c->flags & GBF_FLAG_GRAVITY)) return GBF_OK;
  return launch_volume_force(c, ci, cons, rhs, (cudaStream_t)stream);
}

int gbf_volume_force(const gbf_case* c, const double* cons, double* rhs, void* stream) {
  return record_status(gbf_volume_force_impl(c, cons, rhs, stream));
}

static int gbf_halo_fill_impl(const gbf_case* c, double* prims, double* cons, void* stream) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (!prims) return GBF_ERR_INVALID_ARGUMENT;
  // face halos, then (viscous or heat flux) the edge halos from them
  // (halo_manager.py:126-129; no vertex halos for a single phase)
  st = launch_halo_fill(c, ci, prims, cons, (cudaStream_t)stream);
  if (st != GBF_OK || !(c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT))) return st;
  return launch_halo_edges(c, ci, prims, cons, (cudaStream_t)stream);
}

int gbf_halo_fill(const gbf_case* c, double* prims, double* cons, void* stream) {
  return record_status(gbf_halo_fill_impl(c, prims, cons, stream));
}

static int gbf_prims_from_cons_impl(const gbf_case* c, const double* cons, double* prims, int64_t count,
                        void* stream) {
  if (!c || !cons || !prims || count < 0) return GBF_ERR_INVALID_ARGUMENT;
  return launch_convert(c, cons, prims, count, 1, (cudaStream_t)stream);
}

int gbf_prims_from_cons(const gbf_case* c, const double* cons, double* prims, int64_t count,
                        void* stream) {
  return record_status(gbf_prims_from_cons_impl(c, cons, prims, count, stream));
}

static int gbf_cons_from_prims_impl(const gbf_case* c, const double* prims, double* cons, int64_t count,
                        void* stream) {
  if (!c || !cons || !prims || count < 0) return GBF_ERR_INVALID_ARGUMENT;
  return launch_convert(c, prims, cons, count, 0, (cudaStream_t)stream);
}

int gbf_cons_from_prims(const gbf_case* c, const double* prims, double* cons, int64_t count,
                        void* stream) {
  return record_status(gbf_cons_from_prims_impl(c, prims, cons, count, stream));
}

static int gbf_stage_integrate_impl(const gbf_case* c, double* cons, const double* cons0, const double* rhs,
                        const double* dt, int stage, void* stream) {
  CaseInfo ci;
  int st = make_case_info(c, &ci);
  if (st != GBF_OK) return st;
  if (stage < 0 || stage > 2 || !cons || !rhs || !dt) return GBF_ERR_INVALID_ARGUMENT;
  if (stage > 0 && !cons0) return GBF_ERR_INVALID_ARGUMENT;
  return launch_stage_integrate(c, ci, cons, cons0, rhs, dt, stage, (cudaStream_t)stream);
}

int gbf_stage_integrate(const gbf_case* c, double* cons, const double* cons0, const double* rhs,
                        const double* dt, int stage, void* stream) {
  return record_status(gbf_stage_integrate_impl(c, cons, cons0, rhs, dt, stage, stream));
}

size_t gbf_dt_workspace_bytes(void) { return 2 * sizeof(unsigned long long); }

static int gbf_dt_impl(const gbf_case* c, const double* prims, double* dt_out, void* workspace, void* stream) {
  CaseInfo ci;
  int st = make_case_info(c, &ci);
  if (st != GBF_OK) return st;
  if (!prims || !dt_out || !workspace) return GBF_ERR_INVALID_ARGUMENT;
  if (!aligned8(workspace)) return GBF_ERR_ALIGNMENT;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long* red = (unsigned long long*)workspace;
  if ((st = launch_reduce_init(red, s)) != GBF_OK) return st;
  if ((st = launch_reduce_halo_prims(ci, prims, red, s)) != GBF_OK) return st;
  return launch_dt_finalize(c, ci, red, dt_out, nullptr, 0, s);
}

int gbf_dt(const gbf_case* c, const double* prims, double* dt_out, void* workspace, void* stream) {
  return record_status(gbf_dt_impl(c, prims, dt_out, workspace, stream));
}

// Fused-path workspace: the stage buffers A, B (U^1, U^2), two primitive
// buffers (the stage primitives, alternating) and the face buffers of a stage.
size_t gbf_rk3_workspace_bytes(const gbf_case* c) {
  CaseInfo ci;
  if (make_case_info(c, &ci) != GBF_OK) return 0;
  return ((size_t)4 * 5 * (size_t)ci.cells + (size_t)stage_face_doubles(c, ci)) * sizeof(double);
}

// dt_state = {dt, t, max signal speed bits, min density bits}
static int gbf_rk3_init_impl(const gbf_case* c, const double* cons, const double* prims, double* dt_state,
                             double t0, void* stream) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (!cons || !dt_state) return GBF_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  if ((st = launch_set_scalar(dt_state + 1, t0, s)) != GBF_OK) return st;
  unsigned long long* red = (unsigned long long*)(dt_state + 2);
  if ((st = launch_reduce_init(red, s)) != GBF_OK) return st;
  // the initial time step from the primitives the state was built from
  // (time_control_initializer.py:34-70), else from the conservatives
  st = prims ? launch_reduce_prims(ci, prims, red, s) : launch_reduce_cons(ci, cons, red, s);
  if (st != GBF_OK) return st;
  return launch_dt_finalize(c, ci, red, dt_state, dt_state + 1, 0, s);
}

int gbf_rk3_init(const gbf_case* c, const double* cons, const double* prims, double* dt_state, double t0,
                 void* stream) {
  return record_status(gbf_rk3_init_impl(c, cons, prims, dt_state, t0, stream));
}


static int gbf_rk3_advance_impl(const gbf_case* c, double* cons, const double* prims, double* dt_state,
                                void* workspace, int steps, const gbf_tile* tile, void* stream) {
  if (!c || !workspace) return GBF_ERR_INVALID_ARGUMENT;
  return rk3_advance_on(c, cons, prims, dt_state, (double*)workspace, steps, tile, (cudaStream_t)stream);
}

int gbf_rk3_advance(const gbf_case* c, double* cons, const double* prims, double* dt_state, void* workspace,
                    int steps, const gbf_tile* tile, void* stream) {
  return record_status(gbf_rk3_advance_impl(c, cons, prims, dt_state, workspace, steps, tile, stream));
}

static int gbf_state_check_impl(const gbf_case* c, const double* cons, uint64_t* counts, void* stream) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (!cons || !counts) return GBF_ERR_INVALID_ARGUMENT;
  if (!aligned8(cons) || !aligned8(counts)) return GBF_ERR_ALIGNMENT;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(counts, 0, 3 * sizeof(uint64_t), s) != cudaSuccess) return GBF_ERR_CUDA;
  return launch_state_check(ci, cons, (unsigned long long*)counts, s);
}

int gbf_state_check(const gbf_case* c, const double* cons, uint64_t* counts, void* stream) {
  return record_status(gbf_state_check_impl(c, cons, counts, stream));
}

static int gbf_rk3_stage_impl(const gbf_case* c, int stage, const double* cons_k, const double* cons_n,
                              double* out, double* dt_state, void* workspace, const gbf_tile* tile,
                              void* stream) {
  CaseInfo ci;
  int st = check_case(c, &ci);
  if (st != GBF_OK) return st;
  if (stage < 0 || stage > 2 || !cons_k || !cons_n || !out || !dt_state || !workspace)
    return GBF_ERR_INVALID_ARGUMENT;
  if (out == cons_k) return GBF_ERR_INVALID_ARGUMENT;  // the faces read neighbours of U^k
  if (stage == 0 && cons_k != cons_n) return GBF_ERR_INVALID_ARGUMENT;
  if (!aligned8(cons_k) || !aligned8(cons_n) || !aligned8(out) || !aligned8(dt_state) || !aligned8(workspace))
    return GBF_ERR_ALIGNMENT;
  SweepParams p;
  int threads;
  size_t smem;
  if ((st = make_sweep_params(c, ci, tile, &p, &threads, &smem)) != GBF_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // workspace as gbf_rk3_advance's: the stage primitives in the first
  // primitive buffer, the face buffers behind them
  double* Pk = (double*)workspace + 10 * ci.cells;
  FaceBuffers fb;
  stage_face_buffers(c, ci, (double*)workspace + 20 * ci.cells, &fb);
  if ((st = launch_convert(c, cons_k, Pk, ci.cells, 1, s)) != GBF_OK) return st;
  p.dt_state = dt_state;
  p.stage = stage;
  p.cons = cons_k;
  p.cons0 = cons_n;
  p.out = out;
  p.prims = Pk;
  p.reduce_dt = (stage == 2);
  if ((st = launch_rk3_stage(c, ci, tile, p, fb, nullptr, s)) != GBF_OK) return st;
  if (stage != 2) return GBF_OK;
  // the step is complete: next time step from the new state, time advanced
  unsigned long long* red = (unsigned long long*)(dt_state + 2);
  return launch_dt_finalize(c, ci, red, dt_state, dt_state + 1, 1, s);
}

int gbf_rk3_stage(const gbf_case* c, int stage, const double* cons_k, const double* cons_n, double* out,
                  double* dt_state, void* workspace, const gbf_tile* tile, void* stream) {
  return record_status(gbf_rk3_stage_impl(c, stage, cons_k, cons_n, out, dt_state, workspace, tile, stream));
}

}  // extern "C"
