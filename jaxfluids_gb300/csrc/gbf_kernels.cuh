// Launch-side declarations shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include "gbf_faces.cuh"
#include "gbf_sweep.cuh"

namespace gbf {

// Streaming multiprocessors of a GB300 (the grid-size rules count waves of them).
constexpr int kSms = 152;

// Host-side view of a validated case.
struct CaseInfo {
  int n[3];
  int active_mask;
  int nh;
  int hs[3];               // halo-buffer extents
  long long cells;         // interior cells
  long long halo_cells;    // cells of a halo buffer
  double min_dx;
  FaceParams fp;
};

int make_case_info(const gbf_case* c, CaseInfo* ci);

// Records the status an entry point returns for gbf_last_status (per host
// thread) and passes it through.
int record_status(int status);

// per-face boundary constants for the kernels (gbf_sweep.cu)
void fill_bc_constants(const gbf_case* c, int f, double out[5]);
// Boundary value fields of the case (null where a face is uniform).
void fill_bc_fields(const gbf_case* c, BcFields* bf);

// fills p.{n,t,tiles,...} from the case and tile (tile null or all zero:
// the default shape, for_vjp picking the adjoint kernel's); returns status
int make_sweep_params(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, SweepParams* p,
                      int* threads, size_t* smem, bool for_vjp = false);

// The drop-in right-hand side (gbf_stage.cu): doubles of its workspace (the
// face buffers, N + 1 faces per line on every active axis, and the
// Lax-Friedrichs speed slots) and the face kernels plus divergence on the
// halo buffers p.prims_halo (p.cons_halo), into the interior buffer p.out.
long long rhs_face_doubles(const CaseInfo& ci);
int launch_rhs_faces(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, const SweepParams& p,
                     double* workspace, cudaStream_t s);

// Dynamic shared memory of a face kernel of axis `axis` with face tile ft
// (gbf_stage.cu).
size_t face_smem(const gbf_case* c, const FaceTile& ft, int axis);

// Lax-Friedrichs speed (mode 1) and tie (mode 2) passes of the face kernels
// for the adjoint (gbf_stage.cu).
int launch_lf_face_pass(const gbf_case* c, const CaseInfo& ci, const double* U, const double* P, double* alpha,
                        unsigned long long* ties, long long cap, int mode, int axis, SweepParams* out,
                        cudaStream_t s);

// The fused RK stage (gbf_stage.cu): doubles of the three face buffers (and
// the Lax-Friedrichs speed slots), their layout in a block of that size, and
// one stage (p: prims, cons, cons0, out,
// stage, reduce_dt, dt_state; prims_out, may be null, receives the primitives
// of the new state).
long long stage_face_doubles(const gbf_case* c, const CaseInfo& ci);
void stage_face_buffers(const gbf_case* c, const CaseInfo& ci, double* base, FaceBuffers* fb);
int launch_rk3_stage(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, const SweepParams& p,
                     const FaceBuffers& fb, double* prims_out, cudaStream_t s);

// The fused RK3 steps on a caller-provided workspace of
// gbf_rk3_workspace_bytes(c) bytes (gbf_api.cu); prims: the primitives of
// cons for the first stage, or null.
int rk3_advance_on(const gbf_case* c, double* cons, const double* prims, double* dt_state, double* workspace,
                   int steps, const gbf_tile* tile, cudaStream_t s);
bool aligned8(const void* p);

// auxiliary kernels (gbf_aux.cu)
// rhs[1:5] += gravity forces of the interior of the halo-buffer conservatives
int launch_volume_force(const gbf_case* c, const CaseInfo& ci, const double* cons, double* rhs, cudaStream_t s);
int launch_halo_fill(const gbf_case* c, const CaseInfo& ci, double* prims, double* cons,
                     cudaStream_t s);
// edge halos from the filled face halos (viscous / heat; no vertex halos)
int launch_halo_edges(const gbf_case* c, const CaseInfo& ci, double* prims, double* cons,
                      cudaStream_t s);
int launch_convert(const gbf_case* c, const double* in, double* out, long long count, int to_prims,
                   cudaStream_t s);
int launch_stage_integrate(const gbf_case* c, const CaseInfo& ci, double* cons,
                           const double* cons0, const double* rhs, const double* dt, int stage,
                           cudaStream_t s);
int launch_set_scalar(double* dst, double v, cudaStream_t s);
// reduction slots: red[0] = max signal speed bits, red[1] = min density bits
int launch_reduce_init(unsigned long long* red, cudaStream_t s);
int launch_reduce_halo_prims(const CaseInfo& ci, const double* prims, unsigned long long* red,
                             cudaStream_t s);
// cells with non-finite values, rho <= 0, p <= 0 added to counts[0..2]
int launch_state_check(const CaseInfo& ci, const double* cons, unsigned long long* counts, cudaStream_t s);
int launch_reduce_cons(const CaseInfo& ci, const double* cons, unsigned long long* red,
                       cudaStream_t s);
// the same reduction from an interior primitive buffer
int launch_reduce_prims(const CaseInfo& ci, const double* prims, unsigned long long* red, cudaStream_t s);
// dt from reduction slots; when advance_time, dt_state[1] += previous dt first
int launch_dt_finalize(const gbf_case* c, const CaseInfo& ci, unsigned long long* red,
                       double* dt_out, double* t_inout, int advance_time, cudaStream_t s);

}  // namespace gbf
