// Batched fused TVD-RK3 over many independent cases of uneven size.
//
// Each RK stage walks a work list of (case, tile) pairs: one face-kernel
// launch for every active axis and one epilogue launch (gbf_batch.cuh), with the
// case's sizes, cell widths, state offsets and time-step slots.  Small cases
// that would each leave most of the GPU idle (a 64^2 case is 16 tiles of
// 16 x 16) thereby share every launch, and the whole step (per stage the face
// launches and the epilogue, then one time-step launch) has a fixed launch
// sequence that can be captured in a CUDA graph.
#include <algorithm>
#include <vector>

#include "gbf_batch.cuh"

namespace gbf {

namespace {

// Per-case maximum signal speed and minimum density of the packed states
// (time_step_size.py:96-109), one tile per work item.
__global__ void batch_reduce_kernel(const BatchParams bp, double gm1, double gamma) {
  for (int item = blockIdx.x; item < bp.ntiles; item += gridDim.x) {
    const int c = bp.worklist[2 * item];
    const int tile = bp.worklist[2 * item + 1];
    const gbf_batch_case& cs = bp.cases[c];
    const int t0 = bp.base.t[0], t1 = bp.base.t[1], t2 = bp.base.t[2];
    const int b2 = tile % cs.tiles[2];
    const int b1 = (tile / cs.tiles[2]) % cs.tiles[1];
    const int b0 = tile / (cs.tiles[2] * cs.tiles[1]);
    const int o[3] = {b0 * t0, b1 * t1, b2 * t2};
    const int e[3] = {min(t0, cs.n[0] - o[0]), min(t1, cs.n[1] - o[1]), min(t2, cs.n[2] - o[2])};
    const long long ncs = (long long)cs.n[0] * cs.n[1] * cs.n[2];
    double smax = 0.0;
    double rmin = __longlong_as_double(0x7ff0000000000000LL);
    for (int i = threadIdx.x; i < e[0] * e[1] * e[2]; i += blockDim.x) {
      const int i2 = i % e[2], i1 = (i / e[2]) % e[1], i0 = i / (e[2] * e[1]);
      const long long off = ((long long)(o[0] + i0) * cs.n[1] + (o[1] + i1)) * cs.n[2] + (o[2] + i2);
      double U[5], P[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) U[v] = bp.cons[cs.offset + v * ncs + off];
      prims_from_cons(U, P, gm1);
      const double cc = sqrt(gamma * P[4] / P[0]);
      double s = 0.0;
      if (cs.n[0] > 1) s = s + (fabs(P[1]) + cc);
      if (cs.n[1] > 1) s = s + (fabs(P[2]) + cc);
      if (cs.n[2] > 1) s = s + (fabs(P[3]) + cc);
      smax = fmax(smax, s);
      rmin = fmin(rmin, P[0]);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, d));
      rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, d));
    }
    if ((threadIdx.x & 31) == 0) {
      unsigned long long* red = reinterpret_cast<unsigned long long*>(bp.dt_states + 4 * c + 2);
      atomicMax(red, (unsigned long long)__double_as_longlong(smax));
      atomicMin(red + 1, (unsigned long long)__double_as_longlong(rmin));
    }
  }
}

// Every case's next dt from its reduction slots (time_step_size.py:97-155);
// t += previous dt when advance_time.  Resets the slots.
__global__ void batch_dt_kernel(const gbf_batch_case* cases, int ncases, double* dt_states,
                                double cfl, double eps, double fixed_dt, int advance_time,
                                double t0, int set_time) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncases) return;
  double* st = dt_states + 4 * c;
  unsigned long long* red = reinterpret_cast<unsigned long long*>(st + 2);
  if (set_time) st[1] = t0;
  if (advance_time) st[1] = st[1] + st[0];
  double dt;
  if (fixed_dt > 0.0) {
    dt = fixed_dt;
  } else {
    double mdx = INFINITY;
    for (int a = 0; a < 3; ++a)
      if (cases[c].n[a] > 1) mdx = fmin(mdx, cases[c].dx[a]);
    const double smax = __longlong_as_double((long long)red[0]);
    dt = mdx / (smax + eps);
    dt = dt * cfl;
  }
  st[0] = dt;
  red[0] = 0ull;
  red[1] = (unsigned long long)0x7ff0000000000000ull;
}

// The primitives of the packed states (per work item, its tile's cells).
__global__ void batch_prims_kernel(const BatchParams bp, double gm1, double* prims) {
  for (int item = blockIdx.x; item < bp.ntiles; item += gridDim.x) {
    const int c = bp.worklist[2 * item];
    const int tile = bp.worklist[2 * item + 1];
    SweepParams p;
    batch_case_params(bp, c, p);
    const gbf_batch_case& cs = bp.cases[c];
    int b[3], o[3], e[3];
    batch_tile(p, cs, tile, b, o, e);
    const long long ncs = (long long)cs.n[0] * cs.n[1] * cs.n[2];
    for (int j = threadIdx.x; j < e[0] * e[1] * e[2]; j += blockDim.x) {
      const int j2 = j % e[2], j1 = (j / e[2]) % e[1], j0 = j / (e[2] * e[1]);
      const long long off = ((long long)(o[0] + j0) * cs.n[1] + (o[1] + j1)) * cs.n[2] + (o[2] + j2);
      double U[5], P[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) U[v] = bp.cons[cs.offset + v * ncs + off];
      prims_from_cons(U, P, gm1);
#pragma unroll
      for (int v = 0; v < 5; ++v) prims[cs.offset + v * ncs + off] = P[v];
    }
  }
}

// The stage epilogue of every work item's cells (epilogue_cell): divergence of
// the case's face fluxes, RK combination, primitives of the new state, and in
// the last stage the case's time-step reductions.
__global__ void __launch_bounds__(256) batch_epilogue_kernel(const BatchParams bp) {
  for (int item = blockIdx.x; item < bp.ntiles; item += gridDim.x) {
    const int c = bp.worklist[2 * item];
    const int tile = bp.worklist[2 * item + 1];
    SweepParams p;
    batch_case_params(bp, c, p);
    const gbf_batch_case& cs = bp.cases[c];
    FaceBuffers fb;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const bool active = (p.active_mask >> a) & 1;
      fb.nf[a] = active ? batch_faces_per_line(p, a) : 0;
      fb.flux[a] = active ? bp.faces[a] + 2 * cs.offset : nullptr;
    }
    fb.lf_alpha = nullptr;
    double* prims_out = bp.prims_out ? bp.prims_out + cs.offset : nullptr;
    int b[3], o[3], e[3];
    batch_tile(p, cs, tile, b, o, e);
    const long long ncs = (long long)cs.n[0] * cs.n[1] * cs.n[2];
    const double dt = p.dt_state[0];
    double smax = 0.0;
    double rmin = __longlong_as_double(0x7ff0000000000000LL);
    for (int j = threadIdx.x; j < e[0] * e[1] * e[2]; j += blockDim.x) {
      const int j2 = j % e[2], j1 = (j / e[2]) % e[1], j0 = j / (e[2] * e[1]);
      const int cc[3] = {o[0] + j0, o[1] + j1, o[2] + j2};
      const long long i = ((long long)cc[0] * cs.n[1] + cc[1]) * cs.n[2] + cc[2];
      epilogue_cell(p, fb, prims_out, i, cc, ncs, dt, smax, rmin);
    }
    if (bp.reduce_dt) dt_block_reduce(p.dt_state, smax, rmin);
  }
}

__global__ void batch_slot_init_kernel(double* dt_states, int ncases) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncases) return;
  unsigned long long* red = reinterpret_cast<unsigned long long*>(dt_states + 4 * c + 2);
  red[0] = 0ull;
  red[1] = (unsigned long long)0x7ff0000000000000ull;
}

// The face kernel (every active axis) for the batch's scheme.
int launch_batch_faces(const gbf_case* c, const BatchParams& bp, int threads, size_t smem, int ctas,
                       cudaStream_t s) {
  int na = 0;
  for (int a = 0; a < 3; ++a) na += (bp.base.active_mask >> a) & 1;
  const int grid = (int)std::max(1LL, std::min((long long)ctas, (long long)na * bp.ntiles));
  // WENO5-Z / MUSCL / CHAR-ROE with HLLC or Rusanov here, the other inviscid
  // schemes in gbf_batch_schemes.cu
  const bool here = (c->riemann == GBF_RIEMANN_HLLC || c->riemann == GBF_RIEMANN_RUSANOV) &&
                    (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE || c->recon <= GBF_RECON_MINMOD_AD);
  if (!here) return launch_batch_faces_schemes(c, bp, grid, threads, smem, s);
  const bool hllc = c->riemann == GBF_RIEMANN_HLLC;
  if (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE)
    return hllc ? launch_batch_faces_one<RECON_WENO5Z_CHAR, GBF_RIEMANN_HLLC>(bp, grid, threads, smem, s)
                : launch_batch_faces_one<RECON_WENO5Z_CHAR, GBF_RIEMANN_RUSANOV>(bp, grid, threads, smem, s);
  switch (c->recon) {
    case GBF_RECON_WENO5Z:
      return hllc ? launch_batch_faces_one<GBF_RECON_WENO5Z, GBF_RIEMANN_HLLC>(bp, grid, threads, smem, s)
                  : launch_batch_faces_one<GBF_RECON_WENO5Z, GBF_RIEMANN_RUSANOV>(bp, grid, threads, smem, s);
    case GBF_RECON_MINMOD:
      return hllc ? launch_batch_faces_one<GBF_RECON_MINMOD, GBF_RIEMANN_HLLC>(bp, grid, threads, smem, s)
                  : launch_batch_faces_one<GBF_RECON_MINMOD, GBF_RIEMANN_RUSANOV>(bp, grid, threads, smem, s);
    default:
      return hllc ? launch_batch_faces_one<GBF_RECON_MINMOD_AD, GBF_RIEMANN_HLLC>(bp, grid, threads, smem, s)
                  : launch_batch_faces_one<GBF_RECON_MINMOD_AD, GBF_RIEMANN_RUSANOV>(bp, grid, threads, smem, s);
  }
}

// One batched stage: the face kernel (every active axis), then the epilogue.
int launch_batch_stage(const gbf_case* c, const BatchParams& bp, size_t smem, int threads, int ctas,
                       cudaStream_t s) {
  int st;
  if ((st = launch_batch_faces(c, bp, threads, smem, ctas, s)) != GBF_OK) return st;
  const int grid = std::max(1, std::min(ctas, bp.ntiles));
  batch_epilogue_kernel<<<grid, threads, 0, s>>>(bp);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

// Scheme checks shared by init and advance; fills the base params from a
// representative case (the largest tile shape fits every case).
int batch_setup(const gbf_case* scheme, const gbf_batch_case* cases, int ncases,
                const int32_t* worklist, int ntiles, const gbf_tile* tile, BatchParams* bp,
                int* threads, size_t* smem) {
  if (!scheme || !cases || !worklist || ncases <= 0 || ntiles <= 0 || !tile) return GBF_ERR_INVALID_ARGUMENT;
  if (scheme->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT | GBF_FLAG_INTERPOLATION_LIMITER | GBF_FLAG_GRAVITY))
    return GBF_ERR_UNSUPPORTED;
  // every inviscid PRIMITIVE and CHAR-PRIMITIVE scheme but Lax-Friedrichs, whose
  // global speed pass is per case
  if (scheme->riemann == GBF_RIEMANN_LAXFRIEDRICHS || scheme->recon_var > GBF_RECVAR_CHAR_PRIMITIVE)
    return GBF_ERR_UNSUPPORTED;
  for (int f = 0; f < 6; ++f)  // boundary value fields are per case size: not batched
    if (scheme->bc_field_values[f] || scheme->bc_field_types[f] || scheme->bc[f] == GBF_BC_MIXED)
      return GBF_ERR_UNSUPPORTED;
  // validate the scheme on a case of the tile's size (sizes vary per case)
  gbf_case rep = *scheme;
  int st = gbf_case_check(&rep);
  if (st != GBF_OK) return st;
  CaseInfo ci;
  if ((st = make_case_info(&rep, &ci)) != GBF_OK) return st;
  SweepParams p;
  size_t sweep_smem;
  if ((st = make_sweep_params(&rep, ci, tile, &p, threads, &sweep_smem)) != GBF_OK) return st;
  // the tile shape must be the one the work list was built with
  for (int a = 0; a < 3; ++a)
    if (p.t[a] != std::max(1, tile->t[a]) && rep.n[a] > 1) return GBF_ERR_INVALID_ARGUMENT;
  // shared memory of the face kernel: the largest of the axes' (a tile's faces
  // along the axis, one more on the last tile of a line)
  *smem = 0;
  for (int a = 0; a < 3; ++a) {
    if (!((ci.active_mask >> a) & 1)) continue;
    FaceTile ft{};
    for (int b = 0; b < 3; ++b) ft.t[b] = p.t[b] + (b == a ? 1 : 0);
    *smem = std::max(*smem, face_smem(&rep, ft, a));
  }
  // (plus the kernel's static copy of an item's parameters)
  if (*smem + sizeof(SweepParams) > 227 * 1024) return GBF_ERR_INVALID_ARGUMENT;
  BatchParams b{};
  b.base = p;
  b.cases = cases;
  b.worklist = worklist;
  b.ntiles = ntiles;
  *bp = b;
  return GBF_OK;
}

}  // namespace

}  // namespace gbf

using namespace gbf;

// Host-side case table and (case, tile) work list of a batch, largest cases
// first (the layout jaxfluids_gb300.batch.build_worklist builds).
static int batch_worklist(const int32_t* cells, const double* dx, int ncases, const gbf_tile* tile,
                          gbf_batch_case* cases, int32_t* worklist, int64_t capacity, int64_t* nitems,
                          int64_t* total_doubles) {
  if (!cells || !dx || ncases <= 0 || !tile || !cases || !nitems || !total_doubles) return GBF_ERR_INVALID_ARGUMENT;
  int t[3];
  for (int a = 0; a < 3; ++a) {
    bool active = false;
    for (int c = 0; c < ncases; ++c) {
      if (cells[3 * c + a] < 1) return GBF_ERR_INVALID_ARGUMENT;
      active |= cells[3 * c + a] > 1;
    }
    t[a] = active ? std::max(1, (int)tile->t[a]) : 1;
  }
  std::vector<long long> cellcount(ncases);
  long long offset = 0, items = 0;
  for (int c = 0; c < ncases; ++c) {
    gbf_batch_case& bc = cases[c];
    long long nc = 1, nt = 1;
    for (int a = 0; a < 3; ++a) {
      bc.n[a] = cells[3 * c + a];
      bc.tiles[a] = (cells[3 * c + a] + t[a] - 1) / t[a];
      bc.dx[a] = dx[3 * c + a];
      nc *= bc.n[a];
      nt *= bc.tiles[a];
    }
    bc.offset = offset;
    offset += 5 * nc;
    cellcount[c] = nc;
    items += nt;
  }
  *total_doubles = offset;
  *nitems = items;
  if (!worklist || capacity < items) return GBF_ERR_SIZE;
  std::vector<int> order(ncases);
  for (int c = 0; c < ncases; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cellcount[x] > cellcount[y]; });
  long long k = 0;
  for (int c : order) {
    const long long nt = (long long)cases[c].tiles[0] * cases[c].tiles[1] * cases[c].tiles[2];
    for (long long i = 0; i < nt; ++i) {
      worklist[2 * k] = c;
      worklist[2 * k + 1] = (int32_t)i;
      ++k;
    }
  }
  return GBF_OK;
}

extern "C" int gbf_batch_worklist(const int32_t* cells, const double* dx, int ncases, const gbf_tile* tile,
                                  gbf_batch_case* cases, int32_t* worklist, int64_t capacity, int64_t* nitems,
                                  int64_t* total_doubles) {
  return record_status(batch_worklist(cells, dx, ncases, tile, cases, worklist, capacity, nitems, total_doubles));
}

// Workspace: two stage states and two primitive buffers (total_doubles each)
// and the face fluxes of three axes (2 total_doubles each: a case's faces of
// an axis are at most 2 N per variable).
extern "C" size_t gbf_batch_workspace_bytes(int64_t total_doubles) {
  return total_doubles > 0 ? (size_t)10 * (size_t)total_doubles * sizeof(double) : 0;
}

static int gbf_batch_init_impl(const gbf_case* scheme, const gbf_batch_case* cases, int ncases,
                              const int32_t* worklist, int ntiles, const gbf_tile* tile,
                              const double* cons, double* dt_states, double t0, void* stream) {
  BatchParams bp;
  int threads;
  size_t smem;
  int st = batch_setup(scheme, cases, ncases, worklist, ntiles, tile, &bp, &threads, &smem);
  if (st != GBF_OK) return st;
  if (!cons || !dt_states) return GBF_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  const int cb = (ncases + 127) / 128;
  batch_slot_init_kernel<<<cb, 128, 0, s>>>(dt_states, ncases);
  bp.cons = cons;
  bp.dt_states = dt_states;
  batch_reduce_kernel<<<std::min(ntiles, 152 * 8), 256, 0, s>>>(bp, scheme->gamma - 1.0, scheme->gamma);
  batch_dt_kernel<<<cb, 128, 0, s>>>(cases, ncases, dt_states, scheme->cfl, scheme->eps, scheme->fixed_dt,
                                     0, t0, 1);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

extern "C" int gbf_batch_init(const gbf_case* scheme, const gbf_batch_case* cases, int ncases,
                              const int32_t* worklist, int ntiles, const gbf_tile* tile,
                              const double* cons, double* dt_states, double t0, void* stream) {
  return record_status(gbf_batch_init_impl(scheme, cases, ncases, worklist, ntiles, tile, cons, dt_states, t0, stream));
}

static int gbf_batch_advance_impl(const gbf_case* scheme, const gbf_batch_case* cases, int ncases,
                                 const int32_t* worklist, int ntiles, const gbf_tile* tile, int ctas,
                                 double* cons, double* dt_states, void* workspace,
                                 int64_t total_doubles, int steps, void* stream) {
  BatchParams bp;
  int threads;
  size_t smem;
  int st = batch_setup(scheme, cases, ncases, worklist, ntiles, tile, &bp, &threads, &smem);
  if (st != GBF_OK) return st;
  if (!cons || !dt_states || !workspace || steps < 0 || total_doubles <= 0) return GBF_ERR_INVALID_ARGUMENT;
  if (ctas <= 0) {
    int dev = 0, sms = kSms;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    ctas = 2 * sms;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* A = (double*)workspace;
  double* B = A + total_doubles;
  double* W[2] = {B + total_doubles, B + 2 * total_doubles};
  for (int a = 0; a < 3; ++a) bp.faces[a] = B + (3 + 2 * a) * total_doubles;
  const int cb = (ncases + 127) / 128;
  const int grid = std::max(1, std::min(ctas, ntiles));
  bp.dt_states = dt_states;
  if (steps == 0) return GBF_OK;
  // the primitives of U^n, once per call; every stage then writes those of its new state
  bp.cons = cons;
  batch_prims_kernel<<<grid, threads, 0, s>>>(bp, scheme->gamma - 1.0, W[0]);
  int wn = 0;
  for (int step = 0; step < steps; ++step) {
    const int w1 = 1 - wn, w2 = wn;
    bp.stage = 0; bp.cons = cons; bp.cons0 = cons; bp.out = A; bp.reduce_dt = 0;
    bp.prims = W[wn]; bp.prims_out = W[w1];
    if ((st = launch_batch_stage(scheme, bp, smem, threads, ctas, s)) != GBF_OK) return st;
    bp.stage = 1; bp.cons = A; bp.cons0 = cons; bp.out = B;
    bp.prims = W[w1]; bp.prims_out = W[w2];
    if ((st = launch_batch_stage(scheme, bp, smem, threads, ctas, s)) != GBF_OK) return st;
    bp.stage = 2; bp.cons = B; bp.cons0 = cons; bp.out = cons; bp.reduce_dt = 1;
    bp.prims = W[w2]; bp.prims_out = W[w1];
    if ((st = launch_batch_stage(scheme, bp, smem, threads, ctas, s)) != GBF_OK) return st;
    batch_dt_kernel<<<cb, 128, 0, s>>>(cases, ncases, dt_states, scheme->cfl, scheme->eps,
                                       scheme->fixed_dt, 1, 0.0, 0);
    if (cudaGetLastError() != cudaSuccess) return GBF_ERR_CUDA;
    wn = w1;
  }
  return GBF_OK;
}

extern "C" int gbf_batch_advance(const gbf_case* scheme, const gbf_batch_case* cases, int ncases,
                                 const int32_t* worklist, int ntiles, const gbf_tile* tile, int ctas,
                                 double* cons, double* dt_states, void* workspace,
                                 int64_t total_doubles, int steps, void* stream) {
  return record_status(gbf_batch_advance_impl(scheme, cases, ncases, worklist, ntiles, tile, ctas, cons, dt_states, workspace, total_doubles, steps, stream));
}
