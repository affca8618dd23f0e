// One fused TVD-RK3 stage on interior buffers: the face kernels of every
// active axis (gbf_faces.cuh), then the cell epilogue.  Used by the fused
// stepping (gbf_rk3_advance, gbf_rk3_stage, the allocation-free variant) and
// by the adjoint's recomputation of stage states.  The drop-in right-hand side
// runs the same face kernels on the caller's halo buffers and a divergence
// epilogue (launch_rhs_faces).
#include <algorithm>

#include "gbf_sweep_launch.cuh"

namespace gbf {

namespace {

// The cell epilogue of a stage over every cell of the case (epilogue_cell,
// dt_block_reduce in gbf_faces.cuh).
__global__ void __launch_bounds__(256) stage_epilogue_kernel(const SweepParams p, const FaceBuffers fb,
                                                             double* prims_out) {
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const double dt = p.dt_state[0];
  double smax = 0.0;
  double rmin = __longlong_as_double(0x7ff0000000000000LL);  // +inf
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cs;
       i += (long long)gridDim.x * blockDim.x) {
    const int c2 = (int)(i % p.n[2]);
    const long long r = i / p.n[2];
    const int c1 = (int)(r % p.n[1]);
    const int c0 = (int)(r / p.n[1]);
    const int c[3] = {c0, c1, c2};
    epilogue_cell(p, fb, prims_out, i, c, cs, dt, smax, rmin);
  }
  if (p.reduce_dt) dt_block_reduce(p.dt_state, smax, rmin);
}

// The drop-in right-hand side of every cell: the divergence of the face
// buffers into p.out (interior layout), nothing else.
__global__ void __launch_bounds__(256) rhs_epilogue_kernel(const SweepParams p, const FaceBuffers fb) {
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cs;
       i += (long long)gridDim.x * blockDim.x) {
    const int c2 = (int)(i % p.n[2]);
    const long long r = i / p.n[2];
    const int c1 = (int)(r % p.n[1]);
    const int c0 = (int)(r / p.n[1]);
    const int c[3] = {c0, c1, c2};
    double acc[5];
    divergence_cell(p, fb, c, acc);
#pragma unroll
    for (int v = 0; v < 5; ++v) p.out[v * cs + i] = acc[v];
  }
}

bool periodic_axis(const gbf_case* c, int a) { return c->bc[2 * a] == GBF_BC_PERIODIC; }

// Face tile of the faces of `axis`.  Each face is a long FP64 computation, so
// the tiles of a launch finish together and an SM idles once its last tile is
// done: the tile count per SM sets the tail.  Tiles of 512 faces on 256
// threads (16 along the axis; across it 2 x 16 in 3-D, 32 in 2-D, the
// contiguous axis widest) when the case has at least 12 x 512 cells per SM
// (TGV 128^3: 27 tiles per SM and axis), else 128 faces on 128 threads (16
// along the axis, 8 across; KH 512^2: 13 tiles per SM instead of 3.4,
// measured 14 % faster; the larger tiles coalesce and reuse L1 better,
// 0.4-1.5 % on the 3-D workloads).  The choice is the same for every axis,
// whose tiles share one launch.  In 1-D the tile runs along the axis.  A user
// tile (gbf_tile) gives the extents of every face kernel directly.

int make_face_tile(const CaseInfo& ci, const gbf_tile* tile, int axis, int nf, FaceTile* ft, int* threads) {
  int t[3] = {1, 1, 1};
  int thr = 256;
  const bool user = tile && (tile->t[0] > 0 || tile->t[1] > 0 || tile->t[2] > 0);
  if (user) {
    for (int a = 0; a < 3; ++a) t[a] = std::max(1, tile->t[a]);
    if (tile->threads > 0) thr = tile->threads;
  } else {
    int others[2], k = 0;
    for (int a = 0; a < 3; ++a)
      if (a != axis && (ci.active_mask & (1 << a))) others[k++] = a;
    const bool large = ci.cells >= 12LL * kSms * 512;
    thr = large ? 256 : 128;
    if (k == 0) {
      t[axis] = thr;
    } else {
      t[axis] = 16;
      if (!large) {
        t[others[k - 1]] = 8;
      } else if (k == 1) {
        t[others[0]] = 32;
      } else {
        t[others[0]] = 2;
        t[others[1]] = 16;
      }
    }
  }
  if (thr % 32 != 0 || thr < 32 || thr > 256) return GBF_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; ++a) {
    const int ext = (a == axis) ? nf : ci.n[a];
    if (ci.n[a] == 1) t[a] = 1;
    t[a] = std::min(t[a], ext);
    ft->t[a] = t[a];
    ft->tiles[a] = (ext + t[a] - 1) / t[a];
  }
  ft->nf = nf;
  *threads = thr;
  return GBF_OK;
}

// The face tiles of the axes in `mask` (nf faces per line each), one launch.
int make_face_tiles(const CaseInfo& ci, const gbf_tile* tile, int mask, const int nf[3], FaceTiles* fts,
                    int* threads) {
  int start = 0;
  *threads = 0;
  for (int a = 0; a < 3; ++a) {
    fts->start[a] = start;
    fts->ft[a] = FaceTile{{1, 1, 1}, {1, 1, 1}, 0};
    if (!(mask & (1 << a))) continue;
    int thr;
    const int st = make_face_tile(ci, tile, a, nf[a], &fts->ft[a], &thr);
    if (st != GBF_OK) return st;
    if (*threads && thr != *threads) return GBF_ERR_INVALID_ARGUMENT;
    *threads = thr;
    start += fts->ft[a].tiles[0] * fts->ft[a].tiles[1] * fts->ft[a].tiles[2];
  }
  fts->start[3] = start;
  return GBF_OK;
}

}  // namespace

// Shared memory of the face kernel of a tile set: the largest of its axes'.
size_t face_smem_tiles(const gbf_case* c, const FaceTiles& fts) {
  size_t m = 0;
  for (int a = 0; a < 3; ++a)
    if (fts.start[a + 1] > fts.start[a]) m = std::max(m, face_smem(c, fts.ft[a], a));
  return m;
}

// Shared memory of a face kernel: the pencil (primitives; conservatives too for
// the conservative reconstructions) and, for the kernels of FaceShare
// (gbf_faces.cuh), the three window-term arrays of the smoothness indicators.
size_t face_smem(const gbf_case* c, const FaceTile& ft, int axis) {
  const int R = recon_radius(c->recon);
  long long pv = 1;
  for (int b = 0; b < 3; ++b) pv *= ft.t[b] + (b == axis ? 2 * R - 1 : 0);
  const bool cons_pencil =
      c->recon_var == GBF_RECVAR_CONSERVATIVE || c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE;
  const bool share = !(c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT | GBF_FLAG_NO_CONVECTIVE)) &&
                     c->recon_var == GBF_RECVAR_PRIMITIVE &&
                     (c->recon == GBF_RECON_WENO5Z || c->recon == GBF_RECON_WENO5JS || c->recon == GBF_RECON_TENO5);
  // the dissipative fluxes' per-cell values: 5 doubles per cell of the faces'
  // normal stencils (face_flux_kernel, DissShared)
  long long sv = 0;
  if (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) {
    sv = 1;
    for (int b = 0; b < 3; ++b) sv *= ft.t[b] + (b == axis ? 3 : 0);
  }
  return (size_t)((cons_pencil ? 10 : (share ? 20 : 5)) * pv + 5 * sv) * sizeof(double);
}

namespace {

// The face kernel of the case's scheme family (as launch_sweep_schemes picks
// the tile kernel's).
int launch_faces(const gbf_case* c, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
                 int threads, size_t smem, cudaStream_t s) {
  const bool visc = (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) != 0;
  const bool chr = c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE;
  const bool cons = c->recon_var == GBF_RECVAR_CONSERVATIVE || c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE;
  const int r = c->riemann;
  if (cons && !(c->flags & GBF_FLAG_NO_CONVECTIVE)) {
    if (c->recon_var == GBF_RECVAR_CONSERVATIVE)
      return visc ? launch_faces_cons_visc(r, p, ft, fb, threads, smem, s)
                  : launch_faces_cons(r, p, ft, fb, threads, smem, s);
    return visc ? launch_faces_charcons_visc(r, p, ft, fb, threads, smem, s)
                : launch_faces_charcons(r, p, ft, fb, threads, smem, s);
  }
  if (visc) {
    if (c->flags & GBF_FLAG_NO_CONVECTIVE) return launch_faces_dissipative(p, ft, fb, threads, smem, s);
    const bool c4 = c->dissipative_stencil[0] == GBF_CENTRAL4 && c->dissipative_stencil[1] == GBF_CENTRAL4 &&
                    c->dissipative_stencil[2] == GBF_CENTRAL4;
    if (chr)
      return c4 ? launch_faces_char_visc_c4(r, p, ft, fb, threads, smem, s)
                : launch_faces_char_visc(r, p, ft, fb, threads, smem, s);
    switch (c->recon) {
      case GBF_RECON_WENO5Z:
        return c4 ? launch_faces_weno_visc_c4(r, p, ft, fb, threads, smem, s)
                  : launch_faces_weno_visc(r, p, ft, fb, threads, smem, s);
      case GBF_RECON_WENO5JS: return launch_faces_weno5js_visc(r, p, ft, fb, threads, smem, s);
      case GBF_RECON_TENO5: return launch_faces_teno5_visc(r, p, ft, fb, threads, smem, s);
      case GBF_RECON_WENO3JS: return launch_faces_visc_weno3js(r, p, ft, fb, threads, smem, s);
      case GBF_RECON_WENO3Z: return launch_faces_visc_weno3z(r, p, ft, fb, threads, smem, s);
      case GBF_RECON_MINMOD: return launch_faces_visc_minmod(r, p, ft, fb, threads, smem, s);
      case GBF_RECON_MINMOD_AD: return launch_faces_visc_minmod_ad(r, p, ft, fb, threads, smem, s);
      default: return GBF_ERR_UNSUPPORTED;
    }
  }
  if (chr) return launch_faces_char(r, p, ft, fb, threads, smem, s);
  switch (c->recon) {
    case GBF_RECON_WENO5Z: return launch_faces_weno(r, p, ft, fb, threads, smem, s);
    case GBF_RECON_WENO5JS: return launch_faces_weno5js(r, p, ft, fb, threads, smem, s);
    case GBF_RECON_TENO5: return launch_faces_teno5(r, p, ft, fb, threads, smem, s);
    case GBF_RECON_WENO3JS: return launch_faces_weno3js(r, p, ft, fb, threads, smem, s);
    case GBF_RECON_WENO3Z: return launch_faces_weno3z(r, p, ft, fb, threads, smem, s);
    case GBF_RECON_MINMOD: return launch_faces_minmod(r, p, ft, fb, threads, smem, s);
    case GBF_RECON_MINMOD_AD: return launch_faces_minmod_ad(r, p, ft, fb, threads, smem, s);
    default: return GBF_ERR_UNSUPPORTED;
  }
}

}  // namespace

// The face buffers plus 4 doubles: the Lax-Friedrichs speed slots (3) and padding.
long long stage_face_doubles(const gbf_case* c, const CaseInfo& ci) {
  long long total = 4;
  for (int a = 0; a < 3; ++a) {
    if (!(ci.active_mask & (1 << a))) continue;
    long long f = periodic_axis(c, a) ? ci.n[a] : ci.n[a] + 1;
    for (int b = 0; b < 3; ++b)
      if (b != a) f *= ci.n[b];
    total += 5 * f;
  }
  return total;
}

void stage_face_buffers(const gbf_case* c, const CaseInfo& ci, double* base, FaceBuffers* fb) {
  for (int a = 0; a < 3; ++a) {
    fb->flux[a] = nullptr;
    fb->nf[a] = 0;
    if (!(ci.active_mask & (1 << a))) continue;
    fb->nf[a] = periodic_axis(c, a) ? ci.n[a] : ci.n[a] + 1;
    long long f = fb->nf[a];
    for (int b = 0; b < 3; ++b)
      if (b != a) f *= ci.n[b];
    fb->flux[a] = base;
    base += 5 * f;
  }
  fb->lf_alpha = base;
}

// Lax-Friedrichs passes of the face kernels over a state's interior
// primitives P (U its conservatives), for the adjoint: mode 1 reduces every
// active axis' speed into alpha[0..2] (zeroed by the caller), mode 2 lists
// the ties of axis `axis` with alpha[axis] into ties (counters zeroed by the
// caller, cap entries).  The launch parameters go to *out.
int launch_lf_face_pass(const gbf_case* c, const CaseInfo& ci, const double* U, const double* P, double* alpha,
                        unsigned long long* ties, long long cap, int mode, int axis, SweepParams* out,
                        cudaStream_t s) {
  SweepParams q;
  int thr;
  size_t sm;
  int st = make_sweep_params(c, ci, nullptr, &q, &thr, &sm);
  if (st != GBF_OK) return st;
  q.cons = U;
  q.cons0 = U;
  q.prims = P;
  q.lf_alpha = alpha;
  q.speed_pass = mode;
  q.lf_ties = ties;
  q.lf_ties_cap = cap;
  q.reduce_dt = 0;
  FaceBuffers fb{};
  for (int a = 0; a < 3; ++a)
    if (ci.active_mask & (1 << a)) fb.nf[a] = periodic_axis(c, a) ? ci.n[a] : ci.n[a] + 1;
  fb.lf_alpha = alpha;
  const int mask = (mode == 2) ? (ci.active_mask & (1 << axis)) : ci.active_mask;
  FaceTiles fts;
  int threads;
  if ((st = make_face_tiles(ci, nullptr, mask, fb.nf, &fts, &threads)) != GBF_OK) return st;
  const size_t smem = face_smem_tiles(c, fts);
  if (smem > 227 * 1024) return GBF_ERR_INVALID_ARGUMENT;
  if ((st = launch_faces(c, q, fts, fb, threads, smem, s)) != GBF_OK) return st;
  if (out) *out = q;
  return GBF_OK;
}

// p carries the stage: prims (primitives of p.cons), cons, cons0, out, stage,
// reduce_dt, dt_state.  prims_out (may be null) receives the primitives of
// the new state.  Lax-Friedrichs runs a speed pass of the face kernel before
// its flux pass (LaxFriedrichs.py:25-47).
// Drop-in: every face of the reference's face arrays (N + 1 per line, also on
// a PERIODIC axis, whose end faces read the caller's halos as they are).
long long rhs_face_doubles(const CaseInfo& ci) {
  long long total = 4;
  for (int a = 0; a < 3; ++a) {
    if (!(ci.active_mask & (1 << a))) continue;
    long long f = ci.n[a] + 1;
    for (int b = 0; b < 3; ++b)
      if (b != a) f *= ci.n[b];
    total += 5 * f;
  }
  return total;
}

int launch_rhs_faces(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, const SweepParams& p,
                     double* workspace, cudaStream_t s) {
  if (!p.prims_halo || !p.out || !workspace) return GBF_ERR_INVALID_ARGUMENT;
  // the conservative reconstructions read the caller's conservatives
  const bool cons = c->recon_var == GBF_RECVAR_CONSERVATIVE || c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE;
  if (cons && !(c->flags & GBF_FLAG_NO_CONVECTIVE) && !p.cons_halo) return GBF_ERR_INVALID_ARGUMENT;
  FaceBuffers fb;
  double* base = workspace;
  for (int a = 0; a < 3; ++a) {
    fb.flux[a] = nullptr;
    fb.nf[a] = 0;
    if (!(ci.active_mask & (1 << a))) continue;
    fb.nf[a] = ci.n[a] + 1;
    long long f = fb.nf[a];
    for (int b = 0; b < 3; ++b)
      if (b != a) f *= ci.n[b];
    fb.flux[a] = base;
    base += 5 * f;
  }
  fb.lf_alpha = base;
  const bool lf = c->riemann == GBF_RIEMANN_LAXFRIEDRICHS && !(c->flags & GBF_FLAG_NO_CONVECTIVE);
  SweepParams q = p;
  int st;
  if (lf) {
    q.lf_alpha = fb.lf_alpha;
    if (cudaMemsetAsync(q.lf_alpha, 0, 3 * sizeof(double), s) != cudaSuccess) return GBF_ERR_CUDA;
  }
  FaceTiles fts;
  int threads;
  if ((st = make_face_tiles(ci, tile, ci.active_mask, fb.nf, &fts, &threads)) != GBF_OK) return st;
  const size_t smem = face_smem_tiles(c, fts);
  if (smem > 227 * 1024) return GBF_ERR_INVALID_ARGUMENT;
  if (lf) {
    // LaxFriedrichs.py:35-38: the axis speeds over every face state first
    q.speed_pass = 1;
    if ((st = launch_faces(c, q, fts, fb, threads, smem, s)) != GBF_OK) return st;
    q.speed_pass = 0;
  }
  if ((st = launch_faces(c, q, fts, fb, threads, smem, s)) != GBF_OK) return st;
  long long grid = (ci.cells + 255) / 256;
  grid = std::min<long long>(grid, 152 * 8);
  rhs_epilogue_kernel<<<(int)grid, 256, 0, s>>>(q, fb);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_rk3_stage(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, const SweepParams& p,
                     const FaceBuffers& fb, double* prims_out, cudaStream_t s) {
  const bool lf = c->riemann == GBF_RIEMANN_LAXFRIEDRICHS && !(c->flags & GBF_FLAG_NO_CONVECTIVE);
  SweepParams q = p;
  int st;
  if (lf) {
    q.lf_alpha = fb.lf_alpha;
    if (!q.lf_alpha) return GBF_ERR_INVALID_ARGUMENT;
    if (cudaMemsetAsync(q.lf_alpha, 0, 3 * sizeof(double), s) != cudaSuccess) return GBF_ERR_CUDA;
  }
  // the faces of every active axis in one launch
  FaceTiles fts;
  int threads;
  if ((st = make_face_tiles(ci, tile, ci.active_mask, fb.nf, &fts, &threads)) != GBF_OK) return st;
  const size_t smem = face_smem_tiles(c, fts);
  if (smem > 227 * 1024) return GBF_ERR_INVALID_ARGUMENT;
  if (lf) {
    q.speed_pass = 1;
    if ((st = launch_faces(c, q, fts, fb, threads, smem, s)) != GBF_OK) return st;
    q.speed_pass = 0;
  }
  if ((st = launch_faces(c, q, fts, fb, threads, smem, s)) != GBF_OK) return st;
  long long grid = (ci.cells + 255) / 256;
  grid = std::min<long long>(grid, 152 * 8);
  stage_epilogue_kernel<<<(int)grid, 256, 0, s>>>(q, fb, prims_out);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

}  // namespace gbf
