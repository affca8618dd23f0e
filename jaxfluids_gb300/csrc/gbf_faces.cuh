// The fused TVD-RK3 stage as a face kernel plus one cell epilogue.
//
// A stage of the hot path computes every face flux of the grid exactly once.
// One face-kernel launch covers the faces of every active axis with tiles of
// faces of one axis each (16 along the axis, the rest across it; the
// contiguous axis widest); a tile stages the primitives of its stencil cells
// in shared memory (from the stage's primitive buffer, boundary conditions by
// index remap) and writes the face fluxes to the face buffer of its axis.
// The epilogue kernel
// (stage_epilogue_kernel, gbf_stage.cu) then forms, per cell, the divergence
// in the reference's axis order, the RK stage combination, the primitives of
// the new state (the next stage's input, simulation_manager.py:943-944) and,
// in the last stage, the next CFL time step's reductions.
//
// Against a fused 3-D tile that sweeps all axes in shared memory, this drops
// the duplicated faces on tile boundaries ((T + 1) / T per axis, 12.5 % of
// the face work of 8^3 tiles) and the per-pencil conservative-to-primitive
// conversions (about five per cell and stage): the path is bound by FP64
// arithmetic, and the face buffers cost HBM bytes, which are not the bound.
// The face and cell arithmetic is the tile kernel's (face_flux, the same
// divergence and RK expressions), so both give bitwise equal results.
//
// Faces of an axis: N + 1 per line, N on a PERIODIC axis, whose face N - 1/2
// has the stencil of face -1/2 after the periodic wrap (the epilogue reads
// face 0 for it).
#pragma once

#include "gbf_sweep.cuh"

namespace gbf {

// Face tile of one face kernel: t[AX] faces along the axis, t[b] cells across
// it; tiles[] per axis; nf faces along AX per line.
struct FaceTile {
  int t[3];
  int tiles[3];
  int nf;
};

// The face tiles of one launch over several axes: the blocks of axis a are
// start[a] .. start[a + 1] - 1 (none for an axis not launched); start[3] is
// the grid.
struct FaceTiles {
  FaceTile ft[3];
  int start[4];
};

// Face buffers of a stage: flux[a][v * faces_a + face], faces of axis a laid
// out [E0][E1][E2] with E_a = nf[a] and the other extents the cell counts;
// lf_alpha: the Lax-Friedrichs speed slots (3 doubles of the same workspace).
struct FaceBuffers {
  double* flux[3];
  int nf[3];
  double* lf_alpha;
};

// Whether a face kernel shares the smoothness indicators' window terms
// between faces (reconstruct_pair_shared): the WENO5 family on primitive
// variables without dissipative fluxes (whose stencils read the primitive
// buffer through L1, which the larger shared-memory footprint would shrink).
// The host sizes shared memory by the same rule (gbf_stage.cu, face_smem).
template <int RECON, int RIEMANN, int VISC>
struct FaceShare {
  static constexpr bool value = VISC == 0 && RIEMANN != RIEMANN_NONE &&
                                (RECON == GBF_RECON_WENO5Z || RECON == GBF_RECON_WENO5JS || RECON == GBF_RECON_TENO5);
};

// The faces of axis AX in one face tile: origin o (logical face coordinates),
// fe faces per axis, nf faces per line along AX; fluxes to out[v * faces +
// face] (faces of the axis laid out [E0][E1][E2], E_AX = nf).  MODE_STAGE_P:
// reads the stage primitives p.prims (and, for the conservative
// reconstructions, p.cons), boundary conditions by index remapping; MODE_RHS:
// reads the caller's halo buffers p.prims_halo (and p.cons_halo) as they are
// (the drop-in right-hand side).  smem: the pencil (and the shared terms)
// sized by face_smem.  Returns the thread's Lax-Friedrichs face speed maximum
// (speed pass 1).
template <int AX, int RECON, int RIEMANN, int VISC, int MODE = MODE_STAGE_P>
__device__ __forceinline__ double face_tile_body(const SweepParams& p, const int o[3], const int fe[3], int nf,
                                                 double* out, double* smem) {
  constexpr int R = ReconTraits<RECON>::R;
  constexpr bool CONS = RECON == RECON_WENO5Z_CONS || RECON == RECON_WENO5Z_CHARCONS;
  // pencil: the stencil cells of the tile's faces, o[AX] - R .. o[AX] + fe[AX] - 2 + R
  int pe[3] = {fe[0], fe[1], fe[2]};
  pe[AX] += 2 * R - 1;
  const int pvol = pe[0] * pe[1] * pe[2];
  if (RIEMANN != RIEMANN_NONE) {
    stage_pencil<AX, R, MODE, CONS>(p, o, pe, pvol, smem);
    __syncthreads();
  }
  const int fvol = fe[0] * fe[1] * fe[2];
  const int pstride = (AX == 0) ? pe[1] * pe[2] : ((AX == 1) ? pe[2] : 1);
  // the smoothness indicators' window terms, once per pencil cell (cells with
  // both neighbours along AX in the pencil) instead of three times per face side
  constexpr bool SHARE = FaceShare<RECON, RIEMANN, VISC>::value;
  double* sm_win = smem + 5 * pvol;
  if constexpr (SHARE) {
    for (int i = threadIdx.x; i < pvol; i += blockDim.x) {
      const int i2 = i % pe[2];
      const int r = i / pe[2];
      const int i1 = r % pe[1];
      const int i0 = r / pe[1];
      const int k = (AX == 0) ? i0 : ((AX == 1) ? i1 : i2);
      if (k == 0 || k == pe[AX] - 1) continue;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double dl, dr, e;
        weno5_window_terms(smem[v * pvol + i - pstride], smem[v * pvol + i], smem[v * pvol + i + pstride], dl, dr,
                           e);
        sm_win[v * pvol + i] = dl;
        sm_win[(5 + v) * pvol + i] = dr;
        sm_win[(10 + v) * pvol + i] = e;
      }
    }
    __syncthreads();
  }
  // the dissipative fluxes' per-cell values (DissShared), once per cell of the
  // tile's faces' normal stencils (normal offsets -2..1 around each face)
  // instead of once per face reading them: the temperature and the centre
  // derivatives of the tangential velocity gradient, with the same reads and
  // arithmetic as the per-face forms
  double* sm_vis = smem + (CONS ? 10 : 5) * pvol;
  int se[3] = {fe[0], fe[1], fe[2]};
  se[AX] += 3;
  const int svol = se[0] * se[1] * se[2];
  const int sstride = (AX == 0) ? se[1] * se[2] : ((AX == 1) ? se[2] : 1);
  if (VISC > 0 && !(RIEMANN == GBF_RIEMANN_RUSANOV && p.speed_pass)) {
    // CENTRAL2 everywhere reads only normal offsets -1 and 0
    const bool c4any = VISC == 2 || p.diss_face == 0 || p.diss_recon == 0;
    for (int i = threadIdx.x; i < svol; i += blockDim.x) {
      const int s2 = i % se[2];
      const int r = i / se[2];
      const int s1 = r % se[1];
      const int s0 = r / se[1];
      const int k = (AX == 0) ? s0 : ((AX == 1) ? s1 : s2);
      if (!c4any && (k == 0 || k == se[AX] - 1)) continue;
      int gc[3] = {o[0] + s0, o[1] + s1, o[2] + s2};
      gc[AX] -= 2;
      auto cell = [&](int v, int kax, int ax2, int k2) {
        int g[3] = {gc[0], gc[1], gc[2]};
        g[AX] += kax;
        g[ax2] += k2;
        return global_prim<MODE>(p, v, g[0], g[1], g[2]);
      };
      if (p.heat) sm_vis[i] = cell(4, 0, AX, 0) / (cell(0, 0, AX, 0) * p.R);
      if (p.viscous) {
        int t = 0;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          if (ax == AX || !(p.active_mask & (1 << ax))) continue;
          sm_vis[(1 + 2 * t) * svol + i] = centre_deriv_at<VISC == 2>(p, cell, AX, ax, 0);
          sm_vis[(2 + 2 * t) * svol + i] = centre_deriv_at<VISC == 2>(p, cell, ax, ax, 0);
          ++t;
        }
      }
    }
    __syncthreads();
  }
  int ext[3] = {p.n[0], p.n[1], p.n[2]};
  ext[AX] = nf;
  const long long nfaces = (long long)ext[0] * ext[1] * ext[2];
  double smax_faces = 0.0;
  for (int f = threadIdx.x; f < fvol; f += blockDim.x) {
    const int f2 = f % fe[2];
    const int r = f / fe[2];
    const int f1 = r % fe[1];
    const int f0 = r / fe[1];
    const int base = idx3(f0, f1, f2, pe[1], pe[2]);
    const int q[3] = {o[0] + f0, o[1] + f1, o[2] + f2};
    int sf[3] = {f0, f1, f2};
    sf[AX] += 2;
    const DissShared ds{VISC > 0 ? sm_vis + idx3(sf[0], sf[1], sf[2], se[1], se[2]) : nullptr, svol, sstride};
    double F[5];
    if (!face_flux<AX, RECON, RIEMANN, MODE, VISC, SHARE>(p, smem, pvol, pstride, base, q, F, smax_faces,
                                                                   sm_win, ds))
      continue;
    const long long g = ((long long)q[0] * ext[1] + q[1]) * ext[2] + q[2];
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * nfaces + g] = F[v];
  }
  return smax_faces;
}

// The faces of axis AX in face tile b of ft, fluxes to fb; Lax-Friedrichs'
// speed pass 1 reduces the tile's face speeds.
template <int AX, int RECON, int RIEMANN, int VISC, int MODE>
__device__ __forceinline__ void face_tile(const SweepParams& p, const FaceTile& ft, const FaceBuffers& fb, int b,
                                          double* smem) {
  const int b2 = b % ft.tiles[2];
  const int b1 = (b / ft.tiles[2]) % ft.tiles[1];
  const int b0 = b / (ft.tiles[2] * ft.tiles[1]);
  const int o[3] = {b0 * ft.t[0], b1 * ft.t[1], b2 * ft.t[2]};
  int fe[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) fe[a] = min(ft.t[a], ((a == AX) ? ft.nf : p.n[a]) - o[a]);
  const double smax_faces = face_tile_body<AX, RECON, RIEMANN, VISC, MODE>(p, o, fe, ft.nf, fb.flux[AX], smem);
  if (RIEMANN == GBF_RIEMANN_RUSANOV && p.speed_pass == 1) lf_speed_reduce<AX>(p, smax_faces);
}

// One face kernel for the listed axes: block blockIdx.x is a face tile of the
// axis whose block range holds it, so the tiles of all axes share one launch
// (the last wave of one axis overlaps the next axis' tiles).  Two CTAs per SM
// (at most 128 registers; the inviscid kernels use about 110 and spill
// nothing).  The kernels issue FP64 instructions at the rate of a pure DFMA
// chain on this part; a third CTA (at most 85 registers, spilling) measured
// the same time on TGV 128^3.
template <int RECON, int RIEMANN, int VISC, int MODE>
__global__ void __launch_bounds__(256, 2)
    face_flux_kernel(const SweepParams p, const FaceTiles fts, const FaceBuffers fb) {
  extern __shared__ double smem[];
  const int b = blockIdx.x;
  if (b < fts.start[1])
    face_tile<0, RECON, RIEMANN, VISC, MODE>(p, fts.ft[0], fb, b - fts.start[0], smem);
  else if (b < fts.start[2])
    face_tile<1, RECON, RIEMANN, VISC, MODE>(p, fts.ft[1], fb, b - fts.start[1], smem);
  else
    face_tile<2, RECON, RIEMANN, VISC, MODE>(p, fts.ft[2], fb, b - fts.start[2], smem);
}

// The right-hand side of cell c (logical coordinates) from the face buffers:
// acc = ((0 + d_x) + d_y) + d_z with d_a = (1/dx_a)(F[i - 1/2] - F[i + 1/2])
// (space_solver.py:266-314, :597-599).
__device__ __forceinline__ void divergence_cell(const SweepParams& p, const FaceBuffers& fb, const int c[3],
                                                double acc[5]) {
  bool first = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (!(p.active_mask & (1 << a))) continue;
    int ext[3] = {p.n[0], p.n[1], p.n[2]};
    ext[a] = fb.nf[a];
    const long long nfaces = (long long)ext[0] * ext[1] * ext[2];
    int lo[3] = {c[0], c[1], c[2]};
    const long long flo = ((long long)lo[0] * ext[1] + lo[1]) * ext[2] + lo[2];
    lo[a] = (c[a] + 1 == fb.nf[a]) ? 0 : c[a] + 1;  // periodic: face N - 1/2 is face -1/2
    const long long fhi = ((long long)lo[0] * ext[1] + lo[1]) * ext[2] + lo[2];
    const double* F = fb.flux[a];
    const double odx = p.one_dx[a];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double d = odx * (F[v * nfaces + flo] - F[v * nfaces + fhi]);
      acc[v] = first ? d : __dadd_rn(acc[v], d);
    }
    first = false;
  }
}

// The cell epilogue of a stage at cell i (logical coordinates c, cs cells):
// the right-hand side (divergence_cell), gravity (space_solver.py:377-384), the
// RK combination (RK3.py:27-62, time_integrator.py:34-58) into p.out, the
// primitives of the new state into prims_out, and (p.reduce_dt) the maximum
// signal speed and minimum density of the new state (time_step_size.py:96-109)
// folded into smax, rmin.
__device__ __forceinline__ void epilogue_cell(const SweepParams& p, const FaceBuffers& fb, double* prims_out,
                                              long long i, const int c[3], long long cs, double dt, double& smax,
                                              double& rmin) {
  double acc[5];
  divergence_cell(p, fb, c, acc);
  double U[5], Un[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) U[v] = p.cons[v * cs + i];
  if (p.gravity) add_gravity(acc, U, p.g);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double U0 = (p.stage == 0) ? U[v] : p.cons0[v * cs + i];
    Un[v] = rk3_combine(p.stage, U[v], U0, acc[v], dt);
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) p.out[v * cs + i] = Un[v];
  if (!prims_out && !p.reduce_dt) return;
  double P[5];
  prims_from_cons(Un, P, p.fp.gm1);
  if (prims_out) {
#pragma unroll
    for (int v = 0; v < 5; ++v) prims_out[v * cs + i] = P[v];
  }
  if (p.reduce_dt) {
    const double cc = speed_of_sound(P[4], P[0], p.fp);
    double s = 0.0;
    if (p.active_mask & 1) s = s + (fabs(P[1]) + cc);
    if (p.active_mask & 2) s = s + (fabs(P[2]) + cc);
    if (p.active_mask & 4) s = s + (fabs(P[3]) + cc);
    smax = fmax(smax, s);
    rmin = fmin(rmin, P[0]);
  }
}

// The block's maximum signal speed and minimum density into the time-step
// slots dt_state[2], dt_state[3] (order-preserving bits): warp shuffle ->
// shared memory -> one atomic per CTA (max / min are exact).  Every thread
// of the block calls it.
__device__ __forceinline__ void dt_block_reduce(double* dt_state, double smax, double rmin) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, d));
    rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, d));
  }
  __shared__ double red[2][32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = smax;
    red[1][w] = rmin;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    smax = (threadIdx.x < nw) ? red[0][threadIdx.x] : 0.0;
    rmin = (threadIdx.x < nw) ? red[1][threadIdx.x] : __longlong_as_double(0x7ff0000000000000LL);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, d));
      rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, d));
    }
    if (threadIdx.x == 0) {
      atomicMax(reinterpret_cast<unsigned long long*>(dt_state + 2), ordered_bits(smax));
      atomicMin(reinterpret_cast<unsigned long long*>(dt_state + 3), ordered_bits(rmin));
    }
  }
  __syncthreads();
}

// Host side ------------------------------------------------------------------

// Launch the face kernel of the axes fts lists for one scheme (instantiated
// per scheme family in gbf_sweep_<family>.cu): MODE_RHS when p carries the
// caller's halo buffers (p.prims_halo, the drop-in right-hand side), else
// MODE_STAGE_P (the fused stages).
template <int RECON, int RIEMANN, int VISC>
int launch_faces_one(const SweepParams& p, const FaceTiles& fts, const FaceBuffers& fb, int threads, size_t smem,
                     cudaStream_t s) {
  auto kern = p.prims_halo ? face_flux_kernel<RECON, RIEMANN, VISC, MODE_RHS>
                           : face_flux_kernel<RECON, RIEMANN, VISC, MODE_STAGE_P>;
  if (fts.start[3] <= 0) return GBF_OK;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return GBF_ERR_CUDA;
  kern<<<fts.start[3], threads, smem, s>>>(p, fts, fb);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

template <int RECON, int VISC>
int launch_faces_riemann(int riemann, const SweepParams& p, const FaceTiles& fts, const FaceBuffers& fb,
                         int threads, size_t smem, cudaStream_t s) {
  if (riemann == GBF_RIEMANN_HLLC) return launch_faces_one<RECON, GBF_RIEMANN_HLLC, VISC>(p, fts, fb, threads, smem, s);
  if (riemann == GBF_RIEMANN_HLL) return launch_faces_one<RECON, GBF_RIEMANN_HLL, VISC>(p, fts, fb, threads, smem, s);
  return launch_faces_one<RECON, GBF_RIEMANN_RUSANOV, VISC>(p, fts, fb, threads, smem, s);
}

}  // namespace gbf
