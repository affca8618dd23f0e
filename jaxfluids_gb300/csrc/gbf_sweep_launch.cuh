// Host launch templates of the sweep kernel, shared by the translation units
// that instantiate one scheme family each (compiled in parallel).
#pragma once

#include "gbf_faces.cuh"
#include "gbf_kernels.cuh"

namespace gbf {

constexpr int kSweepMaxCellsPerThread = 4;

template <int RECON, int RIEMANN, int MODE, int VISC>
int launch_sweep_one(const SweepParams& p, int threads, size_t smem, cudaStream_t s) {
  auto kern = sweep_kernel<RECON, RIEMANN, MODE, kSweepMaxCellsPerThread, VISC>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return GBF_ERR_CUDA;
  const int grid = p.tiles[0] * p.tiles[1] * p.tiles[2];
  kern<<<grid, threads, smem, s>>>(p);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

template <int RECON, int MODE, int VISC>
int launch_sweep_riemann(int riemann, const SweepParams& p, int threads, size_t smem, cudaStream_t s) {
  if (riemann == GBF_RIEMANN_HLLC) return launch_sweep_one<RECON, GBF_RIEMANN_HLLC, MODE, VISC>(p, threads, smem, s);
  if (riemann == GBF_RIEMANN_HLL) return launch_sweep_one<RECON, GBF_RIEMANN_HLL, MODE, VISC>(p, threads, smem, s);
  return launch_sweep_one<RECON, GBF_RIEMANN_RUSANOV, MODE, VISC>(p, threads, smem, s);
}

// One entry per scheme family (gbf_sweep_<family>.cu): the tile kernel of the
// drop-in right-hand side (mode MODE_RHS; other modes return
// GBF_ERR_UNSUPPORTED: the fused stages run the face kernels below).
int launch_sweep_weno(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_weno_visc(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_char(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_char_visc(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_muscl(int recon, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                       cudaStream_t s);
int launch_sweep_weno5js(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_weno_family(int recon, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                             cudaStream_t s);
// viscous / heat fluxes with the other PRIMITIVE reconstructions, and the
// dissipative fluxes alone (no convective flux)
int launch_sweep_weno5js_visc(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_short_visc(int recon, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                            cudaStream_t s);
int launch_sweep_dissipative(int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
// WENO5-Z on the conservatives and on their characteristic variables,
// inviscid (MODE_RHS, MODE_STAGE) and with dissipative fluxes (MODE_RHS,
// MODE_STAGE_P, stencils per case)
int launch_sweep_cons(bool visc, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                      cudaStream_t s);
int launch_sweep_charcons(bool visc, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                          cudaStream_t s);
// TENO5 on primitive variables, inviscid and with viscous / heat fluxes
int launch_sweep_teno5(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_teno5_visc(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
// WENO5-Z (PRIMITIVE and CHAR-PRIMITIVE) with CENTRAL4 dissipative stencils fixed
// at compile time (VISC = 2), the default setups
int launch_sweep_weno_visc_c4(int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                              cudaStream_t s);
int launch_sweep_char_visc_c4(int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                              cudaStream_t s);


// Face kernels of the fused stages, one entry per scheme family
// (gbf_sweep_<family>.cu): the faces of the axes ft lists, one launch.
#define GBF_FACES_ARGS \
  const SweepParams &p, const FaceTiles &ft, const FaceBuffers &fb, int threads, size_t smem, cudaStream_t s
int launch_faces_weno(int riemann, GBF_FACES_ARGS);
int launch_faces_weno_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_weno_visc_c4(int riemann, GBF_FACES_ARGS);
int launch_faces_char(int riemann, GBF_FACES_ARGS);
int launch_faces_char_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_char_visc_c4(int riemann, GBF_FACES_ARGS);
int launch_faces_weno5js(int riemann, GBF_FACES_ARGS);
int launch_faces_weno5js_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_teno5(int riemann, GBF_FACES_ARGS);
int launch_faces_teno5_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_weno3js(int riemann, GBF_FACES_ARGS);
int launch_faces_weno3z(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_weno3js(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_weno3z(int riemann, GBF_FACES_ARGS);
int launch_faces_minmod(int riemann, GBF_FACES_ARGS);
int launch_faces_minmod_ad(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_minmod(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_minmod_ad(int riemann, GBF_FACES_ARGS);
int launch_faces_cons(int riemann, GBF_FACES_ARGS);
int launch_faces_cons_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_charcons(int riemann, GBF_FACES_ARGS);
int launch_faces_charcons_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_dissipative(GBF_FACES_ARGS);
#undef GBF_FACES_ARGS

}  // namespace gbf
