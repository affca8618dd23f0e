// Face kernels: WENO5-Z on primitive variables with viscous / heat fluxes on
// CENTRAL4 stencils fixed at compile time (the dissipative_fluxes defaults).
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_weno_visc_c4(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_WENO5Z, 2>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
