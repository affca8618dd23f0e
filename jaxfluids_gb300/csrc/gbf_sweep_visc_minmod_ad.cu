// Face kernels: MUSCL3 with the MINMOD-AD limiter on primitive variables with viscous / heat fluxes.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_visc_minmod_ad(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_MINMOD_AD, 1>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
