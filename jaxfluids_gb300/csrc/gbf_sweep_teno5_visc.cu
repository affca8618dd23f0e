// Face kernels: TENO5 on primitive variables with viscous / heat fluxes.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_teno5_visc(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_TENO5, 1>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
