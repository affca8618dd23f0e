// Face kernels: WENO5-Z on characteristic variables with viscous / heat fluxes on
// the stencils chosen per case (CENTRAL2 in any of the three).
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_char_visc(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<RECON_WENO5Z_CHAR, 1>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
