// Face kernels: WENO5-Z on the characteristic variables of the conservatives
// (reconstruction_variable CHAR-CONSERVATIVE), inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_charcons(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<RECON_WENO5Z_CHARCONS, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
