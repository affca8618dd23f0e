// Face kernels: WENO5-Z on characteristic variables (CHAR-PRIMITIVE), inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_char(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<RECON_WENO5Z_CHAR, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
