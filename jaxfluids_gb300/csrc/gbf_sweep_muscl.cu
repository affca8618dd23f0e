// Face kernels: MUSCL3 with MINMOD and MINMOD-AD limiters, inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_minmod(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_MINMOD, 0>(riemann, p, ft, fb, threads, smem, s);
}

int launch_faces_minmod_ad(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_MINMOD_AD, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
