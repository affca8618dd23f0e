// Sweep kernels: MUSCL3 with MINMOD and MINMOD-AD limiters, inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_sweep_muscl(int recon, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                       cudaStream_t s) {
  if (recon == GBF_RECON_MINMOD) {
    if (mode == MODE_RHS) return launch_sweep_riemann<GBF_RECON_MINMOD, MODE_RHS, 0>(riemann, p, threads, smem, s);
    return GBF_ERR_UNSUPPORTED;  // fused stages run the face kernels
  }
  if (mode == MODE_RHS) return launch_sweep_riemann<GBF_RECON_MINMOD_AD, MODE_RHS, 0>(riemann, p, threads, smem, s);
  return GBF_ERR_UNSUPPORTED;  // fused stages run the face kernels
}

int launch_faces_minmod(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_MINMOD, 0>(riemann, p, ft, fb, threads, smem, s);
}

int launch_faces_minmod_ad(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_MINMOD_AD, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
