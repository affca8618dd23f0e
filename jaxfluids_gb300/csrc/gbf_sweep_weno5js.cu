// Face kernels: WENO5-JS on primitive variables, inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_weno5js(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_WENO5JS, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
