// Face kernels: WENO3-JS and WENO3-Z on primitive variables, inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_weno3js(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_WENO3JS, 0>(riemann, p, ft, fb, threads, smem, s);
}

int launch_faces_weno3z(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_WENO3Z, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
