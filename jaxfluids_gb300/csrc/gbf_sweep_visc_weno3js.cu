// Face kernels: WENO3-JS on primitive variables with viscous / heat fluxes.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_visc_weno3js(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_WENO3JS, 1>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
