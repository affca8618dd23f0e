// Sweep kernels: WENO3-JS and WENO3-Z on primitive variables, inviscid (and
// the dispatch of the WENO5-JS / WENO3 family).
#include "gbf_sweep_launch.cuh"

namespace gbf {

namespace {

template <int RECON>
int launch_modes(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s) {
  if (mode == MODE_RHS) return launch_sweep_riemann<RECON, MODE_RHS, 0>(riemann, p, threads, smem, s);
  return GBF_ERR_UNSUPPORTED;  // fused stages run the face kernels
}

}  // namespace

int launch_sweep_weno_family(int recon, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                             cudaStream_t s) {
  switch (recon) {
    case GBF_RECON_WENO5JS: return launch_sweep_weno5js(riemann, mode, p, threads, smem, s);
    case GBF_RECON_WENO3JS: return launch_modes<GBF_RECON_WENO3JS>(riemann, mode, p, threads, smem, s);
    case GBF_RECON_WENO3Z: return launch_modes<GBF_RECON_WENO3Z>(riemann, mode, p, threads, smem, s);
    case GBF_RECON_TENO5: return launch_sweep_teno5(riemann, mode, p, threads, smem, s);
    default: return GBF_ERR_UNSUPPORTED;
  }
}

int launch_faces_weno3js(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_WENO3JS, 0>(riemann, p, ft, fb, threads, smem, s);
}

int launch_faces_weno3z(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<GBF_RECON_WENO3Z, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
