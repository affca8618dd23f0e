// Right-hand-side VJP kernels: WENO5-Z and WENO5-JS on primitive variables.
#include "gbf_vjp_kernels.cuh"

namespace gbf {

int launch_vjp_weno5(int recon, int riemann, const VjpParams& vp, int grid, int threads, size_t smem,
                     cudaStream_t s) {
  if (recon == GBF_RECON_WENO5JS) return launch_vjp_riemann<GBF_RECON_WENO5JS>(riemann, vp, grid, threads, smem, s);
  return launch_vjp_riemann<GBF_RECON_WENO5Z>(riemann, vp, grid, threads, smem, s);
}

int launch_lf_ties_weno5(int recon, int axis, const LfTieParams& tp, cudaStream_t s) {
  if (recon == GBF_RECON_WENO5JS) return launch_lf_ties_one<GBF_RECON_WENO5JS>(axis, tp, s);
  return launch_lf_ties_one<GBF_RECON_WENO5Z>(axis, tp, s);
}

}  // namespace gbf
