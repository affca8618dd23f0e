// Right-hand-side VJP kernels: WENO5-Z on the characteristic variables of the
// conservatives (reconstruction_variable CHAR-CONSERVATIVE).
#include "gbf_vjp_kernels.cuh"

namespace gbf {

int launch_vjp_charcons(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s) {
  return launch_vjp_riemann<RECON_WENO5Z_CHARCONS>(riemann, vp, grid, threads, smem, s);
}

int launch_lf_ties_charcons(int axis, const LfTieParams& tp, cudaStream_t s) {
  return launch_lf_ties_window_one<RECON_WENO5Z_CHARCONS>(axis, tp, s);
}

}  // namespace gbf
