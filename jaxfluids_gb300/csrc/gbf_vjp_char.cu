// Right-hand-side VJP kernels: WENO5-Z on characteristic variables (CHAR-PRIMITIVE).
#include "gbf_vjp_kernels.cuh"

namespace gbf {

int launch_vjp_char(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s) {
  return launch_vjp_riemann<RECON_WENO5Z_CHAR>(riemann, vp, grid, threads, smem, s);
}

int launch_lf_ties_char(int axis, const LfTieParams& tp, cudaStream_t s) {
  return launch_lf_ties_window_one<RECON_WENO5Z_CHAR>(axis, tp, s);
}

}  // namespace gbf
