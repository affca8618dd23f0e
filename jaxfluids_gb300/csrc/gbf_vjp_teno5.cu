// Right-hand-side VJP kernels: TENO5 on primitive variables.
#include "gbf_vjp_kernels.cuh"

namespace gbf {

int launch_vjp_teno5(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s) {
  return launch_vjp_riemann<GBF_RECON_TENO5>(riemann, vp, grid, threads, smem, s);
}

int launch_lf_ties_teno5(int axis, const LfTieParams& tp, cudaStream_t s) {
  return launch_lf_ties_one<GBF_RECON_TENO5>(axis, tp, s);
}

}  // namespace gbf
