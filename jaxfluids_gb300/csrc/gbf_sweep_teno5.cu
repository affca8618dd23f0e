// Sweep kernels: TENO5 on primitive variables, inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_sweep_teno5(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s) {
  if (mode == MODE_RHS) return launch_sweep_riemann<GBF_RECON_TENO5, MODE_RHS, 0>(riemann, p, threads, smem, s);
  return launch_sweep_riemann<GBF_RECON_TENO5, MODE_STAGE, 0>(riemann, p, threads, smem, s);
}

}  // namespace gbf
