// Sweep kernels: MUSCL3 with MINMOD and MINMOD-AD limiters, inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_sweep_muscl(int recon, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                       cudaStream_t s) {
  if (recon == GBF_RECON_MINMOD) {
    if (mode == MODE_RHS) return launch_sweep_riemann<GBF_RECON_MINMOD, MODE_RHS, 0>(riemann, p, threads, smem, s);
    return launch_sweep_riemann<GBF_RECON_MINMOD, MODE_STAGE, 0>(riemann, p, threads, smem, s);
  }
  if (mode == MODE_RHS) return launch_sweep_riemann<GBF_RECON_MINMOD_AD, MODE_RHS, 0>(riemann, p, threads, smem, s);
  return launch_sweep_riemann<GBF_RECON_MINMOD_AD, MODE_STAGE, 0>(riemann, p, threads, smem, s);
}

}  // namespace gbf
