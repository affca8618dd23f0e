// Dispatch of the sweep kernels of the three-point reconstructions (WENO3-JS,
// WENO3-Z, MINMOD, MINMOD-AD) with viscous / heat fluxes; one translation
// unit per reconstruction (gbf_sweep_visc_<recon>.cu), compiled in parallel.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_sweep_visc_weno3js(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_visc_weno3z(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_visc_minmod(int riemann, int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s);
int launch_sweep_visc_minmod_ad(int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                                cudaStream_t s);

int launch_sweep_short_visc(int recon, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                            cudaStream_t s) {
  switch (recon) {
    case GBF_RECON_WENO3JS: return launch_sweep_visc_weno3js(riemann, mode, p, threads, smem, s);
    case GBF_RECON_WENO3Z: return launch_sweep_visc_weno3z(riemann, mode, p, threads, smem, s);
    case GBF_RECON_MINMOD: return launch_sweep_visc_minmod(riemann, mode, p, threads, smem, s);
    case GBF_RECON_MINMOD_AD: return launch_sweep_visc_minmod_ad(riemann, mode, p, threads, smem, s);
    default: return GBF_ERR_UNSUPPORTED;
  }
}

}  // namespace gbf
