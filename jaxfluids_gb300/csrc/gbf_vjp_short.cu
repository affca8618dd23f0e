// Right-hand-side VJP kernels: the four-cell stencils (WENO3-JS, WENO3-Z, MINMOD, MINMOD-AD).
#include "gbf_vjp_kernels.cuh"

namespace gbf {

int launch_vjp_short(int recon, int riemann, const VjpParams& vp, int grid, int threads, size_t smem,
                     cudaStream_t s) {
  switch (recon) {
    case GBF_RECON_WENO3JS: return launch_vjp_riemann<GBF_RECON_WENO3JS>(riemann, vp, grid, threads, smem, s);
    case GBF_RECON_WENO3Z: return launch_vjp_riemann<GBF_RECON_WENO3Z>(riemann, vp, grid, threads, smem, s);
    case GBF_RECON_MINMOD: return launch_vjp_riemann<GBF_RECON_MINMOD>(riemann, vp, grid, threads, smem, s);
    case GBF_RECON_MINMOD_AD: return launch_vjp_riemann<GBF_RECON_MINMOD_AD>(riemann, vp, grid, threads, smem, s);
    default: return GBF_ERR_UNSUPPORTED;
  }
}

int launch_lf_ties_short(int recon, int axis, const LfTieParams& tp, cudaStream_t s) {
  switch (recon) {
    case GBF_RECON_WENO3JS: return launch_lf_ties_one<GBF_RECON_WENO3JS>(axis, tp, s);
    case GBF_RECON_WENO3Z: return launch_lf_ties_one<GBF_RECON_WENO3Z>(axis, tp, s);
    case GBF_RECON_MINMOD: return launch_lf_ties_one<GBF_RECON_MINMOD>(axis, tp, s);
    case GBF_RECON_MINMOD_AD: return launch_lf_ties_one<GBF_RECON_MINMOD_AD>(axis, tp, s);
    default: return GBF_ERR_UNSUPPORTED;
  }
}

}  // namespace gbf
