// Batched face kernels of the inviscid schemes beyond gbf_batch.cu's: HLL
// with WENO5-Z, MUSCL and CHAR-PRIMITIVE, and WENO3-JS / WENO3-Z with every
// Riemann solver here; WENO5-JS and TENO5 in gbf_batch_schemes5.cu.
#include "gbf_batch.cuh"

namespace gbf {

int launch_batch_faces_weno5_family(int recon, int riemann, const BatchParams& bp, int grid,
                                    int threads, size_t smem, cudaStream_t s);

namespace {

template <int RECON>
int by_riemann(int riemann, const BatchParams& bp, int grid, int threads, size_t smem, cudaStream_t s) {
  if (riemann == GBF_RIEMANN_HLLC)
    return launch_batch_faces_one<RECON, GBF_RIEMANN_HLLC>(bp, grid, threads, smem, s);
  if (riemann == GBF_RIEMANN_HLL)
    return launch_batch_faces_one<RECON, GBF_RIEMANN_HLL>(bp, grid, threads, smem, s);
  return launch_batch_faces_one<RECON, GBF_RIEMANN_RUSANOV>(bp, grid, threads, smem, s);
}

}  // namespace

int launch_batch_faces_schemes(const gbf_case* c, const BatchParams& bp, int grid, int threads, size_t smem,
                               cudaStream_t s) {
  if (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE) {
    if (c->riemann != GBF_RIEMANN_HLL) return GBF_ERR_UNSUPPORTED;
    return launch_batch_faces_one<RECON_WENO5Z_CHAR, GBF_RIEMANN_HLL>(bp, grid, threads, smem, s);
  }
  switch (c->recon) {
    case GBF_RECON_WENO5Z:
    case GBF_RECON_MINMOD:
    case GBF_RECON_MINMOD_AD:
      if (c->riemann != GBF_RIEMANN_HLL) return GBF_ERR_UNSUPPORTED;
      if (c->recon == GBF_RECON_WENO5Z)
        return launch_batch_faces_one<GBF_RECON_WENO5Z, GBF_RIEMANN_HLL>(bp, grid, threads, smem, s);
      if (c->recon == GBF_RECON_MINMOD)
        return launch_batch_faces_one<GBF_RECON_MINMOD, GBF_RIEMANN_HLL>(bp, grid, threads, smem, s);
      return launch_batch_faces_one<GBF_RECON_MINMOD_AD, GBF_RIEMANN_HLL>(bp, grid, threads, smem, s);
    case GBF_RECON_WENO3JS: return by_riemann<GBF_RECON_WENO3JS>(c->riemann, bp, grid, threads, smem, s);
    case GBF_RECON_WENO3Z: return by_riemann<GBF_RECON_WENO3Z>(c->riemann, bp, grid, threads, smem, s);
    case GBF_RECON_WENO5JS:
    case GBF_RECON_TENO5:
      return launch_batch_faces_weno5_family(c->recon, c->riemann, bp, grid, threads, smem, s);
    default: return GBF_ERR_UNSUPPORTED;
  }
}

}  // namespace gbf
