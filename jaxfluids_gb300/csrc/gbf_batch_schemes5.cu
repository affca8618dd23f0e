// Batched face kernels: WENO5-JS and TENO5 with HLLC, HLL or Rusanov.
#include "gbf_batch.cuh"

namespace gbf {

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

int launch_batch_faces_weno5_family(int recon, int riemann, const BatchParams& bp, int grid,
                                    int threads, size_t smem, cudaStream_t s) {
  if (recon == GBF_RECON_WENO5JS) return by_riemann<GBF_RECON_WENO5JS>(riemann, bp, grid, threads, smem, s);
  return by_riemann<GBF_RECON_TENO5>(riemann, bp, grid, threads, smem, s);
}

}  // namespace gbf
