// Sweep kernels: WENO5-Z on the conservative variables (reconstruction_variable
// CONSERVATIVE), inviscid.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_sweep_cons_visc(int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                           cudaStream_t s);

int launch_sweep_cons(bool visc, int riemann, int mode, const SweepParams& p, int threads, size_t smem,
                      cudaStream_t s) {
  if (visc) return launch_sweep_cons_visc(riemann, mode, p, threads, smem, s);
  if (mode == MODE_RHS) return launch_sweep_riemann<RECON_WENO5Z_CONS, MODE_RHS, 0>(riemann, p, threads, smem, s);
  return GBF_ERR_UNSUPPORTED;  // fused stages run the face kernels
}

int launch_faces_cons(int riemann, const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
    int threads, size_t smem, cudaStream_t s) {
  return launch_faces_riemann<RECON_WENO5Z_CONS, 0>(riemann, p, ft, fb, threads, smem, s);
}

}  // namespace gbf
