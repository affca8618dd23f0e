// Sweep kernels: viscous / heat fluxes alone (active_physics.is_convective_flux
// = false, space_solver.py:512-587); the face flux starts at zero.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_sweep_dissipative(int mode, const SweepParams& p, int threads, size_t smem, cudaStream_t s) {
  // the reconstruction parameter only sizes the (unused) pencil box
  if (mode == MODE_RHS) return launch_sweep_one<GBF_RECON_MINMOD, RIEMANN_NONE, MODE_RHS, 1>(p, threads, smem, s);
  return GBF_ERR_UNSUPPORTED;  // fused stages run the face kernels
}

int launch_faces_dissipative(const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
                             int threads, size_t smem, cudaStream_t s) {
  return launch_faces_one<GBF_RECON_MINMOD, RIEMANN_NONE, 1>(p, ft, fb, threads, smem, s);
}

}  // namespace gbf
