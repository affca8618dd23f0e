// Face kernels: viscous / heat fluxes alone (active_physics.is_convective_flux
// = false, space_solver.py:512-587); the face flux starts at zero.
#include "gbf_sweep_launch.cuh"

namespace gbf {

int launch_faces_dissipative(const SweepParams& p, const FaceTiles& ft, const FaceBuffers& fb,
                             int threads, size_t smem, cudaStream_t s) {
  return launch_faces_one<GBF_RECON_MINMOD, RIEMANN_NONE, 1>(p, ft, fb, threads, smem, s);
}

}  // namespace gbf
