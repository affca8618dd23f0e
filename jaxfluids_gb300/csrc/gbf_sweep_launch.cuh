// Face-kernel launch entries, one per scheme family, each defined in its own
// translation unit (gbf_sweep_<family>.cu, compiled in parallel).
#pragma once

#include "gbf_faces.cuh"
#include "gbf_kernels.cuh"

namespace gbf {

// The face kernels of one scheme family: the faces of the axes ft lists, one
// launch; the drop-in right-hand side (p.prims_halo set) or a fused stage.
#define GBF_FACES_ARGS \
  const SweepParams &p, const FaceTiles &ft, const FaceBuffers &fb, int threads, size_t smem, cudaStream_t s
int launch_faces_weno(int riemann, GBF_FACES_ARGS);
int launch_faces_weno_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_weno_visc_c4(int riemann, GBF_FACES_ARGS);
int launch_faces_char(int riemann, GBF_FACES_ARGS);
int launch_faces_char_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_char_visc_c4(int riemann, GBF_FACES_ARGS);
int launch_faces_weno5js(int riemann, GBF_FACES_ARGS);
int launch_faces_weno5js_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_teno5(int riemann, GBF_FACES_ARGS);
int launch_faces_teno5_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_weno3js(int riemann, GBF_FACES_ARGS);
int launch_faces_weno3z(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_weno3js(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_weno3z(int riemann, GBF_FACES_ARGS);
int launch_faces_minmod(int riemann, GBF_FACES_ARGS);
int launch_faces_minmod_ad(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_minmod(int riemann, GBF_FACES_ARGS);
int launch_faces_visc_minmod_ad(int riemann, GBF_FACES_ARGS);
int launch_faces_cons(int riemann, GBF_FACES_ARGS);
int launch_faces_cons_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_charcons(int riemann, GBF_FACES_ARGS);
int launch_faces_charcons_visc(int riemann, GBF_FACES_ARGS);
int launch_faces_dissipative(GBF_FACES_ARGS);
#undef GBF_FACES_ARGS

}  // namespace gbf
