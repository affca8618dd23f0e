// Per-face finite-volume building blocks.
//
// face_flux (one face from a staged pencil: reconstruction, limiter, Riemann
// flux, dissipative flux) is shared by the face kernels (gbf_faces.cuh: the
// fused stages and the drop-in right-hand side) and the batched stages
// (gbf_batch.cuh); stage_pencil stages the primitives of a tile's stencil
// cells (a "pencil box": the tile extended by the stencil radius R along the
// face axis) in shared memory from the caller's halo buffer or the stage's
// interior buffer, boundary conditions by index remapping.
//
// The path is FP64-arithmetic bound on GB300 (about 2 FP64 lanes per SM and
// clock against kilobytes of FP64 work per cell), so the layouts minimise
// repeated FP64 work rather than HBM traffic.
#pragma once

#include "gbf_physics.cuh"

namespace gbf {

// Where a stencil's primitives come from:
// MODE_RHS: a halo primitive buffer (the drop-in right-hand side).
// MODE_STAGE: interior conservatives, the primitives of each staged cell
//   derived on the way in, boundary rules by index remapping (the adjoint's
//   pencils).
// MODE_STAGE_P: an interior primitive buffer computed once per stage,
//   boundary rules by index remapping (the fused and batched stages' face
//   kernels; the dissipative stencils read it directly).
enum { MODE_RHS = 0, MODE_STAGE = 1, MODE_STAGE_P = 2 };

// Boundary values that vary along a face (gbf_case::bc_field_values /
// bc_field_types): per face the raw boundary values of every boundary cell
// (5 x nt, variable-major; WALL velocity in 1..3, DIRICHLET primitives,
// NEUMANN normal derivatives) and, for faces of several types, the type of
// every boundary cell; null where the face is uniform.
struct BcFields {
  const double* val[6];
  const signed char* type[6];
};

struct SweepParams {
  int n[3];          // interior cells per axis (1 = inactive)
  int t[3];          // tile extents
  int tiles[3];      // tiles per axis
  int nh;            // halo width of the halo buffer (MODE_RHS)
  int hs[3];         // halo buffer extents (MODE_RHS)
  int bc[6];         // boundary types, GBF_FACE_* order (MODE_STAGE)
  // per-face boundary constants: WALL [1..3] = 2 u_wall, DIRICHLET [0..4] =
  // primitives, NEUMANN [0..4] = (gradient * sign) * dx
  double bcv[6][5];
  BcFields bf;       // boundary values varying along a face
  double dx[3];      // cell size per axis (NEUMANN fields)
  double one_dx[3];  // 1 / dx per axis
  FaceParams fp;
  const double* prims_halo;  // MODE_RHS input
  const double* cons_halo;   // MODE_RHS input of the conservative reconstructions
  const double* cons;        // MODE_STAGE: stage state U^k (interior layout)
  const double* cons0;       // MODE_STAGE: step state U^n (interior layout)
  double* out;               // MODE_RHS: rhs; MODE_STAGE: U^{k+1}
  double* dt_state;          // {dt, t, max_signal, min_rho}
  int stage;                 // RK stage 0, 1, 2
  int reduce_dt;             // reduce the next time step of the new state
  int active_mask;           // bit a set when axis a is active
  // dissipative fluxes (CENTRAL4, constant transport properties)
  const double* prims;       // MODE_STAGE_P: interior primitives of the stage state
  int viscous;               // viscous flux on
  int heat;                  // heat flux on
  int heat_production;       // viscous energy flux sum_k tau_k u_k (is_viscous_heat_production)
  double mu1;                // dynamic viscosity
  double mu2;                // bulk viscosity - 2/3 mu
  double kappa;              // thermal conductivity
  double R;                  // specific gas constant
  // dissipative stencils: 0 CENTRAL4, 1 CENTRAL2 (reconstruction, centre
  // derivative, face derivative)
  int diss_recon, diss_center, diss_face;
  // interpolation limiter: 0 off, 1 density and pressure, 2 every primitive
  int limiter;
  int gravity;               // volume force on
  double g[3];               // gravity vector
  // Lax-Friedrichs (Rusanov instantiations): the per-axis dissipation speeds;
  // speed_pass 1 reduces them (max of |u| + c over the face states, as bits)
  // instead of computing fluxes; speed_pass 2 (face kernels, for the
  // adjoint) lists the face states whose speed equals the reduced one
  double* lf_alpha;
  int speed_pass;
  // speed_pass 2: lf_ties[0] entries listed, lf_ties[1 + side] ties of the
  // left (0) and right (1) states counted as the reference's face arrays hold
  // them, then the entries (LfTie) from lf_ties[4], at most lf_ties_cap
  unsigned long long* lf_ties;
  long long lf_ties_cap;
};

// One listed Lax-Friedrichs tie: bits 3.. the face's index in its axis' face
// buffer layout, bit 2 the side (0 left state, 1 right state), bits 0..1 its
// multiplicity in the reference's face arrays (2 for face -1/2 of a PERIODIC
// axis, which the arrays also hold as face N - 1/2).
struct LfTie {
  static __host__ __device__ unsigned long long pack(long long face, int side, int mult) {
    return ((unsigned long long)face << 3) | ((unsigned long long)side << 2) | (unsigned long long)mult;
  }
  static __host__ __device__ long long face(unsigned long long e) { return (long long)(e >> 3); }
  static __host__ __device__ int side(unsigned long long e) { return (int)((e >> 2) & 1); }
  static __host__ __device__ int mult(unsigned long long e) { return (int)(e & 3); }
};

// Gravity forces added to a cell's right-hand side (source_term_solver.py:165-186,
// space_solver.py:377-384): rhs[1 + i] += g_i rho, rhs[4] += (g_0 m_0 + g_1 m_1) + g_2 m_2
// from the cell's conservatives U.
__device__ __forceinline__ void add_gravity(double rhs[5], const double U[5], const double g[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) rhs[1 + i] = __dadd_rn(rhs[1 + i], __dmul_rn(g[i], U[0]));
  const double e = __dadd_rn(__dadd_rn(__dmul_rn(g[0], U[1]), __dmul_rn(g[1], U[2])), __dmul_rn(g[2], U[3]));
  rhs[4] = __dadd_rn(rhs[4], e);
}

// Boundary rule of one face (halos/outer/material.py:140-210 with the
// retrieve slices of halos/outer/boundary_condition.py:539-604): bc_src is
// the interior index along the face's axis that halo coordinate g reads
// (PERIODIC image, SYMMETRY/WALL mirror: halo layer j <- interior cell j,
// ZEROGRADIENT/NEUMANN boundary cell; DIRICHLET reads nothing), bc_apply the
// value of primitive v from the retrieved value x.
__device__ __forceinline__ int bc_src(int g, int n, int type) {
  if (g < 0) {
    if (type == GBF_BC_PERIODIC) return g + n;
    if (type == GBF_BC_SYMMETRY || type == GBF_BC_WALL) return -1 - g;
    return 0;
  }
  if (type == GBF_BC_PERIODIC) return g - n;
  if (type == GBF_BC_SYMMETRY || type == GBF_BC_WALL) return 2 * n - 1 - g;
  return n - 1;
}

__device__ __forceinline__ double bc_apply(int type, const double* bcv, int ax, int v, double x) {
  switch (type) {
    case GBF_BC_SYMMETRY:
      return (v == ax + 1) ? -x : x;
    case GBF_BC_WALL:  // 2 u_wall - u (material.py:511-513), 2 u_wall precomputed exactly
      return (v >= 1 && v <= 3) ? bcv[v] - x : x;
    case GBF_BC_DIRICHLET:
      return bcv[v];
    case GBF_BC_NEUMANN:  // P + (g sign) dx (material.py:860-862)
      return x + bcv[v];
    default:
      return x;
  }
}

// d bc_apply / d x (the adjoint's boundary transpose)
__device__ __forceinline__ double bc_apply_grad(int type, int ax, int v) {
  switch (type) {
    case GBF_BC_SYMMETRY:
      return (v == ax + 1) ? -1.0 : 1.0;
    case GBF_BC_WALL:
      return (v >= 1 && v <= 3) ? -1.0 : 1.0;
    case GBF_BC_DIRICHLET:
      return 0.0;
    default:
      return 1.0;
  }
}

// Tangential position of cell g on a face of axis a (the other two axes in
// axis order, interior coordinates) and the number of such positions.
__device__ __forceinline__ long long face_pos(const int n[3], int a, const int g[3]) {
  const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
  return (long long)g[b] * n[c] + g[c];
}
__device__ __forceinline__ long long face_npos(const int n[3], int a) {
  const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
  return (long long)n[b] * n[c];
}

// Boundary type of face f at tangential position k: per boundary cell on a
// face of several types (bounding_domain masks, outer/material.py:252-266),
// else the face's type.
__device__ __forceinline__ int face_type_at(const int bc[6], const BcFields& bf, int f, long long k) {
  return bf.type[f] ? (int)bf.type[f][k] : bc[f];
}

// bc_apply with the values of boundary cell k where face f carries a value
// field, transformed as the reference transforms the callables' values:
// 2 u_wall - u (material.py:511-513), P + (g sign) dx (material.py:860-862).
__device__ __forceinline__ double bc_apply_at(int type, const double* bcv, const BcFields& bf, int f, long long k,
                                              long long nk, double dx, int ax, int v, double x) {
  const double* fv = bf.val[f];
  if (!fv) return bc_apply(type, bcv, ax, v, x);
  switch (type) {
    case GBF_BC_WALL:
      return (v >= 1 && v <= 3) ? 2.0 * __ldg(fv + v * nk + k) - x : x;
    case GBF_BC_DIRICHLET:
      return __ldg(fv + v * nk + k);
    case GBF_BC_NEUMANN:
      return x + __dmul_rn(__ldg(fv + v * nk + k) * ((f & 1) ? -1.0 : 1.0), dx);
    default:
      return bc_apply(type, bcv, ax, v, x);
  }
}

__device__ __forceinline__ int idx3(int i0, int i1, int i2, int e1, int e2) {
  return (i0 * e1 + i1) * e2 + i2;
}

// Primitive v of an interior cell of the interior primitive buffer.
__device__ __forceinline__ double interior_prim(const SweepParams& p, int v, const int g[3]) {
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  return __ldg(p.prims + v * cs + ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2]);
}

// Primitive v of a cell outside along axis a only: the face rule of that face.
__device__ __forceinline__ double face_halo_prim(const SweepParams& p, int v, int a, int g[3]) {
  const int f = 2 * a + (g[a] >= 0 ? 1 : 0);
  const long long k = face_pos(p.n, a, g);
  const int t = face_type_at(p.bc, p.bf, f, k);
  const int ga = g[a];
  g[a] = bc_src(ga, p.n[a], t);
  const double x = (t == GBF_BC_DIRICHLET) ? 0.0 : interior_prim(p, v, g);
  g[a] = ga;
  return bc_apply_at(t, p.bcv[f], p.bf, f, k, face_npos(p.n, a), p.dx[a], a, v, x);
}

// Primitive v of a logical cell outside the interior along one or two axes,
// from the interior primitive buffer: the face rule, and for edge cells the
// edge rule of compute_edge_halos (outer/material.py:339-379, type
// combinations boundary_condition.py:128-177, :606-660): along the edge's
// faces in axis order the first PERIODIC or SYMMETRY face maps the cell onto
// the other face's halo (periodic image, or mirror with that axis' velocity
// negated); otherwise (also where a face has several types) the mean of the
// two face halos nh cells inward.  Kept out of line: only tiles on the domain boundary reach it, and inlining it
// costs the interior path registers.
static __device__ __noinline__ double halo_prim(const SweepParams& p, int v, int g0, int g1, int g2) {
  int g[3] = {g0, g1, g2};
  int out[3], k = 0;
  for (int a = 0; a < 3; ++a)
    if (g[a] < 0 || g[a] >= p.n[a]) out[k++] = a;
  if (k == 1) return face_halo_prim(p, v, out[0], g);
  const int a = out[0], b = out[1];
  const int ta = p.bc[2 * a + (g[a] >= 0 ? 1 : 0)];
  const int tb = p.bc[2 * b + (g[b] >= 0 ? 1 : 0)];
  if (ta == GBF_BC_PERIODIC || ta == GBF_BC_SYMMETRY) {
    g[a] = bc_src(g[a], p.n[a], ta);
    const double x = face_halo_prim(p, v, b, g);
    return (ta == GBF_BC_SYMMETRY && v == a + 1) ? -x : x;
  }
  if (tb == GBF_BC_PERIODIC || tb == GBF_BC_SYMMETRY) {
    g[b] = bc_src(g[b], p.n[b], tb);
    const double x = face_halo_prim(p, v, a, g);
    return (tb == GBF_BC_SYMMETRY && v == b + 1) ? -x : x;
  }
  // ANY_ANY: 0.5 * (edge '_10' + edge '_01')
  int ga[3] = {g[0], g[1], g[2]};
  ga[a] += (g[a] < 0) ? p.nh : -p.nh;
  const double A = face_halo_prim(p, v, b, ga);
  int gb[3] = {g[0], g[1], g[2]};
  gb[b] += (g[b] < 0) ? p.nh : -p.nh;
  const double B = face_halo_prim(p, v, a, gb);
  return 0.5 * (A + B);
}

// Primitive v of the logical cell (g0, g1, g2), which may lie up to nh cells
// outside the interior (face or edge halo): read from the halo buffer
// (MODE_RHS) or from the interior primitive buffer through halo_prim.
template <int MODE>
__device__ __forceinline__ double global_prim(const SweepParams& p, int v, int g0, int g1, int g2) {
  if (MODE == MODE_RHS) {
    const int b0 = (p.n[0] > 1) ? g0 + p.nh : 0;
    const int b1 = (p.n[1] > 1) ? g1 + p.nh : 0;
    const int b2 = (p.n[2] > 1) ? g2 + p.nh : 0;
    const long long cs = (long long)p.hs[0] * p.hs[1] * p.hs[2];
    return __ldg(p.prims_halo + v * cs + ((long long)b0 * p.hs[1] + b1) * p.hs[2] + b2);
  } else {
    const bool inside = (unsigned)g0 < (unsigned)p.n[0] && (unsigned)g1 < (unsigned)p.n[1] &&
                        (unsigned)g2 < (unsigned)p.n[2];
    if (inside) {
      const int g[3] = {g0, g1, g2};
      return interior_prim(p, v, g);
    }
    return halo_prim(p, v, g0, g1, g2);
  }
}

// Orders non-negative doubles as unsigned integers (for atomicMax).
__device__ __forceinline__ unsigned long long ordered_bits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// CENTRAL4 stencils: deriv_center_4.py:37-49, deriv_face_4.py:37-50, central_4.py:39-50
__device__ __forceinline__ double c4_center_deriv(double one_dx, double m2, double m1, double p1, double p2) {
  return one_dx * ((1.0 / 12.0) * (m2 - p2) + (8.0 / 12.0) * (p1 - m1));
}
__device__ __forceinline__ double c4_face_deriv(double one_dx, double m2, double m1, double c0, double p1) {
  return one_dx * ((1.0 / 24.0) * (m2 - p1) + (27.0 / 24.0) * (c0 - m1));
}
__device__ __forceinline__ double c4_face_interp(double m2, double m1, double c0, double p1) {
  return fma(-1.0 / 16.0, m2 + p1, (9.0 / 16.0) * (m1 + c0));  // -1/16 x exact
}
// CENTRAL2 stencils: deriv_center_2.py:33-44 ((1/dx) 1/2 (u[i+1] - u[i-1])),
// deriv_face_2.py:30-45 ((1/dx) (u[i] - u[i-1])), central_2.py:30-41 (1/2 (u[i-1] + u[i]))
__device__ __forceinline__ double c2_center_deriv(double one_dx, double m1, double p1) {
  return (one_dx * 0.5) * (p1 - m1);
}
__device__ __forceinline__ double c2_face_deriv(double one_dx, double m1, double c0) {
  return one_dx * (c0 - m1);
}
__device__ __forceinline__ double c2_face_interp(double m1, double c0) { return 0.5 * (m1 + c0); }

// The dissipative face stencils of one face along AX (CENTRAL4 or CENTRAL2 by
// SweepParams::diss_*).  at(k) is the value at normal offset k (cells k = -2..1
// around face q - 1/2), cell(v, kax, ax2, k2) primitive v at normal offset kax
// and offset k2 along axis ax2.
template <bool C4 = false, class At>
__device__ __forceinline__ double face_deriv_along(const SweepParams& p, double odx, const At& at) {
  return (C4 || p.diss_face == 0) ? c4_face_deriv(odx, at(-2), at(-1), at(0), at(1)) : c2_face_deriv(odx, at(-1), at(0));
}

template <int AX, bool C4 = false, class At>
__device__ __forceinline__ double face_interp_along(const SweepParams& p, const At& at) {
  return (C4 || p.diss_recon == 0) ? c4_face_interp(at(-2), at(-1), at(0), at(1)) : c2_face_interp(at(-1), at(0));
}

// gr[a][b] = d u_a / d x_b at the face (zero for inactive axes and for the
// tangential derivatives tau does not use): normal derivatives by the face
// stencil, tangential ones as face reconstructions of centre derivatives
// (source_term_solver.py compute_velocity_gradient :414-448 and
// compute_xi_derivatives_at_xj :538-580, stencils chosen at :57-118).
// The centre derivative d u_a / d x_i (i != AX) of the cell at normal offset
// kax from the face (deriv_center_4.py / deriv_center_2.py).
template <bool C4, class Cell>
__device__ __forceinline__ double centre_deriv_at(const SweepParams& p, const Cell& cell, int a, int i, int kax) {
  const double odi = p.one_dx[i];
  return (C4 || p.diss_center == 0) ? c4_center_deriv(odi, cell(1 + a, kax, i, -2), cell(1 + a, kax, i, -1),
                                                    cell(1 + a, kax, i, 1), cell(1 + a, kax, i, 2))
                                  : c2_center_deriv(odi, cell(1 + a, kax, i, -1), cell(1 + a, kax, i, 1));
}

// Per-cell values of the dissipative fluxes shared by the faces that read
// them (the face kernels form them once per pencil cell): sv[kax * sstride]
// is the temperature p / (rho R) of the cell at normal offset kax from the
// face, sv[(1 + j) * svol + kax * sstride] its centre derivative j, j = 2 t +
// which over the tangential active axes t in axis order (which 0: d u_AX / d
// x_t, 1: d u_t / d x_t).  Null: formed per face.
struct DissShared {
  const double* sv;
  int svol, sstride;
};

template <int AX, bool C4 = false, class Cell>
__device__ __forceinline__ void face_velocity_gradient(const SweepParams& p, const Cell& cell, double gr[3][3],
                                                       const DissShared& ds = DissShared{nullptr, 0, 0}) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) gr[a][b] = 0.0;
  const double odx = p.one_dx[AX];
#pragma unroll
  for (int a = 0; a < 3; ++a) gr[a][AX] = face_deriv_along<C4>(p, odx, [&](int k) { return cell(1 + a, k, AX, 0); });
  int t = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i == AX || !(p.active_mask & (1 << i))) continue;
    // d u_AX / d x_i and d u_i / d x_i
#pragma unroll
    for (int which = 0; which < 2; ++which) {
      const int a = (which == 0) ? AX : i;
      const double* sj = ds.sv ? ds.sv + (1 + 2 * t + which) * ds.svol : nullptr;
      gr[a][i] = face_interp_along<AX, C4>(p, [&](int kax) {
        return sj ? sj[kax * ds.sstride] : centre_deriv_at<C4>(p, cell, a, i, kax);
      });
    }
    ++t;
  }
}

// Viscous and heat fluxes at the face of axis AX with logical face coordinates
// q (the face lies between cells q[AX]-1 and q[AX]); source_term_solver.py
// compute_viscous_flux_xi (:264-350), compute_velocity_gradient (:414-448),
// compute_xi_derivatives_at_xj (:538-580), compute_tau (:504-536),
// compute_heat_flux_xi (:188-254).  Adds them to the convective flux F the
// way compute_rhs_xi does: F[1:5] += -visc, then F[4] += heat
// (space_solver.py:565-585).
// C4: the stencils are CENTRAL4 at compile time (else chosen by p.diss_*).
template <int AX, int MODE, bool C4>
__device__ __forceinline__ void add_dissipative_flux(const SweepParams& p, const int q[3], double F[5],
                                                     const DissShared& ds = DissShared{nullptr, 0, 0}) {
  auto cell = [&](int v, int kax, int ax2, int k2) {
    int g[3] = {q[0], q[1], q[2]};
    g[AX] += kax;
    g[ax2] += k2;
    return global_prim<MODE>(p, v, g[0], g[1], g[2]);
  };
  const double odx = p.one_dx[AX];
  if (p.viscous) {
    double gr[3][3];
    face_velocity_gradient<AX, C4>(p, cell, gr, ds);
    double tau[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      tau[k] = (p.active_mask & (1 << k)) ? p.mu1 * (gr[AX][k] + gr[k][AX]) : 0.0;
    double tr = 0.0;
    bool first = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!(p.active_mask & (1 << k))) continue;
      tr = first ? gr[k][k] : tr + gr[k][k];
      first = false;
    }
    tau[AX] = tau[AX] + p.mu2 * tr;
    double vt = 0.0;
    if (p.heat_production) {
      first = true;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (!(p.active_mask & (1 << k))) continue;
        const double vf = face_interp_along<AX, C4>(p, [&](int kax) { return cell(1 + k, kax, AX, 0); });
        vt = first ? tau[k] * vf : vt + tau[k] * vf;
        first = false;
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) F[1 + k] = F[1 + k] + (-tau[k]);
    F[4] = F[4] + (-vt);
  }
  if (p.heat) {
    const double dT = face_deriv_along<C4>(p, odx, [&](int k) {
      return ds.sv ? ds.sv[k * ds.sstride] : cell(4, k, AX, 0) / (cell(0, k, AX, 0) * p.R);
    });
    F[4] = F[4] + (-p.kappa) * dT;
  }
}

// Interpolation limiter of one reconstructed face state
// (limiter_interpolation.py:82-125, :170-188, SINGLE-PHASE): where the density
// is below 1e-12, then where the pressure (+ the ideal gas' zero background
// pressure) is below 1e-10 (precision.py:54), the first-order state w (the cell
// beside the face, weno1_js.py; w[v * stride]) replaces density and pressure
// (mode 1) or every primitive (mode 2, limit_velocity).  The reference's
// x (1 - mask) + w mask with mask 0 or 1 is this selection.  Returns the
// replaced primitives as bits (bit v), for the adjoint.
__device__ __forceinline__ unsigned positivity_limit(double P[5], const double* w, int stride, int mode) {
  unsigned replaced = 0;
#pragma unroll
  for (int check = 0; check < 2; ++check) {
    const bool m = (check == 0) ? (P[0] < 1e-12) : (P[4] < 1e-10);
    if (m) {
      if (mode == 2) {
#pragma unroll
        for (int v = 0; v < 5; ++v) P[v] = w[v * stride];
        replaced = 31u;
      } else {
        P[0] = w[0];
        P[4] = w[4 * stride];
        replaced |= 17u;
      }
    }
  }
  return replaced;
}

// Primitives of the pencil box (tile extended by R cells along AX) into
// shared memory, variable-major: from the halo buffer (MODE_RHS), from the
// interior primitive buffer (MODE_STAGE_P) or derived from the interior
// conservatives (MODE_STAGE); boundary conditions by index remapping.  CONS
// also stages the conservatives behind the primitives (sm_prim[(5 + v) pvol]):
// the halo buffer's (MODE_RHS), the state's in the interior, and in the halos
// the conservatives of the halo primitives (material.py:248-250).
template <int AX, int R, int MODE, bool CONS = false>
__device__ __forceinline__ void stage_pencil(const SweepParams& p, const int o[3], const int pe[3], int pvol,
                                             double* sm_prim) {
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  for (int i = tid; i < pvol; i += nthr) {
    const int i2 = i % pe[2];
    const int r = i / pe[2];
    const int i1 = r % pe[1];
    const int i0 = r / pe[1];
    int g[3] = {o[0] + i0, o[1] + i1, o[2] + i2};
    g[AX] -= R;
    double P[5], U[5];
    if (MODE == MODE_RHS) {
      int b[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) b[a] = (p.n[a] > 1) ? g[a] + p.nh : 0;
      const long long cs = (long long)p.hs[0] * p.hs[1] * p.hs[2];
      const long long off = ((long long)b[0] * p.hs[1] + b[1]) * p.hs[2] + b[2];
#pragma unroll
      for (int v = 0; v < 5; ++v) P[v] = __ldg(p.prims_halo + v * cs + off);
      if (CONS) {
#pragma unroll
        for (int v = 0; v < 5; ++v) U[v] = __ldg(p.cons_halo + v * cs + off);
      }
    } else {
      // halo cells along AX: the face rule applied to the primitives of the
      // retrieved interior cell (halo prims from interior prims, as the
      // reference's halo update after prims_from_cons over the buffer)
      const int ga = g[AX];
      const bool halo = ga < 0 || ga >= p.n[AX];
      const int f = 2 * AX + (ga >= 0 ? 1 : 0);
      const long long k = halo ? face_pos(p.n, AX, g) : 0;
      const int t = halo ? face_type_at(p.bc, p.bf, f, k) : -1;
      if (halo) g[AX] = bc_src(ga, p.n[AX], t);
      const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
      const long long off = ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
      if (MODE == MODE_STAGE_P) {
#pragma unroll
        for (int v = 0; v < 5; ++v) P[v] = __ldg(p.prims + v * cs + off);
        if (CONS && !halo) {
#pragma unroll
          for (int v = 0; v < 5; ++v) U[v] = p.cons[v * cs + off];
        }
      } else {
#pragma unroll
        for (int v = 0; v < 5; ++v) U[v] = p.cons[v * cs + off];
        prims_from_cons(U, P, p.fp.gm1);
      }
      if (halo) {
#pragma unroll
        for (int v = 0; v < 5; ++v)
          P[v] = bc_apply_at(t, p.bcv[f], p.bf, f, k, face_npos(p.n, AX), p.dx[AX], AX, v, P[v]);
        if (CONS) cons_from_prims(P, U, p.fp.gm1);
      }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) sm_prim[v * pvol + i] = P[v];
    if (CONS) {
#pragma unroll
      for (int v = 0; v < 5; ++v) sm_prim[(5 + v) * pvol + i] = U[v];
    }
  }
}

// Lax-Friedrichs ties (speed_pass 2): list the face states of face q whose
// speed equals the axis' reduced speed (p.lf_alpha[AX], bitwise: the same
// face states and arithmetic as the reducing pass) and count them with their
// multiplicity in the reference's face arrays (N + 1 faces per line; face
// -1/2 of a PERIODIC axis is also its face N - 1/2, whose states are the same).
template <int AX>
__device__ __forceinline__ void lf_record_ties(const SweepParams& p, const int q[3], double sL, double sR) {
  const double a = p.lf_alpha[AX];
  if (sL != a && sR != a) return;
  const bool periodic = p.bc[2 * AX] == GBF_BC_PERIODIC;
  int ext[3] = {p.n[0], p.n[1], p.n[2]};
  ext[AX] = periodic ? p.n[AX] : p.n[AX] + 1;
  const long long face = ((long long)q[0] * ext[1] + q[1]) * ext[2] + q[2];
  const int mult = (periodic && q[AX] == 0) ? 2 : 1;
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    if ((side == 0 ? sL : sR) != a) continue;
    const unsigned long long i = atomicAdd(p.lf_ties, 1ull);
    if ((long long)i < p.lf_ties_cap) p.lf_ties[4 + i] = LfTie::pack(face, side, mult);
    atomicAdd(p.lf_ties + 1 + side, (unsigned long long)mult);
  }
}

// Flux of one face along AX from a staged pencil (sm_prim, variable stride
// pvol, stride pstride along AX); `base` is the pencil index of the face's
// first stencil cell (R cells left of the face) and q the logical face
// coordinates (the face lies between cells q[AX] - 1 and q[AX]).  In a
// Lax-Friedrichs speed pass (p.speed_pass) it folds max(|u| + c) of the two
// face states into smax_faces and returns false without a flux.
// VISC: 0 no dissipative fluxes, 1 dissipative fluxes with the stencils of
// p.diss_*, 2 dissipative fluxes with CENTRAL4 stencils fixed at compile time
// SHARE (the WENO5 family on primitive variables): the smoothness indicators'
// window terms come from sm_win (weno5_window_terms of every pencil cell,
// arrays dl, dr, e of 5 x pvol each, in that order) instead of being formed
// per face.
// ds: the dissipative fluxes' per-cell values at the face's cells (see
// DissShared; null pointer: formed per face).
template <int AX, int RECON, int RIEMANN, int MODE, int VISC, bool SHARE = false>
__device__ __forceinline__ bool face_flux(const SweepParams& p, const double* sm_prim, int pvol, int pstride,
                                          int base, const int q[3], double F[5], double& smax_faces,
                                          const double* sm_win = nullptr,
                                          const DissShared& ds = DissShared{nullptr, 0, 0}) {
  constexpr int R = ReconTraits<RECON>::R;
  constexpr bool CONS = RECON == RECON_WENO5Z_CONS || RECON == RECON_WENO5Z_CHARCONS;
  double PL[5], PR[5];
  double UL[5], UR[5];  // face conservatives of the conservative reconstructions
  if (RIEMANN == RIEMANN_NONE) {
    // no convective flux: nothing to reconstruct
  } else if (RECON == RECON_WENO5Z_CONS) {
    // high_order_godunov.py:282-296
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double w[2 * R];
#pragma unroll
      for (int k = 0; k < 2 * R; ++k) w[k] = sm_prim[(5 + v) * pvol + base + k * pstride];
      reconstruct_pair<GBF_RECON_WENO5Z>(w, p.fp.stencil_eps, UL[v], UR[v]);
    }
    prims_from_cons(UL, PL, p.fp.gm1);
    prims_from_cons(UR, PR, p.fp.gm1);
  } else if (RECON == RECON_WENO5Z_CHARCONS) {
    const double* b = sm_prim + base;
    auto wu = [&](int v, int k) { return b[(5 + v) * pvol + k * pstride]; };
    auto wp = [&](int v, int k) { return b[v * pvol + k * pstride]; };
    charcons_reconstruct<AX>(wu, wp, p.fp, UL, UR);
    prims_from_cons(UL, PL, p.fp.gm1);
    prims_from_cons(UR, PR, p.fp.gm1);
  } else if (RECON == RECON_WENO5Z_CHAR) {
    const double* b = sm_prim + base;
    auto w = [&](int v, int k) { return b[v * pvol + k * pstride]; };
    char_reconstruct<AX>(w, p.fp, PL, PR);
  } else if constexpr (SHARE) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double w[6], dl[5], dr[5], e[4];
#pragma unroll
      for (int k = 0; k < 6; ++k) w[k] = sm_prim[v * pvol + base + k * pstride];
#pragma unroll
      for (int k = 1; k <= 3; ++k) dl[k] = sm_win[v * pvol + base + k * pstride];
#pragma unroll
      for (int k = 2; k <= 4; ++k) dr[k] = sm_win[(5 + v) * pvol + base + k * pstride];
#pragma unroll
      for (int k = 2; k <= 3; ++k) e[k] = sm_win[(10 + v) * pvol + base + k * pstride];
      reconstruct_pair_shared<RECON>(w, dl, dr, e, p.fp.stencil_eps, PL[v], PR[v]);
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double w[2 * R];
#pragma unroll
      for (int k = 0; k < 2 * R; ++k) w[k] = sm_prim[v * pvol + base + k * pstride];
      reconstruct_pair<(RECON >= RECON_WENO5Z_CHAR) ? GBF_RECON_WENO5Z : RECON>(w, p.fp.stencil_eps,
                                                                                PL[v], PR[v]);
    }
  }
  if (RIEMANN != RIEMANN_NONE && p.limiter) {
    const double* c = sm_prim + base + (R - 1) * pstride;  // the cell left of the face
    positivity_limit(PL, c, pvol, p.limiter);
    positivity_limit(PR, c + pstride, pvol, p.limiter);
  }
  if (RIEMANN == GBF_RIEMANN_RUSANOV && p.speed_pass) {
    // LaxFriedrichs.py:35-38: max(max |u_L| + c_L, max |u_R| + c_R) over the axis
    const double cL = speed_of_sound(PL[4], PL[0], p.fp);
    const double cR = speed_of_sound(PR[4], PR[0], p.fp);
    const double sL = fabs(PL[AX + 1]) + cL, sR = fabs(PR[AX + 1]) + cR;
    if (p.speed_pass == 2) {
      lf_record_ties<AX>(p, q, sL, sR);
      return false;
    }
    smax_faces = fmax(smax_faces, fmax(sL, sR));
    return false;
  }
  if (RIEMANN == GBF_RIEMANN_RUSANOV && p.lf_alpha) {
    double uL[5], uR[5];
    if (CONS && !p.limiter) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        uL[v] = UL[v];
        uR[v] = UR[v];
      }
    } else {
      cons_from_prims(PL, uL, p.fp.gm1);
      cons_from_prims(PR, uR, p.fp.gm1);
    }
    rusanov_alpha<AX>(PL, PR, uL, uR, p.lf_alpha[AX], F);
  } else if (CONS && RIEMANN != RIEMANN_NONE && !p.limiter) {
    riemann_flux_u<AX, RIEMANN>(PL, PR, UL, UR, p.fp, F);
  } else {
    // the limiter returns the conservatives of its primitives
    // (limiter_interpolation.py:206)
    riemann_flux<AX, RIEMANN>(PL, PR, p.fp, F);
  }
  if (VISC) add_dissipative_flux<AX, MODE, VISC == 2>(p, q, F, ds);
  return true;
}

// Warp maximum of the Lax-Friedrichs face speeds, one atomic per warp on the
// order-preserving bits of the non-negative speeds.
template <int AX>
__device__ __forceinline__ void lf_speed_reduce(const SweepParams& p, double smax_faces) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) smax_faces = fmax(smax_faces, __shfl_xor_sync(0xffffffffu, smax_faces, off));
  if ((threadIdx.x & 31) == 0)
    atomicMax(reinterpret_cast<unsigned long long*>(p.lf_alpha) + AX,
              (unsigned long long)__double_as_longlong(smax_faces));
}

// RK3 coefficients (RK3.py:27-29)
__device__ __forceinline__ double rk3_combine(int stage, double U, double U0, double rhs, double dt) {
  // time_integrator.py:34-58 + RK3.py:31-62: buf = a U + b U0 (stages 1, 2),
  // then buf += (dt * m) * rhs; kept un-contracted to follow the reference order.
  if (stage == 0) return __dadd_rn(U, __dmul_rn(__dmul_rn(dt, 1.0), rhs));
  if (stage == 1) {
    const double b = fma(0.25, U, __dmul_rn(0.75, U0));  // 0.25 U exact
    return __dadd_rn(b, __dmul_rn(__dmul_rn(dt, 0.25), rhs));
  }
  const double b = __dadd_rn(__dmul_rn(2.0 / 3.0, U), __dmul_rn(1.0 / 3.0, U0));
  return __dadd_rn(b, __dmul_rn(__dmul_rn(dt, 2.0 / 3.0), rhs));
}

}  // namespace gbf
