/*
 * Test infrastructure, not product code: a second CPU restatement, in plain C,
 * of the single-phase right-hand side for WENO5-Z on primitive or characteristic
 * variables with HLLC, HLL (Einfeldt signal speeds) or Rusanov fluxes, with
 * CENTRAL4 viscous and heat fluxes on periodic boxes, on a
 * halo-filled primitive buffer, with its own face halos, CFL time step and
 * TVD-RK3 steps; multi-threaded with OpenMP where built with it (the CPU
 * baseline of the benchmark).  It is written independently of the torch restatement in
 * jf_oracle.py and follows
 * the same reference operations in the same order, so the two must agree
 * bitwise; the tests check that (tests/test_oracle_c.py).  Compile without
 * contraction (-ffp-contract=off): the reference rounds every product.
 *
 *   reconstruction   stencils/reconstruction/shock_capturing/weno/weno5_z.py:24-58,
 *                    weno5_base.py:24-51 (smoothness, polynomials, eps = 1e-30)
 *   CHAR-PRIMITIVE   high_order_godunov.py:298-316; eigendecomposition.py:120-281
 *                    (frozen state, ARITHMETIC and ROE), :402-433 and :499-523
 *                    (primitive <-> characteristic transforms)
 *   conversions      equation_manager.py:93-101, :164-171; ideal_gas.py:69-88
 *   physical flux    equation_manager.py:237-252
 *   HLLC             solvers/riemann_solvers/HLLC.py:41-126,
 *                    signal_speeds.py:109-133 (Einfeldt), :159-199 (S*)
 *   HLL              solvers/riemann_solvers/HLL.py:28-58 (eps = machine
 *                    epsilon, riemann_solver.py:28)
 *   Rusanov          solvers/riemann_solvers/Rusanov.py:25-47
 *   divergence       solvers/space_solver.py:266-314, :597-599
 *   face halos       halos/outer/material.py:868-894,
 *                    halos/outer/boundary_condition.py:539-604
 *   viscous, heat    solvers/source_term_solver.py:188-254, :264-350,
 *                    :504-580; deriv_center_4.py, deriv_face_4.py, central_4.py;
 *                    space_solver.py:565-585
 *   time step        time_integration/time_step_size.py:15-157 (CFL, viscous
 *                    and heat limits)
 *   TVD-RK3          time_integration/RK3.py:27-62, simulation_manager.py:670-1077
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

/* Built with -fopenmp the cell and face loops run on every host core (the
   arithmetic of each cell and face is unchanged, so the results are too). */
#ifdef _OPENMP
#define JF_OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define JF_OMP_FOR
#endif

static double weno5z(double u0, double u1, double u2, double u3, double u4, double eps) {
  const double t0 = u0 - 2.0 * u1 + u2, t1 = u0 - 4.0 * u1 + 3.0 * u2;
  const double t2 = u1 - 2.0 * u2 + u3, t3 = u1 - u3;
  const double t4 = u2 - 2.0 * u3 + u4, t5 = 3.0 * u2 - 4.0 * u3 + u4;
  const double b0 = 13.0 / 12.0 * (t0 * t0) + 1.0 / 4.0 * (t1 * t1);
  const double b1 = 13.0 / 12.0 * (t2 * t2) + 1.0 / 4.0 * (t3 * t3);
  const double b2 = 13.0 / 12.0 * (t4 * t4) + 1.0 / 4.0 * (t5 * t5);
  const double tau5 = fabs(b0 - b2);
  const double a0 = 0.1 * (1.0 + tau5 / (b0 + eps));
  const double a1 = 0.6 * (1.0 + tau5 / (b1 + eps));
  const double a2 = 0.3 * (1.0 + tau5 / (b2 + eps));
  const double one_a = 1.0 / (a0 + a1 + a2);
  const double w0 = a0 * one_a, w1 = a1 * one_a, w2 = a2 * one_a;
  const double p0 = 1.0 / 3.0 * u0 + -7.0 / 6.0 * u1 + 11.0 / 6.0 * u2;
  const double p1 = -1.0 / 6.0 * u1 + 5.0 / 6.0 * u2 + 1.0 / 3.0 * u3;
  const double p2 = 1.0 / 3.0 * u2 + 5.0 / 6.0 * u3 + -1.0 / 6.0 * u4;
  return w0 * p0 + w1 * p1 + w2 * p2;
}

static void cons_from_prims(const double P[5], double U[5], double gamma) {
  const double rho = P[0];
  const double e = P[4] / (rho * (gamma - 1.0));
  const double s = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
  U[0] = rho;
  U[1] = rho * P[1];
  U[2] = rho * P[2];
  U[3] = rho * P[3];
  U[4] = rho * (0.5 * s + e);
}

static void physical_flux(const double P[5], const double U[5], int n, double F[5]) {
  F[0] = U[n];
  F[1] = U[n] * P[1];
  F[2] = U[n] * P[2];
  F[3] = U[n] * P[3];
  F[4] = P[n] * (U[4] + P[4]);
  F[n] = F[n] + P[4];
}

static void hllc_star_flux(const double P[5], const double U[5], double S, double Ss, int n, int left,
                           double out[5]) {
  const double pre = (S - P[n]) / (S - Ss) * P[0];
  const double e_term = pre * (U[4] / U[0] + (Ss - P[n]) * (Ss + P[4] / P[0] / (S - P[n])));
  double us[5] = {pre, pre, pre, pre, e_term};
  for (int t = 1; t <= 3; ++t) us[t] = (t == n) ? us[t] * Ss : us[t] * P[t];
  double F[5];
  physical_flux(P, U, n, F);
  const double wave = left ? fmin(S, 0.0) : fmax(S, 0.0);
  for (int v = 0; v < 5; ++v) out[v] = F[v] + wave * (us[v] - U[v]);
}

/* Einfeldt's wave-speed estimates (signal_speeds.py:109-133) from the face
   states' normal velocities uL, uR and speeds of sound cL, cR. */
static void einfeldt(const double PL[5], const double PR[5], int n, double cL, double cR, double* SL,
                     double* SR) {
  const double uL = PL[n], uR = PR[n];
  const double sL = sqrt(PL[0]), sR = sqrt(PR[0]);
  const double od = 1.0 / (sL + sR);
  const double eta2 = 0.5 * sL * sR * od * od;
  const double ubar = (sL * uL + sR * uR) * od;
  const double du = uR - uL;
  const double dbar = sqrt((sL * cL * cL + sR * cR * cR) * od + eta2 * (du * du));
  *SL = fmin(ubar - dbar, uL - cL);
  *SR = fmax(ubar + dbar, uR + cR);
}

static void hllc_einfeldt(const double PL[5], const double PR[5], int n, double gamma, double F[5]) {
  double UL[5], UR[5];
  cons_from_prims(PL, UL, gamma);
  cons_from_prims(PR, UR, gamma);
  const double cL = sqrt(gamma * PL[4] / PL[0]);
  const double cR = sqrt(gamma * PR[4] / PR[0]);
  const double uL = PL[n], uR = PR[n];
  double SL, SR;
  einfeldt(PL, PR, n, cL, cR, &SL, &SR);
  const double rdL = PL[0] * (SL - uL);
  const double rdR = PR[0] * (SR - uR);
  const double Ss = ((PR[4] - PL[4]) + (uL * rdL - uR * rdR)) / (rdL - rdR);
  double FL[5], FR[5];
  hllc_star_flux(PL, UL, SL, Ss, n, 1, FL);
  hllc_star_flux(PR, UR, SR, Ss, n, 0, FR);
  const double sg = (Ss > 0.0) ? 1.0 : (Ss < 0.0) ? -1.0 : Ss;  /* sign, 0 and NaN kept */
  for (int v = 0; v < 5; ++v) F[v] = 0.5 * (1.0 + sg) * FL[v] + 0.5 * (1.0 - sg) * FR[v];
}

/* Physical fluxes of both face states (equation_manager.py:237-252). */
static void both_fluxes(const double PL[5], const double PR[5], int n, double gamma, double UL[5], double UR[5],
                        double FL[5], double FR[5]) {
  cons_from_prims(PL, UL, gamma);
  cons_from_prims(PR, UR, gamma);
  physical_flux(PL, UL, n, FL);
  physical_flux(PR, UR, n, FR);
}

/* HLL with Einfeldt speeds clipped at 0: (SR FL - SL FR + SL SR (UR - UL)) /
   (SR - SL + eps), eps the double-precision machine epsilon. */
static void hll_einfeldt(const double PL[5], const double PR[5], int n, double gamma, double F[5]) {
  double UL[5], UR[5], FL[5], FR[5];
  both_fluxes(PL, PR, n, gamma, UL, UR, FL, FR);
  const double cL = sqrt(gamma * PL[4] / PL[0]);
  const double cR = sqrt(gamma * PR[4] / PR[0]);
  double SLs, SRs;
  einfeldt(PL, PR, n, cL, cR, &SLs, &SRs);
  const double SL = fmin(SLs, 0.0), SR = fmax(SRs, 0.0);
  const double den = SR - SL + 2.220446049250313e-16;
  for (int v = 0; v < 5; ++v) F[v] = (SR * FL[v] - SL * FR[v] + SL * SR * (UR[v] - UL[v])) / den;
}

/* Rusanov: 0.5 (FL + FR) - 0.5 alpha (UR - UL), alpha the larger |u| + c. */
static void rusanov(const double PL[5], const double PR[5], int n, double gamma, double F[5]) {
  double UL[5], UR[5], FL[5], FR[5];
  both_fluxes(PL, PR, n, gamma, UL, UR, FL, FR);
  const double cL = sqrt(gamma * PL[4] / PL[0]);
  const double cR = sqrt(gamma * PR[4] / PR[0]);
  const double alpha = fmax(fabs(PL[n]) + cL, fabs(PR[n]) + cR);
  for (int v = 0; v < 5; ++v) F[v] = 0.5 * (FL[v] + FR[v]) - 0.5 * alpha * (UR[v] - UL[v]);
}

/* riemann 0 HLLC, 1 Rusanov, 2 HLL (the ABI's numbering). */
static void riemann_flux(const double PL[5], const double PR[5], int n, double gamma, int riemann, double F[5]) {
  if (riemann == 1)
    rusanov(PL, PR, n, gamma, F);
  else if (riemann == 2)
    hll_einfeldt(PL, PR, n, gamma, F);
  else
    hllc_einfeldt(PL, PR, n, gamma, F);
}

/* velocity_minor_axes and vel_id_eigs per axis (equation_information.py:110,
   eigendecomposition.py:67-71) */
static const int kMinor[3][2] = {{2, 3}, {3, 1}, {1, 2}};
static const int kEig[3][2] = {{2, 3}, {3, 2}, {2, 3}};

/* Frozen density, speed of sound and its square between cells L and R:
   frozen 1 ARITHMETIC, 2 ROE (eigendecomposition.py:120-281). */
static void frozen_state(const double L[5], const double R[5], int frozen, double gamma, double* rho_a,
                         double* c, double* cc) {
  if (frozen == 1) {
    double pa[5];
    for (int v = 0; v < 5; ++v) pa[v] = 0.5 * (L[v] + R[v]);
    *rho_a = pa[0];
    *c = sqrt(gamma * pa[4] / pa[0]);
    *cc = *c * *c;
    return;
  }
  const double ra = sqrt(L[0] * R[0]);
  const double sL = sqrt(L[0]), sR = sqrt(R[0]);
  const double rho_div = 1.0 / (sL + sR);
  const double psi_a = (sL * (L[4] / L[0]) + sR * (R[4] / R[0])) * rho_div;
  const double gr_a = (sL * (gamma - 1) + sR * (gamma - 1)) * rho_div;
  const double d1 = R[1] - L[1], d2 = R[2] - L[2], d3 = R[3] - L[3];
  const double sqvd = d1 * d1 + d2 * d2 + d3 * d3;
  const double p_over_rho = (sL * L[4] / L[0] + sR * R[4] / R[0]) * rho_div + 0.5 * ra * rho_div * rho_div * sqvd;
  *rho_a = ra;
  *cc = psi_a + gr_a * p_over_rho;
  *c = sqrt(*cc);
}

/* Face states of the six window cells w[k][v] (k = 0..5, face between 2 and 3):
   mode 0 WENO5-Z on the primitives, 1 / 2 on the characteristic variables of
   the ARITHMETIC / ROE frozen state. */
static void face_states(double w[6][5], int axis, int mode, double gamma, double eps, double PL[5],
                        double PR[5]) {
  if (mode == 0) {
    for (int v = 0; v < 5; ++v) {
      PL[v] = weno5z(w[0][v], w[1][v], w[2][v], w[3][v], w[4][v], eps);
      PR[v] = weno5z(w[5][v], w[4][v], w[3][v], w[2][v], w[1][v], eps);
    }
    return;
  }
  const int n = axis + 1, m0 = kMinor[axis][0], m1 = kMinor[axis][1];
  const int e0 = kEig[axis][0], e1 = kEig[axis][1];
  double rho_a, c, cc;
  frozen_state(w[2], w[3], mode, gamma, &rho_a, &c, &cc);
  double ch[6][5];
  for (int k = 0; k < 6; ++k) {
    const double* x = w[k];
    ch[k][0] = -0.5 / c * x[n] + 0.5 / (cc * rho_a) * x[4];
    ch[k][1] = x[0] - 1.0 / cc * x[4];
    ch[k][e0] = x[m0];
    ch[k][e1] = x[m1];
    ch[k][4] = 0.5 / c * x[n] + 0.5 / (cc * rho_a) * x[4];
  }
  double cL[5], cR[5];
  for (int v = 0; v < 5; ++v) {
    cL[v] = weno5z(ch[0][v], ch[1][v], ch[2][v], ch[3][v], ch[4][v], eps);
    cR[v] = weno5z(ch[5][v], ch[4][v], ch[3][v], ch[2][v], ch[1][v], eps);
  }
  const double* xs[2] = {cL, cR};
  double* outs[2] = {PL, PR};
  for (int side = 0; side < 2; ++side) {
    const double* x = xs[side];
    double* o = outs[side];
    o[0] = rho_a * (x[0] + x[4]) + x[1];
    o[n] = c * (-x[0] + x[4]);
    o[m0] = x[e0];
    o[m1] = x[e1];
    o[4] = cc * rho_a * (x[0] + x[4]);
  }
}

/*
 * Viscous and heat fluxes with CENTRAL4 stencils on periodic axes
 * (source_term_solver.py:188-254, :264-350, :414-448, :504-580;
 * deriv_center_4.py:37-49, deriv_face_4.py:37-50, central_4.py:39-50), added
 * to a face's convective flux as compute_rhs_xi does (space_solver.py:565-585:
 * F[1:5] += -visc, then F[4] += heat).  The face-normal stencils read the
 * face halos; the centre derivatives of the velocity are evaluated once per
 * interior cell and read across the box's ends by the periodic wrap (the
 * reference reads the same values from its filled edge halos).
 */
typedef struct {
  int viscous, heat, heat_production;
  double mu1, mu2, kappa, R, mu, cp;
} Diss;

typedef struct {
  const double* P;  /* the primitive halo buffer */
  size_t hcs, cs;
  int n[3], h[3], lo[3];
  double* dc[3][3]; /* dc[i][a]: d u_a / d x_i at the interior cell centres, i active */
} DissCells;

/* primitive v of interior-relative cell g (coordinates -nh .. n + nh - 1 on active axes) */
static double hget(const DissCells* b, int v, const int g[3]) {
  return b->P[v * b->hcs + ((size_t)(g[0] + b->lo[0]) * b->h[1] + (g[1] + b->lo[1])) * b->h[2] + (g[2] + b->lo[2])];
}

static double c4_center(double odx, double m2, double m1, double p1, double p2) {
  return odx * (1.0 / 12.0 * (m2 - p2) + 8.0 / 12.0 * (p1 - m1));
}
static double c4_face_deriv(double odx, double m2, double m1, double c0, double p1) {
  return odx * (1.0 / 24.0 * (m2 - p1) + 27.0 / 24.0 * (c0 - m1));
}
static double c4_face_interp(double m2, double m1, double c0, double p1) {
  return -1.0 / 16.0 * (m2 + p1) + 9.0 / 16.0 * (m1 + c0);
}

/* the centre derivatives of every interior cell (viscous cases); 0 or -2 */
static int diss_cells_init(DissCells* b, const Diss* d, const double one_dx[3]) {
  memset(b->dc, 0, sizeof(b->dc));
  if (!d->viscous) return 0;
  for (int i = 0; i < 3; ++i) {
    if (b->n[i] <= 1) continue;
    for (int a = 0; a < 3; ++a) {
      b->dc[i][a] = (double*)malloc(b->cs * sizeof(double));
      if (!b->dc[i][a]) return -2;
    }
  }
  for (int i = 0; i < 3; ++i) {
    if (b->n[i] <= 1) continue;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i0 = 0; i0 < b->n[0]; ++i0)
      for (int i1 = 0; i1 < b->n[1]; ++i1)
        for (int i2 = 0; i2 < b->n[2]; ++i2) {
          const size_t o = ((size_t)i0 * b->n[1] + i1) * b->n[2] + i2;
          for (int a = 0; a < 3; ++a) {
            double u[5];
            for (int k = -2; k <= 2; ++k) {
              int g[3] = {i0, i1, i2};
              g[i] += k;
              u[k + 2] = hget(b, 1 + a, g);
            }
            b->dc[i][a][o] = c4_center(one_dx[i], u[0], u[1], u[3], u[4]);
          }
        }
  }
  return 0;
}

static void diss_cells_free(DissCells* b) {
  for (int i = 0; i < 3; ++i)
    for (int a = 0; a < 3; ++a) free(b->dc[i][a]);
}

static void add_dissipative(const DissCells* b, const Diss* d, const int q[3], int ax, const double one_dx[3],
                            double F[5]) {
  const int* n = b->n;
  const double odx = one_dx[ax];
  /* the four cells q - 2 .. q + 1 along ax of face q */
  int g[4][3];
  size_t wo[4];
  for (int k = 0; k < 4; ++k) {
    g[k][0] = q[0];
    g[k][1] = q[1];
    g[k][2] = q[2];
    g[k][ax] += k - 2;
    int x = g[k][ax];
    x = x < 0 ? x + n[ax] : (x >= n[ax] ? x - n[ax] : x);
    int w[3] = {g[k][0], g[k][1], g[k][2]};
    w[ax] = x;
    wo[k] = ((size_t)w[0] * n[1] + w[1]) * n[2] + w[2];
  }
  if (d->viscous) {
    double vel[3][4];
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 4; ++k) vel[a][k] = hget(b, 1 + a, g[k]);
    double gr[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < 3; ++a) gr[a][ax] = c4_face_deriv(odx, vel[a][0], vel[a][1], vel[a][2], vel[a][3]);
    for (int i = 0; i < 3; ++i) {
      if (i == ax || n[i] <= 1) continue;
      for (int which = 0; which < 2; ++which) {
        const int a = which == 0 ? ax : i;
        const double* dc = b->dc[i][a];
        gr[a][i] = c4_face_interp(dc[wo[0]], dc[wo[1]], dc[wo[2]], dc[wo[3]]);
      }
    }
    double tau[3];
    for (int k = 0; k < 3; ++k) tau[k] = n[k] > 1 ? d->mu1 * (gr[ax][k] + gr[k][ax]) : 0.0;
    double tr = 0.0;
    int first = 1;
    for (int k = 0; k < 3; ++k) {
      if (n[k] <= 1) continue;
      tr = first ? gr[k][k] : tr + gr[k][k];
      first = 0;
    }
    tau[ax] = tau[ax] + d->mu2 * tr;
    double vt = 0.0;
    if (d->heat_production) {
      first = 1;
      for (int k = 0; k < 3; ++k) {
        if (n[k] <= 1) continue;
        const double vf = c4_face_interp(vel[k][0], vel[k][1], vel[k][2], vel[k][3]);
        vt = first ? tau[k] * vf : vt + tau[k] * vf;
        first = 0;
      }
    }
    for (int k = 0; k < 3; ++k) F[1 + k] = F[1 + k] + -tau[k];
    F[4] = F[4] + -vt;
  }
  if (d->heat) {
    double T[4];
    for (int k = 0; k < 4; ++k) T[k] = hget(b, 4, g[k]) / (hget(b, 0, g[k]) * d->R);
    const double dT = c4_face_deriv(odx, T[0], T[1], T[2], T[3]);
    F[4] = F[4] + -d->kappa * dT;
  }
}

static int rhs_impl(const double* P, const int n[3], int nh, const double one_dx[3], double gamma, double eps,
                    int mode, int riemann, const Diss* diss, double* rhs);

/*
 * rhs[5][n0][n1][n2] of the primitive halo buffer P[5][h0][h1][h2]
 * (h_a = n_a + 2 nh on active axes, 1 on inactive ones), axes summed in order
 * from the first active one; mode as face_states, riemann as riemann_flux.
 * Returns 0, or -2 when out of memory.
 */
int jf_rhs_weno5z(const double* P, const int n[3], int nh, const double one_dx[3], double gamma, double eps,
                  int mode, int riemann, double* rhs) {
  return rhs_impl(P, n, nh, one_dx, gamma, eps, mode, riemann, NULL, rhs);
}

/* As jf_rhs_weno5z with CENTRAL4 viscous (viscous != 0) and heat (heat != 0)
   fluxes on a periodic box: mu, bulk viscosity, kappa, cp and R of the
   material, heat_production as is_viscous_heat_production. */
int jf_rhs_weno5z_visc(const double* P, const int n[3], int nh, const double one_dx[3], double gamma, double eps,
                       int mode, int riemann, double mu, double bulk, double kappa, double cp, double R,
                       int viscous, int heat, int heat_production, double* rhs) {
  const Diss d = {viscous, heat, heat_production, mu, bulk - 2.0 / 3.0 * mu, kappa, R, mu, cp};
  return rhs_impl(P, n, nh, one_dx, gamma, eps, mode, riemann, &d, rhs);
}

static int rhs_impl(const double* P, const int n[3], int nh, const double one_dx[3], double gamma, double eps,
                    int mode, int riemann, const Diss* diss, double* rhs) {
  int h[3], lo[3];
  for (int a = 0; a < 3; ++a) {
    h[a] = n[a] > 1 ? n[a] + 2 * nh : 1;
    lo[a] = n[a] > 1 ? nh : 0;
  }
  const size_t hcs = (size_t)h[0] * h[1] * h[2];
  const size_t cs = (size_t)n[0] * n[1] * n[2];
  DissCells db = {P, hcs, cs, {n[0], n[1], n[2]}, {h[0], h[1], h[2]}, {lo[0], lo[1], lo[2]}, {{0}}};
  if (diss && diss_cells_init(&db, diss, one_dx) != 0) {
    diss_cells_free(&db);
    return -2;
  }
  int first = 1;
  for (int a = 0; a < 3; ++a) {
    if (n[a] <= 1) continue;
    const size_t stride = (a == 0) ? (size_t)h[1] * h[2] : (a == 1) ? (size_t)h[2] : 1;
    /* the N + 1 faces of every line along a, each once (face f between cells
       f - 1 and f), laid out [f0][f1][f2] with N + 1 along a */
    int e[3] = {n[0], n[1], n[2]};
    e[a] = n[a] + 1;
    const size_t nfaces = (size_t)e[0] * e[1] * e[2];
    double* F = (double*)malloc(5 * nfaces * sizeof(double));
    if (!F) {
      if (diss) diss_cells_free(&db);
      return -2;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i0 = 0; i0 < e[0]; ++i0)
      for (int i1 = 0; i1 < e[1]; ++i1)
        for (int i2 = 0; i2 < e[2]; ++i2) {
          const int g[3] = {i0 + lo[0], i1 + lo[1], i2 + lo[2]};
          const size_t c0 = ((size_t)g[0] * h[1] + g[1]) * h[2] + g[2];
          double w[6][5], PL[5], PR[5], Ff[5];
          for (int v = 0; v < 5; ++v)
            for (int k = 0; k < 6; ++k) w[k][v] = P[v * hcs + c0 + (ptrdiff_t)(k - 3) * (ptrdiff_t)stride];
          face_states(w, a, mode, gamma, eps, PL, PR);
          riemann_flux(PL, PR, a + 1, gamma, riemann, Ff);
          if (diss) {
            const int q[3] = {i0, i1, i2};
            add_dissipative(&db, diss, q, a, one_dx, Ff);
          }
          const size_t o = ((size_t)i0 * e[1] + i1) * e[2] + i2;
          for (int v = 0; v < 5; ++v) F[v * nfaces + o] = Ff[v];
        }
    const size_t fstride = (a == 0) ? (size_t)e[1] * e[2] : (a == 1) ? (size_t)e[2] : 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i0 = 0; i0 < n[0]; ++i0)
      for (int i1 = 0; i1 < n[1]; ++i1)
        for (int i2 = 0; i2 < n[2]; ++i2) {
          const size_t fo = ((size_t)i0 * e[1] + i1) * e[2] + i2;  /* the face left of the cell */
          const size_t o = ((size_t)i0 * n[1] + i1) * n[2] + i2;
          for (int v = 0; v < 5; ++v) {
            const double r = one_dx[a] * (F[v * nfaces + fo] - F[v * nfaces + fo + fstride]);
            rhs[v * cs + o] = first ? r : rhs[v * cs + o] + r;
          }
        }
    free(F);
    first = 0;
  }
  if (diss) diss_cells_free(&db);
  return 0;
}


/*
 * Face halos of the primitive halo buffer P[5][h0][h1][h2] (as jf_rhs_weno5z)
 * from its interior, for PERIODIC (0), ZEROGRADIENT (1) and SYMMETRY (2)
 * faces (halos/outer/material.py:868-894 with the retrieve slices of
 * halos/outer/boundary_condition.py:539-604): halo layer g = 1..nh outside a
 * face takes interior cell n - g + 1 counted from the opposite face
 * (periodic), the boundary cell (zero gradient), or interior cell g with the
 * face-normal velocity negated (symmetry).  bc[2 a + hi]: faces west, east,
 * south, north, bottom, top.  Edge and corner halos are left as they are (the
 * inviscid right-hand side reads none).  Returns 0, or -1 for another type.
 */
int jf_fill_face_halos(double* P, const int n[3], int nh, const int bc[6]) {
  int h[3];
  for (int a = 0; a < 3; ++a) h[a] = n[a] > 1 ? n[a] + 2 * nh : 1;
  const size_t hcs = (size_t)h[0] * h[1] * h[2];
  for (int a = 0; a < 3; ++a) {
    if (n[a] <= 1) continue;
    const int b = (a + 1) % 3, c = (a + 2) % 3;  /* the two tangential axes */
    for (int hi = 0; hi < 2; ++hi) {
      const int type = bc[2 * a + hi];
      if (type < 0 || type > 2) return -1;
      for (int g = 1; g <= nh; ++g) {
        const int dst = hi ? nh + n[a] + g - 1 : nh - g;
        int src;
        if (type == 0)
          src = hi ? nh + g - 1 : nh + n[a] - g;
        else if (type == 1)
          src = hi ? nh + n[a] - 1 : nh;
        else
          src = hi ? nh + n[a] - g : nh + g - 1;
        for (int ib = 0; ib < h[b]; ++ib)
          for (int ic = 0; ic < h[c]; ++ic) {
            int id[3], is[3];
            id[a] = dst; is[a] = src;
            id[b] = is[b] = ib;
            id[c] = is[c] = ic;
            const size_t od = ((size_t)id[0] * h[1] + id[1]) * h[2] + id[2];
            const size_t os = ((size_t)is[0] * h[1] + is[1]) * h[2] + is[2];
            for (int v = 0; v < 5; ++v) {
              const double x = P[v * hcs + os];
              P[v * hcs + od] = (type == 2 && v == a + 1) ? -1.0 * x : x;
            }
          }
      }
    }
  }
  return 0;
}

/* Primitives of one cell's conservatives (equation_manager.py:164-171,
   ideal_gas.py:73-75: p = (gamma - 1) e rho). */
static void prims_from_cons(const double U[5], double P[5], double gamma) {
  const double rho = U[0];
  const double one_rho = 1.0 / rho;
  const double u = U[1] * one_rho, v = U[2] * one_rho, w = U[3] * one_rho;
  const double e = U[4] * one_rho - 0.5 * (u * u + v * v + w * w);
  P[0] = rho; P[1] = u; P[2] = v; P[3] = w;
  P[4] = (gamma - 1.0) * e * rho;
}

/*
 * `steps` TVD-RK3 steps with the CFL time step (simulation_manager.py:670-1077;
 * time_integration/RK3.py:27-62; time_step_size.py:15-157 for inviscid cases).
 * U, P: interior conservatives and primitives [5][n0][n1][n2]; P is used for
 * the first stage (as the reference's initial primitive buffer) and both are
 * advanced in place.  After each stage the primitives are recomputed from the
 * conservatives and the face halos refilled (bc as jf_fill_face_halos).  dt of
 * each step: min_cell_size / (max over cells of the sum over active axes of
 * |u_i| + c, plus eps) times cfl.  *t is advanced by the dts.  Returns 0, -1
 * for a boundary type it does not fill, -2 when out of memory.
 */
static int rk3_steps(double* U, double* P, const int n[3], int nh, const double one_dx[3], double min_cell_size,
                     double cfl, double fixed_dt, double gamma, double eps, int mode, int riemann, const int bc[6],
                     const Diss* diss, int steps, double* t);

int jf_rk3_steps(double* U, double* P, const int n[3], int nh, const double one_dx[3], double min_cell_size,
                 double cfl, double gamma, double eps, int mode, int riemann, const int bc[6], int steps,
                 double* t) {
  return rk3_steps(U, P, n, nh, one_dx, min_cell_size, cfl, 0.0, gamma, eps, mode, riemann, bc, NULL, steps, t);
}

/* As jf_rk3_steps with CENTRAL4 viscous and heat fluxes (as
   jf_rhs_weno5z_visc; every face PERIODIC) and their time-step limits
   (time_step_size.py:111-150). */
int jf_rk3_steps_visc(double* U, double* P, const int n[3], int nh, const double one_dx[3], double min_cell_size,
                      double cfl, double gamma, double eps, int mode, int riemann, double mu, double bulk,
                      double kappa, double cp, double R, int viscous, int heat, int heat_production, int steps,
                      double* t) {
  static const int kPeriodic[6] = {0, 0, 0, 0, 0, 0};
  const Diss d = {viscous, heat, heat_production, mu, bulk - 2.0 / 3.0 * mu, kappa, R, mu, cp};
  return rk3_steps(U, P, n, nh, one_dx, min_cell_size, cfl, 0.0, gamma, eps, mode, riemann, kPeriodic, &d, steps,
                   t);
}

/* As jf_rk3_steps with a fixed time step dt (time_control's fixed_timestep,
   the feed-forward semantics). */
int jf_rk3_steps_fixed_dt(double* U, double* P, const int n[3], int nh, const double one_dx[3], double dt,
                          double gamma, double eps, int mode, int riemann, const int bc[6], int steps, double* t) {
  return rk3_steps(U, P, n, nh, one_dx, 1.0, 1.0, dt, gamma, eps, mode, riemann, bc, NULL, steps, t);
}

static int rk3_steps(double* U, double* P, const int n[3], int nh, const double one_dx[3], double min_cell_size,
                     double cfl, double fixed_dt, double gamma, double eps, int mode, int riemann, const int bc[6],
                     const Diss* diss, int steps, double* t) {
  int h[3], lo[3];
  for (int a = 0; a < 3; ++a) {
    h[a] = n[a] > 1 ? n[a] + 2 * nh : 1;
    lo[a] = n[a] > 1 ? nh : 0;
  }
  const size_t hcs = (size_t)h[0] * h[1] * h[2];
  const size_t cs = (size_t)n[0] * n[1] * n[2];
  double* Ph = (double*)calloc(5 * hcs, sizeof(double));
  double* Un = (double*)malloc(5 * cs * sizeof(double));
  double* rhs = (double*)malloc(5 * cs * sizeof(double));
  int st = 0;
  if (!Ph || !Un || !rhs) st = -2;
  /* interior primitives -> halo buffer, then its face halos */
#define JF_LOAD_HALO()                                                                    \
  JF_OMP_FOR                                                                              \
  for (int i0 = 0; i0 < n[0]; ++i0)                                                       \
    for (int i1 = 0; i1 < n[1]; ++i1)                                                     \
      for (int i2 = 0; i2 < n[2]; ++i2) {                                                 \
        const size_t o = ((size_t)i0 * n[1] + i1) * n[2] + i2;                             \
        const size_t q = ((size_t)(i0 + lo[0]) * h[1] + (i1 + lo[1])) * h[2] + (i2 + lo[2]); \
        for (int v = 0; v < 5; ++v) Ph[v * hcs + q] = P[v * cs + o];                       \
      }                                                                                   \
  if (st == 0 && jf_fill_face_halos(Ph, n, nh, bc) != 0) st = -1;
  if (st == 0) { JF_LOAD_HALO() }
  static const double kDtMult[3] = {1.0, 0.25, 2.0 / 3.0};
  static const double kCons[2][2] = {{0.25, 0.75}, {2.0 / 3.0, 1.0 / 3.0}};
  for (int step = 0; st == 0 && step < steps; ++step) {
    /* the largest signal speed sum (non-negative: the maximum is exact in any order) */
    double amax = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : amax)
#endif
    for (size_t o = 0; o < cs; ++o) {
      const double c = sqrt(gamma * P[4 * cs + o] / P[o]);
      double s = 0.0;
      for (int a = 0; a < 3; ++a)
        if (n[a] > 1) s = s + (fabs(P[(a + 1) * cs + o]) + c);
      if (s > amax) amax = s;
    }
    double dt = min_cell_size / (amax + 2.220446049250313e-16);
    if (diss && diss->viscous) {
      /* nu = mu / rho, dt_v = (3/14) dx^2 / (max nu + eps) */
      double numax = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : numax)
#endif
      for (size_t o = 0; o < cs; ++o) {
        const double nu = diss->mu / P[o];
        if (nu > numax) numax = nu;
      }
      const double dt_v = 3.0 / 14.0 * (min_cell_size * min_cell_size) / (numax + 2.220446049250313e-16);
      if (dt_v < dt) dt = dt_v;
    }
    if (diss && diss->heat) {
      /* alpha = kappa / (rho cp), dt_h = 0.1 dx^2 / (max alpha + eps) */
      double amx = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : amx)
#endif
      for (size_t o = 0; o < cs; ++o) {
        const double al = diss->kappa / (P[o] * diss->cp);
        if (al > amx) amx = al;
      }
      const double dt_h = 0.1 * (min_cell_size * min_cell_size) / (amx + 2.220446049250313e-16);
      if (dt_h < dt) dt = dt_h;
    }
    dt = fixed_dt > 0.0 ? fixed_dt : dt * cfl;
    memcpy(Un, U, 5 * cs * sizeof(double));
    for (int stage = 0; stage < 3; ++stage) {
      if (rhs_impl(Ph, n, nh, one_dx, gamma, eps, mode, riemann, diss, rhs) != 0) {
        st = -2;
        break;
      }
      const double ts = dt * kDtMult[stage];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
      for (size_t k = 0; k < 5 * cs; ++k) {
        const double base = stage > 0 ? kCons[stage - 1][0] * U[k] + kCons[stage - 1][1] * Un[k] : U[k];
        U[k] = base + ts * rhs[k];
      }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
      for (size_t o = 0; o < cs; ++o) {
        double u5[5], p5[5];
        for (int v = 0; v < 5; ++v) u5[v] = U[v * cs + o];
        prims_from_cons(u5, p5, gamma);
        for (int v = 0; v < 5; ++v) P[v * cs + o] = p5[v];
      }
      JF_LOAD_HALO()
    }
    *t += dt;
  }
#undef JF_LOAD_HALO
  free(Ph);
  free(Un);
  free(rhs);
  return st;
}
