// Tile kernel of the right-hand-side VJP (the inviscid part), shared by the
// translation units that instantiate one scheme family each
// (gbf_vjp_<family>.cu, compiled in parallel); launched by gbf_adjoint.cu.
#pragma once

#include "gbf_adjoint.cuh"
#include "gbf_kernels.cuh"

namespace gbf {

struct VjpParams {
  SweepParams sp;       // state U (sp.cons), sizes, tile, scheme
  const double* w;      // cotangent of the rhs, interior [5][N]
  double* dP;           // primitive cotangent accumulator, interior [5][N]
  double* dU;           // conservative cotangent accumulator (CONSERVATIVE reconstruction), interior [5][N]
  // Lax-Friedrichs (Rusanov instantiations, PRIMITIVE reconstructions): the
  // axes' speeds of the state (null: Rusanov's local speeds) and the
  // accumulators of their cotangents
  const double* lf_alpha;
  double* lf_dalpha;
  // Lax-Friedrichs tie pullback (lf_tie_side 0 / 1, -1 off): the face states'
  // cotangents are those of the speed of side lf_tie_side, lf_tie_ds, in place
  // of the flux's
  int lf_tie_side;
  double lf_tie_ds;
};

// Lax-Friedrichs flux VJP with the axis' speed fixed, or the scheme's own;
// in a tie pullback, the speed's cotangent on one face state.
template <int AX, int RIEMANN>
__device__ __forceinline__ void face_riemann_vjp(const VjpParams& vp, const double PL[5], const double PR[5],
                                                 const double dF[5], double dPL[5], double dPR[5],
                                                 double& dalpha) {
  if (RIEMANN == GBF_RIEMANN_RUSANOV && vp.lf_tie_side >= 0)
    lf_speed_vjp<AX>(vp.lf_tie_side == 0 ? PL : PR, vp.sp.fp, vp.lf_tie_ds, vp.lf_tie_side == 0 ? dPL : dPR);
  else if (RIEMANN == GBF_RIEMANN_RUSANOV && vp.lf_alpha)
    lf_vjp<AX>(PL, PR, vp.sp.fp, vp.lf_alpha[AX], dF, dPL, dPR, dalpha);
  else
    riemann_flux_vjp<AX, RIEMANN>(PL, PR, vp.sp.fp, dF, dPL, dPR);
}

// face_riemann_vjp on the face states after the interpolation limiter
// (positivity_limit against the primitives of window cells 2 and 3: variable
// stride pvol, cell stride ps from win): PL, PR are limited in place, and the
// cotangent of a replaced face primitive, which is the cell's primitive, goes
// to limL / limR instead of dPL / dPR.
template <int AX, int RIEMANN>
__device__ __forceinline__ void face_riemann_limited_vjp(const VjpParams& vp, const double* win, int pvol, int ps,
                                                         double PL[5], double PR[5], const double dF[5],
                                                         double dPL[5], double dPR[5], double limL[5],
                                                         double limR[5], double& dalpha) {
  unsigned mL = 0, mR = 0;
  if (vp.sp.limiter) {
    mL = positivity_limit(PL, win + 2 * ps, pvol, vp.sp.limiter);
    mR = positivity_limit(PR, win + 3 * ps, pvol, vp.sp.limiter);
  }
  face_riemann_vjp<AX, RIEMANN>(vp, PL, PR, dF, dPL, dPR, dalpha);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    limL[v] = (mL & (1u << v)) ? dPL[v] : 0.0;
    limR[v] = (mR & (1u << v)) ? dPR[v] : 0.0;
    if (mL & (1u << v)) dPL[v] = 0.0;
    if (mR & (1u << v)) dPR[v] = 0.0;
  }
}

// Cotangents of the primitives of window cells 2 and 3 (limL, limR) onto
// their conservatives (the staged conservatives behind the primitives,
// win + 5 pvol), added to slot(v, 2) and slot(v, 3) = slot[(v * 6 + k) * fvol].
__device__ __forceinline__ void cell_prims_cotangent_to_cons(const VjpParams& vp, const double* win, int pvol,
                                                             int ps, const double limL[5], const double limR[5],
                                                             double* slot, int fvol) {
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const double* lim = side == 0 ? limL : limR;
    if (lim[0] == 0.0 && lim[1] == 0.0 && lim[2] == 0.0 && lim[3] == 0.0 && lim[4] == 0.0) continue;
    const int k = 2 + side;
    double Uc[5], dUc[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int v = 0; v < 5; ++v) Uc[v] = win[(5 + v) * pvol + k * ps];
    prims_from_cons_vjp(Uc, lim, vp.sp.fp.gm1, dUc);
#pragma unroll
    for (int v = 0; v < 5; ++v) slot[(v * 6 + k) * fvol] += dUc[v];
  }
}

// CHAR-PRIMITIVE face (char_reconstruct of the forward): frozen state of the
// two cells adjacent to the face, characteristic variables of the six window
// cells, WENO5-Z with its gradients on each, back-projection, Riemann VJP, and
// the reverse of all of it onto the window cells' primitives.  win points at
// window cell 0 of variable 0 in the staged pencil (variable stride pvol, cell
// stride ps); slot(v, k) = slot[(v * 6 + k) * fvol] receives the cotangent of
// primitive v of window cell k; jr is this thread's private row block.
template <int AX, int RIEMANN>
__device__ __forceinline__ void char_face_vjp(const VjpParams& vp, const double* win, int pvol, int ps,
                                              const double dF[5], double* slot, int fvol, double* jr_rows,
                                              int nthr, double& dalpha) {
  const FaceParams& fp = vp.sp.fp;
  constexpr int N = AX + 1;
  using I = CharIds<AX>;
  auto x = [&](int v, int k) { return win[v * pvol + k * ps]; };
  auto SL = [&](int j, int k) -> double& { return slot[(j * 6 + k) * fvol]; };
  auto JR = [&](int j, int i) -> double& { return jr_rows[(j * 5 + i) * nthr]; };
  double Lc[5], Rc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    Lc[v] = x(v, 2);
    Rc[v] = x(v, 3);
  }
  double rho_a, c, cc;
  frozen_state(Lc, Rc, fp, rho_a, c, cc);
  const double ic = 1.0 / c;
  const double k_m = -0.5 * ic, k_p = 0.5 * ic;
  const double k_e = 0.5 / (cc * rho_a);
  const double k_s = 1.0 / cc;
  const double eps = fp.stencil_eps;
  // characteristic face values cL[j], cR[j]; gradients of char var j: left in
  // slot(j, 0..4), right in the private rows
  double cL[5], cR[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    double ch[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      if (j == 0) ch[k] = k_m * x(N, k) + k_e * x(4, k);
      else if (j == 1) ch[k] = x(0, k) - k_s * x(4, k);
      else if (j == 4) ch[k] = k_p * x(N, k) + k_e * x(4, k);
      else ch[k] = x(j == I::e0 ? I::m0 : I::m1, k);
    }
    double jl[5], jr[5];
    weno5z_jac(ch[0], ch[1], ch[2], ch[3], ch[4], eps, cL[j], jl);
    weno5z_jac(ch[5], ch[4], ch[3], ch[2], ch[1], eps, cR[j], jr);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      SL(j, k) = jl[k];
      JR(j, k) = jr[k];
    }
  }
  double PL[5], PR[5];
  PL[0] = rho_a * (cL[0] + cL[4]) + cL[1];
  PL[N] = c * (-cL[0] + cL[4]);
  PL[I::m0] = cL[I::e0];
  PL[I::m1] = cL[I::e1];
  PL[4] = cc * rho_a * (cL[0] + cL[4]);
  PR[0] = rho_a * (cR[0] + cR[4]) + cR[1];
  PR[N] = c * (-cR[0] + cR[4]);
  PR[I::m0] = cR[I::e0];
  PR[I::m1] = cR[I::e1];
  PR[4] = cc * rho_a * (cR[0] + cR[4]);
  // the interpolation limiter on the back-projected face primitives: a
  // replaced primitive is the one of the cell beside the face (window cells
  // 2 and 3), which takes its cotangent directly
  unsigned mL = 0, mR = 0;
  if (vp.sp.limiter) {
    mL = positivity_limit(PL, win + 2 * ps, pvol, vp.sp.limiter);
    mR = positivity_limit(PR, win + 3 * ps, pvol, vp.sp.limiter);
  }
  double dPL[5] = {0, 0, 0, 0, 0}, dPR[5] = {0, 0, 0, 0, 0};
  face_riemann_vjp<AX, RIEMANN>(vp, PL, PR, dF, dPL, dPR, dalpha);
  double limL[5], limR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    limL[v] = (mL & (1u << v)) ? dPL[v] : 0.0;
    limR[v] = (mR & (1u << v)) ? dPR[v] : 0.0;
    if (mL & (1u << v)) dPL[v] = 0.0;
    if (mR & (1u << v)) dPR[v] = 0.0;
  }
  // back-projection reverse
  double drho_a = 0.0, dc = 0.0, dcc = 0.0;
  double gL[5], gR[5];
  {
    const double sL4 = cL[0] + cL[4], sR4 = cR[0] + cR[4];
    const double ccr = cc * rho_a;
    gL[0] = rho_a * dPL[0] - c * dPL[N] + ccr * dPL[4];
    gL[4] = rho_a * dPL[0] + c * dPL[N] + ccr * dPL[4];
    gL[1] = dPL[0];
    gL[I::e0] = dPL[I::m0];
    gL[I::e1] = dPL[I::m1];
    gR[0] = rho_a * dPR[0] - c * dPR[N] + ccr * dPR[4];
    gR[4] = rho_a * dPR[0] + c * dPR[N] + ccr * dPR[4];
    gR[1] = dPR[0];
    gR[I::e0] = dPR[I::m0];
    gR[I::e1] = dPR[I::m1];
    drho_a = (dPL[0] + cc * dPL[4]) * sL4 + (dPR[0] + cc * dPR[4]) * sR4;
    dc = dPL[N] * (cL[4] - cL[0]) + dPR[N] * (cR[4] - cR[0]);
    dcc = dPL[4] * rho_a * sL4 + dPR[4] * rho_a * sR4;
  }
  // per window cell: cotangents of the char variables, then of the primitives
  double dk_m = 0.0, dk_p = 0.0, dk_e = 0.0, dk_s = 0.0;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double dch[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      double d = (k <= 4) ? gL[j] * SL(j, k) : 0.0;
      if (k >= 1) d += gR[j] * JR(j, 5 - k);
      dch[j] = d;
    }
    const double xn = x(N, k), x4 = x(4, k);
    dk_m += dch[0] * xn;
    dk_p += dch[4] * xn;
    dk_e += (dch[0] + dch[4]) * x4;
    dk_s -= dch[1] * x4;
    double dx[5];
    dx[0] = dch[1];
    dx[N] = k_m * dch[0] + k_p * dch[4];
    dx[4] = k_e * (dch[0] + dch[4]) - k_s * dch[1];
    dx[I::m0] = dch[I::e0];
    dx[I::m1] = dch[I::e1];
#pragma unroll
    for (int v = 0; v < 5; ++v) SL(v, k) = dx[v];
  }
  // k_m = -0.5/c, k_p = 0.5/c, k_e = 0.5/(cc rho_a), k_s = 1/cc
  dc += (dk_m - dk_p) * 0.5 * ic * ic;
  const double dden = -dk_e * k_e / (cc * rho_a);
  dcc += dden * rho_a - dk_s * k_s * k_s;
  drho_a += dden * cc;
  double dLc[5] = {0, 0, 0, 0, 0}, dRc[5] = {0, 0, 0, 0, 0};
  frozen_state_vjp(Lc, Rc, fp, drho_a, dc, dcc, dLc, dRc);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    SL(v, 2) += dLc[v] + limL[v];
    SL(v, 3) += dRc[v] + limR[v];
  }
}

// CHAR-CONSERVATIVE face (charcons_reconstruct of the forward,
// high_order_godunov.py:404-416, eigendecomposition.py:576-742): the full
// frozen state of the primitives of the two cells beside the face, the
// window conservatives to characteristic variables with the left
// eigenvectors, WENO5-Z with its gradients on each, back with the right ones,
// the face conservatives' primitives, the Riemann VJP, and the reverse of all
// of it: the window cells' conservative cotangents to slot(v, k) =
// slot[(v * 6 + k) * fvol] (cells 2 and 3 also receive the frozen state's
// cotangents, carried from their primitives to their conservatives).  win
// points at window cell 0 of the staged pencil (primitives in rows 0..4,
// conservatives in rows 5..9); jr is this thread's private row block.
template <int AX, int RIEMANN>
__device__ __forceinline__ void charcons_face_vjp(const VjpParams& vp, const double* win, int pvol, int ps,
                                                  const double dF[5], double* slot, int fvol, double* jr_rows,
                                                  int nthr, double& dalpha) {
  const FaceParams& fp = vp.sp.fp;
  auto w = [&](int v, int k) { return win[v * pvol + k * ps]; };
  auto u = [&](int v, int k) { return win[(5 + v) * pvol + k * ps]; };
  auto SL = [&](int j, int k) -> double& { return slot[(j * 6 + k) * fvol]; };
  auto JR = [&](int j, int i) -> double& { return jr_rows[(j * 5 + i) * nthr]; };
  double L[5], R[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    L[v] = w(v, 2);
    R[v] = w(v, 3);
  }
  FrozenFull z;
  frozen_state_full(L, R, fp, z);
  double Lm[5][5];
  left_eigvecs_cons<AX>(z, Lm);
  const double eps = fp.stencil_eps;
  double cL[5], cR[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    double ch[6];
#pragma unroll
    for (int k = 0; k < 6; ++k)
      ch[k] = Lm[i][0] * u(0, k) + Lm[i][1] * u(1, k) + Lm[i][2] * u(2, k) + Lm[i][3] * u(3, k) + Lm[i][4] * u(4, k);
    double jl[5], jr[5];
    weno5z_jac(ch[0], ch[1], ch[2], ch[3], ch[4], eps, cL[i], jl);
    weno5z_jac(ch[5], ch[4], ch[3], ch[2], ch[1], eps, cR[i], jr);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      SL(i, k) = jl[k];
      JR(i, k) = jr[k];
    }
  }
  double Rm[5][5];
  right_eigvecs_cons<AX>(z, Rm);
  double UL[5], UR[5], PL[5], PR[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    UL[i] = Rm[i][0] * cL[0] + Rm[i][1] * cL[1] + Rm[i][2] * cL[2] + Rm[i][3] * cL[3] + Rm[i][4] * cL[4];
    UR[i] = Rm[i][0] * cR[0] + Rm[i][1] * cR[1] + Rm[i][2] * cR[2] + Rm[i][3] * cR[3] + Rm[i][4] * cR[4];
  }
  prims_from_cons(UL, PL, fp.gm1);
  prims_from_cons(UR, PR, fp.gm1);
  double limL[5], limR[5];
  double dPL[5] = {0, 0, 0, 0, 0}, dPR[5] = {0, 0, 0, 0, 0};
  face_riemann_limited_vjp<AX, RIEMANN>(vp, win, pvol, ps, PL, PR, dF, dPL, dPR, limL, limR, dalpha);
  double dUL[5] = {0, 0, 0, 0, 0}, dUR[5] = {0, 0, 0, 0, 0};
  prims_from_cons_vjp(UL, dPL, fp.gm1, dUL);
  prims_from_cons_vjp(UR, dPR, fp.gm1, dUR);
  // U = Rm c: cotangents of the right eigenvectors and of the face chars
  FrozenFull dz{};
  double G[5][5];
  double gL[5], gR[5];
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    gL[j] = 0.0;
    gR[j] = 0.0;
  }
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      G[i][j] = dUL[i] * cL[j] + dUR[i] * cR[j];
      gL[j] += Rm[i][j] * dUL[i];
      gR[j] += Rm[i][j] * dUR[i];
    }
  right_eigvecs_cons_vjp<AX>(z, G, dz);
  // per window cell: char cotangents, then conservative ones; G collects the
  // left eigenvectors' cotangent
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) G[i][j] = 0.0;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    double dch[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      double d = (k <= 4) ? gL[i] * SL(i, k) : 0.0;
      if (k >= 1) d += gR[i] * JR(i, 5 - k);
      dch[i] = d;
    }
    double uk[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) uk[j] = u(j, k);
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
      for (int j = 0; j < 5; ++j) G[i][j] += dch[i] * uk[j];
#pragma unroll
    for (int j = 0; j < 5; ++j)
      SL(j, k) = Lm[0][j] * dch[0] + Lm[1][j] * dch[1] + Lm[2][j] * dch[2] + Lm[3][j] * dch[3] + Lm[4][j] * dch[4];
  }
  left_eigvecs_cons_vjp<AX>(z, G, dz);
  double dLp[5] = {0, 0, 0, 0, 0}, dRp[5] = {0, 0, 0, 0, 0};
  frozen_state_full_vjp(L, R, fp, z, dz, dLp, dRp);
  // the limiter's replaced face primitives are those of cells 2 and 3 too
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    dLp[v] += limL[v];
    dRp[v] += limR[v];
  }
  // the frozen state reads the primitives of cells 2 and 3: on to their conservatives
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int k = 2 + side;
    double Uc[5], dUc[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int v = 0; v < 5; ++v) Uc[v] = u(v, k);
    prims_from_cons_vjp(Uc, side == 0 ? dLp : dRp, fp.gm1, dUc);
#pragma unroll
    for (int v = 0; v < 5; ++v) SL(v, k) += dUc[v];
  }
}

// CONSERVATIVE face (high_order_godunov.py:282-296 reversed): WENO5-Z on the
// window conservatives with its gradients, primitives of the face
// conservatives, Riemann VJP, then the face conservatives' cotangents through
// the stencil gradients into slot(v, k) = slot[(v * 6 + k) * fvol] (the
// window cells' conservative cotangents).  win: window cell 0 of the staged
// pencil (conservatives in rows 5..9); jr: this thread's private row block.
template <int AX, int RIEMANN>
__device__ __forceinline__ void cons_face_vjp(const VjpParams& vp, const double* win, int pvol, int ps,
                                              const double dF[5], double* slot, int fvol, double* jr_rows,
                                              int nthr, double& dalpha) {
  const FaceParams& fp = vp.sp.fp;
  auto SL = [&](int v, int k) -> double& { return slot[(v * 6 + k) * fvol]; };
  auto JR = [&](int v, int i) -> double& { return jr_rows[(v * 5 + i) * nthr]; };
  double UL[5], UR[5], PL[5], PR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double wv[6], jl[5], jr[5];
#pragma unroll
    for (int k = 0; k < 6; ++k) wv[k] = win[(5 + v) * pvol + k * ps];
    weno5z_jac(wv[0], wv[1], wv[2], wv[3], wv[4], fp.stencil_eps, UL[v], jl);
    weno5z_jac(wv[5], wv[4], wv[3], wv[2], wv[1], fp.stencil_eps, UR[v], jr);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      SL(v, k) = jl[k];
      JR(v, k) = jr[k];
    }
  }
  prims_from_cons(UL, PL, fp.gm1);
  prims_from_cons(UR, PR, fp.gm1);
  double limL[5], limR[5];
  double dPL[5] = {0, 0, 0, 0, 0}, dPR[5] = {0, 0, 0, 0, 0};
  face_riemann_limited_vjp<AX, RIEMANN>(vp, win, pvol, ps, PL, PR, dF, dPL, dPR, limL, limR, dalpha);
  double dUL[5] = {0, 0, 0, 0, 0}, dUR[5] = {0, 0, 0, 0, 0};
  prims_from_cons_vjp(UL, dPL, fp.gm1, dUL);
  prims_from_cons_vjp(UR, dPR, fp.gm1, dUR);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double gL = dUL[v], gR = dUR[v];
    double jl[5], jr[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      jl[k] = SL(v, k);
      jr[k] = JR(v, k);
    }
    SL(v, 0) = gL * jl[0];
#pragma unroll
    for (int k = 1; k < 5; ++k) SL(v, k) = gL * jl[k] + gR * jr[5 - k];
    SL(v, 5) = gR * jr[0];
  }
  cell_prims_cotangent_to_cons(vp, win, pvol, ps, limL, limR, slot, fvol);
}

template <int AX, int RECON, int RIEMANN>
__device__ __forceinline__ void vjp_axis(const VjpParams& vp, const int o[3], const int ext[3],
                                         double* sm_prim, double* sm_slot, double* sm_jr) {
  constexpr int R = ReconTraits<RECON>::R;
  constexpr int K = 2 * R;
  // CONSERVATIVE, CHAR-CONSERVATIVE: the stencils read the staged
  // conservatives (pencil rows 5..9); the face slots hold conservative cotangents
  constexpr bool CONS = RECON == RECON_WENO5Z_CONS || RECON == RECON_WENO5Z_CHARCONS;
  const SweepParams& p = vp.sp;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  int pe[3] = {ext[0], ext[1], ext[2]};
  pe[AX] += 2 * R;
  const int pvol = pe[0] * pe[1] * pe[2];
  stage_pencil<AX, R, MODE_STAGE, CONS>(p, o, pe, pvol, sm_prim);
  __syncthreads();

  int fe[3] = {ext[0], ext[1], ext[2]};
  fe[AX] += 1;
  const int fvol = fe[0] * fe[1] * fe[2];
  const int pstride = (AX == 0) ? pe[1] * pe[2] : ((AX == 1) ? pe[2] : 1);
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const double odx = p.one_dx[AX];
  double dalpha = 0.0;  // Lax-Friedrichs: this thread's share of the speed's cotangent
  for (int f = tid; f < fvol; f += nthr) {
    const int f2 = f % fe[2];
    const int r = f / fe[2];
    const int f1 = r % fe[1];
    const int f0 = r / fe[1];
    // cotangent of the face flux: rhs_i = odx (F_i - F_{i+1}).  A face on a
    // tile boundary is computed by both tiles, and each tile's forward uses
    // it only for its own cell, so each tile pulls back only the share of
    // its own cells (this also drops cells outside the domain).
    int gc[3] = {o[0] + f0, o[1] + f1, o[2] + f2};  // cell right of the face
    const long long offR = ((long long)gc[0] * p.n[1] + gc[1]) * p.n[2] + gc[2];
    gc[AX] -= 1;
    const long long offL = ((long long)gc[0] * p.n[1] + gc[1]) * p.n[2] + gc[2];
    const int fl = (AX == 0) ? f0 : ((AX == 1) ? f1 : f2);  // tile-local face index
    const bool hasR = fl < ext[AX];
    const bool hasL = fl >= 1;
    double dF[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double wr = hasR ? __ldg(vp.w + v * cs + offR) : 0.0;
      const double wl = hasL ? __ldg(vp.w + v * cs + offL) : 0.0;
      dF[v] = odx * (wr - wl);
    }
    const int base = idx3(f0, f1, f2, pe[1], pe[2]);
    double PL[5], PR[5];
    if constexpr (RECON == RECON_WENO5Z_CHARCONS) {
      charcons_face_vjp<AX, RIEMANN>(vp, sm_prim + base, pvol, pstride, dF, sm_slot + f, fvol, sm_jr + tid, nthr,
                                     dalpha);
    } else if constexpr (CONS) {
      cons_face_vjp<AX, RIEMANN>(vp, sm_prim + base, pvol, pstride, dF, sm_slot + f, fvol, sm_jr + tid, nthr,
                                 dalpha);
    } else if constexpr (RECON == GBF_RECON_WENO5Z || RECON == GBF_RECON_WENO5JS || RECON == GBF_RECON_TENO5) {
      // one pass gives the face states and the stencil gradients; the left
      // gradient waits in the face's slots 0..4, the right one in this
      // thread's private rows, until the Riemann cotangents are known
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double wv[K], jl[5], jr[5];
#pragma unroll
        for (int k = 0; k < K; ++k) wv[k] = sm_prim[v * pvol + base + k * pstride];
        if constexpr (RECON == GBF_RECON_WENO5Z) {
          weno5z_jac(wv[0], wv[1], wv[2], wv[3], wv[4], p.fp.stencil_eps, PL[v], jl);
          weno5z_jac(wv[5], wv[4], wv[3], wv[2], wv[1], p.fp.stencil_eps, PR[v], jr);
        } else if constexpr (RECON == GBF_RECON_TENO5) {
          teno5_jac(wv[0], wv[1], wv[2], wv[3], wv[4], p.fp.stencil_eps, PL[v], jl);
          teno5_jac(wv[5], wv[4], wv[3], wv[2], wv[1], p.fp.stencil_eps, PR[v], jr);
        } else {
          weno5js_jac(wv[0], wv[1], wv[2], wv[3], wv[4], p.fp.stencil_eps, PL[v], jl);
          weno5js_jac(wv[5], wv[4], wv[3], wv[2], wv[1], p.fp.stencil_eps, PR[v], jr);
        }
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          sm_slot[(v * K + k) * fvol + f] = jl[k];
          sm_jr[(v * 5 + k) * nthr + tid] = jr[k];
        }
      }
      if (p.limiter) {
        // limited primitives are the cells beside the face (slot R - 1 on
        // the left, R on the right): unit stencil gradients
        const double* c = sm_prim + base + (R - 1) * pstride;
        const unsigned mL = positivity_limit(PL, c, pvol, p.limiter);
        const unsigned mR = positivity_limit(PR, c + pstride, pvol, p.limiter);
#pragma unroll
        for (int v = 0; v < 5; ++v)
#pragma unroll
          for (int k = 0; k < 5; ++k) {
            if (mL & (1u << v)) sm_slot[(v * K + k) * fvol + f] = (k == R - 1) ? 1.0 : 0.0;
            if (mR & (1u << v)) sm_jr[(v * 5 + k) * nthr + tid] = (k == R - 1) ? 1.0 : 0.0;
          }
      }
      double dPL[5] = {0, 0, 0, 0, 0}, dPR[5] = {0, 0, 0, 0, 0};
      face_riemann_vjp<AX, RIEMANN>(vp, PL, PR, dF, dPL, dPR, dalpha);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double gL = dPL[v], gR = dPR[v];
        double jl[5], jr[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          jl[k] = sm_slot[(v * K + k) * fvol + f];
          jr[k] = sm_jr[(v * 5 + k) * nthr + tid];
        }
        sm_slot[(v * K + 0) * fvol + f] = gL * jl[0];
#pragma unroll
        for (int k = 1; k < 5; ++k) sm_slot[(v * K + k) * fvol + f] = gL * jl[k] + gR * jr[5 - k];
        sm_slot[(v * K + 5) * fvol + f] = gR * jr[0];
      }
    } else if constexpr (RECON == RECON_WENO5Z_CHAR) {
      char_face_vjp<AX, RIEMANN>(vp, sm_prim + base, pvol, pstride, dF, sm_slot + f, fvol, sm_jr + tid, nthr,
                                 dalpha);
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double wv[K];
#pragma unroll
        for (int k = 0; k < K; ++k) wv[k] = sm_prim[v * pvol + base + k * pstride];
        reconstruct_pair<RECON>(wv, p.fp.stencil_eps, PL[v], PR[v]);
      }
      unsigned mL = 0, mR = 0;
      if (p.limiter) {
        const double* c = sm_prim + base + (R - 1) * pstride;
        mL = positivity_limit(PL, c, pvol, p.limiter);
        mR = positivity_limit(PR, c + pstride, pvol, p.limiter);
      }
      double dPL[5] = {0, 0, 0, 0, 0}, dPR[5] = {0, 0, 0, 0, 0};
      face_riemann_vjp<AX, RIEMANN>(vp, PL, PR, dF, dPL, dPR, dalpha);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double wv[K], dw[K];
#pragma unroll
        for (int k = 0; k < K; ++k) wv[k] = sm_prim[v * pvol + base + k * pstride];
        // limited primitives take the cell beside the face (slot R - 1 left, R right)
        const double gL = (mL & (1u << v)) ? 0.0 : dPL[v];
        const double gR = (mR & (1u << v)) ? 0.0 : dPR[v];
        reconstruct_pair_vjp<RECON>(wv, p.fp.stencil_eps, gL, gR, dw);
        if (mL & (1u << v)) dw[R - 1] += dPL[v];
        if (mR & (1u << v)) dw[R] += dPR[v];
#pragma unroll
        for (int k = 0; k < K; ++k) sm_slot[(v * K + k) * fvol + f] = dw[k];
      }
    }
  }
  if (RIEMANN == GBF_RIEMANN_RUSANOV && vp.lf_alpha) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) dalpha += __shfl_xor_sync(0xffffffffu, dalpha, off);
    if ((tid & 31) == 0 && dalpha != 0.0) atomicAdd(vp.lf_dalpha + AX, dalpha);
  }
  __syncthreads();

  // gather per pencil cell (fixed order), map back through the boundary
  // remap and accumulate into the primitive cotangent
  for (int i = tid; i < pvol; i += nthr) {
    const int i2 = i % pe[2];
    const int r = i / pe[2];
    const int i1 = r % pe[1];
    const int i0 = r / pe[1];
    const int ia = (AX == 0) ? i0 : ((AX == 1) ? i1 : i2);
    double d[5] = {0, 0, 0, 0, 0};
    bool any = false;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int fa = ia - k;  // face whose stencil slot k is this cell
      if (fa < 0 || fa >= fe[AX]) continue;
      int fi[3] = {i0, i1, i2};
      fi[AX] = fa;
      const int f = idx3(fi[0], fi[1], fi[2], fe[1], fe[2]);
#pragma unroll
      for (int v = 0; v < 5; ++v) d[v] += sm_slot[(v * K + k) * fvol + f];
      any = true;
    }
    if (!any) continue;
    int g[3] = {o[0] + i0, o[1] + i1, o[2] + i2};
    g[AX] -= R;
    const bool halo = g[AX] < 0 || g[AX] >= p.n[AX];
    if constexpr (CONS) {
      if (!halo) {
        // an interior cell's conservatives are the state itself
        const long long off = ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
#pragma unroll
        for (int v = 0; v < 5; ++v)
          if (d[v] != 0.0) atomicAdd(vp.dU + v * cs + off, d[v]);
        continue;
      }
      // a halo cell's conservatives are those of its halo primitives
      // (material.py:248-250): on to the primitives, then the face rule
      double P[5], dPh[5] = {0, 0, 0, 0, 0};
#pragma unroll
      for (int v = 0; v < 5; ++v) P[v] = sm_prim[v * pvol + i];
      cons_from_prims_vjp(P, d, 1.0 / P[0], 1.0 / p.fp.gm1, dPh);
#pragma unroll
      for (int v = 0; v < 5; ++v) d[v] = dPh[v];
    }
    if (halo) {
      // halo cell: transpose of the face rule (DIRICHLET halos are constants)
      const int t = face_type_at(p.bc, p.bf, 2 * AX + (g[AX] >= 0 ? 1 : 0), face_pos(p.n, AX, g));
      g[AX] = bc_src(g[AX], p.n[AX], t);
#pragma unroll
      for (int v = 0; v < 5; ++v) d[v] *= bc_apply_grad(t, AX, v);
    }
    const long long off = ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      if (d[v] != 0.0) atomicAdd(vp.dP + v * cs + off, d[v]);
  }
  __syncthreads();
}

template <int RECON, int RIEMANN>
__global__ void __launch_bounds__(256) rhs_vjp_kernel(const VjpParams vp) {
  extern __shared__ double smem[];
  const SweepParams& p = vp.sp;
  const int b = blockIdx.x;
  const int b2 = b % p.tiles[2];
  const int b1 = (b / p.tiles[2]) % p.tiles[1];
  const int b0 = b / (p.tiles[2] * p.tiles[1]);
  const int o[3] = {b0 * p.t[0], b1 * p.t[1], b2 * p.t[2]};
  const int ext[3] = {min(p.t[0], p.n[0] - o[0]), min(p.t[1], p.n[1] - o[1]), min(p.t[2], p.n[2] - o[2])};
  constexpr int R = ReconTraits<RECON>::R;
  int pmax = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
    if (p.active_mask & (1 << a))
      pmax = max(pmax, (p.t[0] + (a == 0 ? 2 * R : 0)) * (p.t[1] + (a == 1 ? 2 * R : 0)) *
                           (p.t[2] + (a == 2 ? 2 * R : 0)));
  // pencil primitives (and conservatives) | per-thread right-stencil gradients
  // (WENO only) | face slots
  double* sm_prim = smem;
  double* sm_jr = smem + ((RECON == RECON_WENO5Z_CONS || RECON == RECON_WENO5Z_CHARCONS) ? 10 : 5) * pmax;
  double* sm_slot = sm_jr + (ReconTraits<RECON>::R == 3 ? 25 * blockDim.x : 0);
  if (p.active_mask & 1) vjp_axis<0, RECON, RIEMANN>(vp, o, ext, sm_prim, sm_slot, sm_jr);
  if (p.active_mask & 2) vjp_axis<1, RECON, RIEMANN>(vp, o, ext, sm_prim, sm_slot, sm_jr);
  if (p.active_mask & 4) vjp_axis<2, RECON, RIEMANN>(vp, o, ext, sm_prim, sm_slot, sm_jr);
}

// Lax-Friedrichs: the cotangent of each axis' speed alpha = max(max s_L,
// max s_R), s = |u_n| + c of the face states (LaxFriedrichs.py:35-38), goes
// to the face states that attain it, as jax.grad divides it: jnp.maximum
// gives half to each side when both maxima are equal, jnp.max equal shares to
// the ties of a side.  One thread per listed tie (the face kernels' tie pass,
// speed_pass 2, on the same primitives): the tie's face states and stencil
// gradients, the speed's pullback, then the stencil cells' cotangents
// through the boundary remap into dP.  PRIMITIVE reconstructions.
struct LfTieParams {
  SweepParams sp;                   // the state's interior primitives (sp.prims), sizes, boundaries, scheme
  const unsigned long long* ties;   // the tie pass's counters and LfTie entries
  long long cap;                    // entries the list holds
  const double* dalpha;             // cotangent of each axis' speed
  double* dP;                       // primitive cotangent accumulator, interior [5][N]
  double* dU;                       // conservative cotangent accumulator (conservative reconstructions)
};

template <int AX, int RECON>
__global__ void __launch_bounds__(128) lf_tie_vjp_kernel(const LfTieParams tp) {
  const SweepParams& p = tp.sp;
  constexpr int R = ReconTraits<RECON>::R;
  constexpr int K = 2 * R;
  const unsigned long long listed = tp.ties[0];
  const long long n = (long long)listed < tp.cap ? (long long)listed : tp.cap;
  const double nL = (double)tp.ties[1], nR = (double)tp.ties[2];
  const double share = tp.dalpha[AX] * ((nL > 0.0 && nR > 0.0) ? 0.5 : 1.0);
  const bool periodic = p.bc[2 * AX] == GBF_BC_PERIODIC;
  int ext[3] = {p.n[0], p.n[1], p.n[2]};
  ext[AX] = periodic ? p.n[AX] : p.n[AX] + 1;
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const double eps = p.fp.stencil_eps;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const unsigned long long t = tp.ties[4 + e];
    const long long face = LfTie::face(t);
    const int side = LfTie::side(t);
    const double ds = share * LfTie::mult(t) / (side == 0 ? nL : nR);
    int q[3];
    q[2] = (int)(face % ext[2]);
    const long long r = face / ext[2];
    q[1] = (int)(r % ext[1]);
    q[0] = (int)(r / ext[1]);
    // stencil cells q[AX] - R .. q[AX] + R - 1 (face q[AX] - 1/2)
    double wv[5][K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      int g[3] = {q[0], q[1], q[2]};
      g[AX] += k - R;
#pragma unroll
      for (int v = 0; v < 5; ++v) wv[v][k] = global_prim<MODE_STAGE_P>(p, v, g[0], g[1], g[2]);
    }
    double PL[5], PR[5], jl[5][5], jr[5][5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double* w = wv[v];
      if constexpr (RECON == GBF_RECON_WENO5Z) {
        weno5z_jac(w[0], w[1], w[2], w[3], w[4], eps, PL[v], jl[v]);
        weno5z_jac(w[5], w[4], w[3], w[2], w[1], eps, PR[v], jr[v]);
      } else if constexpr (RECON == GBF_RECON_TENO5) {
        teno5_jac(w[0], w[1], w[2], w[3], w[4], eps, PL[v], jl[v]);
        teno5_jac(w[5], w[4], w[3], w[2], w[1], eps, PR[v], jr[v]);
      } else if constexpr (RECON == GBF_RECON_WENO5JS) {
        weno5js_jac(w[0], w[1], w[2], w[3], w[4], eps, PL[v], jl[v]);
        weno5js_jac(w[5], w[4], w[3], w[2], w[1], eps, PR[v], jr[v]);
      } else {
        reconstruct_pair<RECON>(w, eps, PL[v], PR[v]);
      }
    }
    unsigned mL = 0, mR = 0;
    if (p.limiter) {
      // the limited primitives are those of the cell beside the face
      mL = positivity_limit(PL, &wv[0][R - 1], K, p.limiter);
      mR = positivity_limit(PR, &wv[0][R], K, p.limiter);
    }
    double dPs[5] = {0, 0, 0, 0, 0};
    lf_speed_vjp<AX>(side == 0 ? PL : PR, p.fp, ds, dPs);
    const unsigned m = side == 0 ? mL : mR;
    double dw[5][K];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
#pragma unroll
      for (int k = 0; k < K; ++k) dw[v][k] = 0.0;
      const double gv = dPs[v];
      if (m & (1u << v)) {
        dw[v][side == 0 ? R - 1 : R] = gv;
      } else if constexpr (R == 3) {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          if (side == 0) dw[v][k] += gv * jl[v][k];
          else dw[v][5 - k] += gv * jr[v][k];
        }
      } else {
        double d[K];
        reconstruct_pair_vjp<RECON>(wv[v], eps, side == 0 ? gv : 0.0, side == 1 ? gv : 0.0, d);
#pragma unroll
        for (int k = 0; k < K; ++k) dw[v][k] = d[k];
      }
    }
    // stencil cells' cotangents, halo cells through the transpose of their face rule
#pragma unroll
    for (int k = 0; k < K; ++k) {
      int g[3] = {q[0], q[1], q[2]};
      g[AX] += k - R;
      double d[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) d[v] = dw[v][k];
      if (g[AX] < 0 || g[AX] >= p.n[AX]) {
        const int ty = face_type_at(p.bc, p.bf, 2 * AX + (g[AX] >= 0 ? 1 : 0), face_pos(p.n, AX, g));
        g[AX] = bc_src(g[AX], p.n[AX], ty);
#pragma unroll
        for (int v = 0; v < 5; ++v) d[v] *= bc_apply_grad(ty, AX, v);
      }
      const long long off = ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (d[v] != 0.0) atomicAdd(tp.dP + v * cs + off, d[v]);
    }
  }
}

template <int RECON>
int launch_lf_ties_one(int axis, const LfTieParams& tp, cudaStream_t s) {
  const int grid = 152 * 4, threads = 128;
  if (axis == 0) lf_tie_vjp_kernel<0, RECON><<<grid, threads, 0, s>>>(tp);
  else if (axis == 1) lf_tie_vjp_kernel<1, RECON><<<grid, threads, 0, s>>>(tp);
  else lf_tie_vjp_kernel<2, RECON><<<grid, threads, 0, s>>>(tp);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

// The ties of the characteristic and conservative reconstructions (WENO5-Z
// on the six-cell window): the window's primitives (and conservatives, those
// of a halo cell from its halo primitives, material.py:248-250) in local
// memory, the scheme's own face VJP with the speed's cotangent on the tie's
// face state in place of the flux's (VjpParams::lf_tie_side), then the window
// cells' cotangents as the VJP kernel gathers them.
template <int AX, int RECON>
__global__ void __launch_bounds__(128) lf_tie_window_vjp_kernel(const LfTieParams tp) {
  const SweepParams& p = tp.sp;
  constexpr bool CONS = RECON == RECON_WENO5Z_CONS || RECON == RECON_WENO5Z_CHARCONS;
  const unsigned long long listed = tp.ties[0];
  const long long n = (long long)listed < tp.cap ? (long long)listed : tp.cap;
  const double nL = (double)tp.ties[1], nR = (double)tp.ties[2];
  const double share = tp.dalpha[AX] * ((nL > 0.0 && nR > 0.0) ? 0.5 : 1.0);
  const bool periodic = p.bc[2 * AX] == GBF_BC_PERIODIC;
  int ext[3] = {p.n[0], p.n[1], p.n[2]};
  ext[AX] = periodic ? p.n[AX] : p.n[AX] + 1;
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const unsigned long long t = tp.ties[4 + e];
    const long long face = LfTie::face(t);
    const int side = LfTie::side(t);
    int q[3];
    q[2] = (int)(face % ext[2]);
    const long long r = face / ext[2];
    q[1] = (int)(r % ext[1]);
    q[0] = (int)(r / ext[1]);
    // window cells q[AX] - 3 .. q[AX] + 2: primitives in rows 0..4,
    // conservatives in rows 5..9 (variable stride 6, cell stride 1)
    double win[60], slot[30], jr[25];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      int g[3] = {q[0], q[1], q[2]};
      g[AX] += k - 3;
      double P[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) win[v * 6 + k] = P[v] = global_prim<MODE_STAGE_P>(p, v, g[0], g[1], g[2]);
      if constexpr (CONS) {
        double U[5];
        if (g[AX] >= 0 && g[AX] < p.n[AX]) {
          const long long off = ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
#pragma unroll
          for (int v = 0; v < 5; ++v) U[v] = p.cons[v * cs + off];
        } else {
          cons_from_prims(P, U, p.fp.gm1);
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) win[(5 + v) * 6 + k] = U[v];
      }
    }
    VjpParams vt{};
    vt.sp = p;
    vt.lf_tie_side = side;
    vt.lf_tie_ds = share * LfTie::mult(t) / (side == 0 ? nL : nR);
    const double dF[5] = {0, 0, 0, 0, 0};
    double dal = 0.0;
    if constexpr (RECON == RECON_WENO5Z_CHAR)
      char_face_vjp<AX, GBF_RIEMANN_RUSANOV>(vt, win, 6, 1, dF, slot, 1, jr, 1, dal);
    else if constexpr (RECON == RECON_WENO5Z_CHARCONS)
      charcons_face_vjp<AX, GBF_RIEMANN_RUSANOV>(vt, win, 6, 1, dF, slot, 1, jr, 1, dal);
    else
      cons_face_vjp<AX, GBF_RIEMANN_RUSANOV>(vt, win, 6, 1, dF, slot, 1, jr, 1, dal);
    // the window cells' cotangents: primitive ones (CHAR-PRIMITIVE) or
    // conservative ones (interior cells: the state; halo cells: through the
    // conservatives of their halo primitives), halo cells through the
    // transpose of their face rule
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      int g[3] = {q[0], q[1], q[2]};
      g[AX] += k - 3;
      double d[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) d[v] = slot[v * 6 + k];
      const bool halo = g[AX] < 0 || g[AX] >= p.n[AX];
      if (CONS && !halo) {
        const long long off = ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
#pragma unroll
        for (int v = 0; v < 5; ++v)
          if (d[v] != 0.0) atomicAdd(tp.dU + v * cs + off, d[v]);
        continue;
      }
      if (CONS) {
        double P[5], dPh[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int v = 0; v < 5; ++v) P[v] = win[v * 6 + k];
        cons_from_prims_vjp(P, d, 1.0 / P[0], 1.0 / p.fp.gm1, dPh);
#pragma unroll
        for (int v = 0; v < 5; ++v) d[v] = dPh[v];
      }
      if (halo) {
        const int ty = face_type_at(p.bc, p.bf, 2 * AX + (g[AX] >= 0 ? 1 : 0), face_pos(p.n, AX, g));
        g[AX] = bc_src(g[AX], p.n[AX], ty);
#pragma unroll
        for (int v = 0; v < 5; ++v) d[v] *= bc_apply_grad(ty, AX, v);
      }
      const long long off = ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
#pragma unroll
      for (int v = 0; v < 5; ++v)
        if (d[v] != 0.0) atomicAdd(tp.dP + v * cs + off, d[v]);
    }
  }
}

template <int RECON>
int launch_lf_ties_window_one(int axis, const LfTieParams& tp, cudaStream_t s) {
  const int grid = 152 * 4, threads = 128;
  if (axis == 0) lf_tie_window_vjp_kernel<0, RECON><<<grid, threads, 0, s>>>(tp);
  else if (axis == 1) lf_tie_window_vjp_kernel<1, RECON><<<grid, threads, 0, s>>>(tp);
  else lf_tie_window_vjp_kernel<2, RECON><<<grid, threads, 0, s>>>(tp);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_lf_ties_char(int axis, const LfTieParams& tp, cudaStream_t s);
int launch_lf_ties_cons(int axis, const LfTieParams& tp, cudaStream_t s);
int launch_lf_ties_charcons(int axis, const LfTieParams& tp, cudaStream_t s);

// The tie kernels per reconstruction family (gbf_vjp_<family>.cu).
int launch_lf_ties_weno5(int recon, int axis, const LfTieParams& tp, cudaStream_t s);
int launch_lf_ties_teno5(int axis, const LfTieParams& tp, cudaStream_t s);
int launch_lf_ties_short(int recon, int axis, const LfTieParams& tp, cudaStream_t s);

// Launch of rhs_vjp_kernel for one reconstruction family (mode of the
// gbf_vjp_<family>.cu units): recon and riemann select the instantiation.
int launch_vjp_weno5(int recon, int riemann, const VjpParams& vp, int grid, int threads, size_t smem,
                     cudaStream_t s);
int launch_vjp_char(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s);
int launch_vjp_teno5(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s);
int launch_vjp_cons(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s);
int launch_vjp_charcons(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s);
int launch_vjp_short(int recon, int riemann, const VjpParams& vp, int grid, int threads, size_t smem,
                     cudaStream_t s);

template <int RECON, int RIEMANN>
int launch_vjp_one(const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s) {
  auto k = rhs_vjp_kernel<RECON, RIEMANN>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return GBF_ERR_CUDA;
  k<<<grid, threads, smem, s>>>(vp);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

template <int RECON>
int launch_vjp_riemann(int riemann, const VjpParams& vp, int grid, int threads, size_t smem, cudaStream_t s) {
  if (riemann == GBF_RIEMANN_HLLC) return launch_vjp_one<RECON, GBF_RIEMANN_HLLC>(vp, grid, threads, smem, s);
  if (riemann == GBF_RIEMANN_HLL) return launch_vjp_one<RECON, GBF_RIEMANN_HLL>(vp, grid, threads, smem, s);
  return launch_vjp_one<RECON, GBF_RIEMANN_RUSANOV>(vp, grid, threads, smem, s);
}

}  // namespace gbf
