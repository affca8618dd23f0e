// Hand-written reverse mode (vector-Jacobian products) of the right-hand side.
//
// Each function recomputes the forward intermediates of its counterpart in
// gbf_physics.cuh and propagates a cotangent backwards through them, with
// jax.grad's conventions at the non-smooth points the reference hits:
//   d|x|/dx        = +1 at x = 0  (select(x >= 0, g, -g))
//   max / min tie  = half of the cotangent to each argument
//   sign(x)        : zero derivative
//   where(c, a, b) : cotangent to the selected branch only.
#pragma once

#include "gbf_physics.cuh"

namespace gbf {

__device__ __forceinline__ double jabs_grad(double x) { return (x >= 0.0) ? 1.0 : -1.0; }

// d min(a, b): weight of a (1, 0.5 at a tie, 0)
__device__ __forceinline__ double min_weight_a(double a, double b) {
  return (a < b) ? 1.0 : ((a == b) ? 0.5 : 0.0);
}
__device__ __forceinline__ double max_weight_a(double a, double b) {
  return (a > b) ? 1.0 : ((a == b) ? 0.5 : 0.0);
}

// Contraction is on in the reverse pass, except where the forward's rounding
// decides a branch of the derivative: the smoothness terms (flat stencils give
// exact zeros, |b0 - b2| ties) and the HLLC contact-speed numerator (mirrored
// wall states give S* = 0 exactly, where jnp.sign blends both star fluxes)
// use non-fusable products (__dmul_rn) to round like the forward.
//
// weno5z(u0..u4) and its gradient J[k] = d out / d u_k (the reverse pass with
// unit cotangent), so a caller can scale J by the cotangent once it is known
// without recomputing the stencil.  One reciprocal per denominator serves the
// forward ratios and the reverse pass (4 divisions instead of 10); values
// differ from the forward's divisions at rounding level only.
__device__ __forceinline__ void weno5z_jac(double u0, double u1, double u2, double u3, double u4,
                                           double eps, double& out, double J[5]) {
  constexpr double c13 = 13.0 / 12.0;
  const double t0 = u0 - 2.0 * u1 + u2;
  const double t1 = (u0 - 4.0 * u1) + __dmul_rn(3.0, u2);
  const double t2 = u1 - 2.0 * u2 + u3;
  const double t3 = u1 - u3;
  const double t4 = u2 - 2.0 * u3 + u4;
  const double t5 = fma(-4.0, u3, __dmul_rn(3.0, u2)) + u4;
  const double b0 = c13 * (t0 * t0) + 0.25 * (t1 * t1);
  const double b1 = c13 * (t2 * t2) + 0.25 * (t3 * t3);
  const double b2 = c13 * (t4 * t4) + 0.25 * (t5 * t5);
  const double tau = fabs(b0 - b2);
  const double ie0 = 1.0 / (b0 + eps), ie1 = 1.0 / (b1 + eps), ie2 = 1.0 / (b2 + eps);
  const double q0 = tau * ie0, q1 = tau * ie1, q2 = tau * ie2;
  const double a0 = 0.1 * (1.0 + q0), a1 = 0.6 * (1.0 + q1), a2 = 0.3 * (1.0 + q2);
  const double r = 1.0 / (a0 + a1 + a2);
  const double p0 = (1.0 / 3.0) * u0 + (-7.0 / 6.0) * u1 + (11.0 / 6.0) * u2;
  const double p1 = (-1.0 / 6.0) * u1 + (5.0 / 6.0) * u2 + (1.0 / 3.0) * u3;
  const double p2 = (1.0 / 3.0) * u2 + (5.0 / 6.0) * u3 + (-1.0 / 6.0) * u4;
  // out = (a0 p0 + a1 p1 + a2 p2) r = w0 p0 + w1 p1 + w2 p2
  const double w0 = a0 * r, w1 = a1 * r, w2 = a2 * r;
  out = w0 * p0 + w1 * p1 + w2 * p2;
  J[0] = (1.0 / 3.0) * w0;
  J[1] = (-7.0 / 6.0) * w0 + (-1.0 / 6.0) * w1;
  J[2] = (11.0 / 6.0) * w0 + (5.0 / 6.0) * w1 + (1.0 / 3.0) * w2;
  J[3] = (1.0 / 3.0) * w1 + (5.0 / 6.0) * w2;
  J[4] = (-1.0 / 6.0) * w2;
  // d out / d a_k = r (p_k - out)
  const double da0 = r * (p0 - out), da1 = r * (p1 - out), da2 = r * (p2 - out);
  const double dq0 = 0.1 * da0 * ie0, dq1 = 0.6 * da1 * ie1, dq2 = 0.3 * da2 * ie2;
  const double dtau = dq0 + dq1 + dq2;
  double db0 = -dq0 * q0;
  const double db1 = -dq1 * q1;
  double db2 = -dq2 * q2;
  const double sg = jabs_grad(b0 - b2);
  db0 += dtau * sg;
  db2 -= dtau * sg;
  const double dt0 = db0 * (2.0 * c13) * t0, dt1 = db0 * 0.5 * t1;
  const double dt2 = db1 * (2.0 * c13) * t2, dt3 = db1 * 0.5 * t3;
  const double dt4 = db2 * (2.0 * c13) * t4, dt5 = db2 * 0.5 * t5;
  J[0] += dt0 + dt1;
  J[1] += -2.0 * dt0 - 4.0 * dt1 + dt2 + dt3;
  J[2] += dt0 + 3.0 * dt1 - 2.0 * dt2 + dt4 + 3.0 * dt5;
  J[3] += dt2 - dt3 - 2.0 * dt4 - 4.0 * dt5;
  J[4] += dt4 + dt5;
}

// weno5js(u0..u4) and its gradient (weno/weno5_js.py:33-70): as weno5z_jac
// with alpha_k = d_k / (beta_k^2 + eps), d alpha_k / d beta_k = -2 alpha_k beta_k / (beta_k^2 + eps).
__device__ __forceinline__ void weno5js_jac(double u0, double u1, double u2, double u3, double u4,
                                            double eps, double& out, double J[5]) {
  constexpr double c13 = 13.0 / 12.0;
  const double t0 = u0 - 2.0 * u1 + u2;
  const double t1 = (u0 - 4.0 * u1) + __dmul_rn(3.0, u2);
  const double t2 = u1 - 2.0 * u2 + u3;
  const double t3 = u1 - u3;
  const double t4 = u2 - 2.0 * u3 + u4;
  const double t5 = fma(-4.0, u3, __dmul_rn(3.0, u2)) + u4;
  const double b0 = c13 * (t0 * t0) + 0.25 * (t1 * t1);
  const double b1 = c13 * (t2 * t2) + 0.25 * (t3 * t3);
  const double b2 = c13 * (t4 * t4) + 0.25 * (t5 * t5);
  const double ie0 = 1.0 / (b0 * b0 + eps), ie1 = 1.0 / (b1 * b1 + eps), ie2 = 1.0 / (b2 * b2 + eps);
  const double a0 = 0.1 * ie0, a1 = 0.6 * ie1, a2 = 0.3 * ie2;
  const double r = 1.0 / (a0 + a1 + a2);
  const double p0 = (1.0 / 3.0) * u0 + (-7.0 / 6.0) * u1 + (11.0 / 6.0) * u2;
  const double p1 = (-1.0 / 6.0) * u1 + (5.0 / 6.0) * u2 + (1.0 / 3.0) * u3;
  const double p2 = (1.0 / 3.0) * u2 + (5.0 / 6.0) * u3 + (-1.0 / 6.0) * u4;
  const double w0 = a0 * r, w1 = a1 * r, w2 = a2 * r;
  out = w0 * p0 + w1 * p1 + w2 * p2;
  J[0] = (1.0 / 3.0) * w0;
  J[1] = (-7.0 / 6.0) * w0 + (-1.0 / 6.0) * w1;
  J[2] = (11.0 / 6.0) * w0 + (5.0 / 6.0) * w1 + (1.0 / 3.0) * w2;
  J[3] = (1.0 / 3.0) * w1 + (5.0 / 6.0) * w2;
  J[4] = (-1.0 / 6.0) * w2;
  const double db0 = -2.0 * r * (p0 - out) * a0 * b0 * ie0;
  const double db1 = -2.0 * r * (p1 - out) * a1 * b1 * ie1;
  const double db2 = -2.0 * r * (p2 - out) * a2 * b2 * ie2;
  const double dt0 = db0 * (2.0 * c13) * t0, dt1 = db0 * 0.5 * t1;
  const double dt2 = db1 * (2.0 * c13) * t2, dt3 = db1 * 0.5 * t3;
  const double dt4 = db2 * (2.0 * c13) * t4, dt5 = db2 * 0.5 * t5;
  J[0] += dt0 + dt1;
  J[1] += -2.0 * dt0 - 4.0 * dt1 + dt2 + dt3;
  J[2] += dt0 + 3.0 * dt1 - 2.0 * dt2 + dt4 + 3.0 * dt5;
  J[3] += dt2 - dt3 - 2.0 * dt4 - 4.0 * dt5;
  J[4] += dt4 + dt5;
}

// teno5(u0..u4) and its gradient (teno/teno5.py): the cutoff weights are
// piecewise constant (jnp.where), so d out / d u = sum_k omega_k d p_k / d u.
__device__ __forceinline__ void teno5_jac(double u0, double u1, double u2, double u3, double u4, double eps,
                                          double& out, double J[5]) {
  double b0, b1, b2, o0, o1, o2;
  weno5_smoothness(u0, u1, u2, u3, u4, b0, b1, b2);
  teno5_weights(b0, b1, b2, eps, o0, o1, o2);
  const double p0 = (1.0 / 3.0) * u0 + (-7.0 / 6.0) * u1 + (11.0 / 6.0) * u2;
  const double p1 = (-1.0 / 6.0) * u1 + (5.0 / 6.0) * u2 + (1.0 / 3.0) * u3;
  const double p2 = (1.0 / 3.0) * u2 + (5.0 / 6.0) * u3 + (-1.0 / 6.0) * u4;
  out = o0 * p0 + o1 * p1 + o2 * p2;
  J[0] = (1.0 / 3.0) * o0;
  J[1] = (-7.0 / 6.0) * o0 + (-1.0 / 6.0) * o1;
  J[2] = (11.0 / 6.0) * o0 + (5.0 / 6.0) * o1 + (1.0 / 3.0) * o2;
  J[3] = (1.0 / 3.0) * o1 + (5.0 / 6.0) * o2;
  J[4] = (-1.0 / 6.0) * o2;
}

// weno3<Z>(u0, u1, u2) and its gradient (weno/weno3_js.py:22-45,
// weno/weno3_z.py:24-46, weno3_base.py:20-44).
template <bool Z>
__device__ __forceinline__ void weno3_jac(double u0, double u1, double u2, double eps, double& out, double J[3]) {
  const double e0 = u1 - u0, e1 = u2 - u1;
  const double b0 = e0 * e0, b1 = e1 * e1;
  double a0, a1, da0_db0, da1_db1, tau = 0.0, ie0 = 0.0, ie1 = 0.0;
  if (Z) {
    tau = fabs(b0 - b1);
    ie0 = 1.0 / (b0 + eps);
    ie1 = 1.0 / (b1 + eps);
    a0 = (1.0 / 3.0) * (1.0 + tau * ie0);
    a1 = (2.0 / 3.0) * (1.0 + tau * ie1);
    da0_db0 = da1_db1 = 0.0;
  } else {
    ie0 = 1.0 / (b0 * b0 + eps);
    ie1 = 1.0 / (b1 * b1 + eps);
    a0 = (1.0 / 3.0) * ie0;
    a1 = (2.0 / 3.0) * ie1;
    da0_db0 = -2.0 * a0 * b0 * ie0;
    da1_db1 = -2.0 * a1 * b1 * ie1;
  }
  const double r = 1.0 / (a0 + a1);
  const double p0 = -0.5 * u0 + 1.5 * u1, p1 = 0.5 * u1 + 0.5 * u2;
  const double w0 = a0 * r, w1 = a1 * r;
  out = w0 * p0 + w1 * p1;
  J[0] = -0.5 * w0;
  J[1] = 1.5 * w0 + 0.5 * w1;
  J[2] = 0.5 * w1;
  const double da0 = r * (p0 - out), da1 = r * (p1 - out);
  double db0, db1;
  if (Z) {
    // a_k = d_k (1 + tau / (b_k + eps))
    const double dq0 = (1.0 / 3.0) * da0 * ie0, dq1 = (2.0 / 3.0) * da1 * ie1;
    const double dtau = dq0 + dq1;
    db0 = -dq0 * tau * ie0;
    db1 = -dq1 * tau * ie1;
    const double sg = jabs_grad(b0 - b1);
    db0 += dtau * sg;
    db1 -= dtau * sg;
  } else {
    db0 = da0 * da0_db0;
    db1 = da1 * da1_db1;
  }
  const double de0 = 2.0 * e0 * db0, de1 = 2.0 * e1 * db1;
  J[0] -= de0;
  J[1] += de0 - de1;
  J[2] += de1;
}

// Reverse of minmod_ad<J>(b0, b1, b2): the ratio only selects a branch.
template <int J>
__device__ __forceinline__ void minmod_ad_vjp(double b0, double b1, double b2, double eps, double g,
                                              double& db0, double& db1, double& db2) {
  const double dc = (J == 0) ? b2 - b1 : b1 - b2;
  const double du = (J == 0) ? b1 - b0 : b0 - b1;
  const double r = (du >= eps) ? dc / (du + 1e-100) : (dc + eps) / (du + eps);
  if (r < 0.0) {
    db1 += g;
  } else if (r < 1.0) {
    db1 += 0.5 * g;
    db2 += 0.5 * g;
  } else {
    db1 += 1.5 * g;
    db0 -= 0.5 * g;
  }
}

// Reverse of muscl_minmod<J>(b0, b1, b2) (muscl3.py:53-75, limiter.py:9-10):
// out = b1 +- 0.5 lim du with lim = max(0, min(1, r)); the limiter passes the
// ratio's derivative inside (0, 1) and half of it at r = 0 and at r = 1, where
// jnp.minimum / jnp.maximum split a tie evenly; the ratio's branch is the one
// the forward selects (jnp.where routes no cotangent to the other).
template <int J>
__device__ __forceinline__ void minmod_vjp(double b0, double b1, double b2, double eps, double g,
                                           double& db0, double& db1, double& db2) {
  const double dc = (J == 0) ? b2 - b1 : b1 - b2;
  const double du = (J == 0) ? b1 - b0 : b0 - b1;
  const bool upwind = du >= eps;
  const double num = upwind ? dc : dc + eps;
  const double den = upwind ? du + 1e-10 : du + eps;
  const double r = num / den;
  const double m = fmin(1.0, r);
  const double lim = fmax(0.0, m);
  const double s = (J == 0) ? 0.5 : -0.5;  // out = b1 + s lim du
  const double wmin = (r < 1.0) ? 1.0 : ((r == 1.0) ? 0.5 : 0.0);
  const double wmax = (m > 0.0) ? 1.0 : ((m == 0.0) ? 0.5 : 0.0);
  const double g_r = s * du * g * (wmin * wmax);
  const double g_dc = g_r / den;            // d r / d num = 1 / den
  const double g_du = s * lim * g - g_dc * r;  // explicit du, and d r / d den = -r / den
  if (J == 0) {  // dc = b2 - b1, du = b1 - b0
    db2 += g_dc;
    db1 += g - g_dc + g_du;
    db0 -= g_du;
  } else {  // dc = b1 - b2, du = b0 - b1
    db1 += g + g_dc - g_du;
    db2 -= g_dc;
    db0 += g_du;
  }
}

// Reverse of reconstruct_pair<RECON> for the four-cell stencils (WENO3-JS,
// WENO3-Z, MINMOD, MINMOD-AD): dw[k] = gL dL/dw_k + gR dR/dw_k.  The five-point WENO
// stencils take the single-pass value-and-gradient route (weno5z_jac,
// weno5js_jac) in the tile kernel instead.
template <int RECON>
__device__ __forceinline__ void reconstruct_pair_vjp(const double* w, double eps, double gL, double gR,
                                                     double* dw);

template <bool Z>
__device__ __forceinline__ void weno3_pair_vjp(const double* w, double eps, double gL, double gR, double* dw) {
  // j=0 (w0, w1, w2), j=1 (w3, w2, w1)
  double jl[3], jr[3], vl, vr;
  weno3_jac<Z>(w[0], w[1], w[2], eps, vl, jl);
  weno3_jac<Z>(w[3], w[2], w[1], eps, vr, jr);
  dw[0] = gL * jl[0];
  dw[1] = gL * jl[1] + gR * jr[2];
  dw[2] = gL * jl[2] + gR * jr[1];
  dw[3] = gR * jr[0];
}

template <>
__device__ __forceinline__ void reconstruct_pair_vjp<GBF_RECON_WENO3JS>(const double* w, double eps,
                                                                         double gL, double gR, double* dw) {
  weno3_pair_vjp<false>(w, eps, gL, gR, dw);
}

template <>
__device__ __forceinline__ void reconstruct_pair_vjp<GBF_RECON_WENO3Z>(const double* w, double eps,
                                                                        double gL, double gR, double* dw) {
  weno3_pair_vjp<true>(w, eps, gL, gR, dw);
}

template <>
__device__ __forceinline__ void reconstruct_pair_vjp<GBF_RECON_MINMOD>(const double* w, double eps,
                                                                        double gL, double gR, double* dw) {
  double d[4] = {0, 0, 0, 0};
  minmod_vjp<0>(w[0], w[1], w[2], eps, gL, d[0], d[1], d[2]);
  minmod_vjp<1>(w[3], w[2], w[1], eps, gR, d[3], d[2], d[1]);
  dw[0] = d[0];
  dw[1] = d[1];
  dw[2] = d[2];
  dw[3] = d[3];
}

template <>
__device__ __forceinline__ void reconstruct_pair_vjp<GBF_RECON_MINMOD_AD>(const double* w, double eps,
                                                                           double gL, double gR, double* dw) {
  double d[4] = {0, 0, 0, 0};
  minmod_ad_vjp<0>(w[0], w[1], w[2], eps, gL, d[0], d[1], d[2]);
  minmod_ad_vjp<1>(w[3], w[2], w[1], eps, gR, d[3], d[2], d[1]);
  dw[0] = d[0];
  dw[1] = d[1];
  dw[2] = d[2];
  dw[3] = d[3];
}

// Face states and their reciprocals, shared by the forward recomputation and
// the reverse pass of a Riemann solver: U = cons(P) with e = p / (rho gm1)
// formed as p (1/rho)(1/gm1), and c = sqrt(gamma p / rho) with 1/c from one
// rsqrt.  Results differ from the forward's divisions at rounding level only.
struct FaceSide {
  double U[5];
  double ir;   // 1 / rho
  double y;    // gamma p / rho
  double c;    // speed of sound
  double ic;   // 1 / c
};

__device__ __forceinline__ void face_side(const double P[5], double gamma, double igm1, FaceSide& s) {
  s.ir = 1.0 / P[0];
  const double e = P[4] * s.ir * igm1;
  s.U[0] = P[0];
  s.U[1] = P[0] * P[1];
  s.U[2] = P[0] * P[2];
  s.U[3] = P[0] * P[3];
  s.U[4] = P[0] * (0.5 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]) + e);
  s.y = gamma * P[4] * s.ir;
  s.ic = rsqrt(s.y);
  s.c = s.y * s.ic;
}

// Reverse of cons_from_prims: dP += (dU/dP)^T dU.
__device__ __forceinline__ void cons_from_prims_vjp(const double P[5], const double dU[5], double ir,
                                                    double igm1, double dP[5]) {
  const double rho = P[0];
  const double e = P[4] * ir * igm1;
  const double s = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
  const double h = 0.5 * s + e;
  // U0 = rho, Ui = rho Pi, U4 = rho h
  double drho = dU[0] + dU[1] * P[1] + dU[2] * P[2] + dU[3] * P[3] + dU[4] * h;
  const double dh = dU[4] * rho;
#pragma unroll
  for (int i = 1; i <= 3; ++i) dP[i] += dU[i] * rho + dh * P[i];
  // e = P4 / (rho gm1): de/dP4 = 1/(rho gm1), de/drho = -e/rho
  dP[4] += dh * ir * igm1;
  drho -= dh * e * ir;
  dP[0] += drho;
}

// Reverse of prims_from_cons: dU += (dP/dU)^T dP.
__device__ __forceinline__ void prims_from_cons_vjp(const double U[5], const double dP[5], double gm1,
                                                    double dU[5]) {
  const double rho = U[0];
  const double one_rho = 1.0 / rho;
  const double u = U[1] * one_rho, v = U[2] * one_rho, w = U[3] * one_rho;
  const double e = U[4] * one_rho - 0.5 * (u * u + v * v + w * w);
  // P0 = rho, P1..3 = U1..3 * one_rho, P4 = gm1 e rho
  double drho = dP[0] + dP[4] * gm1 * e;
  const double de = dP[4] * gm1 * rho;
  const double ds = -0.5 * de;
  const double du = dP[1] + ds * 2.0 * u;
  const double dv = dP[2] + ds * 2.0 * v;
  const double dw = dP[3] + ds * 2.0 * w;
  double done = de * U[4] + du * U[1] + dv * U[2] + dw * U[3];
  dU[4] += de * one_rho;
  dU[1] += du * one_rho;
  dU[2] += dv * one_rho;
  dU[3] += dw * one_rho;
  drho += -done * one_rho * one_rho;
  dU[0] += drho;
}


// Reverse of the physical flux F(P, U) along AX (equation_manager.py:237-252).
template <int AX>
__device__ __forceinline__ void physical_flux_vjp(const double P[5], const double U[5], const double dF[5],
                                                  double dP[5], double dU[5]) {
  constexpr int N = AX + 1;
  const double m = U[N];
  dU[N] += dF[0] + dF[1] * P[1] + dF[2] * P[2] + dF[3] * P[3];
  dP[1] += dF[1] * m;
  dP[2] += dF[2] * m;
  dP[3] += dF[3] * m;
  dP[N] += dF[4] * (U[4] + P[4]);
  dU[4] += dF[4] * P[N];
  dP[4] += dF[4] * P[N] + dF[N];
}

// Reverse of hllc_star_flux<AX, J> (HLLC.py:41-78).  Accumulates into dP, dU,
// dS (own wave speed) and dSs (contact speed); ir = 1/rho of this side.
template <int AX, int J>
__device__ __forceinline__ void hllc_star_flux_vjp(const double P[5], const double U[5], double ir, double S,
                                                   double Ss, const double dF[5], double dP[5], double dU[5],
                                                   double& dS, double& dSs) {
  constexpr int N = AX + 1;
  constexpr int T1 = (AX == 0) ? 2 : 1;
  constexpr int T2 = (AX == 2) ? 2 : 3;
  const double n1 = S - P[N];
  const double d1 = S - Ss;
  const double in1 = 1.0 / n1, id1 = 1.0 / d1;
  const double m = n1 * id1;
  const double pre = m * P[0];
  const double A = U[4] * ir;
  const double q = P[4] * ir;
  const double D = q * in1;
  const double B = Ss - P[N];
  const double C = Ss + D;
  const double X = A + B * C;
  const double e_term = pre * X;
  double us[5] = {pre, pre, pre, pre, e_term};
  us[N] *= Ss;
  us[T1] *= P[T1];
  us[T2] *= P[T2];
  const double wave = (J == 0) ? fmin(S, 0.0) : fmax(S, 0.0);
  // F* = F(P, U) + wave (us - U)
  physical_flux_vjp<AX>(P, U, dF, dP, dU);
  double dwave = 0.0;
  double dus[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    dwave += dF[v] * (us[v] - U[v]);
    dus[v] = wave * dF[v];
    dU[v] -= wave * dF[v];
  }
  dS += dwave * ((J == 0) ? min_weight_a(S, 0.0) : max_weight_a(S, 0.0));
  // us components
  const double dpre = dus[0] + dus[N] * Ss + dus[T1] * P[T1] + dus[T2] * P[T2] + dus[4] * X;
  dSs += dus[N] * pre;
  dP[T1] += dus[T1] * pre;
  dP[T2] += dus[T2] * pre;
  const double dX = dus[4] * pre;
  // X = A + B C, A = U4 / U0
  dU[4] += dX * ir;
  dU[0] -= dX * A * ir;
  const double dB = dX * C, dC = dX * B;
  dSs += dB + dC;
  double du = -dB;
  // D = q / n1, q = P4 / P0
  const double dq = dC * in1;
  double dn1 = -dC * D * in1;
  dP[4] += dq * ir;
  dP[0] -= dq * q * ir;
  // pre = m rho, m = n1 / d1
  const double dm = dpre * P[0];
  dP[0] += dpre * m;
  dn1 += dm * id1;
  const double dd1 = -dm * m * id1;
  dS += dn1 + dd1;
  du -= dn1;
  dSs -= dd1;
  dP[N] += du;
}

// Einfeldt wave speeds (signal_speeds.py:109-133) recomputed for a reverse
// pass, with 1/sqrt(rho) and 1/dbar from rsqrt.
struct Einfeldt {
  double isL, isR, sL, sR, od, eta2, ubar, duu, Wn, idbar, X1, X2, Y1, Y2, SL, SR;
};

__device__ __forceinline__ void einfeldt_fwd(double uL, double uR, double rL, double rR, double cL, double cR,
                                             Einfeldt& e) {
  e.isL = rsqrt(rL);
  e.isR = rsqrt(rR);
  e.sL = rL * e.isL;
  e.sR = rR * e.isR;
  e.od = 1.0 / (e.sL + e.sR);
  e.eta2 = 0.5 * e.sL * e.sR * e.od * e.od;
  e.ubar = (e.sL * uL + e.sR * uR) * e.od;
  e.duu = uR - uL;
  e.Wn = e.sL * cL * cL + e.sR * cR * cR;
  const double Z = e.Wn * e.od + e.eta2 * (e.duu * e.duu);
  e.idbar = rsqrt(Z);
  const double dbar = Z * e.idbar;
  e.X1 = e.ubar - dbar;
  e.X2 = uL - cL;
  e.Y1 = e.ubar + dbar;
  e.Y2 = uR + cR;
  e.SL = fmin(e.X1, e.X2);
  e.SR = fmax(e.Y1, e.Y2);
}

// Reverse of einfeldt_fwd: cotangents dSL, dSR of the wave speeds added to
// those of the normal velocities, densities and sounds speeds of both sides.
__device__ __forceinline__ void einfeldt_vjp(const Einfeldt& e, double uL, double uR, double cL, double cR,
                                             double dSL, double dSR, double& duL, double& duR, double& drL,
                                             double& drR, double& dcL, double& dcR) {
  // SL = min(X1, X2), SR = max(Y1, Y2)
  const double wx = min_weight_a(e.X1, e.X2), wy = max_weight_a(e.Y1, e.Y2);
  const double dX1 = dSL * wx, dX2 = dSL * (1.0 - wx);
  const double dY1 = dSR * wy, dY2 = dSR * (1.0 - wy);
  const double dubar = dX1 + dY1;
  const double ddbar = -dX1 + dY1;
  duL += dX2;
  dcL -= dX2;
  duR += dY2;
  dcR += dY2;
  // dbar = sqrt(Z), Z = Wn od + eta2 du^2
  const double dZ = ddbar * 0.5 * e.idbar;
  const double dWn = dZ * e.od;
  double dod = dZ * e.Wn;
  const double deta2 = dZ * (e.duu * e.duu);
  const double dduu = dZ * e.eta2 * 2.0 * e.duu;
  duR += dduu;
  duL -= dduu;
  double dsL = dWn * cL * cL, dsR = dWn * cR * cR;
  dcL += dWn * e.sL * 2.0 * cL;
  dcR += dWn * e.sR * 2.0 * cR;
  // eta2 = 0.5 sL sR od od
  const double od2 = e.od * e.od;
  dsL += deta2 * 0.5 * e.sR * od2;
  dsR += deta2 * 0.5 * e.sL * od2;
  dod += deta2 * e.sL * e.sR * e.od;
  // ubar = (sL uL + sR uR) od
  dsL += dubar * uL * e.od;
  dsR += dubar * uR * e.od;
  duL += dubar * e.sL * e.od;
  duR += dubar * e.sR * e.od;
  dod += dubar * (e.sL * uL + e.sR * uR);
  // od = 1 / (sL + sR)
  const double dsum = -dod * od2;
  dsL += dsum;
  dsR += dsum;
  drL += dsL * 0.5 * e.isL;
  drR += dsR * 0.5 * e.isR;
}

// The wave speeds of every signal_speed estimate (signal_speeds.py:10-157,
// :201-231; the forward's signal_speeds in gbf_physics.cuh) recomputed for a
// reverse pass: EINFELDT through Einfeldt above; DAVIS, ARITHMETIC and RUSANOV
// as min / max of two candidates (X, Y); TORO with the pressure estimate.
struct WaveSpeeds {
  int kind;
  Einfeldt e;
  double X1, X2, Y1, Y2;         // SL = min(X1, X2), SR = max(Y1, Y2) (RUSANOV: Y = |u| + c)
  double ppvrs, pstar, g, qL, qR;  // TORO
  double SL, SR;
};

__device__ __forceinline__ void wave_speeds_fwd(int kind, double uL, double uR, double rL, double rR, double pL,
                                                double pR, double cL, double cR, double gamma, WaveSpeeds& w) {
  w.kind = kind;
  switch (kind) {
    case GBF_SIGNAL_EINFELDT:
      einfeldt_fwd(uL, uR, rL, rR, cL, cR, w.e);
      w.SL = w.e.SL;
      w.SR = w.e.SR;
      break;
    case GBF_SIGNAL_DAVIS:
      w.X1 = uL - cL;
      w.X2 = uR - cR;
      w.Y1 = uL + cL;
      w.Y2 = uR + cR;
      w.SL = fmin(w.X1, w.X2);
      w.SR = fmax(w.Y1, w.Y2);
      break;
    case GBF_SIGNAL_ARITHMETIC: {
      const double um = 0.5 * (uL + uR), am = 0.5 * (cL + cR);
      w.X1 = um - am;
      w.X2 = uL - cL;
      w.Y1 = um + am;
      w.Y2 = uR + cR;
      w.SL = fmin(w.X1, w.X2);
      w.SR = fmax(w.Y1, w.Y2);
      break;
    }
    case GBF_SIGNAL_RUSANOV:
      w.Y1 = fabs(uL) + cL;
      w.Y2 = fabs(uR) + cR;
      w.SR = fmax(w.Y1, w.Y2);
      w.SL = -w.SR;
      break;
    default: {  // TORO
      const double rho_bar = 0.5 * (rL + rR), a_bar = 0.5 * (cL + cR);
      w.ppvrs = 0.5 * (pL + pR) - 0.5 * (uR - uL) * rho_bar * a_bar;
      w.pstar = fmax(0.0, w.ppvrs);
      w.g = (gamma + 1) * 0.5 / gamma;
      w.qL = (w.pstar <= pL) ? 1.0 : sqrt(1 + w.g * (w.pstar / pL - 1));
      w.qR = (w.pstar <= pR) ? 1.0 : sqrt(1 + w.g * (w.pstar / pR - 1));
      w.SL = uL - cL * w.qL;
      w.SR = uR + cR * w.qR;
      break;
    }
  }
}

// Reverse of wave_speeds_fwd: cotangents dSL, dSR added to those of the normal
// velocities, densities, sound speeds and (TORO) pressures of both sides.
__device__ __forceinline__ void wave_speeds_vjp(const WaveSpeeds& w, double uL, double uR, double rL, double rR,
                                                double pL, double pR, double cL, double cR, double dSL, double dSR,
                                                double& duL, double& duR, double& drL, double& drR, double& dcL,
                                                double& dcR, double& dpL, double& dpR) {
  switch (w.kind) {
    case GBF_SIGNAL_EINFELDT:
      einfeldt_vjp(w.e, uL, uR, cL, cR, dSL, dSR, duL, duR, drL, drR, dcL, dcR);
      break;
    case GBF_SIGNAL_DAVIS: {
      const double wx = min_weight_a(w.X1, w.X2), wy = max_weight_a(w.Y1, w.Y2);
      const double dX1 = dSL * wx, dX2 = dSL * (1.0 - wx), dY1 = dSR * wy, dY2 = dSR * (1.0 - wy);
      duL += dX1 + dY1;
      dcL += dY1 - dX1;
      duR += dX2 + dY2;
      dcR += dY2 - dX2;
      break;
    }
    case GBF_SIGNAL_ARITHMETIC: {
      const double wx = min_weight_a(w.X1, w.X2), wy = max_weight_a(w.Y1, w.Y2);
      const double dX1 = dSL * wx, dX2 = dSL * (1.0 - wx), dY1 = dSR * wy, dY2 = dSR * (1.0 - wy);
      const double dum = dX1 + dY1, dam = dY1 - dX1;
      duL += 0.5 * dum + dX2;
      duR += 0.5 * dum + dY2;
      dcL += 0.5 * dam - dX2;
      dcR += 0.5 * dam + dY2;
      break;
    }
    case GBF_SIGNAL_RUSANOV: {
      const double dsp = dSR - dSL;
      const double wy = max_weight_a(w.Y1, w.Y2);
      const double daL = dsp * wy, daR = dsp * (1.0 - wy);
      duL += daL * jabs_grad(uL);
      dcL += daL;
      duR += daR * jabs_grad(uR);
      dcR += daR;
      break;
    }
    default: {  // TORO: SL = uL - cL qL, SR = uR + cR qR
      duL += dSL;
      dcL -= dSL * w.qL;
      const double dqL = -dSL * cL;
      duR += dSR;
      dcR += dSR * w.qR;
      const double dqR = dSR * cR;
      double dps = 0.0;
      // q = sqrt(1 + g (p* / p - 1)) where p* > p: dq/dp* = g / (2 q p), dq/dp = -g p* / (2 q p^2)
      if (w.pstar > pL) {
        const double h = dqL * w.g * 0.5 / (w.qL * pL);
        dps += h;
        dpL -= h * w.pstar / pL;
      }
      if (w.pstar > pR) {
        const double h = dqR * w.g * 0.5 / (w.qR * pR);
        dps += h;
        dpR -= h * w.pstar / pR;
      }
      // p* = max(0, p_pvrs); p_pvrs = (pL + pR) / 2 - (uR - uL) rho_bar a_bar / 2
      const double dpv = dps * max_weight_a(w.ppvrs, 0.0);
      const double rho_bar = 0.5 * (rL + rR), a_bar = 0.5 * (cL + cR);
      dpL += 0.5 * dpv;
      dpR += 0.5 * dpv;
      const double ddu = -0.5 * dpv * rho_bar * a_bar;
      duR += ddu;
      duL -= ddu;
      const double drb = -0.5 * dpv * (uR - uL) * a_bar, dab = -0.5 * dpv * (uR - uL) * rho_bar;
      drL += 0.5 * drb;
      drR += 0.5 * drb;
      dcL += 0.5 * dab;
      dcR += 0.5 * dab;
      break;
    }
  }
}

// Reverse of c = sqrt(y), y = gamma p / rho for one side: dc onto dP[0], dP[4].
__device__ __forceinline__ void sound_speed_vjp(const FaceSide& S, double gamma, double dc, double dP[5]) {
  const double dy = dc * 0.5 * S.ic;
  dP[0] -= dy * S.y * S.ir;
  dP[4] += dy * S.ir * gamma;
}

// Reverse of hllc<AX> with any signal-speed estimate (HLLC.py:80-126,
// signal_speeds.py:10-199); the cons of the face states are
// recomputed and reversed too.  dPL, dPR are accumulated.
template <int AX>
__device__ __forceinline__ void hllc_vjp(const double PL[5], const double PR[5], const FaceParams& fp,
                                         const double dF[5], double dPL[5], double dPR[5]) {
  constexpr int N = AX + 1;
  const double gamma = fp.gamma;
  const double igm1 = 1.0 / fp.gm1;
  FaceSide L, R;
  face_side(PL, gamma, igm1, L);
  face_side(PR, gamma, igm1, R);
  const double uL = PL[N], uR = PR[N], rL = PL[0], rR = PR[0], pL = PL[4], pR = PR[4];
  WaveSpeeds e;
  wave_speeds_fwd(fp.signal_speed, uL, uR, rL, rR, pL, pR, L.c, R.c, gamma, e);
  const double SL = e.SL, SR = e.SR;
  const double rdL = rL * (SL - uL), rdR = rR * (SR - uR);
  const double num = (pR - pL) + (__dmul_rn(uL, rdL) - __dmul_rn(uR, rdR));
  const double den = rdL - rdR;
  const double iden = 1.0 / den;
  const double Ss = num * iden;
  const double sg = (Ss > 0.0) ? 1.0 : ((Ss < 0.0) ? -1.0 : 0.0);
  const double wl = 0.5 * (1.0 + sg), wr = 0.5 * (1.0 - sg);
  double dUL[5] = {0, 0, 0, 0, 0}, dUR[5] = {0, 0, 0, 0, 0};
  double dSL = 0.0, dSR = 0.0, dSs = 0.0;
  if (wl != 0.0) {
    double g[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) g[v] = wl * dF[v];
    hllc_star_flux_vjp<AX, 0>(PL, L.U, L.ir, SL, Ss, g, dPL, dUL, dSL, dSs);
  }
  if (wr != 0.0) {
    double g[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) g[v] = wr * dF[v];
    hllc_star_flux_vjp<AX, 1>(PR, R.U, R.ir, SR, Ss, g, dPR, dUR, dSR, dSs);
  }
  // Ss = num / den
  const double dnum = dSs * iden;
  const double dden = -dSs * Ss * iden;
  dPR[4] += dnum;
  dPL[4] -= dnum;
  double duL = dnum * rdL, duR = -dnum * rdR;
  const double drdL = dnum * uL + dden, drdR = -dnum * uR - dden;
  // rd = rho (S - u)
  double drL = drdL * (SL - uL), drR = drdR * (SR - uR);
  dSL += drdL * rL;
  duL -= drdL * rL;
  dSR += drdR * rR;
  duR -= drdR * rR;
  double dcL = 0.0, dcR = 0.0, dpL = 0.0, dpR = 0.0;
  wave_speeds_vjp(e, uL, uR, rL, rR, pL, pR, L.c, R.c, dSL, dSR, duL, duR, drL, drR, dcL, dcR, dpL, dpR);
  sound_speed_vjp(L, gamma, dcL, dPL);
  sound_speed_vjp(R, gamma, dcR, dPR);
  dPL[0] += drL;
  dPR[0] += drR;
  dPL[N] += duL;
  dPR[N] += duR;
  dPL[4] += dpL;
  dPR[4] += dpR;
  // U = cons(P)
  cons_from_prims_vjp(PL, dUL, L.ir, igm1, dPL);
  cons_from_prims_vjp(PR, dUR, R.ir, igm1, dPR);
}

// Reverse of hll<AX> with any signal-speed estimate (HLL.py:28-58):
// F = N / den, N = SR FL - SL FR + SL SR (UR - UL), den = SR - SL + eps,
// SL = min(sL, 0), SR = max(sR, 0).
template <int AX>
__device__ __forceinline__ void hll_vjp(const double PL[5], const double PR[5], const FaceParams& fp,
                                        const double dF[5], double dPL[5], double dPR[5]) {
  constexpr int N = AX + 1;
  const double gamma = fp.gamma;
  const double igm1 = 1.0 / fp.gm1;
  FaceSide L, R;
  face_side(PL, gamma, igm1, L);
  face_side(PR, gamma, igm1, R);
  const double uL = PL[N], uR = PR[N];
  WaveSpeeds e;
  wave_speeds_fwd(fp.signal_speed, uL, uR, PL[0], PR[0], PL[4], PR[4], L.c, R.c, gamma, e);
  const double SL = fmin(e.SL, 0.0), SR = fmax(e.SR, 0.0);
  double FL[5], FR[5];
  physical_flux<AX>(PL, L.U, FL);
  physical_flux<AX>(PR, R.U, FR);
  const double iden = 1.0 / ((SR - SL) + fp.eps);
  double dSL = 0.0, dSR = 0.0, dden = 0.0;
  double dFL[5], dFR[5], dUL[5], dUR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double dU = R.U[v] - L.U[v];
    const double Fv = ((SR * FL[v] - SL * FR[v]) + (SL * SR) * dU) * iden;
    const double dN = dF[v] * iden;
    dden -= dF[v] * Fv * iden;
    dSR += dN * (FL[v] + SL * dU);
    dSL += dN * (SR * dU - FR[v]);
    dFL[v] = dN * SR;
    dFR[v] = -dN * SL;
    dUR[v] = dN * SL * SR;
    dUL[v] = -dUR[v];
  }
  dSR += dden;
  dSL -= dden;
  const double dsL = dSL * min_weight_a(e.SL, 0.0);
  const double dsR = dSR * max_weight_a(e.SR, 0.0);
  physical_flux_vjp<AX>(PL, L.U, dFL, dPL, dUL);
  physical_flux_vjp<AX>(PR, R.U, dFR, dPR, dUR);
  double duL = 0.0, duR = 0.0, drL = 0.0, drR = 0.0, dcL = 0.0, dcR = 0.0, dpL = 0.0, dpR = 0.0;
  wave_speeds_vjp(e, uL, uR, PL[0], PR[0], PL[4], PR[4], L.c, R.c, dsL, dsR, duL, duR, drL, drR, dcL, dcR, dpL,
                  dpR);
  sound_speed_vjp(L, gamma, dcL, dPL);
  sound_speed_vjp(R, gamma, dcR, dPR);
  dPL[0] += drL;
  dPR[0] += drR;
  dPL[N] += duL;
  dPR[N] += duR;
  dPL[4] += dpL;
  dPR[4] += dpR;
  cons_from_prims_vjp(PL, dUL, L.ir, igm1, dPL);
  cons_from_prims_vjp(PR, dUR, R.ir, igm1, dPR);
}

// Reverse of rusanov<AX> (Rusanov.py:25-47).
template <int AX>
__device__ __forceinline__ void rusanov_vjp(const double PL[5], const double PR[5], const FaceParams& fp,
                                            const double dF[5], double dPL[5], double dPR[5]) {
  constexpr int N = AX + 1;
  const double gamma = fp.gamma;
  const double igm1 = 1.0 / fp.gm1;
  FaceSide L, R;
  face_side(PL, gamma, igm1, L);
  face_side(PR, gamma, igm1, R);
  const double aL = fabs(PL[N]) + L.c, aR = fabs(PR[N]) + R.c;
  const double alpha = fmax(aL, aR);
  double dUL[5] = {0, 0, 0, 0, 0}, dUR[5] = {0, 0, 0, 0, 0};
  // F = 0.5 (FL + FR) - 0.5 alpha (UR - UL)
  double g[5];
  double dalpha = 0.0;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    g[v] = 0.5 * dF[v];
    dalpha += -0.5 * dF[v] * (R.U[v] - L.U[v]);
    dUR[v] += -0.5 * alpha * dF[v];
    dUL[v] += 0.5 * alpha * dF[v];
  }
  physical_flux_vjp<AX>(PL, L.U, g, dPL, dUL);
  physical_flux_vjp<AX>(PR, R.U, g, dPR, dUR);
  const double w = max_weight_a(aL, aR);
  const double daL = dalpha * w, daR = dalpha * (1.0 - w);
  dPL[N] += daL * jabs_grad(PL[N]);
  dPR[N] += daR * jabs_grad(PR[N]);
  const double dyL = daL * 0.5 * L.ic, dyR = daR * 0.5 * R.ic;
  dPL[0] -= dyL * L.y * L.ir;
  dPR[0] -= dyR * R.y * R.ir;
  dPL[4] += dyL * L.ir * gamma;
  dPR[4] += dyR * R.ir * gamma;
  cons_from_prims_vjp(PL, dUL, L.ir, igm1, dPL);
  cons_from_prims_vjp(PR, dUR, R.ir, igm1, dPR);
}

// Lax-Friedrichs flux with the axis' speed alpha held fixed
// (LaxFriedrichs.py:33-45): F = 0.5 (F_L + F_R) - 0.5 alpha (U_R - U_L).  The
// face states' cotangents go to dPL, dPR; the cotangent of alpha,
// -0.5 sum_v dF_v (U_R - U_L)_v, is added to dalpha (the caller reduces it
// over the axis and hands it to the face states that attain the maximum).
template <int AX>
__device__ __forceinline__ void lf_vjp(const double PL[5], const double PR[5], const FaceParams& fp, double alpha,
                                       const double dF[5], double dPL[5], double dPR[5], double& dalpha) {
  const double igm1 = 1.0 / fp.gm1;
  double UL[5], UR[5];
  cons_from_prims(PL, UL, fp.gm1);
  cons_from_prims(PR, UR, fp.gm1);
  double dUL[5], dUR[5], g[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    g[v] = 0.5 * dF[v];
    dalpha += -0.5 * dF[v] * (UR[v] - UL[v]);
    dUR[v] = -0.5 * alpha * dF[v];
    dUL[v] = 0.5 * alpha * dF[v];
  }
  physical_flux_vjp<AX>(PL, UL, g, dPL, dUL);
  physical_flux_vjp<AX>(PR, UR, g, dPR, dUR);
  cons_from_prims_vjp(PL, dUL, 1.0 / PL[0], igm1, dPL);
  cons_from_prims_vjp(PR, dUR, 1.0 / PR[0], igm1, dPR);
}

// Pullback of a cotangent ds on the Lax-Friedrichs speed s = |u_n| + c of a
// face state P (ideal gas, c = sqrt(gamma p / rho)) onto P: jnp.abs has
// derivative +-1 (+1 at 0, jabs_grad), dc/dp = c / (2 p), dc/drho = -c / (2 rho).
template <int AX>
__device__ __forceinline__ void lf_speed_vjp(const double P[5], const FaceParams& fp, double ds, double dP[5]) {
  const double c = sqrt(fp.gamma * P[4] / P[0]);
  dP[AX + 1] += ds * jabs_grad(P[AX + 1]);
  const double h = 0.5 * ds * c;
  dP[4] += h / P[4];
  dP[0] -= h / P[0];
}

// Reverse of frozen_state (eigendecomposition.py:120-281) for the single-phase
// ideal gas: cotangents of (rho_a, c, cc) pulled back onto the primitives of
// the two cells L, R adjacent to the face (accumulated into dL, dR).
__device__ __forceinline__ void frozen_state_vjp(const double L[5], const double R[5], const FaceParams& fp,
                                                 double drho_a, double dc, double dcc, double dL[5],
                                                 double dR[5]) {
  if (fp.frozen_state == GBF_FROZEN_ARITHMETIC) {
    // rho = (L0+R0)/2, p = (L4+R4)/2, c = sqrt(gamma p / rho), cc = c c
    const double rho = 0.5 * (L[0] + R[0]);
    const double p = 0.5 * (L[4] + R[4]);
    const double irho = 1.0 / rho;
    const double y = fp.gamma * p * irho;
    const double c = sqrt(y);
    const double dct = dc + dcc * 2.0 * c;
    const double dy = dct * 0.5 / c;
    const double drho = drho_a - dy * y * irho;
    const double dp = dy * fp.gamma * irho;
    dL[0] += 0.5 * drho;
    dR[0] += 0.5 * drho;
    dL[4] += 0.5 * dp;
    dR[4] += 0.5 * dp;
    return;
  }
  const double gm1 = fp.gm1;
  const double rho_a = sqrt(L[0] * R[0]);
  const double sL = sqrt(L[0]), sR = sqrt(R[0]);
  const double rho_div = 1.0 / (sL + sR);
  const double iL0 = 1.0 / L[0], iR0 = 1.0 / R[0];
  const double qL = L[4] * iL0, qR = R[4] * iR0;
  const double A = sL * qL + sR * qR;  // psi_a and the first term of p_over_rho
  const double gr_a = (sL * gm1 + sR * gm1) * rho_div;
  const double d1 = R[1] - L[1], d2 = R[2] - L[2], d3 = R[3] - L[3];
  const double sqvd = d1 * d1 + d2 * d2 + d3 * d3;
  const double p_over_rho = A * rho_div + 0.5 * rho_a * rho_div * rho_div * sqvd;
  const double cc = A * rho_div + gr_a * p_over_rho;
  const double c = sqrt(cc);
  // c = sqrt(cc)
  const double dcct = dcc + dc * 0.5 / c;
  // cc = psi_a + gr_a p_over_rho
  const double dpor = dcct * gr_a;
  const double dgr = dcct * p_over_rho;
  double dA = dcct * rho_div + dpor * rho_div;
  double drho_div = dcct * A + dpor * A + dpor * rho_a * rho_div * sqvd;
  double drho = drho_a + dpor * 0.5 * rho_div * rho_div * sqvd;
  const double dsq = dpor * 0.5 * rho_a * rho_div * rho_div;
  // gr_a = (sL gm1 + sR gm1) rho_div
  double dsL = dgr * gm1 * rho_div, dsR = dgr * gm1 * rho_div;
  drho_div += dgr * (sL * gm1 + sR * gm1);
  // A = sL L4/L0 + sR R4/R0
  dsL += dA * qL;
  dsR += dA * qR;
  const double dqL = dA * sL, dqR = dA * sR;
  dL[4] += dqL * iL0;
  dR[4] += dqR * iR0;
  dL[0] -= dqL * qL * iL0;
  dR[0] -= dqR * qR * iR0;
  // sqvd
  dR[1] += 2.0 * d1 * dsq;
  dL[1] -= 2.0 * d1 * dsq;
  dR[2] += 2.0 * d2 * dsq;
  dL[2] -= 2.0 * d2 * dsq;
  dR[3] += 2.0 * d3 * dsq;
  dL[3] -= 2.0 * d3 * dsq;
  // rho_div = 1/(sL + sR)
  const double dsum = -drho_div * rho_div * rho_div;
  dsL += dsum;
  dsR += dsum;
  dL[0] += dsL * 0.5 / sL;
  dR[0] += dsR * 0.5 / sR;
  // rho_a = sqrt(L0 R0)
  const double dprod = drho * 0.5 / rho_a;
  dL[0] += dprod * R[0];
  dR[0] += dprod * L[0];
}

// Reverse of total_enthalpy(p, rho, u0, u1, u2): H = (p / gm1 + 0.5 rho |u|^2 + p) / rho.
// P holds (rho, u0, u1, u2, p); dP += dH dH/dP.
__device__ __forceinline__ void total_enthalpy_vjp(const double P[5], double H, double gm1, double dH,
                                                   double dP[5]) {
  const double ir = 1.0 / P[0];
  const double dE = dH * ir;
  dP[4] += dH * ir + dE / gm1;
  dP[0] += -dH * H * ir + dE * 0.5 * (P[1] * P[1] + P[2] * P[2] + P[3] * P[3]);
#pragma unroll
  for (int j = 1; j <= 3; ++j) dP[j] += dE * P[0] * P[j];
}

// Reverse of frozen_state_full (eigendecomposition.py:120-281, both frozen
// states): the cotangents dz of every field of the full frozen state pulled
// back onto the primitives of the two cells L, R beside the face (added to
// dL, dR).  gm1 enters the ROE average's gamma - 1 as a constant.
__device__ __forceinline__ void frozen_state_full_vjp(const double L[5], const double R[5], const FaceParams& fp,
                                                      const FrozenFull& z, const FrozenFull& dz, double dL[5],
                                                      double dR[5]) {
  double dpa[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) dpa[v] = dz.pa[v];
  // vsq = |pa[1..3]|^2
#pragma unroll
  for (int j = 1; j <= 3; ++j) dpa[j] += 2.0 * z.pa[j] * dz.vsq;
  const double gm1 = fp.gm1;
  if (fp.frozen_state == GBF_FROZEN_ARITHMETIC) {
    // c = sqrt(gamma pa4 / pa0), cc = c c, H = total_enthalpy(pa), gr = gm1
    const double dct = dz.c + 2.0 * z.c * dz.cc;
    const double y = z.c * z.c;
    const double dy = dct * 0.5 / z.c;
    dpa[4] += dy * y / z.pa[4];
    dpa[0] -= dy * y / z.pa[0];
    total_enthalpy_vjp(z.pa, z.H, gm1, dz.H, dpa);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      dL[v] += 0.5 * dpa[v];
      dR[v] += 0.5 * dpa[v];
    }
    return;
  }
  const double sL = sqrt(L[0]), sR = sqrt(R[0]);
  const double S = sL + sR;
  const double rho_div = 1.0 / S;
  const double iL0 = 1.0 / L[0], iR0 = 1.0 / R[0];
  const double qL = L[4] * iL0, qR = R[4] * iR0;
  const double A = sL * qL + sR * qR;
  const double HL = total_enthalpy(L[4], L[0], L[1], L[2], L[3], gm1);
  const double HR = total_enthalpy(R[4], R[0], R[1], R[2], R[3], gm1);
  const double d1 = R[1] - L[1], d2 = R[2] - L[2], d3 = R[3] - L[3];
  const double sqvd = d1 * d1 + d2 * d2 + d3 * d3;
  const double p_over_rho = A * rho_div + 0.5 * z.pa[0] * rho_div * rho_div * sqvd;
  // c = sqrt(cc); cc = psi_a + gr p_over_rho, psi_a = A rho_div
  const double dcct = dz.cc + dz.c * 0.5 / z.c;
  const double dgr = dz.gr + dcct * p_over_rho;
  const double dpor = dcct * z.gr;
  double dA = dcct * rho_div + dpor * rho_div;
  double drho_div = dcct * A + dpor * (A + z.pa[0] * rho_div * sqvd);
  dpa[0] += dpor * 0.5 * rho_div * rho_div * sqvd;
  const double dsq = dpor * 0.5 * z.pa[0] * rho_div * rho_div;
  // gr = (sL gm1 + sR gm1) rho_div
  double dsL = dgr * gm1 * rho_div, dsR = dgr * gm1 * rho_div;
  drho_div += dgr * (sL * gm1 + sR * gm1);
  // H = (sL HL + sR HR) rho_div
  dsL += dz.H * HL * rho_div;
  dsR += dz.H * HR * rho_div;
  drho_div += dz.H * (sL * HL + sR * HR);
  total_enthalpy_vjp(L, HL, gm1, dz.H * sL * rho_div, dL);
  total_enthalpy_vjp(R, HR, gm1, dz.H * sR * rho_div, dR);
  // pa[v] = (sL L[v] + sR R[v]) / S, v = 1..4
  double dS = 0.0;
#pragma unroll
  for (int v = 1; v < 5; ++v) {
    const double dn = dpa[v] / S;
    dL[v] += dn * sL;
    dR[v] += dn * sR;
    dsL += dn * L[v];
    dsR += dn * R[v];
    dS -= dn * z.pa[v];
  }
  // A = sL L4/L0 + sR R4/R0
  dsL += dA * qL;
  dsR += dA * qR;
  dL[4] += dA * sL * iL0;
  dR[4] += dA * sR * iR0;
  dL[0] -= dA * sL * qL * iL0;
  dR[0] -= dA * sR * qR * iR0;
  // sqvd
  dR[1] += 2.0 * d1 * dsq;
  dL[1] -= 2.0 * d1 * dsq;
  dR[2] += 2.0 * d2 * dsq;
  dL[2] -= 2.0 * d2 * dsq;
  dR[3] += 2.0 * d3 * dsq;
  dL[3] -= 2.0 * d3 * dsq;
  // rho_div = 1 / S
  dS -= drho_div * rho_div * rho_div;
  dsL += dS;
  dsR += dS;
  dL[0] += dsL * 0.5 / sL;
  dR[0] += dsR * 0.5 / sR;
  // pa0 = sqrt(L0 R0)
  const double dprod = dpa[0] * 0.5 / z.pa[0];
  dL[0] += dprod * R[0];
  dR[0] += dprod * L[0];
}

// Reverse of left_eigvecs_cons: dz += (d Lm / d z)^T G.
template <int AX>
__device__ __forceinline__ void left_eigvecs_cons_vjp(const FrozenFull& z, const double G[5][5], FrozenFull& dz) {
  constexpr int n = AX + 1;
  using I = CharIds<AX>;
  constexpr int m0 = I::m0, m1 = I::m1;
  const double one_cc = 1.0 / z.cc;
  const double one_rho = 1.0 / z.pa[0];
  const double h = 0.5 * one_cc;
  const double pn = z.pa[n], c = z.c, gr = z.gr;
  const double t0 = gr * z.vsq - gr * z.H;
  // rows 0 and 4: h * (...)
  double dh = G[0][0] * (t0 + (pn + c) * c) + G[0][n] * (-pn * gr - c) + G[0][m0] * (-z.pa[m0] * gr) +
              G[0][m1] * (-z.pa[m1] * gr) + G[0][4] * gr + G[4][0] * (t0 - (pn - c) * c) +
              G[4][n] * (-pn * gr + c) + G[4][m0] * (-z.pa[m0] * gr) + G[4][m1] * (-z.pa[m1] * gr) +
              G[4][4] * gr;
  const double a0 = h * G[0][0], a1 = h * G[0][n], a2 = h * G[0][m0], a3 = h * G[0][m1], a4 = h * G[0][4];
  const double b0 = h * G[4][0], b1 = h * G[4][n], b2 = h * G[4][m0], b3 = h * G[4][m1], b4 = h * G[4][4];
  dz.gr += (a0 + b0) * (z.vsq - z.H) - (a1 + b1) * pn - (a2 + b2) * z.pa[m0] - (a3 + b3) * z.pa[m1] + a4 + b4;
  dz.vsq += (a0 + b0) * gr;
  dz.H -= (a0 + b0) * gr;
  dz.pa[n] += a0 * c - b0 * c - (a1 + b1) * gr;
  dz.c += a0 * (pn + 2.0 * c) + b0 * (2.0 * c - pn) - a1 + b1;
  dz.pa[m0] -= (a2 + b2) * gr;
  dz.pa[m1] -= (a3 + b3) * gr;
  // row n: one_cc * (...)
  double done_cc = G[n][0] * (z.H - z.vsq) + G[n][1] * z.pa[1] + G[n][2] * z.pa[2] + G[n][3] * z.pa[3] - G[n][4];
  dz.H += G[n][0] * one_cc;
  dz.vsq -= G[n][0] * one_cc;
#pragma unroll
  for (int j = 1; j <= 3; ++j) dz.pa[j] += G[n][j] * one_cc;
  // rows m0, m1: one_rho * (...)
  const double done_rho = G[m0][0] * z.pa[m0] - G[m0][m0] - G[m1][0] * z.pa[m1] + G[m1][m1];
  dz.pa[m0] += G[m0][0] * one_rho;
  dz.pa[m1] -= G[m1][0] * one_rho;
  done_cc += 0.5 * dh;
  dz.cc -= done_cc * one_cc * one_cc;
  dz.pa[0] -= done_rho * one_rho * one_rho;
}

// Reverse of right_eigvecs_cons: dz += (d Rm / d z)^T G.
template <int AX>
__device__ __forceinline__ void right_eigvecs_cons_vjp(const FrozenFull& z, const double G[5][5], FrozenFull& dz) {
  constexpr int n = AX + 1;
  using I = CharIds<AX>;
  constexpr int m0 = I::m0, m1 = I::m1;
  const double pn = z.pa[n], c = z.c;
  dz.pa[n] += G[n][0] - G[4][0] * c + G[n][4] + G[4][4] * c;
  dz.c += -G[n][0] - G[4][0] * pn + G[n][4] + G[4][4] * pn;
  dz.pa[m0] += G[m0][0] + G[m0][4] - G[4][m0] * z.pa[0];
  dz.pa[m1] += G[m1][0] + G[m1][4] + G[4][m1] * z.pa[0];
  dz.H += G[4][0] + G[4][n] * z.gr + G[4][4];
  dz.gr += G[0][n] + G[1][n] * z.pa[1] + G[2][n] * z.pa[2] + G[3][n] * z.pa[3] + G[4][n] * z.H;
#pragma unroll
  for (int j = 1; j <= 3; ++j) dz.pa[j] += G[j][n] * z.gr;
  dz.cc -= G[4][n];
  dz.pa[0] += -G[m0][m0] - G[4][m0] * z.pa[m0] + G[m1][m1] + G[4][m1] * z.pa[m1];
}

template <int AX, int RIEMANN>
__device__ __forceinline__ void riemann_flux_vjp(const double PL[5], const double PR[5], const FaceParams& fp,
                                                 const double dF[5], double dPL[5], double dPR[5]) {
  if (RIEMANN == GBF_RIEMANN_HLLC)
    hllc_vjp<AX>(PL, PR, fp, dF, dPL, dPR);
  else if (RIEMANN == GBF_RIEMANN_HLL)
    hll_vjp<AX>(PL, PR, fp, dF, dPL, dPR);
  else
    rusanov_vjp<AX>(PL, PR, fp, dF, dPL, dPR);
}

}  // namespace gbf
