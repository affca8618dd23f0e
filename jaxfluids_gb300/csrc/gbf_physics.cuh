// Device-side physics of the single-phase finite-volume right-hand side:
// ideal-gas EOS, cell-face reconstruction, signal speeds and Riemann fluxes.
//
// Every function restates the corresponding JAX-Fluids routine (paths relative
// to src/jaxfluids) in FP64.  Per-face state lives in small register arrays
// indexed only with compile-time constants (the sweep axis is a template
// parameter), so nothing spills to local memory through dynamic indexing.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbfluids.h"

namespace gbf {

struct FaceParams {
  double gamma;        // specific heat ratio
  double gm1;          // gamma - 1.0 (computed once on the host, like ideal_gas.py)
  double stencil_eps;  // WENO / MUSCL epsilon (precision.py:53, 1e-30)
  double eps;          // precision epsilon (float64 machine epsilon; HLL denominator)
  int signal_speed;    // GBF_SIGNAL_*
  int frozen_state;    // GBF_FROZEN_*
};

__device__ __forceinline__ double sq(double x) { return x * x; }

// a / b, the IEEE quotient, with a zero dividend answered without dividing:
// (+-0) / b for a non-zero, non-NaN b (infinities included) is the zero
// carrying the XOR of the operands' signs, exactly what the division returns.  The division takes a
// general path for a zero dividend that costs 19 FP64 instructions on GB300
// against 8 on its common path (measured with ncu), and flat stencils (WENO's
// |beta0 - beta2| = 0), resting fluid and symmetric states give zero
// dividends on many faces.
// The operand tests are integer operations on the halves of the operands (a
// floating-point compare would take an FP64 issue slot).
__device__ __forceinline__ double div0(double a, double b) {
  const unsigned ahi = (unsigned)__double2hiint(a), alo = (unsigned)__double2loint(a);
  const unsigned bhi = (unsigned)__double2hiint(b), blo = (unsigned)__double2loint(b);
  const bool a_zero = ((ahi & 0x7fffffffu) | alo) == 0u;
  const bool b_nonzero = ((bhi & 0x7fffffffu) | blo) != 0u;
  const bool b_nan = (bhi & 0x7ff00000u) == 0x7ff00000u && (((bhi & 0x000fffffu) | blo) != 0u);
  if (a_zero && b_nonzero && !b_nan) return __hiloint2double((int)((ahi ^ bhi) & 0x80000000u), 0);
  return a / b;
}

// ---------------------------------------------------------------------------
// Ideal gas and equation layout
// ---------------------------------------------------------------------------

// materials/single_materials/ideal_gas.py:69-71
__device__ __forceinline__ double speed_of_sound(double p, double rho, const FaceParams& fp) {
  return sqrt(fp.gamma * p / rho);
}

// equation_manager.py:93-101 (E = rho (|u|^2/2 + p / (rho (gamma-1))))
__device__ __forceinline__ void cons_from_prims(const double P[5], double U[5], double gm1) {
  const double rho = P[0];
  const double e = P[4] / (rho * gm1);
  U[0] = rho;
  U[1] = rho * P[1];
  U[2] = rho * P[2];
  U[3] = rho * P[3];
  U[4] = rho * fma(0.5, P[1] * P[1] + P[2] * P[2] + P[3] * P[3], e);  // 0.5 s exact
}

// equation_manager.py:164-171 (p = (gamma-1) e rho)
__device__ __forceinline__ void prims_from_cons(const double U[5], double P[5], double gm1) {
  const double rho = U[0];
  const double one_rho = 1.0 / rho;
  const double u = U[1] * one_rho;
  const double v = U[2] * one_rho;
  const double w = U[3] * one_rho;
  const double e = fma(-0.5, u * u + v * v + w * w, U[4] * one_rho);  // 0.5 s exact
  P[0] = rho;
  P[1] = u;
  P[2] = v;
  P[3] = w;
  P[4] = gm1 * e * rho;
}

// equation_manager.py:237-252
template <int AX>
__device__ __forceinline__ void physical_flux(const double P[5], const double U[5], double F[5]) {
  const double m = U[AX + 1];
  F[0] = m;
  F[1] = m * P[1];
  F[2] = m * P[2];
  F[3] = m * P[3];
  F[4] = P[AX + 1] * (U[4] + P[4]);
  F[AX + 1] += P[4];
}

// ---------------------------------------------------------------------------
// Reconstruction
// ---------------------------------------------------------------------------

// WENO5-Z, Borges et al. 2008 (stencils/reconstruction/shock_capturing/weno/weno5_z.py:24-58,
// weno5_base.py:24-51).  Arguments are (u_imm, u_im, u_i, u_ip, u_ipp) in the
// reference's slice order; the right state passes the mirrored cells.
//
// Products by powers of two (2 u, 4 u, 1/4 t^2) are exact, so fusing them with
// the following addition (explicit fma) rounds exactly like the reference's
// separate multiply and add; the build forbids every other contraction.
// Smoothness indicators and candidate polynomials of the five-point stencils
// (weno5_base.py:34-51).
__device__ __forceinline__ void weno5_smoothness(double u0, double u1, double u2, double u3, double u4,
                                                 double& b0, double& b1, double& b2) {
  b0 = fma(0.25, sq(fma(-4.0, u1, u0) + 3.0 * u2), (13.0 / 12.0) * sq(fma(-2.0, u1, u0) + u2));
  b1 = fma(0.25, sq(u1 - u3), (13.0 / 12.0) * sq(fma(-2.0, u2, u1) + u3));
  b2 = fma(0.25, sq(fma(-4.0, u3, 3.0 * u2) + u4), (13.0 / 12.0) * sq(fma(-2.0, u3, u2) + u4));
}

__device__ __forceinline__ double weno5_combine(double a0, double a1, double a2, double u0, double u1,
                                                double u2, double u3, double u4) {
  const double one_a = 1.0 / (a0 + a1 + a2);
  const double p0 = (1.0 / 3.0) * u0 + (-7.0 / 6.0) * u1 + (11.0 / 6.0) * u2;
  const double p1 = (-1.0 / 6.0) * u1 + (5.0 / 6.0) * u2 + (1.0 / 3.0) * u3;
  const double p2 = (1.0 / 3.0) * u2 + (5.0 / 6.0) * u3 + (-1.0 / 6.0) * u4;
  return (a0 * one_a) * p0 + (a1 * one_a) * p1 + (a2 * one_a) * p2;
}

// The smoothness indicators of weno5_smoothness from window terms computed
// once per cell and shared by the three faces whose stencils hold the window:
// d0, d1, d2 = (13/12) (fma(-2, u_c, u_prev) + u_next)^2 of the windows centred
// on u1, u2, u3, and e1 = (u1 - u3)^2, each formed by the same operations on
// the same operands in the same order as weno5_smoothness forms it, so the
// indicators are bitwise equal.
__device__ __forceinline__ void weno5_smoothness_shared(double u0, double u1, double u2, double u3, double u4,
                                                        double d0, double d1, double d2, double e1, double& b0,
                                                        double& b1, double& b2) {
  b0 = fma(0.25, sq(fma(-4.0, u1, u0) + 3.0 * u2), d0);
  b1 = fma(0.25, e1, d1);
  b2 = fma(0.25, sq(fma(-4.0, u3, 3.0 * u2) + u4), d2);
}

__device__ __forceinline__ double weno5z_from_beta(double b0, double b1, double b2, double u0, double u1,
                                                   double u2, double u3, double u4, double eps) {
  const double tau5 = fabs(b0 - b2);
  const double a0 = 0.1 * (1.0 + div0(tau5, b0 + eps));
  const double a1 = 0.6 * (1.0 + div0(tau5, b1 + eps));
  const double a2 = 0.3 * (1.0 + div0(tau5, b2 + eps));
  return weno5_combine(a0, a1, a2, u0, u1, u2, u3, u4);
}

__device__ __forceinline__ double weno5z(double u0, double u1, double u2, double u3, double u4,
                                         double eps) {
  double b0, b1, b2;
  weno5_smoothness(u0, u1, u2, u3, u4, b0, b1, b2);
  return weno5z_from_beta(b0, b1, b2, u0, u1, u2, u3, u4, eps);
}

// WENO5-JS (shock_capturing/weno/weno5_js.py:33-70): alpha_k = d_k / (beta_k^2 + eps).
__device__ __forceinline__ double weno5js_from_beta(double b0, double b1, double b2, double u0, double u1,
                                                    double u2, double u3, double u4, double eps) {
  const double a0 = 0.1 * (1.0 / (b0 * b0 + eps));
  const double a1 = 0.6 * (1.0 / (b1 * b1 + eps));
  const double a2 = 0.3 * (1.0 / (b2 * b2 + eps));
  return weno5_combine(a0, a1, a2, u0, u1, u2, u3, u4);
}

__device__ __forceinline__ double weno5js(double u0, double u1, double u2, double u3, double u4,
                                          double eps) {
  double b0, b1, b2;
  weno5_smoothness(u0, u1, u2, u3, u4, b0, b1, b2);
  return weno5js_from_beta(b0, b1, b2, u0, u1, u2, u3, u4, eps);
}

// TENO5 (teno/teno5.py, Fu et al. 2016) weights: gamma_k = (1 + tau5 / (beta_k
// + eps))^6 (jnp.power with an integer exponent: x^2 (x^2)^2, the square-and-
// multiply of lax.integer_pow), sharp cutoff (gamma_k / sum gamma < 1e-5 drops
// stencil k), weights d_k = (0.05, 0.55, 0.40) of the kept stencils divided by
// their sum + eps.  Unfused products: the adjoint units recompute the cutoff
// with the forward's rounding.
__device__ __forceinline__ void teno5_weights(double b0, double b1, double b2, double eps, double& o0,
                                              double& o1, double& o2) {
  const double tau5 = fabs(__dsub_rn(b0, b2));
  auto gamma = [&](double b) {
    const double x = __dadd_rn(1.0, div0(tau5, __dadd_rn(b, eps)));
    const double x2 = __dmul_rn(x, x);
    return __dmul_rn(x2, __dmul_rn(x2, x2));
  };
  const double g0 = gamma(b0), g1 = gamma(b1), g2 = gamma(b2);
  const double one_gamma_sum = __ddiv_rn(1.0, __dadd_rn(__dadd_rn(g0, g1), g2));
  const double w0 = (__dmul_rn(g0, one_gamma_sum) < 1e-5) ? 0.0 : 0.05;
  const double w1 = (__dmul_rn(g1, one_gamma_sum) < 1e-5) ? 0.0 : 0.55;
  const double w2 = (__dmul_rn(g2, one_gamma_sum) < 1e-5) ? 0.0 : 0.40;
  const double one_dk = __ddiv_rn(1.0, __dadd_rn(__dadd_rn(__dadd_rn(w0, w1), w2), eps));
  o0 = __dmul_rn(w0, one_dk);
  o1 = __dmul_rn(w1, one_dk);
  o2 = __dmul_rn(w2, one_dk);
}

__device__ __forceinline__ double teno5_from_beta(double b0, double b1, double b2, double u0, double u1,
                                                  double u2, double u3, double u4, double eps) {
  double o0, o1, o2;
  teno5_weights(b0, b1, b2, eps, o0, o1, o2);
  const double p0 = (1.0 / 3.0) * u0 + (-7.0 / 6.0) * u1 + (11.0 / 6.0) * u2;
  const double p1 = (-1.0 / 6.0) * u1 + (5.0 / 6.0) * u2 + (1.0 / 3.0) * u3;
  const double p2 = (1.0 / 3.0) * u2 + (5.0 / 6.0) * u3 + (-1.0 / 6.0) * u4;
  return o0 * p0 + o1 * p1 + o2 * p2;
}

__device__ __forceinline__ double teno5(double u0, double u1, double u2, double u3, double u4, double eps) {
  double b0, b1, b2, o0, o1, o2;
  weno5_smoothness(u0, u1, u2, u3, u4, b0, b1, b2);
  teno5_weights(b0, b1, b2, eps, o0, o1, o2);
  const double p0 = (1.0 / 3.0) * u0 + (-7.0 / 6.0) * u1 + (11.0 / 6.0) * u2;
  const double p1 = (-1.0 / 6.0) * u1 + (5.0 / 6.0) * u2 + (1.0 / 3.0) * u3;
  const double p2 = (1.0 / 3.0) * u2 + (5.0 / 6.0) * u3 + (-1.0 / 6.0) * u4;
  return o0 * p0 + o1 * p1 + o2 * p2;
}

// WENO3-JS (weno/weno3_js.py:22-45) and WENO3-Z (weno/weno3_z.py:24-46) on
// (u_im, u_i, u_ip), weno3_base.py:20-44: d = (1/3, 2/3),
// p0 = -u_im/2 + 3 u_i / 2, p1 = (u_i + u_ip) / 2.
template <bool Z>
__device__ __forceinline__ double weno3(double u0, double u1, double u2, double eps) {
  const double b0 = sq(u1 - u0);
  const double b1 = sq(u2 - u1);
  double a0, a1;
  if (Z) {
    const double tau3 = fabs(b0 - b1);
    a0 = (1.0 / 3.0) * (1.0 + div0(tau3, b0 + eps));
    a1 = (2.0 / 3.0) * (1.0 + div0(tau3, b1 + eps));
  } else {
    a0 = (1.0 / 3.0) * (1.0 / (b0 * b0 + eps));
    a1 = (2.0 / 3.0) * (1.0 / (b1 * b1 + eps));
  }
  const double one_a = 1.0 / (a0 + a1);
  const double p0 = fma(-0.5, u0, 1.5 * u1);   // -0.5 u exact
  const double p1 = fma(0.5, u1, 0.5 * u2);    // both products exact
  return (a0 * one_a) * p0 + (a1 * one_a) * p1;
}

// MUSCL3 with the MINMOD limiter (shock_capturing/muscl/muscl3.py:53-75, limiter.py:9-10).
// (b0, b1, b2) are the reference's s_[0], s_[1], s_[2] for side j.
template <int J>
__device__ __forceinline__ double muscl_minmod(double b0, double b1, double b2, double eps) {
  const double dc = (J == 0) ? b2 - b1 : b1 - b2;
  const double du = (J == 0) ? b1 - b0 : b0 - b1;
  const double r = (du >= eps) ? div0(dc, du + 1e-10) : (dc + eps) / (du + eps);
  const double lim = fmax(0.0, fmin(1.0, r));
  return (J == 0) ? b1 + 0.5 * lim * du : b1 - 0.5 * lim * du;
}

// MINMOD-AD (shock_capturing/muscl/minmod_ad.py:45-66)
template <int J>
__device__ __forceinline__ double minmod_ad(double b0, double b1, double b2, double eps) {
  const double dc = (J == 0) ? b2 - b1 : b1 - b2;
  const double du = (J == 0) ? b1 - b0 : b0 - b1;
  const double r = (du >= eps) ? div0(dc, du + 1e-100) : (dc + eps) / (du + eps);
  return (r < 0.0) ? b1 : ((r < 1.0) ? 0.5 * (b1 + b2) : fma(-0.5, b0, 1.5 * b1));
}

// Internal reconstruction id (outside the GBF_RECON_* range): WENO5-Z on
// Roe-characteristic variables (reconstruction_variable CHAR-PRIMITIVE); same
// six-cell window as WENO5-Z.
constexpr int RECON_WENO5Z_CHAR = 100;
// WENO5-Z on the conservatives (reconstruction_variable CONSERVATIVE) and on
// their characteristic variables (CHAR-CONSERVATIVE); the pencil carries the
// conservatives behind the primitives.
constexpr int RECON_WENO5Z_CONS = 101;
constexpr int RECON_WENO5Z_CHARCONS = 102;

// Halo radius of a GBF_RECON_* stencil (host and device).
__host__ __device__ constexpr int recon_radius(int recon) {
  return (recon == GBF_RECON_WENO5Z || recon == GBF_RECON_WENO5JS || recon == GBF_RECON_TENO5 ||
          recon == RECON_WENO5Z_CHAR)
             ? 3
             : 2;
}

// Halo radius (cells each side of a face) of each reconstruction stencil.
template <int RECON>
struct ReconTraits;
template <>
struct ReconTraits<RECON_WENO5Z_CHAR> {
  static constexpr int R = 3;
};
template <>
struct ReconTraits<RECON_WENO5Z_CONS> {
  static constexpr int R = 3;
};
template <>
struct ReconTraits<RECON_WENO5Z_CHARCONS> {
  static constexpr int R = 3;
};
template <>
struct ReconTraits<GBF_RECON_WENO5Z> {
  static constexpr int R = 3;
};
template <>
struct ReconTraits<GBF_RECON_MINMOD> {
  static constexpr int R = 2;
};
template <>
struct ReconTraits<GBF_RECON_MINMOD_AD> {
  static constexpr int R = 2;
};
template <>
struct ReconTraits<GBF_RECON_WENO5JS> {
  static constexpr int R = 3;
};
template <>
struct ReconTraits<GBF_RECON_TENO5> {
  static constexpr int R = 3;
};
template <>
struct ReconTraits<GBF_RECON_WENO3JS> {
  static constexpr int R = 2;
};
template <>
struct ReconTraits<GBF_RECON_WENO3Z> {
  static constexpr int R = 2;
};

// Left (J=0) and right (J=1) face values from the 2R cells around the face;
// w[k] is the cell at offset k - R from the face (w[R-1] left neighbour,
// w[R] right neighbour).
template <int RECON>
__device__ __forceinline__ void reconstruct_pair(const double* w, double eps, double& L, double& R);

template <>
__device__ __forceinline__ void reconstruct_pair<GBF_RECON_WENO5Z>(const double* w, double eps,
                                                                    double& L, double& R) {
  // j=0 offsets (-3..1) -> w[0..4]; j=1 offsets (2..-2) -> w[5..1]
  L = weno5z(w[0], w[1], w[2], w[3], w[4], eps);
  R = weno5z(w[5], w[4], w[3], w[2], w[1], eps);
}

// The WENO5 family (WENO5-Z, WENO5-JS, TENO5) on primitive variables with the
// window terms of weno5_smoothness_shared read from per-cell arrays: for the
// six cells w[0..5] around the face, dl[k] / dr[k] / e[k] are the terms of the
// window centred on w[k] (k = 1..4) in the left-state / right-state operand
// order.  Equal bitwise to reconstruct_pair<RECON>.
template <int RECON>
__device__ __forceinline__ void reconstruct_pair_shared(const double* w, const double* dl, const double* dr,
                                                        const double* e, double eps, double& L, double& R) {
  double b0, b1, b2;
  // left: (w0 .. w4), windows centred on w1, w2, w3
  weno5_smoothness_shared(w[0], w[1], w[2], w[3], w[4], dl[1], dl[2], dl[3], e[2], b0, b1, b2);
  if (RECON == GBF_RECON_WENO5Z) L = weno5z_from_beta(b0, b1, b2, w[0], w[1], w[2], w[3], w[4], eps);
  if (RECON == GBF_RECON_WENO5JS) L = weno5js_from_beta(b0, b1, b2, w[0], w[1], w[2], w[3], w[4], eps);
  if (RECON == GBF_RECON_TENO5) L = teno5_from_beta(b0, b1, b2, w[0], w[1], w[2], w[3], w[4], eps);
  // right: (w5 .. w1), windows centred on w4, w3, w2
  weno5_smoothness_shared(w[5], w[4], w[3], w[2], w[1], dr[4], dr[3], dr[2], e[3], b0, b1, b2);
  if (RECON == GBF_RECON_WENO5Z) R = weno5z_from_beta(b0, b1, b2, w[5], w[4], w[3], w[2], w[1], eps);
  if (RECON == GBF_RECON_WENO5JS) R = weno5js_from_beta(b0, b1, b2, w[5], w[4], w[3], w[2], w[1], eps);
  if (RECON == GBF_RECON_TENO5) R = teno5_from_beta(b0, b1, b2, w[5], w[4], w[3], w[2], w[1], eps);
}

// The window terms of the cell u_c between u_prev and u_next (along the axis):
// dl = (13/12) (fma(-2, u_c, u_prev) + u_next)^2, dr = (13/12) (fma(-2, u_c,
// u_next) + u_prev)^2, e = (u_prev - u_next)^2 (weno5_smoothness_shared).
__device__ __forceinline__ void weno5_window_terms(double up, double uc, double un, double& dl, double& dr,
                                                   double& e) {
  dl = (13.0 / 12.0) * sq(fma(-2.0, uc, up) + un);
  dr = (13.0 / 12.0) * sq(fma(-2.0, uc, un) + up);
  e = sq(up - un);
}

template <>
__device__ __forceinline__ void reconstruct_pair<GBF_RECON_MINMOD>(const double* w, double eps,
                                                                    double& L, double& R) {
  // j=0 offsets (-2,-1,0) -> w[0],w[1],w[2]; j=1 offsets (1,0,-1) -> w[3],w[2],w[1]
  L = muscl_minmod<0>(w[0], w[1], w[2], eps);
  R = muscl_minmod<1>(w[3], w[2], w[1], eps);
}

template <>
__device__ __forceinline__ void reconstruct_pair<GBF_RECON_MINMOD_AD>(const double* w, double eps,
                                                                       double& L, double& R) {
  L = minmod_ad<0>(w[0], w[1], w[2], eps);
  R = minmod_ad<1>(w[3], w[2], w[1], eps);
}

template <>
__device__ __forceinline__ void reconstruct_pair<GBF_RECON_WENO5JS>(const double* w, double eps,
                                                                     double& L, double& R) {
  L = weno5js(w[0], w[1], w[2], w[3], w[4], eps);
  R = weno5js(w[5], w[4], w[3], w[2], w[1], eps);
}

template <>
__device__ __forceinline__ void reconstruct_pair<GBF_RECON_TENO5>(const double* w, double eps,
                                                                   double& L, double& R) {
  L = teno5(w[0], w[1], w[2], w[3], w[4], eps);
  R = teno5(w[5], w[4], w[3], w[2], w[1], eps);
}

template <>
__device__ __forceinline__ void reconstruct_pair<GBF_RECON_WENO3JS>(const double* w, double eps,
                                                                     double& L, double& R) {
  // j=0 offsets (-2,-1,0) -> w[0],w[1],w[2]; j=1 offsets (1,0,-1) -> w[3],w[2],w[1]
  L = weno3<false>(w[0], w[1], w[2], eps);
  R = weno3<false>(w[3], w[2], w[1], eps);
}

template <>
__device__ __forceinline__ void reconstruct_pair<GBF_RECON_WENO3Z>(const double* w, double eps,
                                                                    double& L, double& R) {
  L = weno3<true>(w[0], w[1], w[2], eps);
  R = weno3<true>(w[3], w[2], w[1], eps);
}

// ---------------------------------------------------------------------------
// Characteristic decomposition (solvers/riemann_solvers/eigendecomposition.py)
// ---------------------------------------------------------------------------

// Eigendecomposition.compute_frozen_state, single phase (:120-281): density,
// speed of sound and its square of the frozen state between cells L and R.
__device__ __forceinline__ void frozen_state(const double L[5], const double R[5],
                                             const FaceParams& fp, double& rho_a, double& c,
                                             double& cc) {
  if (fp.frozen_state == GBF_FROZEN_ARITHMETIC) {
    const double rho = 0.5 * (L[0] + R[0]);
    const double p = 0.5 * (L[4] + R[4]);
    rho_a = rho;
    c = sqrt(fp.gamma * p / rho);
    cc = c * c;
  } else {
    // ROE: cc = psi_ave + grueneisen_ave * p_over_rho_ave (:223-268)
    rho_a = sqrt(L[0] * R[0]);
    const double sL = sqrt(L[0]);
    const double sR = sqrt(R[0]);
    const double rho_div = 1.0 / (sL + sR);
    const double psi_a = (sL * (L[4] / L[0]) + sR * (R[4] / R[0])) * rho_div;
    const double gr_a = (sL * fp.gm1 + sR * fp.gm1) * rho_div;
    const double d1 = R[1] - L[1];
    const double d2 = R[2] - L[2];
    const double d3 = R[3] - L[3];
    const double sqvd = d1 * d1 + d2 * d2 + d3 * d3;
    const double p_over_rho =
        (sL * L[4] / L[0] + sR * R[4] / R[0]) * rho_div + 0.5 * rho_a * rho_div * rho_div * sqvd;
    cc = psi_a + gr_a * p_over_rho;
    c = sqrt(cc);
  }
}

// Every output of compute_frozen_state (eigendecomposition.py:120-281), single
// phase, for the conservative eigenvectors: averaged primitives (ROE:
// compute_roe_cons :283-294, density sqrt(rho_L rho_R)), total enthalpy,
// Grueneisen coefficient (gamma - 1 for the ideal gas), speed of sound, its
// square and the squared averaged velocity.
struct FrozenFull {
  double pa[5];
  double H, gr, c, cc, vsq;
};

// ideal_gas.py:90-110: (p / (gamma - 1) + 0.5 rho (u^2 + v^2 + w^2) + p) / rho
__device__ __forceinline__ double total_enthalpy(double p, double rho, double u0, double u1, double u2,
                                                 double gm1) {
  const double E = p / gm1 + 0.5 * rho * (u0 * u0 + u1 * u1 + u2 * u2);
  return (E + p) / rho;
}

__device__ __forceinline__ void frozen_state_full(const double L[5], const double R[5], const FaceParams& fp,
                                                  FrozenFull& z) {
  if (fp.frozen_state == GBF_FROZEN_ARITHMETIC) {
#pragma unroll
    for (int v = 0; v < 5; ++v) z.pa[v] = 0.5 * (L[v] + R[v]);
    z.gr = fp.gm1;
    z.H = total_enthalpy(z.pa[4], z.pa[0], z.pa[1], z.pa[2], z.pa[3], fp.gm1);
    z.c = sqrt(fp.gamma * z.pa[4] / z.pa[0]);
    z.cc = z.c * z.c;
  } else {
    const double sL = sqrt(L[0]);
    const double sR = sqrt(R[0]);
#pragma unroll
    for (int v = 1; v < 5; ++v) z.pa[v] = div0(sL * L[v] + sR * R[v], sL + sR);
    z.pa[0] = sqrt(L[0] * R[0]);
    const double rho_div = 1.0 / (sL + sR);
    const double HL = total_enthalpy(L[4], L[0], L[1], L[2], L[3], fp.gm1);
    const double HR = total_enthalpy(R[4], R[0], R[1], R[2], R[3], fp.gm1);
    z.H = (sL * HL + sR * HR) * rho_div;
    const double psi_a = (sL * (L[4] / L[0]) + sR * (R[4] / R[0])) * rho_div;
    z.gr = (sL * fp.gm1 + sR * fp.gm1) * rho_div;
    const double d1 = R[1] - L[1];
    const double d2 = R[2] - L[2];
    const double d3 = R[3] - L[3];
    const double sqvd = d1 * d1 + d2 * d2 + d3 * d3;
    const double p_over_rho =
        (sL * L[4] / L[0] + sR * R[4] / R[0]) * rho_div + 0.5 * z.pa[0] * rho_div * rho_div * sqvd;
    z.cc = psi_a + z.gr * p_over_rho;
    z.c = sqrt(z.cc);
  }
  z.vsq = z.pa[1] * z.pa[1] + z.pa[2] * z.pa[2] + z.pa[3] * z.pa[3];
}

// velocity_minor_axes (equation_information.py:110) and vel_id_eigs
// (eigendecomposition.py:67-71) for each sweep axis
template <int AX>
struct CharIds {
  static constexpr int m0 = (AX == 0) ? 2 : ((AX == 1) ? 3 : 1);
  static constexpr int m1 = (AX == 0) ? 3 : ((AX == 1) ? 1 : 2);
  static constexpr int e0 = (AX == 1) ? 3 : 2;
  static constexpr int e1 = (AX == 1) ? 2 : 3;
};

// Left eigenvectors of the conservative flux Jacobian along AX
// (eigendecomposition_conservatives, eigendecomposition.py:576-662, Fedkiw et
// al. 1999), zeros included: the transforms sum over every column in order as
// jnp.einsum("ij...,j...->i...") does.
template <int AX>
__device__ __forceinline__ void left_eigvecs_cons(const FrozenFull& z, double Lm[5][5]) {
  constexpr int n = AX + 1;
  using I = CharIds<AX>;
  constexpr int m0 = I::m0, m1 = I::m1;
  const double one_cc = 1.0 / z.cc;
  const double one_rho = 1.0 / z.pa[0];
  const double h = 0.5 * one_cc;
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) Lm[i][j] = 0.0;
  Lm[0][0] = h * (z.gr * z.vsq - z.gr * z.H + (z.pa[n] + z.c) * z.c);
  Lm[0][n] = h * (-z.pa[n] * z.gr - z.c);
  Lm[0][m0] = h * (-z.pa[m0] * z.gr);
  Lm[0][m1] = h * (-z.pa[m1] * z.gr);
  Lm[0][4] = h * z.gr;
  Lm[n][0] = one_cc * (z.H - z.vsq);
  Lm[n][1] = z.pa[1] * one_cc;
  Lm[n][2] = z.pa[2] * one_cc;
  Lm[n][3] = z.pa[3] * one_cc;
  Lm[n][4] = -one_cc;
  Lm[m0][0] = z.pa[m0] * one_rho;
  Lm[m0][m0] = -one_rho;
  Lm[m1][0] = -z.pa[m1] * one_rho;
  Lm[m1][m1] = one_rho;
  Lm[4][0] = h * (z.gr * z.vsq - z.gr * z.H - (z.pa[n] - z.c) * z.c);
  Lm[4][n] = h * (-z.pa[n] * z.gr + z.c);
  Lm[4][m0] = h * (-z.pa[m0] * z.gr);
  Lm[4][m1] = h * (-z.pa[m1] * z.gr);
  Lm[4][4] = h * z.gr;
}

// Right eigenvectors (the same source), zeros included.
template <int AX>
__device__ __forceinline__ void right_eigvecs_cons(const FrozenFull& z, double Rm[5][5]) {
  constexpr int n = AX + 1;
  using I = CharIds<AX>;
  constexpr int m0 = I::m0, m1 = I::m1;
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) Rm[i][j] = 0.0;
  Rm[0][0] = 1.0;
  Rm[n][0] = z.pa[n] - z.c;
  Rm[m0][0] = z.pa[m0];
  Rm[m1][0] = z.pa[m1];
  Rm[4][0] = z.H - z.pa[n] * z.c;
  Rm[0][n] = z.gr;
  Rm[1][n] = z.gr * z.pa[1];
  Rm[2][n] = z.gr * z.pa[2];
  Rm[3][n] = z.gr * z.pa[3];
  Rm[4][n] = z.gr * z.H - z.cc;
  Rm[m0][m0] = -z.pa[0];
  Rm[4][m0] = -z.pa[0] * z.pa[m0];
  Rm[m1][m1] = z.pa[0];
  Rm[4][m1] = z.pa[0] * z.pa[m1];
  Rm[0][4] = 1.0;
  Rm[n][4] = z.pa[n] + z.c;
  Rm[m0][4] = z.pa[m0];
  Rm[m1][4] = z.pa[m1];
  Rm[4][4] = z.H + z.pa[n] * z.c;
}

// CHAR-CONSERVATIVE face states (high_order_godunov.py:404-416): the window of
// conservatives u(v, k) (k = 0..5, face between cells 2 and 3) to
// characteristic variables with the left eigenvectors of the frozen state of
// the primitives w(v, 2), w(v, 3), WENO5-Z on each, back with the right ones.
template <int AX, typename WU, typename WP>
__device__ __forceinline__ void charcons_reconstruct(const WU& u, const WP& w, const FaceParams& fp, double UL[5],
                                                     double UR[5]) {
  double L[5], R[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    L[v] = w(v, 2);
    R[v] = w(v, 3);
  }
  FrozenFull z;
  frozen_state_full(L, R, fp, z);
  double cL[5], cR[5];
  {
    double Lm[5][5];
    left_eigvecs_cons<AX>(z, Lm);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      double ch[6];
#pragma unroll
      for (int k = 0; k < 6; ++k)
        ch[k] = Lm[i][0] * u(0, k) + Lm[i][1] * u(1, k) + Lm[i][2] * u(2, k) + Lm[i][3] * u(3, k) +
                Lm[i][4] * u(4, k);
      cL[i] = weno5z(ch[0], ch[1], ch[2], ch[3], ch[4], fp.stencil_eps);
      cR[i] = weno5z(ch[5], ch[4], ch[3], ch[2], ch[1], fp.stencil_eps);
    }
  }
  double Rm[5][5];
  right_eigvecs_cons<AX>(z, Rm);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    UL[i] = Rm[i][0] * cL[0] + Rm[i][1] * cL[1] + Rm[i][2] * cL[2] + Rm[i][3] * cL[3] + Rm[i][4] * cL[4];
    UR[i] = Rm[i][0] * cR[0] + Rm[i][1] * cR[1] + Rm[i][2] * cR[2] + Rm[i][3] * cR[3] + Rm[i][4] * cR[4];
  }
}

// CHAR-PRIMITIVE face states (high_order_godunov.py:298-316): transform the six
// window cells to characteristic variables with the face's frozen state
// (get_characteristics_from_primitives, :402-433), WENO5-Z each variable on
// both sides, transform back (get_primitives_from_characteristics, :499-523).
// w(v, k) returns primitive v of window cell k (k = 0..5, face between 2 and 3).
template <int AX, typename W>
__device__ __forceinline__ void char_reconstruct(const W& w, const FaceParams& fp, double PL[5],
                                                 double PR[5]) {
  constexpr int N = AX + 1;
  using I = CharIds<AX>;
  double L[5], R[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    L[v] = w(v, 2);
    R[v] = w(v, 3);
  }
  double rho_a, c, cc;
  frozen_state(L, R, fp, rho_a, c, cc);
  const double k_m = -0.5 / c;
  const double k_p = 0.5 / c;
  const double k_e = 0.5 / (cc * rho_a);
  const double k_s = 1.0 / cc;
  double ch0[6], ch1[6], ch4[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double xn = w(N, k);
    const double x0 = w(0, k);
    const double x4 = w(4, k);
    ch0[k] = k_m * xn + k_e * x4;
    ch1[k] = x0 - k_s * x4;
    ch4[k] = k_p * xn + k_e * x4;
  }
  const double eps = fp.stencil_eps;
  double cL[5], cR[5];
  cL[0] = weno5z(ch0[0], ch0[1], ch0[2], ch0[3], ch0[4], eps);
  cR[0] = weno5z(ch0[5], ch0[4], ch0[3], ch0[2], ch0[1], eps);
  cL[1] = weno5z(ch1[0], ch1[1], ch1[2], ch1[3], ch1[4], eps);
  cR[1] = weno5z(ch1[5], ch1[4], ch1[3], ch1[2], ch1[1], eps);
  cL[4] = weno5z(ch4[0], ch4[1], ch4[2], ch4[3], ch4[4], eps);
  cR[4] = weno5z(ch4[5], ch4[4], ch4[3], ch4[2], ch4[1], eps);
  // shear waves: the characteristic variables are the transverse velocities
  cL[I::e0] = weno5z(w(I::m0, 0), w(I::m0, 1), w(I::m0, 2), w(I::m0, 3), w(I::m0, 4), eps);
  cR[I::e0] = weno5z(w(I::m0, 5), w(I::m0, 4), w(I::m0, 3), w(I::m0, 2), w(I::m0, 1), eps);
  cL[I::e1] = weno5z(w(I::m1, 0), w(I::m1, 1), w(I::m1, 2), w(I::m1, 3), w(I::m1, 4), eps);
  cR[I::e1] = weno5z(w(I::m1, 5), w(I::m1, 4), w(I::m1, 3), w(I::m1, 2), w(I::m1, 1), eps);
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
}

// ---------------------------------------------------------------------------
// Signal speeds and Riemann solvers (solvers/riemann_solvers/)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void signal_speeds(int kind, double uL, double uR, double aL, double aR,
                                              double rhoL, double rhoR, double pL, double pR,
                                              double gamma, double& SL, double& SR) {
  switch (kind) {
    case GBF_SIGNAL_EINFELDT: {  // signal_speeds.py:109-133
      const double sL = sqrt(rhoL);
      const double sR = sqrt(rhoR);
      const double od = 1.0 / (sL + sR);
      const double eta2 = 0.5 * sL * sR * od * od;
      const double ubar = (sL * uL + sR * uR) * od;
      const double dbar = sqrt((sL * aL * aL + sR * aR * aR) * od + eta2 * sq(uR - uL));
      SL = fmin(ubar - dbar, uL - aL);
      SR = fmax(ubar + dbar, uR + aR);
      break;
    }
    case GBF_SIGNAL_DAVIS:  // :51-69
      SL = fmin(uL - aL, uR - aR);
      SR = fmax(uL + aL, uR + aR);
      break;
    case GBF_SIGNAL_ARITHMETIC: {  // :10-29
      const double um = 0.5 * (uL + uR);
      const double am = 0.5 * (aL + aR);
      SL = fmin(um - am, uL - aL);
      SR = fmax(um + am, uR + aR);
      break;
    }
    case GBF_SIGNAL_RUSANOV: {  // :31-49
      const double sp = fmax(fabs(uL) + aL, fabs(uR) + aR);
      SL = -sp;
      SR = sp;
      break;
    }
    default: {  // GBF_SIGNAL_TORO, :135-157 with estimate_pressure :201-231
      const double rho_bar = 0.5 * (rhoL + rhoR);
      const double a_bar = 0.5 * (aL + aR);
      const double p_pvrs = 0.5 * (pL + pR) - 0.5 * (uR - uL) * rho_bar * a_bar;
      const double p_star = fmax(0.0, p_pvrs);
      const double g_ = (gamma + 1) * 0.5 / gamma;
      const double qL = (p_star <= pL) ? 1.0 : sqrt(1 + g_ * (p_star / pL - 1));
      const double qR = (p_star <= pR) ? 1.0 : sqrt(1 + g_ * (p_star / pR - 1));
      SL = uL - aL * qL;
      SR = uR + aR * qR;
      break;
    }
  }
}

// HLLC star-state flux of side K (HLLC.py:41-78), J=0 left (min(S,0)), J=1 right (max(S,0)).
template <int AX, int J>
__device__ __forceinline__ void hllc_star_flux(const double P[5], const double U[5], double S,
                                               double Ss, double F[5]) {
  constexpr int N = AX + 1;
  constexpr int T1 = (AX == 0) ? 2 : 1;
  constexpr int T2 = (AX == 2) ? 2 : 3;
  const double pre = (S - P[N]) / (S - Ss) * P[0];
  const double e_term = pre * (U[4] / U[0] + (Ss - P[N]) * (Ss + P[4] / P[0] / (S - P[N])));
  double us[5] = {pre, pre, pre, pre, e_term};
  us[N] *= Ss;
  us[T1] *= P[T1];
  us[T2] *= P[T2];
  physical_flux<AX>(P, U, F);
  const double wave = (J == 0) ? fmin(S, 0.0) : fmax(S, 0.0);
#pragma unroll
  for (int v = 0; v < 5; ++v) F[v] = F[v] + wave * (us[v] - U[v]);
}

// HLLC._solve_riemann_problem_xi_single_phase (HLLC.py:80-126).  GIVEN: the
// face conservatives come with the primitives (the conservative
// reconstructions) instead of being formed from them.
template <int AX, bool GIVEN = false>
__device__ __forceinline__ void hllc(const double PL[5], const double PR[5], const FaceParams& fp, double F[5],
                                     const double* gUL = nullptr, const double* gUR = nullptr) {
  constexpr int N = AX + 1;
  const double cL = speed_of_sound(PL[4], PL[0], fp);
  const double cR = speed_of_sound(PR[4], PR[0], fp);
  double SL, SR;
  signal_speeds(fp.signal_speed, PL[N], PR[N], cL, cR, PL[0], PR[0], PL[4], PR[4], fp.gamma, SL,
                SR);
  // compute_sstar, signal_speeds.py:159-199
  const double rdL = PL[0] * (SL - PL[N]);
  const double rdR = PR[0] * (SR - PR[N]);
  const double Ss = div0((PR[4] - PL[4]) + (PL[N] * rdL - PR[N] * rdR), rdL - rdR);
  // F = 0.5 (1 + sign S*) F*_L + 0.5 (1 - sign S*) F*_R.  With S* != 0 one
  // weight is exactly 0 and the other exactly 1, so only the upwind star flux
  // is formed (a finite F* times 0 adds a signed zero, which changes nothing
  // downstream); S* = 0 and NaN take the general blend.
  double UL[5], UR[5];
  auto side = [&](const double* P, const double* gU, double* U) {
    if (GIVEN) {
#pragma unroll
      for (int v = 0; v < 5; ++v) U[v] = gU[v];
    } else {
      cons_from_prims(P, U, fp.gm1);
    }
  };
  if (Ss > 0.0) {
    side(PL, gUL, UL);
    hllc_star_flux<AX, 0>(PL, UL, SL, Ss, F);
    return;
  }
  if (Ss < 0.0) {
    side(PR, gUR, UR);
    hllc_star_flux<AX, 1>(PR, UR, SR, Ss, F);
    return;
  }
  side(PL, gUL, UL);
  side(PR, gUR, UR);
  double FL[5], FR[5];
  hllc_star_flux<AX, 0>(PL, UL, SL, Ss, FL);
  hllc_star_flux<AX, 1>(PR, UR, SR, Ss, FR);
  const double sg = (Ss == 0.0) ? 0.0 : Ss;  // jnp.sign (NaN propagates)
  const double wl = 0.5 * (1.0 + sg);
  const double wr = 0.5 * (1.0 - sg);
#pragma unroll
  for (int v = 0; v < 5; ++v) F[v] = fma(wl, FL[v], wr * FR[v]);  // wl in {0, 1/2, 1}: exact product
}

// 0.5 (F_L + F_R) - 0.5 alpha (U_R - U_L): Rusanov's flux with its local alpha,
// Lax-Friedrichs' (LaxFriedrichs.py:25-47) with the axis' global one.
template <int AX>
__device__ __forceinline__ void rusanov_alpha(const double PL[5], const double PR[5], const double UL[5],
                                              const double UR[5], double alpha, double F[5]) {
  double FL[5], FR[5];
  physical_flux<AX>(PL, UL, FL);
  physical_flux<AX>(PR, UR, FR);
#pragma unroll
  for (int v = 0; v < 5; ++v) F[v] = fma(0.5, FL[v] + FR[v], -(0.5 * alpha * (UR[v] - UL[v])));
}

// Rusanov._solve_riemann_problem_xi_single_phase (Rusanov.py:25-47)
template <int AX>
__device__ __forceinline__ void rusanov(const double PL[5], const double PR[5], const double UL[5],
                                        const double UR[5], const FaceParams& fp, double F[5]) {
  constexpr int N = AX + 1;
  const double cL = speed_of_sound(PL[4], PL[0], fp);
  const double cR = speed_of_sound(PR[4], PR[0], fp);
  const double alpha = fmax(fabs(PL[N]) + cL, fabs(PR[N]) + cR);
  rusanov_alpha<AX>(PL, PR, UL, UR, alpha, F);
}

// HLL._solve_riemann_problem_xi_single_phase (HLL.py:28-58):
// F = (S_R F_L - S_L F_R + S_L S_R (U_R - U_L)) / (S_R - S_L + eps) with
// S_L = min(s_L, 0), S_R = max(s_R, 0) from the configured signal speeds.
template <int AX>
__device__ __forceinline__ void hll(const double PL[5], const double PR[5], const double UL[5],
                                    const double UR[5], const FaceParams& fp, double F[5]) {
  constexpr int N = AX + 1;
  const double cL = speed_of_sound(PL[4], PL[0], fp);
  const double cR = speed_of_sound(PR[4], PR[0], fp);
  double sL, sR;
  signal_speeds(fp.signal_speed, PL[N], PR[N], cL, cR, PL[0], PR[0], PL[4], PR[4], fp.gamma, sL, sR);
  const double SL = fmin(sL, 0.0);
  const double SR = fmax(sR, 0.0);
  double FL[5], FR[5];
  physical_flux<AX>(PL, UL, FL);
  physical_flux<AX>(PR, UR, FR);
  const double SLR = SL * SR;
  const double den = (SR - SL) + fp.eps;
#pragma unroll
  for (int v = 0; v < 5; ++v) F[v] = div0((SR * FL[v] - SL * FR[v]) + SLR * (UR[v] - UL[v]), den);
}

// Face flux without a convective part (GBF_FLAG_NO_CONVECTIVE): flux_xi =
// zeros, the dissipative fluxes are added to it.
constexpr int RIEMANN_NONE = 100;

// Face flux from face primitives and the given face conservatives (the
// conservative reconstructions).
template <int AX, int RIEMANN>
__device__ __forceinline__ void riemann_flux_u(const double PL[5], const double PR[5], const double UL[5],
                                               const double UR[5], const FaceParams& fp, double F[5]) {
  if (RIEMANN == GBF_RIEMANN_HLLC) {
    hllc<AX, true>(PL, PR, fp, F, UL, UR);
  } else if (RIEMANN == GBF_RIEMANN_HLL) {
    hll<AX>(PL, PR, UL, UR, fp, F);
  } else {
    rusanov<AX>(PL, PR, UL, UR, fp, F);
  }
}

template <int AX, int RIEMANN>
__device__ __forceinline__ void riemann_flux(const double PL[5], const double PR[5],
                                             const FaceParams& fp, double F[5]) {
  double UL[5], UR[5];
  if (RIEMANN == RIEMANN_NONE) {
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = 0.0;
  } else if (RIEMANN == GBF_RIEMANN_HLLC) {
    hllc<AX>(PL, PR, fp, F);  // forms the conservatives of the side(s) it uses
  } else if (RIEMANN == GBF_RIEMANN_HLL) {
    cons_from_prims(PL, UL, fp.gm1);
    cons_from_prims(PR, UR, fp.gm1);
    hll<AX>(PL, PR, UL, UR, fp, F);
  } else {
    cons_from_prims(PL, UL, fp.gm1);
    cons_from_prims(PR, UR, fp.gm1);
    rusanov<AX>(PL, PR, UL, UR, fp, F);
  }
}

}  // namespace gbf
