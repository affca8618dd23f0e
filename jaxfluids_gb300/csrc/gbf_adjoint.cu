// Adjoint of the fused TVD-RK3 step: vector-Jacobian products of the
// right-hand side and of one RK3 step on interior conservatives.
//
// The reference differentiates its step with jax.grad through
// SimulationManager._feed_forward (fixed time step, feed_forward.py:231-524);
// here the reverse sweep is hand written:
//   rhs VJP  w -> J(U)^T w, J = d rhs / d U:  per tile and axis the face
//            cotangents dF = (1/dx)(w[i] - w[i-1]) are pulled back through the
//            Riemann solver and the reconstruction onto the primitives of the
//            stencil cells (deterministically gathered per cell in shared
//            memory), mapped back through the boundary remap, accumulated in a
//            primitive cotangent buffer, and finally pulled back through the
//            primitive/conservative conversion per cell;
//   step VJP lambda^{n+1} -> lambda^n through the three RK stages with the
//            stage states recomputed from U^n.
#include <algorithm>

#include "gbf_vjp_kernels.cuh"

namespace gbf {

namespace {

// ---------------------------------------------------------------------------
// Viscous and heat fluxes (CENTRAL4, any boundary types): the flux at a face
// is a function of the velocity gradient at the face (normal derivatives by
// the face stencil, tangential ones as face interpolations of centre
// derivatives), the face-interpolated velocity and the face derivative of T.
// Every axis has N+1 faces (face i-1/2 at index i; the end faces take the
// one-sided cotangent of their single interior cell, which is exact for
// periodic axes too).  Pass 1 (one thread per face) turns the face-flux
// cotangent into the cotangents of the 11 stencil outputs; pass 2 (one thread
// per interior cell) applies the transposed stencils to every face whose
// stencil reads the cell, pulls dT back through T = p / (rho R) and adds to
// the primitive cotangent in a fixed order; pass 3 (one thread per face, only
// faces whose stencil leaves the domain) sends the cotangents of halo cells
// back through the transposed boundary rules (face rule, and the edge rule of
// compute_edge_halos) with atomics.
// ---------------------------------------------------------------------------
constexpr int VISC_SLOTS = 11;  // dg[a][AX] (3), tangential (2 x 2), dvf (3), dTn

struct ViscVjpParams {
  SweepParams sp;       // sizes, boundary rules, transport, interior primitives (sp.prims)
  const double* w;      // rhs cotangent [5][N]
  double* fc;           // face cotangents: axis a at fc + foff[a], [VISC_SLOTS][faces of axis a]
  long long foff[3];
  double* dP;           // primitive cotangent accumulator [5][N]
};

__device__ __forceinline__ long long cell_off(const SweepParams& p, const int g[3]) {
  return ((long long)g[0] * p.n[1] + g[1]) * p.n[2] + g[2];
}

__device__ __forceinline__ bool cell_inside(const SweepParams& p, const int g[3]) {
  return (unsigned)g[0] < (unsigned)p.n[0] && (unsigned)g[1] < (unsigned)p.n[1] &&
         (unsigned)g[2] < (unsigned)p.n[2];
}

// faces of axis AX: index q[AX] in [0, n], the others in [0, n)
template <int AX>
__device__ __forceinline__ long long face_count(const SweepParams& p) {
  return (long long)(p.n[0] + (AX == 0)) * (p.n[1] + (AX == 1)) * (p.n[2] + (AX == 2));
}

template <int AX>
__device__ __forceinline__ bool face_valid(const SweepParams& p, const int q[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
    if (q[a] < 0 || q[a] > p.n[a] - (a == AX ? 0 : 1)) return false;
  return true;
}

template <int AX>
__device__ __forceinline__ long long face_off(const SweepParams& p, const int q[3]) {
  return ((long long)q[0] * (p.n[1] + (AX == 1)) + q[1]) * (p.n[2] + (AX == 2)) + q[2];
}

// tangential axes of AX in ascending order (the ones that are active)
template <int AX>
__device__ __forceinline__ int tangential(int t) {
  return (AX == 0) ? 1 + t : ((AX == 1) ? 2 * t : t);
}

// Transpose of the face rule of the face beyond which g lies along axis a
// (bc_src / bc_apply): the cotangent d of the halo primitives goes to the
// retrieved interior cell, scaled by d bc_apply / d x (DIRICHLET: nothing).
__device__ __forceinline__ void face_halo_transpose(const SweepParams& p, int a, int g[3], const double d[5],
                                                    double* dP) {
  const int f = 2 * a + (g[a] >= 0 ? 1 : 0);
  const int t = face_type_at(p.bc, p.bf, f, face_pos(p.n, a, g));
  if (t == GBF_BC_DIRICHLET) return;
  const int ga = g[a];
  g[a] = bc_src(ga, p.n[a], t);
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const long long off = cell_off(p, g);
  g[a] = ga;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double x = d[v] * bc_apply_grad(t, a, v);
    if (x != 0.0) atomicAdd(dP + v * cs + off, x);
  }
}

// Transpose of halo_prim: the cotangent d of the primitives of halo cell g
// (outside along one or two axes) onto interior cells.
__device__ __noinline__ void scatter_halo_cotangent(const SweepParams& p, int g0, int g1, int g2, double d0,
                                                    double d1, double d2, double d3, double d4, double* dP) {
  int g[3] = {g0, g1, g2};
  double d[5] = {d0, d1, d2, d3, d4};
  int out[3], k = 0;
  for (int a = 0; a < 3; ++a)
    if (g[a] < 0 || g[a] >= p.n[a]) out[k++] = a;
  if (k == 1) {
    face_halo_transpose(p, out[0], g, d, dP);
    return;
  }
  const int a = out[0], b = out[1];
  const int ta = p.bc[2 * a + (g[a] >= 0 ? 1 : 0)];
  const int tb = p.bc[2 * b + (g[b] >= 0 ? 1 : 0)];
  if (ta == GBF_BC_PERIODIC || ta == GBF_BC_SYMMETRY) {
    g[a] = bc_src(g[a], p.n[a], ta);
    if (ta == GBF_BC_SYMMETRY) d[a + 1] = -d[a + 1];
    face_halo_transpose(p, b, g, d, dP);
    return;
  }
  if (tb == GBF_BC_PERIODIC || tb == GBF_BC_SYMMETRY) {
    g[b] = bc_src(g[b], p.n[b], tb);
    if (tb == GBF_BC_SYMMETRY) d[b + 1] = -d[b + 1];
    face_halo_transpose(p, a, g, d, dP);
    return;
  }
  // ANY_ANY: 0.5 (edge '_10' + edge '_01')
  double h[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) h[v] = 0.5 * d[v];
  int ga[3] = {g[0], g[1], g[2]};
  ga[a] += (g[a] < 0) ? p.nh : -p.nh;
  face_halo_transpose(p, b, ga, h, dP);
  int gb[3] = {g[0], g[1], g[2]};
  gb[b] += (g[b] < 0) ? p.nh : -p.nh;
  face_halo_transpose(p, a, gb, h, dP);
}

// C4: CENTRAL4 stencils fixed at compile time (the default setups), else the
// per-case stencils of p.diss_*.
template <int AX, bool C4>
__global__ void __launch_bounds__(256) visc_face_vjp_kernel(const ViscVjpParams vp) {
  const SweepParams& p = vp.sp;
  const long long nf = face_count<AX>(p);
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nf) return;
  const int e1 = p.n[1] + (AX == 1), e2 = p.n[2] + (AX == 2);
  const int q[3] = {(int)(i / ((long long)e2 * e1)), (int)((i / e2) % e1), (int)(i % e2)};
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  auto cell = [&](int v, int kax, int ax2, int k2) {
    int g[3] = {q[0], q[1], q[2]};
    g[AX] += kax;
    g[ax2] += k2;
    return global_prim<MODE_STAGE_P>(p, v, g[0], g[1], g[2]);
  };
  const double odx = p.one_dx[AX];
  // face cotangent: rhs_c = odx (F_{c-1/2} - F_{c+1/2}) over interior cells c
  int gl[3] = {q[0], q[1], q[2]};
  gl[AX] -= 1;
  const bool hasR = q[AX] < p.n[AX], hasL = q[AX] >= 1;
  double dF[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double wr = hasR ? __ldg(vp.w + v * cs + cell_off(p, q)) : 0.0;
    const double wl = hasL ? __ldg(vp.w + v * cs + cell_off(p, gl)) : 0.0;
    dF[v] = odx * (wr - wl);
  }
  double out[VISC_SLOTS];
#pragma unroll
  for (int k = 0; k < VISC_SLOTS; ++k) out[k] = 0.0;
  if (p.viscous) {
    double dtau[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dtau[k] = (p.active_mask & (1 << k)) ? -dF[1 + k] : 0.0;
    if (p.heat_production) {
      // tau and the face velocity of the forward (energy flux sum_k tau_k vf_k)
      double gr[3][3];
      face_velocity_gradient<AX, C4>(p, cell, gr);
      double tau[3], tr = 0.0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const bool act = p.active_mask & (1 << k);
        tau[k] = act ? p.mu1 * (gr[AX][k] + gr[k][AX]) : 0.0;
        if (act) tr += gr[k][k];
      }
      tau[AX] += p.mu2 * tr;
      const double dvt = -dF[4];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (!(p.active_mask & (1 << k))) continue;
        const double vf = face_interp_along<AX, C4>(p, [&](int kax) { return cell(1 + k, kax, AX, 0); });
        dtau[k] += dvt * vf;
        out[7 + k] = dvt * tau[k];
      }
    }
    const double dtr = p.mu2 * dtau[AX];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (!(p.active_mask & (1 << a))) continue;
      out[a] = p.mu1 * dtau[a] + ((a == AX) ? p.mu1 * dtau[AX] + dtr : 0.0);
    }
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int ii = tangential<AX>(t);
      if (!(p.active_mask & (1 << ii))) continue;
      out[3 + 2 * t] = p.mu1 * dtau[ii];  // d u_AX / d x_i
      out[4 + 2 * t] = dtr;               // d u_i / d x_i
    }
  }
  if (p.heat) out[10] = -p.kappa * dF[4];
  double* fc = vp.fc + vp.foff[AX];
#pragma unroll
  for (int k = 0; k < VISC_SLOTS; ++k) fc[k * nf + i] = out[k];
}

// Weights of the dissipative stencils, [CENTRAL4, CENTRAL2]: face derivative
// and face interpolation at normal offsets -2..1, centre derivative at offsets
// -2, -1, +1, +2 (CENTRAL2 zero at the outer points)
__device__ __constant__ double kFd[2][4] = {{1.0 / 24.0, -27.0 / 24.0, 27.0 / 24.0, -1.0 / 24.0},
                                            {0.0, -1.0, 1.0, 0.0}};
__device__ __constant__ double kFi[2][4] = {{-1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0},
                                            {0.0, 0.5, 0.5, 0.0}};
__device__ __constant__ double kCd[2][4] = {{1.0 / 12.0, -8.0 / 12.0, 8.0 / 12.0, -1.0 / 12.0},
                                            {0.0, -0.5, 0.5, 0.0}};
__device__ __constant__ int kCj[4] = {-2, -1, 1, 2};

// Stencil weight k of the face derivative, face interpolation and centre
// derivative: CENTRAL4 as immediates when C4, else the case's row of the tables.
template <bool C4>
__device__ __forceinline__ double w_fd(const SweepParams& p, int k) {
  if (C4) return (k == 0) ? 1.0 / 24.0 : (k == 1) ? -27.0 / 24.0 : (k == 2) ? 27.0 / 24.0 : -1.0 / 24.0;
  return kFd[p.diss_face][k];
}
template <bool C4>
__device__ __forceinline__ double w_fi(const SweepParams& p, int k) {
  if (C4) return (k == 0 || k == 3) ? -1.0 / 16.0 : 9.0 / 16.0;
  return kFi[p.diss_recon][k];
}
template <bool C4>
__device__ __forceinline__ double w_cd(const SweepParams& p, int k) {
  if (C4) return (k == 0) ? 1.0 / 12.0 : (k == 1) ? -8.0 / 12.0 : (k == 2) ? 8.0 / 12.0 : -1.0 / 12.0;
  return kCd[p.diss_center][k];
}

template <bool C4>
__global__ void __launch_bounds__(256) visc_cell_gather_kernel(const ViscVjpParams vp) {
  const SweepParams& p = vp.sp;
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= cs) return;
  const int c[3] = {(int)(i / ((long long)p.n[2] * p.n[1])), (int)((i / p.n[2]) % p.n[1]), (int)(i % p.n[2])};
  double du[3] = {0.0, 0.0, 0.0}, dT = 0.0;
#pragma unroll
  for (int AX = 0; AX < 3; ++AX) {
    if (!(p.active_mask & (1 << AX))) continue;
    const long long nf = (long long)(p.n[0] + (AX == 0)) * (p.n[1] + (AX == 1)) * (p.n[2] + (AX == 2));
    const double* fc = vp.fc + vp.foff[AX];
    const int e1 = p.n[1] + (AX == 1), e2 = p.n[2] + (AX == 2);
    const double odx = p.one_dx[AX];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      // this cell is stencil point k (offset k-2) of the face at q = c - (k-2) along AX
      int q[3] = {c[0], c[1], c[2]};
      q[AX] -= k - 2;
      if (q[AX] < 0 || q[AX] > p.n[AX]) continue;
      const long long f = ((long long)q[0] * e1 + q[1]) * e2 + q[2];
      const double wd = odx * w_fd<C4>(p, k);
      if (wd != 0.0 || w_fi<C4>(p, k) != 0.0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) du[a] += wd * fc[a * nf + f] + w_fi<C4>(p, k) * fc[(7 + a) * nf + f];
        dT += wd * fc[10 * nf + f];
      }
      if (w_fi<C4>(p, k) == 0.0) continue;
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int ii = (AX == 0) ? 1 + t : ((AX == 1) ? 2 * t : t);
        if (!(p.active_mask & (1 << ii))) continue;
        const double odi = p.one_dx[ii];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          if (w_cd<C4>(p, jj) == 0.0) continue;
          int h[3] = {q[0], q[1], q[2]};
          h[ii] -= kCj[jj];
          if (h[ii] < 0 || h[ii] >= p.n[ii]) continue;
          const long long ff = ((long long)h[0] * e1 + h[1]) * e2 + h[2];
          const double wt = w_fi<C4>(p, k) * odi * w_cd<C4>(p, jj);
          du[AX] += wt * fc[(3 + 2 * t) * nf + ff];
          du[ii] += wt * fc[(4 + 2 * t) * nf + ff];
        }
      }
    }
  }
  const double rho = __ldg(p.prims + i);
  const double pr = __ldg(p.prims + 4 * cs + i);
  // T = p / (rho R)
  const double iden = 1.0 / (rho * p.R);
  vp.dP[i] += -dT * pr * iden / rho;
  vp.dP[cs + i] += du[0];
  vp.dP[2 * cs + i] += du[1];
  vp.dP[3 * cs + i] += du[2];
  vp.dP[4 * cs + i] += dT * iden;
}

// Pass 3: the stencil cells of face q (axis AX) that lie outside the domain.
template <int AX, bool C4>
__global__ void __launch_bounds__(256) visc_halo_scatter_kernel(const ViscVjpParams vp) {
  const SweepParams& p = vp.sp;
  const long long nf = face_count<AX>(p);
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nf) return;
  const int e1 = p.n[1] + (AX == 1), e2 = p.n[2] + (AX == 2);
  const int q[3] = {(int)(i / ((long long)e2 * e1)), (int)((i / e2) % e1), (int)(i % e2)};
  // faces whose whole stencil is interior have nothing to send
  bool reaches_out = q[AX] < 2 || q[AX] > p.n[AX] - 2;
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const int ii = tangential<AX>(t);
    if (p.viscous && (p.active_mask & (1 << ii)) && (q[ii] < 2 || q[ii] > p.n[ii] - 3)) reaches_out = true;
  }
  if (!reaches_out) return;
  const double* fc = vp.fc + vp.foff[AX];
  double s[VISC_SLOTS];
#pragma unroll
  for (int k = 0; k < VISC_SLOTS; ++k) s[k] = fc[k * nf + i];
  const double odx = p.one_dx[AX];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (w_fd<C4>(p, k) == 0.0 && w_fi<C4>(p, k) == 0.0) continue;
    int g[3] = {q[0], q[1], q[2]};
    g[AX] += k - 2;
    if (g[AX] < 0 || g[AX] >= p.n[AX]) {
      // normal stencil cell in the halo: velocity and temperature cotangents
      const double wd = odx * w_fd<C4>(p, k);
      double d[5];
      d[1] = wd * s[0] + w_fi<C4>(p, k) * s[7];
      d[2] = wd * s[1] + w_fi<C4>(p, k) * s[8];
      d[3] = wd * s[2] + w_fi<C4>(p, k) * s[9];
      const double dT = wd * s[10];
      const double rho = global_prim<MODE_STAGE_P>(p, 0, g[0], g[1], g[2]);
      const double pr = global_prim<MODE_STAGE_P>(p, 4, g[0], g[1], g[2]);
      const double iden = 1.0 / (rho * p.R);
      d[0] = -dT * pr * iden / rho;
      d[4] = dT * iden;
      scatter_halo_cotangent(p, g[0], g[1], g[2], d[0], d[1], d[2], d[3], d[4], vp.dP);
    }
    if (!p.viscous || w_fi<C4>(p, k) == 0.0) continue;
    for (int t = 0; t < 2; ++t) {
      const int ii = tangential<AX>(t);
      if (!(p.active_mask & (1 << ii))) continue;
      const double odi = p.one_dx[ii];
      for (int jj = 0; jj < 4; ++jj) {
        if (w_cd<C4>(p, jj) == 0.0) continue;
        int h[3] = {g[0], g[1], g[2]};
        h[ii] += kCj[jj];
        if (cell_inside(p, h)) continue;
        const double wt = w_fi<C4>(p, k) * odi * w_cd<C4>(p, jj);
        double d[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        d[1 + AX] = wt * s[3 + 2 * t];
        d[1 + ii] = wt * s[4 + 2 * t];
        scatter_halo_cotangent(p, h[0], h[1], h[2], d[0], d[1], d[2], d[3], d[4], vp.dP);
      }
    }
  }
}

// The three passes of the dissipative-flux reverse.
template <bool C4>
void launch_visc_vjp(const ViscVjpParams& q, const long long nface[3], long long cells, cudaStream_t s) {
  auto blocks = [](long long n) { return (unsigned)((n + 255) / 256); };
  if (nface[0]) visc_face_vjp_kernel<0, C4><<<blocks(nface[0]), 256, 0, s>>>(q);
  if (nface[1]) visc_face_vjp_kernel<1, C4><<<blocks(nface[1]), 256, 0, s>>>(q);
  if (nface[2]) visc_face_vjp_kernel<2, C4><<<blocks(nface[2]), 256, 0, s>>>(q);
  visc_cell_gather_kernel<C4><<<blocks(cells), 256, 0, s>>>(q);
  if (nface[0]) visc_halo_scatter_kernel<0, C4><<<blocks(nface[0]), 256, 0, s>>>(q);
  if (nface[1]) visc_halo_scatter_kernel<1, C4><<<blocks(nface[1]), 256, 0, s>>>(q);
  if (nface[2]) visc_halo_scatter_kernel<2, C4><<<blocks(nface[2]), 256, 0, s>>>(q);
}

// out = (dP/dU)^T dP per cell, dP is cleared for the next use.
// With gravity (g non-null) the transpose of add_gravity joins: d rho += g . w[1:4],
// d m_j += g_j w[4], w the right-hand side's cotangent.  dU (non-null: the
// CONSERVATIVE reconstruction) adds the cotangent that reached the state's
// conservatives directly, and is cleared.
__global__ void dp_to_du_kernel(const double* U, double* dP, double* out, long long n, double gm1,
                                const double* w, double g0, double g1, double g2, double* dU) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double u[5], d[5], o[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      u[v] = U[v * n + i];
      d[v] = dP[v * n + i];
      dP[v * n + i] = 0.0;
    }
    prims_from_cons_vjp(u, d, gm1, o);
    if (w) {
      const double w1 = w[n + i], w2 = w[2 * n + i], w3 = w[3 * n + i], w4 = w[4 * n + i];
      o[0] += (g0 * w1 + g1 * w2) + g2 * w3;
      o[1] += g0 * w4;
      o[2] += g1 * w4;
      o[3] += g2 * w4;
    }
    if (dU) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        o[v] += dU[v * n + i];
        dU[v * n + i] = 0.0;
      }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * n + i] = o[v];
  }
}

// y = a x + b * (*dt) * z (elementwise, interior buffers of 5 n doubles)
__global__ void axpy_dt_kernel(double* y, const double* x, double a, const double* z, double b,
                               const double* dtp, long long m) {
  const double s = b * (*dtp);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x)
    y[i] = a * x[i] + s * z[i];
}

// lam_n = acc + lam1 + dt * j1  where acc = 1/3 lam3 + 3/4 lam2
__global__ void step_combine_kernel(double* out, const double* lam3, const double* lam2, const double* lam1,
                                    const double* j1, const double* dtp, long long m) {
  const double dt = *dtp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = ((1.0 / 3.0) * lam3[i] + 0.75 * lam2[i]) + lam1[i] + dt * j1[i];
}

// y += b x (elementwise)
__global__ void add_scaled_kernel(double* y, const double* x, double b, long long m) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x)
    y[i] += b * x[i];
}

__global__ void zero_kernel(double* x, long long m) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = 0.0;
}

inline int grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (int)std::max(1LL, std::min(g, 152LL * 16));
}

int vjp_check(const gbf_case* c) {
  if (c->flags & GBF_FLAG_NO_CONVECTIVE) return GBF_OK;  // no convective scheme to reverse
  if (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE && c->recon != GBF_RECON_WENO5Z) return GBF_ERR_UNSUPPORTED;
  return GBF_OK;
}

inline bool vjp_dissipative(const gbf_case* c) { return (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) != 0; }

// doubles of rhs-VJP scratch beyond the primitive cotangent: interior
// primitives and the viscous face cotangents of every active axis
// faces of axis a: N_a + 1 along a
long long visc_faces(const CaseInfo& ci, int a) { return ci.cells / ci.n[a] * (ci.n[a] + 1); }

long long vjp_visc_doubles(const gbf_case* c, const CaseInfo& ci) {
  if (!vjp_dissipative(c)) return 0;
  long long faces = 0;
  for (int a = 0; a < 3; ++a)
    if (ci.active_mask & (1 << a)) faces += visc_faces(ci, a);
  return 5 * ci.cells + VISC_SLOTS * faces;
}

// the conservative reconstructions' (CONSERVATIVE, CHAR-CONSERVATIVE)
// conservative cotangent follows the dissipative part
inline bool vjp_cons(const gbf_case* c) {
  return (c->recon_var == GBF_RECVAR_CONSERVATIVE || c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE) &&
         !(c->flags & GBF_FLAG_NO_CONVECTIVE);
}

inline bool vjp_lf(const gbf_case* c) {
  return c->riemann == GBF_RIEMANN_LAXFRIEDRICHS && !(c->flags & GBF_FLAG_NO_CONVECTIVE);
}

// Lax-Friedrichs tie list: two entries (both face states) per face of the
// axis with the most faces
long long lf_ties_cap(const gbf_case* c, const CaseInfo& ci) {
  long long cap = 0;
  for (int a = 0; a < 3; ++a) {
    if (!(ci.active_mask & (1 << a))) continue;
    const long long nf = c->bc[2 * a] == GBF_BC_PERIODIC ? ci.n[a] : ci.n[a] + 1;
    cap = std::max(cap, 2 * (ci.cells / ci.n[a]) * nf);
  }
  return cap;
}

// Lax-Friedrichs scratch: the state's primitives, the speeds and their
// cotangents (8 doubles), the tie counters (4) and list
long long vjp_lf_doubles(const gbf_case* c, const CaseInfo& ci) {
  return vjp_lf(c) ? 5 * ci.cells + 8 + 4 + lf_ties_cap(c, ci) : 0;
}

long long vjp_extra_doubles(const gbf_case* c, const CaseInfo& ci) {
  return vjp_visc_doubles(c, ci) + (vjp_cons(c) ? 5 * ci.cells : 0) + vjp_lf_doubles(c, ci);
}

// VJP of the rhs at state U (interior): out = J(U)^T w.  dP: zeroed scratch of 5 n doubles
// (left zeroed on return).
int launch_rhs_vjp(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, const double* U,
                   const double* w, double* out, double* dP, double* extra, cudaStream_t s) {
  // the CONSERVATIVE pencil carries primitives and conservatives: the 3-D
  // default tile is one cell shorter (6 x 8 x 8) to stay within 227 KB of
  // shared memory with the WENO5 gradient rows and face slots
  gbf_tile cons_tile{{6, 8, 8}, 256};
  const bool user_tile = tile && (tile->t[0] > 0 || tile->t[1] > 0 || tile->t[2] > 0);
  if (vjp_cons(c) && !user_tile && ci.active_mask == 7) tile = &cons_tile;
  VjpParams vp;
  int threads;
  size_t smem;
  int st = make_sweep_params(c, ci, tile, &vp.sp, &threads, &smem, true);
  if (st != GBF_OK) return st;
  const int R = recon_radius(c->recon);
  // shared memory: pencil primitives + 2R x 5 slots per face (replaces the
  // flux slots) + 25 doubles per thread for WENO's right-stencil gradients
  // (primitive or characteristic)
  long long pmax = 0, fmax = 0;
  for (int a = 0; a < 3; ++a) {
    if (!(ci.active_mask & (1 << a))) continue;
    long long pv = 1, fv = 1;
    for (int b = 0; b < 3; ++b) {
      pv *= vp.sp.t[b] + (b == a ? 2 * R : 0);
      fv *= vp.sp.t[b] + (b == a ? 1 : 0);
    }
    pmax = std::max(pmax, pv);
    fmax = std::max(fmax, fv);
  }
  // (the CONSERVATIVE pencil stages the conservatives too)
  smem = (size_t)((vjp_cons(c) ? 10 : 5) * pmax + 10 * R * fmax + (R == 3 ? 25 * threads : 0)) * sizeof(double);
  if (smem > 227 * 1024) return GBF_ERR_INVALID_ARGUMENT;
  vp.sp.cons = U;
  vp.w = w;
  vp.dP = dP;
  vp.dU = vjp_cons(c) ? extra + vjp_visc_doubles(c, ci) : nullptr;
  if (vp.dU) zero_kernel<<<grid_for(5 * ci.cells), 256, 0, s>>>(vp.dU, 5 * ci.cells);
  vp.lf_alpha = nullptr;
  vp.lf_dalpha = nullptr;
  vp.lf_tie_side = -1;
  vp.lf_tie_ds = 0.0;
  // Lax-Friedrichs: the axes' speeds of U from the forward face kernels'
  // speed pass on U's primitives (the same face states and arithmetic as the
  // forward, so the ties below are the forward's)
  double* lfP = nullptr;
  double* lfa = nullptr;
  unsigned long long* ties = nullptr;
  if (vjp_lf(c)) {
    lfP = extra + vjp_visc_doubles(c, ci) + (vjp_cons(c) ? 5 * ci.cells : 0);
    lfa = lfP + 5 * ci.cells;
    ties = reinterpret_cast<unsigned long long*>(lfa + 8);
    if ((st = launch_convert(c, U, lfP, ci.cells, 1, s)) != GBF_OK) return st;
    if (cudaMemsetAsync(lfa, 0, 8 * sizeof(double), s) != cudaSuccess) return GBF_ERR_CUDA;
    if ((st = launch_lf_face_pass(c, ci, U, lfP, lfa, nullptr, 0, 1, -1, nullptr, s)) != GBF_OK) return st;
    vp.lf_alpha = lfa;
    vp.lf_dalpha = lfa + 3;
  }
  const int grid = vp.sp.tiles[0] * vp.sp.tiles[1] * vp.sp.tiles[2];
  if (c->flags & GBF_FLAG_NO_CONVECTIVE)
    st = GBF_OK;  // dissipative fluxes only
  else if (vjp_cons(c))
    st = (c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE) ? launch_vjp_charcons(c->riemann, vp, grid, threads, smem, s)
                                                        : launch_vjp_cons(c->riemann, vp, grid, threads, smem, s);
  else if (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE)
    st = launch_vjp_char(c->riemann, vp, grid, threads, smem, s);
  else if (c->recon == GBF_RECON_WENO5Z || c->recon == GBF_RECON_WENO5JS)
    st = launch_vjp_weno5(c->recon, c->riemann, vp, grid, threads, smem, s);
  else if (c->recon == GBF_RECON_TENO5)
    st = launch_vjp_teno5(c->riemann, vp, grid, threads, smem, s);
  else
    st = launch_vjp_short(c->recon, c->riemann, vp, grid, threads, smem, s);
  if (st != GBF_OK) return st;
  if (cudaGetLastError() != cudaSuccess) return GBF_ERR_CUDA;
  if (vjp_lf(c)) {
    // the speeds' cotangents to the face states attaining them, axis by axis
    const long long cap = lf_ties_cap(c, ci);
    for (int a = 0; a < 3; ++a) {
      if (!(ci.active_mask & (1 << a))) continue;
      LfTieParams tp;
      if (cudaMemsetAsync(ties, 0, 4 * sizeof(unsigned long long), s) != cudaSuccess) return GBF_ERR_CUDA;
      if ((st = launch_lf_face_pass(c, ci, U, lfP, lfa, ties, cap, 2, a, &tp.sp, s)) != GBF_OK) return st;
      tp.ties = ties;
      tp.cap = cap;
      tp.dalpha = lfa + 3;
      tp.dP = dP;
      tp.dU = vp.dU;
      if (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE)
        st = launch_lf_ties_char(a, tp, s);
      else if (c->recon_var == GBF_RECVAR_CONSERVATIVE)
        st = launch_lf_ties_cons(a, tp, s);
      else if (c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE)
        st = launch_lf_ties_charcons(a, tp, s);
      else if (c->recon == GBF_RECON_WENO5Z || c->recon == GBF_RECON_WENO5JS)
        st = launch_lf_ties_weno5(c->recon, a, tp, s);
      else if (c->recon == GBF_RECON_TENO5)
        st = launch_lf_ties_teno5(a, tp, s);
      else
        st = launch_lf_ties_short(c->recon, a, tp, s);
      if (st != GBF_OK) return st;
    }
  }
  if (vjp_dissipative(c)) {
    ViscVjpParams q;
    q.sp = vp.sp;
    double* P = extra;
    q.sp.prims = P;
    q.w = w;
    q.fc = P + 5 * ci.cells;
    q.dP = dP;
    long long off = 0, nface[3];
    for (int a = 0; a < 3; ++a) {
      nface[a] = (ci.active_mask & (1 << a)) ? visc_faces(ci, a) : 0;
      q.foff[a] = off;
      off += VISC_SLOTS * nface[a];
    }
    if ((st = launch_convert(c, U, P, ci.cells, 1, s)) != GBF_OK) return st;
    const bool c4 = c->dissipative_stencil[0] == GBF_CENTRAL4 && c->dissipative_stencil[1] == GBF_CENTRAL4 &&
                    c->dissipative_stencil[2] == GBF_CENTRAL4;
    if (c4)
      launch_visc_vjp<true>(q, nface, ci.cells, s);
    else
      launch_visc_vjp<false>(q, nface, ci.cells, s);
    if (cudaGetLastError() != cudaSuccess) return GBF_ERR_CUDA;
  }
  const bool grav = (c->flags & GBF_FLAG_GRAVITY) != 0;
  dp_to_du_kernel<<<grid_for(ci.cells), 256, 0, s>>>(U, dP, out, ci.cells, ci.fp.gm1, grav ? w : nullptr,
                                                     c->gravity[0], c->gravity[1], c->gravity[2], vp.dU);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

}  // namespace

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_vjp_workspace_bytes(const gbf_case* c) {
  CaseInfo ci;
  if (make_case_info(c, &ci) != GBF_OK || vjp_check(c) != GBF_OK) return 0;  // no adjoint for this case
  // step VJP: U1, U2, lam2, lam1, j, dP (6 interior states); dissipative
  // cases add the primitives and the viscous face cotangents; the forward
  // recomputation of U1, U2 adds two primitive buffers and the face buffers
  return ((size_t)8 * 5 * (size_t)ci.cells + (size_t)vjp_extra_doubles(c, ci) +
          (size_t)stage_face_doubles(c, ci)) * sizeof(double);
}

static int gbf_rhs_vjp_impl(const gbf_case* c, const double* cons, const double* w, double* out,
                           void* workspace, const gbf_tile* tile, void* stream) {
  int st = gbf_case_check(c);
  if (st != GBF_OK) return st;
  if ((st = vjp_check(c)) != GBF_OK) return st;
  if (!cons || !w || !out || !workspace) return GBF_ERR_INVALID_ARGUMENT;
  CaseInfo ci;
  make_case_info(c, &ci);
  cudaStream_t s = (cudaStream_t)stream;
  double* dP = (double*)workspace;
  zero_kernel<<<grid_for(5 * ci.cells), 256, 0, s>>>(dP, 5 * ci.cells);
  return launch_rhs_vjp(c, ci, tile, cons, w, out, dP, dP + 5 * ci.cells, s);
}

extern "C" int gbf_rhs_vjp(const gbf_case* c, const double* cons, const double* w, double* out,
                           void* workspace, const gbf_tile* tile, void* stream) {
  return record_status(gbf_rhs_vjp_impl(c, cons, w, out, workspace, tile, stream));
}

static int step_vjp(const gbf_case* c, const double* cons, const double* u1_in, const double* u2_in,
                    const double* dt, const double* lam, double* lam_out, void* workspace, const gbf_tile* tile,
                    void* stream) {
  int st = gbf_case_check(c);
  if (st != GBF_OK) return st;
  if ((st = vjp_check(c)) != GBF_OK) return st;
  if (!cons || !dt || !lam || !lam_out || !workspace || lam_out == lam) return GBF_ERR_INVALID_ARGUMENT;
  CaseInfo ci;
  make_case_info(c, &ci);
  cudaStream_t s = (cudaStream_t)stream;
  const long long m = 5 * ci.cells;
  double* U1 = (double*)workspace;
  double* U2 = U1 + m;
  double* lam2 = U2 + m;
  double* lam1 = lam2 + m;
  double* j = lam1 + m;
  double* dP = j + m;
  double* extra = dP + m;
  const double* S1 = u1_in;
  const double* S2 = u2_in;
  if (!S1 || !S2) {
    // recompute the stage states U1, U2 from U^n with the forward stage
    // kernels (gbf_rk3_advance's stages 0 and 1)
    SweepParams p;
    int threads;
    size_t smem;
    if ((st = make_sweep_params(c, ci, tile, &p, &threads, &smem)) != GBF_OK) return st;
    double* Pa = extra + vjp_extra_doubles(c, ci);
    double* Pb = Pa + m;
    FaceBuffers fb;
    stage_face_buffers(c, ci, Pb + m, &fb);
    // the forward kernels read dt from dt_state[0]; dt points at a device scalar
    p.dt_state = const_cast<double*>(dt);
    p.reduce_dt = 0;
    if ((st = launch_convert(c, cons, Pa, ci.cells, 1, s)) != GBF_OK) return st;
    p.stage = 0; p.cons = cons; p.cons0 = cons; p.out = U1; p.prims = Pa;
    if ((st = launch_rk3_stage(c, ci, tile, p, fb, Pb, s)) != GBF_OK) return st;
    p.stage = 1; p.cons = U1; p.cons0 = cons; p.out = U2; p.prims = Pb;
    if ((st = launch_rk3_stage(c, ci, tile, p, fb, nullptr, s)) != GBF_OK) return st;
    S1 = U1;
    S2 = U2;
  }
  zero_kernel<<<grid_for(m), 256, 0, s>>>(dP, m);
  // stage 3: U3 = 1/3 Un + 2/3 U2 + 2/3 dt L(U2)
  if ((st = launch_rhs_vjp(c, ci, tile, S2, lam, j, dP, extra, s)) != GBF_OK) return st;
  axpy_dt_kernel<<<grid_for(m), 256, 0, s>>>(lam2, lam, 2.0 / 3.0, j, 2.0 / 3.0, dt, m);
  // stage 2: U2 = 3/4 Un + 1/4 U1 + 1/4 dt L(U1)
  if ((st = launch_rhs_vjp(c, ci, tile, S1, lam2, j, dP, extra, s)) != GBF_OK) return st;
  axpy_dt_kernel<<<grid_for(m), 256, 0, s>>>(lam1, lam2, 0.25, j, 0.25, dt, m);
  // stage 1: U1 = Un + dt L(Un)
  if ((st = launch_rhs_vjp(c, ci, tile, cons, lam1, j, dP, extra, s)) != GBF_OK) return st;
  step_combine_kernel<<<grid_for(m), 256, 0, s>>>(lam_out, lam, lam2, lam1, j, dt, m);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

static int gbf_rk3_step_vjp_impl(const gbf_case* c, const double* cons, const double* dt, const double* lam,
                                double* lam_out, void* workspace, const gbf_tile* tile, void* stream) {
  return step_vjp(c, cons, nullptr, nullptr, dt, lam, lam_out, workspace, tile, stream);
}

// Reverse of one fused stage U_out = a U_k + b U^n + c dt L(U_k)
// (RK3.py:27-29: stage 0 a = 1, b = 0, c = 1 with U_k = U^n; stage 1
// a = 1/4, b = 3/4, c = 1/4; stage 2 a = 2/3, b = 1/3, c = 2/3):
// lam_k = a lam + c dt J(U_k)^T lam, lam_n += b lam (stages 1 and 2).
static int gbf_rk3_stage_vjp_impl(const gbf_case* c, int stage, const double* cons_k, const double* dt,
                                  const double* lam, double* lam_k, double* lam_n, void* workspace,
                                  const gbf_tile* tile, void* stream) {
  int st = gbf_case_check(c);
  if (st != GBF_OK) return st;
  if ((st = vjp_check(c)) != GBF_OK) return st;
  if (stage < 0 || stage > 2 || !cons_k || !dt || !lam || !lam_k || !workspace || lam_k == lam)
    return GBF_ERR_INVALID_ARGUMENT;
  if (stage > 0 && (!lam_n || lam_n == lam || lam_n == lam_k)) return GBF_ERR_INVALID_ARGUMENT;
  CaseInfo ci;
  make_case_info(c, &ci);
  cudaStream_t s = (cudaStream_t)stream;
  const long long m = 5 * ci.cells;
  double* dP = (double*)workspace;
  double* j = dP + m;
  double* extra = j + m;
  static const double kA[3] = {1.0, 0.25, 2.0 / 3.0};
  static const double kB[3] = {0.0, 0.75, 1.0 / 3.0};
  static const double kC[3] = {1.0, 0.25, 2.0 / 3.0};
  zero_kernel<<<grid_for(m), 256, 0, s>>>(dP, m);
  if ((st = launch_rhs_vjp(c, ci, tile, cons_k, lam, j, dP, extra, s)) != GBF_OK) return st;
  axpy_dt_kernel<<<grid_for(m), 256, 0, s>>>(lam_k, lam, kA[stage], j, kC[stage], dt, m);
  if (stage > 0) add_scaled_kernel<<<grid_for(m), 256, 0, s>>>(lam_n, lam, kB[stage], m);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

extern "C" int gbf_rk3_stage_vjp(const gbf_case* c, int stage, const double* cons_k, const double* dt,
                                 const double* lam, double* lam_k, double* lam_n, void* workspace,
                                 const gbf_tile* tile, void* stream) {
  return record_status(gbf_rk3_stage_vjp_impl(c, stage, cons_k, dt, lam, lam_k, lam_n, workspace, tile, stream));
}

extern "C" int gbf_rk3_step_vjp(const gbf_case* c, const double* cons, const double* dt, const double* lam,
                                double* lam_out, void* workspace, const gbf_tile* tile, void* stream) {
  return record_status(gbf_rk3_step_vjp_impl(c, cons, dt, lam, lam_out, workspace, tile, stream));
}

static int gbf_rk3_step_vjp_stages_impl(const gbf_case* c, const double* cons, const double* u1,
                                       const double* u2, const double* dt, const double* lam, double* lam_out,
                                       void* workspace, const gbf_tile* tile, void* stream) {
  if (!u1 || !u2) return GBF_ERR_INVALID_ARGUMENT;
  return step_vjp(c, cons, u1, u2, dt, lam, lam_out, workspace, tile, stream);
}

extern "C" int gbf_rk3_step_vjp_stages(const gbf_case* c, const double* cons, const double* u1,
                                       const double* u2, const double* dt, const double* lam, double* lam_out,
                                       void* workspace, const gbf_tile* tile, void* stream) {
  return record_status(gbf_rk3_step_vjp_stages_impl(c, cons, u1, u2, dt, lam, lam_out, workspace, tile, stream));
}
