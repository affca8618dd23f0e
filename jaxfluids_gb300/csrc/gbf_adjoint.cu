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
// Viscous and heat fluxes (CENTRAL4, periodic boundaries): the flux at a face
// is a function of the velocity gradient at the face (normal derivatives by
// the face stencil, tangential ones as face interpolations of centre
// derivatives), the face-interpolated velocity and the face derivative of T.
// Pass 1 (one thread per face) turns the face-flux cotangent into the
// cotangents of those 11 stencil outputs; pass 2 (one thread per cell) applies
// the transposed stencils, gathers over every face whose stencil reads the
// cell, pulls dT back through T = p / (rho R) and adds to the primitive
// cotangent.  Fixed summation order: deterministic.
// ---------------------------------------------------------------------------
constexpr int VISC_SLOTS = 11;  // dg[a][AX] (3), tangential (2 x 2), dvf (3), dTn

struct ViscVjpParams {
  int n[3];
  int active_mask;
  double one_dx[3];
  const double* prims;  // interior primitives [5][N]
  const double* w;      // rhs cotangent [5][N]
  double* fc;           // face cotangents [3][VISC_SLOTS][N]; face i-1/2 of axis a stored at cell i
  double* dP;           // primitive cotangent accumulator [5][N]
  double mu1, mu2, kappa, R;
  int viscous, heat, heat_production;
};

__device__ __forceinline__ long long wrap_off(const ViscVjpParams& p, int g0, int g1, int g2) {
  g0 = (g0 < 0) ? g0 + p.n[0] : ((g0 >= p.n[0]) ? g0 - p.n[0] : g0);
  g1 = (g1 < 0) ? g1 + p.n[1] : ((g1 >= p.n[1]) ? g1 - p.n[1] : g1);
  g2 = (g2 < 0) ? g2 + p.n[2] : ((g2 >= p.n[2]) ? g2 - p.n[2] : g2);
  return ((long long)g0 * p.n[1] + g1) * p.n[2] + g2;
}

// tangential axes of AX in ascending order (the ones that are active)
template <int AX>
__device__ __forceinline__ int tangential(int t) {
  return (AX == 0) ? 1 + t : ((AX == 1) ? 2 * t : t);
}

template <int AX>
__global__ void __launch_bounds__(256) visc_face_vjp_kernel(const ViscVjpParams p) {
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= cs) return;
  const int q2 = (int)(i % p.n[2]);
  const int q1 = (int)((i / p.n[2]) % p.n[1]);
  const int q0 = (int)(i / ((long long)p.n[2] * p.n[1]));
  const int q[3] = {q0, q1, q2};
  auto cell = [&](int v, int kax, int ax2, int k2) {
    int g[3] = {q[0], q[1], q[2]};
    g[AX] += kax;
    g[ax2] += k2;
    return __ldg(p.prims + v * cs + wrap_off(p, g[0], g[1], g[2]));
  };
  const double odx = p.one_dx[AX];
  int gl[3] = {q0, q1, q2};
  gl[AX] -= 1;
  const long long offL = wrap_off(p, gl[0], gl[1], gl[2]);
  double dF[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) dF[v] = odx * (__ldg(p.w + v * cs + i) - __ldg(p.w + v * cs + offL));
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
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) gr[a][b] = 0.0;
#pragma unroll
      for (int a = 0; a < 3; ++a)
        gr[a][AX] = c4_face_deriv(odx, cell(1 + a, -2, AX, 0), cell(1 + a, -1, AX, 0), cell(1 + a, 0, AX, 0),
                                  cell(1 + a, 1, AX, 0));
#pragma unroll
      for (int ii = 0; ii < 3; ++ii) {
        if (ii == AX || !(p.active_mask & (1 << ii))) continue;
        const double odi = p.one_dx[ii];
#pragma unroll
        for (int which = 0; which < 2; ++which) {
          const int a = (which == 0) ? AX : ii;
          double d[4];
#pragma unroll
          for (int k = 0; k < 4; ++k)
            d[k] = c4_center_deriv(odi, cell(1 + a, k - 2, ii, -2), cell(1 + a, k - 2, ii, -1),
                                   cell(1 + a, k - 2, ii, 1), cell(1 + a, k - 2, ii, 2));
          gr[a][ii] = c4_face_interp(d[0], d[1], d[2], d[3]);
        }
      }
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
        const double vf = c4_face_interp(cell(1 + k, -2, AX, 0), cell(1 + k, -1, AX, 0), cell(1 + k, 0, AX, 0),
                                         cell(1 + k, 1, AX, 0));
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
  double* fc = p.fc + (long long)AX * VISC_SLOTS * cs;
#pragma unroll
  for (int k = 0; k < VISC_SLOTS; ++k) fc[k * cs + i] = out[k];
}

__global__ void __launch_bounds__(256) visc_cell_gather_kernel(const ViscVjpParams p) {
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= cs) return;
  const int c2 = (int)(i % p.n[2]);
  const int c1 = (int)((i / p.n[2]) % p.n[1]);
  const int c0 = (int)(i / ((long long)p.n[2] * p.n[1]));
  constexpr double fd[4] = {1.0 / 24.0, -27.0 / 24.0, 27.0 / 24.0, -1.0 / 24.0};
  constexpr double fi[4] = {-1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0};
  constexpr double cd[4] = {1.0 / 12.0, -8.0 / 12.0, 8.0 / 12.0, -1.0 / 12.0};  // offsets -2, -1, +1, +2
  constexpr int cj[4] = {-2, -1, 1, 2};
  double du[3] = {0.0, 0.0, 0.0}, dT = 0.0;
#pragma unroll
  for (int AX = 0; AX < 3; ++AX) {
    if (!(p.active_mask & (1 << AX))) continue;
    const double* fc = p.fc + (long long)AX * VISC_SLOTS * cs;
    const double odx = p.one_dx[AX];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      // this cell is stencil point k (offset k-2) of the face at q = c - (k-2) along AX
      int g[3] = {c0, c1, c2};
      g[AX] -= k - 2;
      const long long f = wrap_off(p, g[0], g[1], g[2]);
      const double wd = odx * fd[k];
#pragma unroll
      for (int a = 0; a < 3; ++a) du[a] += wd * fc[a * cs + f] + fi[k] * fc[(7 + a) * cs + f];
      dT += wd * fc[10 * cs + f];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int ii = (AX == 0) ? 1 + t : ((AX == 1) ? 2 * t : t);
        if (!(p.active_mask & (1 << ii))) continue;
        const double odi = p.one_dx[ii];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          int h[3] = {g[0], g[1], g[2]};
          h[ii] -= cj[jj];
          const long long ff = wrap_off(p, h[0], h[1], h[2]);
          const double wt = fi[k] * odi * cd[jj];
          du[AX] += wt * fc[(3 + 2 * t) * cs + ff];
          du[ii] += wt * fc[(4 + 2 * t) * cs + ff];
        }
      }
    }
  }
  const double rho = __ldg(p.prims + i);
  const double pr = __ldg(p.prims + 4 * cs + i);
  // T = p / (rho R)
  const double iden = 1.0 / (rho * p.R);
  p.dP[i] += -dT * pr * iden / rho;
  p.dP[cs + i] += du[0];
  p.dP[2 * cs + i] += du[1];
  p.dP[3 * cs + i] += du[2];
  p.dP[4 * cs + i] += dT * iden;
}

// out = (dP/dU)^T dP per cell, dP is cleared for the next use.
__global__ void dp_to_du_kernel(const double* U, double* dP, double* out, long long n, double gm1) {
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
  // every reconstruction but MINMOD (whose differentiable form is MINMOD-AD)
  if (c->recon == GBF_RECON_MINMOD) return GBF_ERR_UNSUPPORTED;
  if (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE && c->recon != GBF_RECON_WENO5Z) return GBF_ERR_UNSUPPORTED;
  // HLLC and HLL are reversed with Einfeldt wave speeds; Rusanov has its own
  if (c->riemann != GBF_RIEMANN_RUSANOV && c->signal_speed != GBF_SIGNAL_EINFELDT) return GBF_ERR_UNSUPPORTED;
  // the viscous reverse pass indexes faces periodically (one face per cell)
  if (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT))
    for (int f = 0; f < 6; ++f)
      if (c->n[f >> 1] > 1 && c->bc[f] != GBF_BC_PERIODIC) return GBF_ERR_UNSUPPORTED;
  return GBF_OK;
}

inline bool vjp_dissipative(const gbf_case* c) { return (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) != 0; }

// doubles of rhs-VJP scratch beyond the primitive cotangent: interior
// primitives and the viscous face cotangents of every active axis
long long vjp_extra_doubles(const gbf_case* c, const CaseInfo& ci) {
  if (!vjp_dissipative(c)) return 0;
  return 5 * ci.cells + 3LL * VISC_SLOTS * ci.cells;
}

// VJP of the rhs at state U (interior): out = J(U)^T w.  dP: zeroed scratch of 5 n doubles
// (left zeroed on return).
int launch_rhs_vjp(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, const double* U,
                   const double* w, double* out, double* dP, double* extra, cudaStream_t s) {
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
  smem = (size_t)(5 * pmax + 10 * R * fmax + (R == 3 ? 25 * threads : 0)) * sizeof(double);
  if (smem > 227 * 1024) return GBF_ERR_INVALID_ARGUMENT;
  vp.sp.cons = U;
  vp.w = w;
  vp.dP = dP;
  const int grid = vp.sp.tiles[0] * vp.sp.tiles[1] * vp.sp.tiles[2];
  if (c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE)
    st = launch_vjp_char(c->riemann, vp, grid, threads, smem, s);
  else if (c->recon == GBF_RECON_WENO5Z || c->recon == GBF_RECON_WENO5JS)
    st = launch_vjp_weno5(c->recon, c->riemann, vp, grid, threads, smem, s);
  else
    st = launch_vjp_short(c->recon, c->riemann, vp, grid, threads, smem, s);
  if (st != GBF_OK) return st;
  if (cudaGetLastError() != cudaSuccess) return GBF_ERR_CUDA;
  if (vjp_dissipative(c)) {
    ViscVjpParams q;
    for (int a = 0; a < 3; ++a) {
      q.n[a] = ci.n[a];
      q.one_dx[a] = vp.sp.one_dx[a];
    }
    q.active_mask = ci.active_mask;
    double* P = extra;
    q.prims = P;
    q.w = w;
    q.fc = P + 5 * ci.cells;
    q.dP = dP;
    q.mu1 = vp.sp.mu1;
    q.mu2 = vp.sp.mu2;
    q.kappa = vp.sp.kappa;
    q.R = vp.sp.R;
    q.viscous = vp.sp.viscous;
    q.heat = vp.sp.heat;
    q.heat_production = vp.sp.heat_production;
    if ((st = launch_convert(c, U, P, ci.cells, 1, s)) != GBF_OK) return st;
    const unsigned g = (unsigned)((ci.cells + 255) / 256);
    if (ci.active_mask & 1) visc_face_vjp_kernel<0><<<g, 256, 0, s>>>(q);
    if (ci.active_mask & 2) visc_face_vjp_kernel<1><<<g, 256, 0, s>>>(q);
    if (ci.active_mask & 4) visc_face_vjp_kernel<2><<<g, 256, 0, s>>>(q);
    visc_cell_gather_kernel<<<g, 256, 0, s>>>(q);
    if (cudaGetLastError() != cudaSuccess) return GBF_ERR_CUDA;
  }
  dp_to_du_kernel<<<grid_for(ci.cells), 256, 0, s>>>(U, dP, out, ci.cells, ci.fp.gm1);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

}  // namespace

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_vjp_workspace_bytes(const gbf_case* c) {
  CaseInfo ci;
  if (make_case_info(c, &ci) != GBF_OK) return 0;
  // step VJP: U1, U2, lam2, lam1, j, dP (6 interior states); dissipative
  // cases add the primitives and the viscous face cotangents
  return ((size_t)6 * 5 * (size_t)ci.cells + (size_t)vjp_extra_doubles(c, ci)) * sizeof(double);
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
    // recompute the stage states U1, U2 from U^n with the forward stage kernels
    SweepParams p;
    int threads;
    size_t smem;
    if ((st = make_sweep_params(c, ci, tile, &p, &threads, &smem)) != GBF_OK) return st;
    // the forward kernels read dt from dt_state[0]; dt points at a device scalar
    p.dt_state = const_cast<double*>(dt);
    p.reduce_dt = 0;
    const bool diss = vjp_dissipative(c);
    const int mode = diss ? MODE_STAGE_P : MODE_STAGE;
    p.prims = extra;  // dissipative stages read the stage primitives
    if (diss && (st = launch_convert(c, cons, extra, ci.cells, 1, s)) != GBF_OK) return st;
    p.stage = 0; p.cons = cons; p.cons0 = cons; p.out = U1;
    if ((st = launch_sweep(c, p, threads, smem, s, mode)) != GBF_OK) return st;
    if (diss && (st = launch_convert(c, U1, extra, ci.cells, 1, s)) != GBF_OK) return st;
    p.stage = 1; p.cons = U1; p.cons0 = cons; p.out = U2;
    if ((st = launch_sweep(c, p, threads, smem, s, mode)) != GBF_OK) return st;
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
