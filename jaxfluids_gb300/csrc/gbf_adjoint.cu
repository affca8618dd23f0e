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

#include "gbf_adjoint.cuh"
#include "gbf_kernels.cuh"

namespace gbf {

namespace {

struct VjpParams {
  SweepParams sp;       // state U (sp.cons), sizes, tile, scheme
  const double* w;      // cotangent of the rhs, interior [5][N]
  double* dP;           // primitive cotangent accumulator, interior [5][N]
};

template <int AX, int RECON, int RIEMANN>
__device__ __forceinline__ void vjp_axis(const VjpParams& vp, const int o[3], const int ext[3],
                                         double* sm_prim, double* sm_slot, double* sm_jr) {
  constexpr int R = ReconTraits<RECON>::R;
  constexpr int K = 2 * R;
  const SweepParams& p = vp.sp;
  const int tid = threadIdx.x;
  const int nthr = blockDim.x;
  int pe[3] = {ext[0], ext[1], ext[2]};
  pe[AX] += 2 * R;
  const int pvol = pe[0] * pe[1] * pe[2];
  stage_pencil<AX, R, MODE_STAGE>(p, o, pe, pvol, sm_prim);
  __syncthreads();

  int fe[3] = {ext[0], ext[1], ext[2]};
  fe[AX] += 1;
  const int fvol = fe[0] * fe[1] * fe[2];
  const int pstride = (AX == 0) ? pe[1] * pe[2] : ((AX == 1) ? pe[2] : 1);
  const long long cs = (long long)p.n[0] * p.n[1] * p.n[2];
  const double odx = p.one_dx[AX];
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
    if constexpr (RECON == GBF_RECON_WENO5Z) {
      // one pass gives the face states and the stencil gradients; the left
      // gradient waits in the face's slots 0..4, the right one in this
      // thread's private rows, until the Riemann cotangents are known
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double wv[K], jl[5], jr[5];
#pragma unroll
        for (int k = 0; k < K; ++k) wv[k] = sm_prim[v * pvol + base + k * pstride];
        weno5z_jac(wv[0], wv[1], wv[2], wv[3], wv[4], p.fp.stencil_eps, PL[v], jl);
        weno5z_jac(wv[5], wv[4], wv[3], wv[2], wv[1], p.fp.stencil_eps, PR[v], jr);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          sm_slot[(v * K + k) * fvol + f] = jl[k];
          sm_jr[(v * 5 + k) * nthr + tid] = jr[k];
        }
      }
      double dPL[5] = {0, 0, 0, 0, 0}, dPR[5] = {0, 0, 0, 0, 0};
      riemann_flux_vjp<AX, RIEMANN>(PL, PR, p.fp, dF, dPL, dPR);
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
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double wv[K];
#pragma unroll
        for (int k = 0; k < K; ++k) wv[k] = sm_prim[v * pvol + base + k * pstride];
        reconstruct_pair<RECON>(wv, p.fp.stencil_eps, PL[v], PR[v]);
      }
      double dPL[5] = {0, 0, 0, 0, 0}, dPR[5] = {0, 0, 0, 0, 0};
      riemann_flux_vjp<AX, RIEMANN>(PL, PR, p.fp, dF, dPL, dPR);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double wv[K], dw[K];
#pragma unroll
        for (int k = 0; k < K; ++k) wv[k] = sm_prim[v * pvol + base + k * pstride];
        reconstruct_pair_vjp<RECON>(wv, p.fp.stencil_eps, dPL[v], dPR[v], dw);
#pragma unroll
        for (int k = 0; k < K; ++k) sm_slot[(v * K + k) * fvol + f] = dw[k];
      }
    }
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
    bool flip;
    g[AX] = remap_bc(g[AX], p.n[AX], p.bc[2 * AX], p.bc[2 * AX + 1], flip);
    if (flip) d[AX + 1] = -d[AX + 1];
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
  // pencil primitives | per-thread right-stencil gradients (WENO only) | face slots
  double* sm_prim = smem;
  double* sm_jr = smem + 5 * pmax;
  double* sm_slot = sm_jr + ((RECON == GBF_RECON_WENO5Z) ? 25 * blockDim.x : 0);
  if (p.active_mask & 1) vjp_axis<0, RECON, RIEMANN>(vp, o, ext, sm_prim, sm_slot, sm_jr);
  if (p.active_mask & 2) vjp_axis<1, RECON, RIEMANN>(vp, o, ext, sm_prim, sm_slot, sm_jr);
  if (p.active_mask & 4) vjp_axis<2, RECON, RIEMANN>(vp, o, ext, sm_prim, sm_slot, sm_jr);
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
  if (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) return GBF_ERR_UNSUPPORTED;
  if (c->recon_var != GBF_RECVAR_PRIMITIVE) return GBF_ERR_UNSUPPORTED;
  if (c->recon != GBF_RECON_WENO5Z && c->recon != GBF_RECON_MINMOD_AD) return GBF_ERR_UNSUPPORTED;
  if (c->riemann == GBF_RIEMANN_HLLC && c->signal_speed != GBF_SIGNAL_EINFELDT) return GBF_ERR_UNSUPPORTED;
  return GBF_OK;
}

// VJP of the rhs at state U (interior): out = J(U)^T w.  dP: zeroed scratch of 5 n doubles
// (left zeroed on return).
int launch_rhs_vjp(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, const double* U,
                   const double* w, double* out, double* dP, cudaStream_t s) {
  VjpParams vp;
  int threads;
  size_t smem;
  int st = make_sweep_params(c, ci, tile, &vp.sp, &threads, &smem);
  if (st != GBF_OK) return st;
  const int R = (c->recon == GBF_RECON_WENO5Z) ? 3 : 2;
  // shared memory: pencil primitives + 2R x 5 slots per face (replaces the
  // flux slots) + 25 doubles per thread for WENO's right-stencil gradients
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
#define GBF_VJP(RC, RM)                                                                              \
  {                                                                                                  \
    auto k = rhs_vjp_kernel<RC, RM>;                                                                 \
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) \
      return GBF_ERR_CUDA;                                                                           \
    k<<<grid, threads, smem, s>>>(vp);                                                               \
  }
  const bool hllc = c->riemann == GBF_RIEMANN_HLLC;
  if (c->recon == GBF_RECON_WENO5Z) {
    if (hllc) GBF_VJP(GBF_RECON_WENO5Z, GBF_RIEMANN_HLLC) else GBF_VJP(GBF_RECON_WENO5Z, GBF_RIEMANN_RUSANOV)
  } else {
    if (hllc) GBF_VJP(GBF_RECON_MINMOD_AD, GBF_RIEMANN_HLLC) else GBF_VJP(GBF_RECON_MINMOD_AD, GBF_RIEMANN_RUSANOV)
  }
#undef GBF_VJP
  if (cudaGetLastError() != cudaSuccess) return GBF_ERR_CUDA;
  dp_to_du_kernel<<<grid_for(ci.cells), 256, 0, s>>>(U, dP, out, ci.cells, ci.fp.gm1);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

}  // namespace

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_vjp_workspace_bytes(const gbf_case* c) {
  CaseInfo ci;
  if (make_case_info(c, &ci) != GBF_OK) return 0;
  // step VJP: U1, U2, lam2, lam1, j, dP (6 interior states)
  return (size_t)6 * 5 * (size_t)ci.cells * sizeof(double);
}

extern "C" int gbf_rhs_vjp(const gbf_case* c, const double* cons, const double* w, double* out,
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
  return launch_rhs_vjp(c, ci, tile, cons, w, out, dP, s);
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
    p.stage = 0; p.cons = cons; p.cons0 = cons; p.out = U1;
    if ((st = launch_sweep(c, p, threads, smem, s, MODE_STAGE)) != GBF_OK) return st;
    p.stage = 1; p.cons = U1; p.cons0 = cons; p.out = U2;
    if ((st = launch_sweep(c, p, threads, smem, s, MODE_STAGE)) != GBF_OK) return st;
    S1 = U1;
    S2 = U2;
  }
  zero_kernel<<<grid_for(m), 256, 0, s>>>(dP, m);
  // stage 3: U3 = 1/3 Un + 2/3 U2 + 2/3 dt L(U2)
  if ((st = launch_rhs_vjp(c, ci, tile, S2, lam, j, dP, s)) != GBF_OK) return st;
  axpy_dt_kernel<<<grid_for(m), 256, 0, s>>>(lam2, lam, 2.0 / 3.0, j, 2.0 / 3.0, dt, m);
  // stage 2: U2 = 3/4 Un + 1/4 U1 + 1/4 dt L(U1)
  if ((st = launch_rhs_vjp(c, ci, tile, S1, lam2, j, dP, s)) != GBF_OK) return st;
  axpy_dt_kernel<<<grid_for(m), 256, 0, s>>>(lam1, lam2, 0.25, j, 0.25, dt, m);
  // stage 1: U1 = Un + dt L(Un)
  if ((st = launch_rhs_vjp(c, ci, tile, cons, lam1, j, dP, s)) != GBF_OK) return st;
  step_combine_kernel<<<grid_for(m), 256, 0, s>>>(lam_out, lam, lam2, lam1, j, dt, m);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

extern "C" int gbf_rk3_step_vjp(const gbf_case* c, const double* cons, const double* dt, const double* lam,
                                double* lam_out, void* workspace, const gbf_tile* tile, void* stream) {
  return step_vjp(c, cons, nullptr, nullptr, dt, lam, lam_out, workspace, tile, stream);
}

extern "C" int gbf_rk3_step_vjp_stages(const gbf_case* c, const double* cons, const double* u1,
                                       const double* u2, const double* dt, const double* lam, double* lam_out,
                                       void* workspace, const gbf_tile* tile, void* stream) {
  if (!u1 || !u2) return GBF_ERR_INVALID_ARGUMENT;
  return step_vjp(c, cons, u1, u2, dt, lam, lam_out, workspace, tile, stream);
}
