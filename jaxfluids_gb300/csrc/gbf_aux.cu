// Auxiliary kernels of the drop-in path: halo fill, primitive/conservative
// conversion, RK stage integration and the CFL time-step reduction.
#include <math.h>

#include "gbf_kernels.cuh"

namespace gbf {

namespace {

constexpr int kThreads = 256;

inline int grid_for(long long n, int threads = kThreads) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > (1LL << 30)) g = (1LL << 30);
  return (int)g;
}

struct HaloParams {
  int n[3];
  int hs[3];
  int nh;
  int bc[6];
  int active_mask;
  long long face_count[6];  // halo cells per face (0 for inactive axes)
  long long face_start[6];
  long long total;
  double gm1;
  double bcv[6][5];  // per-face boundary constants (fill_bc_constants)
  BcFields bf;       // boundary values varying along a face
  double dx[3];
};

// halos/outer/material.py:94-287 (face halos) with the retrieve slices of
// halos/outer/boundary_condition.py:539-604 and fill slices of
// halos/halo_slices.py:46-75.  One thread per halo cell of every active face.
__global__ void halo_fill_kernel(const HaloParams hp, double* prims, double* cons) {
  const long long cs = (long long)hp.hs[0] * hp.hs[1] * hp.hs[2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < hp.total;
       i += (long long)gridDim.x * blockDim.x) {
    int face = 0;
#pragma unroll
    for (int f = 1; f < 6; ++f)
      if (i >= hp.face_start[f] && hp.face_count[f] > 0) face = f;
    const long long j = i - hp.face_start[face];
    const int ax = face >> 1;
    const bool hi = face & 1;
    const int oa = (ax == 0) ? 1 : 0;          // first other axis
    const int ob = (ax == 2) ? 1 : 2;          // second other axis
    const int eb = hp.n[ob];
    const int ea = hp.n[oa];
    const int ib = (int)(j % eb);
    const int ia = (int)((j / eb) % ea);
    const int layer = (int)(j / ((long long)eb * ea));  // 0..nh-1, buffer order
    int dst[3], src[3];
    dst[oa] = (hp.n[oa] > 1) ? ia + hp.nh : 0;
    dst[ob] = (hp.n[ob] > 1) ? ib + hp.nh : 0;
    src[oa] = dst[oa];
    src[ob] = dst[ob];
    const int n = hp.n[ax];
    const int nh = hp.nh;
    const long long k = (long long)ia * eb + ib;  // boundary cell along the face
    const int bct = face_type_at(hp.bc, hp.bf, face, k);
    // logical halo coordinate of this layer and the interior cell it reads
    const int g = hi ? n + layer : layer - nh;
    dst[ax] = g + nh;
    src[ax] = bc_src(g, n, bct) + nh;
    const long long so = ((long long)src[0] * hp.hs[1] + src[1]) * hp.hs[2] + src[2];
    const long long d = ((long long)dst[0] * hp.hs[1] + dst[1]) * hp.hs[2] + dst[2];
    double P[5];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      P[v] = bc_apply_at(bct, hp.bcv[face], hp.bf, face, k, (long long)ea * eb, hp.dx[ax], ax, v, prims[v * cs + so]);
#pragma unroll
    for (int v = 0; v < 5; ++v) prims[v * cs + d] = P[v];
    if (cons) {
      double U[5];
      cons_from_prims(P, U, hp.gm1);
#pragma unroll
      for (int v = 0; v < 5; ++v) cons[v * cs + d] = U[v];
    }
  }
}

// Edge halos (outer/material.py:289-379) of the halo buffer, after its face
// halos: one thread per buffer cell outside the interior along exactly two
// active axes a < b.  Type combination of boundary_condition.py:128-177 and
// retrieve locations :606-660: the first of the two faces (axis order) that is
// PERIODIC or SYMMETRY takes the other face's halo cell at its periodic image
// or mirror (that axis' velocity negated); otherwise (ANY_ANY) the mean of the
// two face-halo cells nh cells inward ('_10' then '_01' slices,
// halo_slices.py:77-149); a face of several types counts as neither.  Halo
// conservatives from the halo primitives.
__global__ void halo_edge_kernel(const HaloParams hp, double* prims, double* cons) {
  const long long cs = (long long)hp.hs[0] * hp.hs[1] * hp.hs[2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cs;
       i += (long long)gridDim.x * blockDim.x) {
    int b[3] = {(int)(i / ((long long)hp.hs[1] * hp.hs[2])), (int)((i / hp.hs[2]) % hp.hs[1]),
                (int)(i % hp.hs[2])};
    int out[3], k = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if (hp.n[a] > 1 && (b[a] < hp.nh || b[a] >= hp.n[a] + hp.nh)) out[k++] = a;
    if (k != 2) continue;
    const int a0 = out[0], a1 = out[1];
    auto lo = [&](int a) { return b[a] < hp.nh; };
    const int t0 = hp.bc[2 * a0 + (lo(a0) ? 0 : 1)];
    const int t1 = hp.bc[2 * a1 + (lo(a1) ? 0 : 1)];
    auto at = [&](const int q[3]) { return ((long long)q[0] * hp.hs[1] + q[1]) * hp.hs[2] + q[2]; };
    double P[5];
    if (t0 == GBF_BC_PERIODIC || t0 == GBF_BC_SYMMETRY || t1 == GBF_BC_PERIODIC || t1 == GBF_BC_SYMMETRY) {
      const bool first = (t0 == GBF_BC_PERIODIC || t0 == GBF_BC_SYMMETRY);
      const int a = first ? a0 : a1;
      const int t = first ? t0 : t1;
      int q[3] = {b[0], b[1], b[2]};
      q[a] = bc_src(b[a] - hp.nh, hp.n[a], t) + hp.nh;
      const long long so = at(q);
#pragma unroll
      for (int v = 0; v < 5; ++v) P[v] = prims[v * cs + so];
      if (t == GBF_BC_SYMMETRY) P[a + 1] = -P[a + 1];
    } else {
      int qa[3] = {b[0], b[1], b[2]}, qb[3] = {b[0], b[1], b[2]};
      qa[a0] += lo(a0) ? hp.nh : -hp.nh;
      qb[a1] += lo(a1) ? hp.nh : -hp.nh;
      const long long sa = at(qa), sb = at(qb);
#pragma unroll
      for (int v = 0; v < 5; ++v) P[v] = 0.5 * (prims[v * cs + sa] + prims[v * cs + sb]);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) prims[v * cs + i] = P[v];
    if (cons) {
      double U[5];
      cons_from_prims(P, U, hp.gm1);
#pragma unroll
      for (int v = 0; v < 5; ++v) cons[v * cs + i] = U[v];
    }
  }
}

__global__ void convert_kernel(const double* in, double* out, long long count, double gm1,
                               int to_prims) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    double a[5], b[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) a[v] = in[v * count + i];
    if (to_prims)
      prims_from_cons(a, b, gm1);
    else
      cons_from_prims(a, b, gm1);
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * count + i] = b[v];
  }
}

struct StageParams {
  int n[3];
  int hs[3];
  int nh;
  long long total;
  int stage;
};

// time_integrator.py:34-58, :108-226 and RK3.py:31-62 on a halo buffer.
__global__ void stage_integrate_kernel(const StageParams sp, double* cons, const double* cons0,
                                       const double* rhs, const double* dtp) {
  const double dt = *dtp;
  const long long cs = sp.total;
  const long long rs = (long long)sp.n[0] * sp.n[1] * sp.n[2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cs;
       i += (long long)gridDim.x * blockDim.x) {
    const int b2 = (int)(i % sp.hs[2]);
    const int b1 = (int)((i / sp.hs[2]) % sp.hs[1]);
    const int b0 = (int)(i / ((long long)sp.hs[2] * sp.hs[1]));
    int c[3] = {b0, b1, b2};
    bool interior = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (sp.n[a] > 1) {
        c[a] -= sp.nh;
        interior = interior && c[a] >= 0 && c[a] < sp.n[a];
      }
    }
    const long long ro = ((long long)c[0] * sp.n[1] + c[1]) * sp.n[2] + c[2];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double U = cons[v * cs + i];
      if (sp.stage == 1) U = __dadd_rn(__dmul_rn(0.25, U), __dmul_rn(0.75, cons0[v * cs + i]));
      if (sp.stage == 2)
        U = __dadd_rn(__dmul_rn(2.0 / 3.0, U), __dmul_rn(1.0 / 3.0, cons0[v * cs + i]));
      if (interior) {
        const double m = (sp.stage == 0) ? 1.0 : ((sp.stage == 1) ? 0.25 : 2.0 / 3.0);
        U = __dadd_rn(U, __dmul_rn(__dmul_rn(dt, m), rhs[v * rs + ro]));
      }
      cons[v * cs + i] = U;
    }
  }
}

__global__ void set_scalar_kernel(double* dst, double v) { *dst = v; }

__global__ void reduce_init_kernel(unsigned long long* red) {
  red[0] = 0ull;                                   // bits of +0.0
  red[1] = (unsigned long long)0x7ff0000000000000ull;  // bits of +inf
}

__device__ __forceinline__ void block_reduce_store(double smax, double rmin, unsigned long long* red) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, d));
    rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, d));
  }
  __shared__ double r[2][32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    r[0][w] = smax;
    r[1][w] = rmin;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    smax = (threadIdx.x < nw) ? r[0][threadIdx.x] : 0.0;
    rmin = (threadIdx.x < nw) ? r[1][threadIdx.x] : __longlong_as_double(0x7ff0000000000000LL);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, d));
      rmin = fmin(rmin, __shfl_xor_sync(0xffffffffu, rmin, d));
    }
    if (threadIdx.x == 0) {
      atomicMax(red, (unsigned long long)__double_as_longlong(smax));
      atomicMin(red + 1, (unsigned long long)__double_as_longlong(rmin));
    }
  }
}

struct ReduceParams {
  int n[3];
  int hs[3];
  int nh;
  int active_mask;
  long long cells;
  double gamma;
  double gm1;
  int from_cons;  // 1: interior conservative buffer, 0: halo primitive buffer, 2: interior primitives
};

// time_step_size.py:96-109: max over interior cells of sum_active(|u_i| + c);
// also the minimum density (for the viscous and heat-conduction limits).
__global__ void reduce_kernel(const ReduceParams rp, const double* buf, unsigned long long* red) {
  double smax = 0.0;
  double rmin = __longlong_as_double(0x7ff0000000000000LL);
  const long long hcs = (long long)rp.hs[0] * rp.hs[1] * rp.hs[2];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rp.cells;
       i += (long long)gridDim.x * blockDim.x) {
    double P[5];
    if (rp.from_cons == 2) {
#pragma unroll
      for (int v = 0; v < 5; ++v) P[v] = buf[v * rp.cells + i];
    } else if (rp.from_cons) {
      double U[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) U[v] = buf[v * rp.cells + i];
      prims_from_cons(U, P, rp.gm1);
    } else {
      const int c2 = (int)(i % rp.n[2]);
      const int c1 = (int)((i / rp.n[2]) % rp.n[1]);
      const int c0 = (int)(i / ((long long)rp.n[2] * rp.n[1]));
      const int b0 = (rp.n[0] > 1) ? c0 + rp.nh : 0;
      const int b1 = (rp.n[1] > 1) ? c1 + rp.nh : 0;
      const int b2 = (rp.n[2] > 1) ? c2 + rp.nh : 0;
      const long long o = ((long long)b0 * rp.hs[1] + b1) * rp.hs[2] + b2;
#pragma unroll
      for (int v = 0; v < 5; ++v) P[v] = buf[v * hcs + o];
    }
    const double c = sqrt(rp.gamma * P[4] / P[0]);
    double s = 0.0;
    if (rp.active_mask & 1) s = s + (fabs(P[1]) + c);
    if (rp.active_mask & 2) s = s + (fabs(P[2]) + c);
    if (rp.active_mask & 4) s = s + (fabs(P[3]) + c);
    smax = fmax(smax, s);
    rmin = fmin(rmin, P[0]);
  }
  block_reduce_store(smax, rmin, red);
}

struct DtParams {
  double min_dx;
  double eps;
  double cfl;
  double fixed_dt;
  double mu;
  double kappa;
  double cp;
  int viscous;
  int heat;
  int advance_time;
};

// time_step_size.py:97-155
__global__ void dt_finalize_kernel(const DtParams dp, unsigned long long* red, double* dt_out,
                                   double* t_inout) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (dp.advance_time && t_inout) *t_inout = *t_inout + *dt_out;
  double dt;
  if (dp.fixed_dt > 0.0) {
    dt = dp.fixed_dt;
  } else {
    const double smax = __longlong_as_double((long long)red[0]);
    const double rmin = __longlong_as_double((long long)red[1]);
    dt = dp.min_dx / (smax + dp.eps);
    const double mdx2 = dp.min_dx * dp.min_dx;
    if (dp.viscous) {
      // max(mu / rho) == mu / min(rho): correctly rounded division is monotone
      const double dtv = (3.0 / 14.0) * mdx2 / (dp.mu / rmin + dp.eps);
      dt = fmin(dt, dtv);
    }
    if (dp.heat) {
      // max(kappa / (rho cp)) == kappa / (min(rho) cp)
      const double dth = 0.1 * mdx2 / (dp.kappa / (rmin * dp.cp) + dp.eps);
      dt = fmin(dt, dth);
    }
    dt = dt * dp.cfl;
  }
  *dt_out = dt;
  red[0] = 0ull;
  red[1] = (unsigned long long)0x7ff0000000000000ull;
}

}  // namespace

namespace {

// Gravity forces of the drop-in right-hand side: one thread per interior
// cell, conservatives read from the halo buffer.
__global__ void volume_force_kernel(const double* cons, double* rhs, int n0, int n1, int n2, int hs1, int hs2,
                                    int h0, int h1, int h2, long long hcs, double g0, double g1, double g2) {
  const long long cs = (long long)n0 * n1 * n2;
  const double g[3] = {g0, g1, g2};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cs;
       i += (long long)gridDim.x * blockDim.x) {
    const int i2 = (int)(i % n2), i1 = (int)((i / n2) % n1), i0 = (int)(i / ((long long)n2 * n1));
    const long long hoff = ((long long)(i0 + h0) * hs1 + (i1 + h1)) * hs2 + (i2 + h2);
    double U[5], r[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      U[v] = cons[v * hcs + hoff];
      r[v] = rhs[v * cs + i];
    }
    add_gravity(r, U, g);
#pragma unroll
    for (int v = 1; v < 5; ++v) rhs[v * cs + i] = r[v];
  }
}

}  // namespace

int launch_volume_force(const gbf_case* c, const CaseInfo& ci, const double* cons, double* rhs, cudaStream_t s) {
  int h[3];
  for (int a = 0; a < 3; ++a) h[a] = (ci.n[a] > 1) ? ci.nh : 0;
  const long long hcs = (long long)ci.hs[0] * ci.hs[1] * ci.hs[2];
  volume_force_kernel<<<grid_for(ci.cells), kThreads, 0, s>>>(cons, rhs, ci.n[0], ci.n[1], ci.n[2], ci.hs[1],
                                                               ci.hs[2], h[0], h[1], h[2], hcs, c->gravity[0],
                                                               c->gravity[1], c->gravity[2]);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_halo_fill(const gbf_case* c, const CaseInfo& ci, double* prims, double* cons,
                     cudaStream_t s) {
  HaloParams hp;
  for (int a = 0; a < 3; ++a) {
    hp.n[a] = ci.n[a];
    hp.hs[a] = ci.hs[a];
  }
  hp.nh = ci.nh;
  for (int f = 0; f < 6; ++f) {
    hp.bc[f] = c->bc[f];
    fill_bc_constants(c, f, hp.bcv[f]);
  }
  fill_bc_fields(c, &hp.bf);
  for (int a = 0; a < 3; ++a) hp.dx[a] = c->dx[a];
  hp.active_mask = ci.active_mask;
  hp.gm1 = ci.fp.gm1;
  long long start = 0;
  for (int f = 0; f < 6; ++f) {
    const int ax = f >> 1;
    long long cnt = 0;
    if (ci.active_mask & (1 << ax)) {
      cnt = ci.nh;
      for (int a = 0; a < 3; ++a)
        if (a != ax) cnt *= ci.n[a];
    }
    hp.face_start[f] = start;
    hp.face_count[f] = cnt;
    start += cnt;
  }
  hp.total = start;
  if (hp.total == 0) return GBF_OK;
  halo_fill_kernel<<<grid_for(hp.total), kThreads, 0, s>>>(hp, prims, cons);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_halo_edges(const gbf_case* c, const CaseInfo& ci, double* prims, double* cons,
                      cudaStream_t s) {
  HaloParams hp{};
  for (int a = 0; a < 3; ++a) {
    hp.n[a] = ci.n[a];
    hp.hs[a] = ci.hs[a];
  }
  hp.nh = ci.nh;
  for (int f = 0; f < 6; ++f) hp.bc[f] = c->bc[f];
  hp.gm1 = ci.fp.gm1;
  halo_edge_kernel<<<grid_for(ci.halo_cells), kThreads, 0, s>>>(hp, prims, cons);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_convert(const gbf_case* c, const double* in, double* out, long long count, int to_prims,
                   cudaStream_t s) {
  if (count <= 0) return GBF_OK;
  const double gm1 = c->gamma - 1.0;
  convert_kernel<<<grid_for(count), kThreads, 0, s>>>(in, out, count, gm1, to_prims);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_stage_integrate(const gbf_case* c, const CaseInfo& ci, double* cons,
                           const double* cons0, const double* rhs, const double* dt, int stage,
                           cudaStream_t s) {
  StageParams sp;
  for (int a = 0; a < 3; ++a) {
    sp.n[a] = ci.n[a];
    sp.hs[a] = ci.hs[a];
  }
  sp.nh = ci.nh;
  sp.total = ci.halo_cells;
  sp.stage = stage;
  stage_integrate_kernel<<<grid_for(sp.total), kThreads, 0, s>>>(sp, cons, cons0, rhs, dt);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_set_scalar(double* dst, double v, cudaStream_t s) {
  set_scalar_kernel<<<1, 1, 0, s>>>(dst, v);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_reduce_init(unsigned long long* red, cudaStream_t s) {
  reduce_init_kernel<<<1, 1, 0, s>>>(red);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

static int launch_reduce(const CaseInfo& ci, const double* buf, unsigned long long* red, int from_cons,
                         cudaStream_t s) {
  ReduceParams rp;
  for (int a = 0; a < 3; ++a) {
    rp.n[a] = ci.n[a];
    rp.hs[a] = ci.hs[a];
  }
  rp.nh = ci.nh;
  rp.active_mask = ci.active_mask;
  rp.cells = ci.cells;
  rp.gamma = ci.fp.gamma;
  rp.gm1 = ci.fp.gm1;
  rp.from_cons = from_cons;
  int grid = grid_for(ci.cells);
  if (grid > 152 * 8) grid = 152 * 8;
  reduce_kernel<<<grid, kThreads, 0, s>>>(rp, buf, red);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_reduce_halo_prims(const CaseInfo& ci, const double* prims, unsigned long long* red,
                             cudaStream_t s) {
  return launch_reduce(ci, prims, red, 0, s);
}

// Numerical health of an interior conservative state: cells with a
// non-finite conservative, with rho <= 0, and with p <= 0 (p from the ideal-gas
// EOS, equation_manager.py:164-171), counted into counts[0..2] (accumulated).
__global__ void state_check_kernel(const double* cons, long long n, double gm1, unsigned long long* counts) {
  unsigned long long bad = 0, neg_rho = 0, neg_p = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double U[5], P[5];
    bool finite = true;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      U[v] = cons[v * n + i];
      finite &= isfinite(U[v]);
    }
    prims_from_cons(U, P, gm1);
    bad += finite ? 0 : 1;
    neg_rho += (U[0] <= 0.0) ? 1 : 0;
    neg_p += (P[4] <= 0.0) ? 1 : 0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    bad += __shfl_down_sync(0xffffffffu, bad, o);
    neg_rho += __shfl_down_sync(0xffffffffu, neg_rho, o);
    neg_p += __shfl_down_sync(0xffffffffu, neg_p, o);
  }
  if ((threadIdx.x & 31) == 0 && (bad | neg_rho | neg_p)) {
    atomicAdd(counts + 0, bad);
    atomicAdd(counts + 1, neg_rho);
    atomicAdd(counts + 2, neg_p);
  }
}

int launch_state_check(const CaseInfo& ci, const double* cons, unsigned long long* counts, cudaStream_t s) {
  state_check_kernel<<<grid_for(ci.cells), kThreads, 0, s>>>(cons, ci.cells, ci.fp.gm1, counts);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

int launch_reduce_cons(const CaseInfo& ci, const double* cons, unsigned long long* red,
                       cudaStream_t s) {
  return launch_reduce(ci, cons, red, 1, s);
}

int launch_reduce_prims(const CaseInfo& ci, const double* prims, unsigned long long* red, cudaStream_t s) {
  return launch_reduce(ci, prims, red, 2, s);
}

int launch_dt_finalize(const gbf_case* c, const CaseInfo& ci, unsigned long long* red,
                       double* dt_out, double* t_inout, int advance_time, cudaStream_t s) {
  DtParams dp;
  dp.min_dx = ci.min_dx;
  dp.eps = c->eps;
  dp.cfl = c->cfl;
  dp.fixed_dt = c->fixed_dt;
  dp.mu = c->mu;
  // thermal diffusivity kappa / (rho cp), cp = gamma / (gamma - 1) R (ideal_gas.py:32)
  dp.cp = c->gamma / (c->gamma - 1.0) * c->R;
  dp.kappa = c->kappa;
  dp.viscous = (c->flags & GBF_FLAG_VISCOUS) ? 1 : 0;
  dp.heat = (c->flags & GBF_FLAG_HEAT) ? 1 : 0;
  dp.advance_time = advance_time;
  dt_finalize_kernel<<<1, 32, 0, s>>>(dp, red, dt_out, t_inout);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

}  // namespace gbf
