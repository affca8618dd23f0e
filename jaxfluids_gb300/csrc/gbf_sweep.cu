// Launch parameters of the sweep kernel and dispatch to the scheme families
// (gbf_sweep_<family>.cu instantiate the kernels).
#include <algorithm>

#include "gbf_sweep_launch.cuh"

namespace gbf {

namespace {

int radius_of(int recon) {
  return recon_radius(recon);
}

}  // namespace

// Per-face boundary constants of the kernels, rounded as the reference rounds
// them: WALL 2 u_wall (exact), DIRICHLET the primitives, NEUMANN
// (gradient * sign) * dx with sign +1 at the low and -1 at the high face
// (halos/outer/material.py:41-44, :860-861).
void fill_bc_constants(const gbf_case* c, int f, double out[5]) {
  const int ax = f >> 1;
  const double sign = (f & 1) ? -1.0 : 1.0;
  for (int v = 0; v < 5; ++v) {
    const double x = c->bc_value[f][v];
    switch (c->bc[f]) {
      case GBF_BC_WALL: out[v] = 2.0 * x; break;
      case GBF_BC_DIRICHLET: out[v] = x; break;
      case GBF_BC_NEUMANN: out[v] = (x * sign) * c->dx[ax]; break;
      default: out[v] = 0.0;
    }
  }
}

void fill_bc_fields(const gbf_case* c, BcFields* bf) {
  for (int f = 0; f < 6; ++f) {
    bf->val[f] = c->bc_field_values[f];
    bf->type[f] = reinterpret_cast<const signed char*>(c->bc_field_types[f]);
  }
}

int make_sweep_params(const gbf_case* c, const CaseInfo& ci, const gbf_tile* tile, SweepParams* p,
                      int* threads, size_t* smem, bool for_vjp) {
  SweepParams q{};
  int t[3];
  int thr = 256;
  const int dim = ((ci.active_mask & 1) ? 1 : 0) + ((ci.active_mask & 2) ? 1 : 0) +
                  ((ci.active_mask & 4) ? 1 : 0);
  const bool user = tile && (tile->t[0] > 0 || tile->t[1] > 0 || tile->t[2] > 0);
  if (user) {
    for (int a = 0; a < 3; ++a) t[a] = std::max(1, tile->t[a]);
    if (tile->threads > 0) thr = tile->threads;
  } else {
    // defaults: ~512-cell tiles, longest along the contiguous (last active)
    // axis.  A face sweep runs one face per thread; 15 x 32 (2-D) and
    // 7 x 8 x 8 (3-D) tiles have 495..512 faces per axis, two full rounds of
    // 256 threads instead of a third round on a quarter of the warps (measured
    // on GB300: 2-D forward -9 %, 3-D viscous CHAR forward -4 %, 3-D adjoint
    // -6 %).  The inviscid 3-D forward, two CTAs per SM, is flat across shapes
    // and keeps 8 x 8 x 8.
    for (int a = 0; a < 3; ++a) t[a] = 1;
    if (dim == 1) {
      for (int a = 0; a < 3; ++a)
        if (ci.active_mask & (1 << a)) t[a] = 256;
    } else if (dim == 2) {
      int ax[2], k = 0;
      for (int a = 0; a < 3; ++a)
        if (ci.active_mask & (1 << a)) ax[k++] = a;
      t[ax[0]] = 15;
      t[ax[1]] = 32;
      if (for_vjp) {
        // the adjoint kernel runs one CTA per SM (registers): of shapes with
        // the same two rounds of faces per axis, take the one whose tile
        // count fills its last wave of 152 CTAs best (KH 512^2: 16 x 27, 608
        // tiles = 4 full waves, 7 % faster than 15 x 32's 560)
        static const int cand[3][2] = {{15, 32}, {16, 27}, {14, 32}};
        double best = -1.0;
        for (const auto& cd : cand) {
          const long long tiles = (long long)((ci.n[ax[0]] + cd[0] - 1) / cd[0]) * ((ci.n[ax[1]] + cd[1] - 1) / cd[1]);
          const long long waves = (tiles + kSms - 1) / kSms;
          const double fill = (double)tiles / (double)(waves * kSms);
          if (fill > best + 1e-9) {
            best = fill;
            t[ax[0]] = cd[0];
            t[ax[1]] = cd[1];
          }
        }
      }
    } else {
      const bool heavy = for_vjp || (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) ||
                         c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE;
      t[0] = heavy ? 7 : 8;
      t[1] = 8;
      t[2] = 8;
    }
  }
  for (int a = 0; a < 3; ++a) {
    if (ci.n[a] == 1) t[a] = 1;
    t[a] = std::min(t[a], ci.n[a]);
  }
  if (thr % 32 != 0 || thr < 32 || thr > 256) return GBF_ERR_INVALID_ARGUMENT;
  const long long tvol = (long long)t[0] * t[1] * t[2];
  if (tvol > (long long)kSweepMaxCellsPerThread * thr) return GBF_ERR_INVALID_ARGUMENT;
  const int R = radius_of(c->recon);
  long long pmax = 0, fmax = 0;
  for (int a = 0; a < 3; ++a) {
    if (!(ci.active_mask & (1 << a))) continue;
    long long pv = 1, fv = 1;
    for (int b = 0; b < 3; ++b) {
      pv *= t[b] + (b == a ? 2 * R : 0);
      fv *= t[b] + (b == a ? 1 : 0);
    }
    pmax = std::max(pmax, pv);
    fmax = std::max(fmax, fv);
  }
  const bool cons_pencil =
      c->recon_var == GBF_RECVAR_CONSERVATIVE || c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE;
  const size_t bytes = (size_t)((cons_pencil ? 2 : 1) * pmax + fmax) * 5 * sizeof(double);
  if (bytes > 227 * 1024) return GBF_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; ++a) {
    q.n[a] = ci.n[a];
    q.t[a] = t[a];
    q.tiles[a] = (ci.n[a] + t[a] - 1) / t[a];
    q.hs[a] = ci.hs[a];
    q.one_dx[a] = 1.0 / c->dx[a];
  }
  q.nh = ci.nh;
  for (int f = 0; f < 6; ++f) {
    q.bc[f] = c->bc[f];
    fill_bc_constants(c, f, q.bcv[f]);
  }
  fill_bc_fields(c, &q.bf);
  for (int a = 0; a < 3; ++a) q.dx[a] = c->dx[a];
  q.fp = ci.fp;
  q.active_mask = ci.active_mask;
  q.viscous = (c->flags & GBF_FLAG_VISCOUS) ? 1 : 0;
  q.heat = (c->flags & GBF_FLAG_HEAT) ? 1 : 0;
  q.heat_production = (c->flags & GBF_FLAG_VISCOUS_HEAT_PRODUCTION) ? 1 : 0;
  q.mu1 = c->mu;
  q.mu2 = c->bulk_mu - 2.0 / 3.0 * c->mu;  // compute_tau: bulk - 2/3 mu
  q.kappa = c->kappa;
  q.R = c->R;
  q.diss_recon = c->dissipative_stencil[0];
  q.diss_center = c->dissipative_stencil[1];
  q.diss_face = c->dissipative_stencil[2];
  q.limiter = (c->flags & GBF_FLAG_INTERPOLATION_LIMITER) ? ((c->flags & GBF_FLAG_LIMIT_VELOCITY) ? 2 : 1) : 0;
  q.gravity = (c->flags & GBF_FLAG_GRAVITY) ? 1 : 0;
  for (int a = 0; a < 3; ++a) q.g[a] = q.gravity ? c->gravity[a] : 0.0;
  *p = q;
  *threads = thr;
  *smem = bytes;
  return GBF_OK;
}

namespace {

// Lax-Friedrichs dissipation speeds (bits of three non-negative doubles), one
// array per device; its address is looked up once per device, before any
// graph capture (the first launch of a case).
__device__ unsigned long long g_lf_alpha[3];
constexpr int kLfMaxDevices = 64;
double* g_lf_alpha_ptr[kLfMaxDevices] = {};

}  // namespace

int lf_alpha_on_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GBF_ERR_CUDA;
  if (dev < 0 || dev >= kLfMaxDevices) return GBF_ERR_UNSUPPORTED;
  if (!g_lf_alpha_ptr[dev]) {
    void* a = nullptr;
    if (cudaGetSymbolAddress(&a, g_lf_alpha) != cudaSuccess || !a) return GBF_ERR_CUDA;
    g_lf_alpha_ptr[dev] = static_cast<double*>(a);
  }
  *out = g_lf_alpha_ptr[dev];
  return GBF_OK;
}

namespace {

int launch_sweep_schemes(const gbf_case* c, const SweepParams& p, int threads, size_t smem, cudaStream_t s,
                         int mode);

}  // namespace

// Lax-Friedrichs (LaxFriedrichs.py:25-47) runs the Rusanov instantiation twice:
// a pass reducing the axis' max |u| + c over the face states (into lf_ws, or
// the per-device slots), then the flux pass with that speed.
int launch_sweep(const gbf_case* c, const SweepParams& p, int threads, size_t smem, cudaStream_t s, int mode,
                 double* lf_ws) {
  if (c->riemann != GBF_RIEMANN_LAXFRIEDRICHS || (c->flags & GBF_FLAG_NO_CONVECTIVE))
    return launch_sweep_schemes(c, p, threads, smem, s, mode);
  double* alpha = lf_ws;
  int st = GBF_OK;
  if (!alpha && (st = lf_alpha_on_current_device(&alpha)) != GBF_OK) return st;
  if (cudaMemsetAsync(alpha, 0, 3 * sizeof(double), s) != cudaSuccess) return GBF_ERR_CUDA;
  SweepParams q = p;
  q.lf_alpha = alpha;
  q.speed_pass = 1;
  q.reduce_dt = 0;
  if ((st = launch_sweep_schemes(c, q, threads, smem, s, mode)) != GBF_OK) return st;
  q.speed_pass = 0;
  q.reduce_dt = p.reduce_dt;
  return launch_sweep_schemes(c, q, threads, smem, s, mode);
}

namespace {

int launch_sweep_schemes(const gbf_case* c, const SweepParams& p, int threads, size_t smem, cudaStream_t s,
                         int mode) {
  const bool visc = (c->flags & (GBF_FLAG_VISCOUS | GBF_FLAG_HEAT)) != 0;
  const bool chr = c->recon_var == GBF_RECVAR_CHAR_PRIMITIVE;
  const bool cons = c->recon_var == GBF_RECVAR_CONSERVATIVE || c->recon_var == GBF_RECVAR_CHAR_CONSERVATIVE;
  if (cons && !(c->flags & GBF_FLAG_NO_CONVECTIVE)) {
    if (visc && mode == MODE_STAGE) return GBF_ERR_UNSUPPORTED;
    if (!visc && mode == MODE_STAGE_P) return GBF_ERR_UNSUPPORTED;
    if (mode == MODE_RHS && !p.cons_halo) return GBF_ERR_INVALID_ARGUMENT;  // needs the conservatives
    return (c->recon_var == GBF_RECVAR_CONSERVATIVE)
               ? launch_sweep_cons(visc, c->riemann, mode, p, threads, smem, s)
               : launch_sweep_charcons(visc, c->riemann, mode, p, threads, smem, s);
  }
  if (visc) {
    // dissipative fluxes read the primitive buffer (MODE_STAGE_P) or the halo buffer
    if (mode == MODE_STAGE) return GBF_ERR_UNSUPPORTED;
    if (c->flags & GBF_FLAG_NO_CONVECTIVE) return launch_sweep_dissipative(mode, p, threads, smem, s);
    const bool c4 = c->dissipative_stencil[0] == GBF_CENTRAL4 && c->dissipative_stencil[1] == GBF_CENTRAL4 &&
                    c->dissipative_stencil[2] == GBF_CENTRAL4;
    if (chr)
      return c4 ? launch_sweep_char_visc_c4(c->riemann, mode, p, threads, smem, s)
                : launch_sweep_char_visc(c->riemann, mode, p, threads, smem, s);
    if (c->recon == GBF_RECON_WENO5Z)
      return c4 ? launch_sweep_weno_visc_c4(c->riemann, mode, p, threads, smem, s)
                : launch_sweep_weno_visc(c->riemann, mode, p, threads, smem, s);
    if (c->recon == GBF_RECON_WENO5JS) return launch_sweep_weno5js_visc(c->riemann, mode, p, threads, smem, s);
    if (c->recon == GBF_RECON_TENO5) return launch_sweep_teno5_visc(c->riemann, mode, p, threads, smem, s);
    return launch_sweep_short_visc(c->recon, c->riemann, mode, p, threads, smem, s);
  }
  if (mode == MODE_STAGE_P) return GBF_ERR_UNSUPPORTED;
  if (chr) return launch_sweep_char(c->riemann, mode, p, threads, smem, s);
  if (c->recon == GBF_RECON_WENO5Z) return launch_sweep_weno(c->riemann, mode, p, threads, smem, s);
  if (c->recon == GBF_RECON_MINMOD || c->recon == GBF_RECON_MINMOD_AD)
    return launch_sweep_muscl(c->recon, c->riemann, mode, p, threads, smem, s);
  return launch_sweep_weno_family(c->recon, c->riemann, mode, p, threads, smem, s);
}

}  // namespace

}  // namespace gbf
