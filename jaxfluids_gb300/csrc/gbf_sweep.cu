// Kernel parameters of a case (SweepParams) and its boundary constants and
// fields, shared by the face kernels, the batched stages and the adjoint.
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
    // defaults of the cell tiles (the adjoint's tile kernels; the face
    // kernels take their own face tiles, gbf_stage.cu): ~512-cell tiles,
    // longest along the contiguous (last active) axis.  15 x 32 (2-D) and
    // 7 x 8 x 8 (3-D) tiles have 495..512 faces per axis, two full rounds of
    // 256 threads instead of a third round on a quarter of the warps
    // (measured on GB300: 3-D adjoint -6 %).
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

}  // namespace gbf
