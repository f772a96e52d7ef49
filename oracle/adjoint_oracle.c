/*
 * CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Gradient oracles for the discrete adjoint.  The reference has no gradient
 * entry point; these functions differentiate its RK step map
 * (src/ivp/rk.rs:370-398: stages, then y += sum_j b_j K_j) along the
 * accepted-step sequence of a forward solve, with every step size frozen at
 * the value the forward solve used.
 *
 *   oracle_rk_adjoint_one    reverse sweep (the operation order the CUDA
 *                            adjoint kernel executes)
 *   oracle_rk_frozen_fd_one  central differences of the replayed step map
 *   oracle_rk_fwdsens_one    forward (tangent-linear) sensitivities
 *
 * Loss per system: L = sum_d (y_T[d] - target[d])^2.
 * Only the as_written / fehlberg readings define a one-step map; the
 * as_compiled reading feeds stage values across attempts and is rejected.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"
#include "oracle_internal.h"

#define ORC_MAX_P 16

/* ---- right-hand-side derivatives ---------------------------------------- */
/* ubar = J(y)^T v, and mu += (df/dp)(y)^T v: the adjoint's own arithmetic,
 * fused multiply-adds (C's fma, one rounding each) in the order the CUDA
 * reverse kernel executes (Vjp<> in bacon_gb300/csrc/rhs.cuh). */
static int rhs_vjp(int32_t rhs, int32_t dim, const double* y, const double* p, const double* v,
                   double* ubar, double* mu) {
  switch (rhs) {
    case ORC_RHS_EXP:
      for (int d = 0; d < dim; ++d) ubar[d] = v[d];
      return 0;
    case ORC_RHS_DECAY:
      for (int d = 0; d < dim; ++d) ubar[d] = -v[d];
      return 0;
    case ORC_RHS_HARMONIC:
      ubar[0] = -v[1];
      ubar[1] = v[0];
      return 0;
    case ORC_RHS_VDP: {
      const double m = p[0], y0 = y[0], y1 = y[1];
      const double w = fma(-y0, y0, 1.0);
      ubar[0] = fma((-2.0 * m) * y0, y1, -1.0) * v[1];
      ubar[1] = fma(m * w, v[1], v[0]);
      mu[0] = fma(w * y1, v[1], mu[0]);
      return 0;
    }
    case ORC_RHS_LORENZ: {
      const double s = p[0], r = p[1], b = p[2];
      ubar[0] = fma(y[1], v[2], fma(r - y[2], v[1], (-s) * v[0]));
      ubar[1] = fma(y[0], v[2], fma(s, v[0], -v[1]));
      ubar[2] = fma(-y[0], v[1], -(b * v[2]));
      mu[0] = fma(y[1] - y[0], v[0], mu[0]);
      mu[1] = fma(y[0], v[1], mu[1]);
      mu[2] = fma(-y[2], v[2], mu[2]);
      return 0;
    }
    case ORC_RHS_LOTKA: {
      const double a = p[0], b = p[1], c = p[2], dd = p[3];
      const double x = y[0], w = y[1];
      ubar[0] = fma(c * w, v[1], fma(-b, w, a) * v[0]);
      ubar[1] = fma(fma(c, x, -dd), v[1], (-(b * x)) * v[0]);
      const double xw = x * w;
      mu[0] = fma(x, v[0], mu[0]);
      mu[1] = fma(-xw, v[0], mu[1]);
      mu[2] = fma(xw, v[1], mu[2]);
      mu[3] = fma(-w, v[1], mu[3]);
      return 0;
    }
    default:
      return -1;
  }
}

/* du = J(y) dy + (df/dp)(y) dp (tangent-linear), any order. */
static int rhs_jvp(int32_t rhs, int32_t dim, const double* y, const double* p, const double* dy,
                   const double* dp, double* du) {
  switch (rhs) {
    case ORC_RHS_EXP:
      for (int d = 0; d < dim; ++d) du[d] = dy[d];
      return 0;
    case ORC_RHS_DECAY:
      for (int d = 0; d < dim; ++d) du[d] = -dy[d];
      return 0;
    case ORC_RHS_HARMONIC:
      du[0] = dy[1];
      du[1] = -dy[0];
      return 0;
    case ORC_RHS_VDP: {
      const double mu = p[0], y0 = y[0], y1 = y[1];
      du[0] = dy[1];
      du[1] = (-2.0 * mu * y0 * y1 - 1.0) * dy[0] + mu * (1.0 - y0 * y0) * dy[1] +
              (1.0 - y0 * y0) * y1 * dp[0];
      return 0;
    }
    case ORC_RHS_LORENZ: {
      const double s = p[0], r = p[1], b = p[2];
      du[0] = s * (dy[1] - dy[0]) + (y[1] - y[0]) * dp[0];
      du[1] = (r - y[2]) * dy[0] - y[0] * dy[2] - dy[1] + y[0] * dp[1];
      du[2] = y[1] * dy[0] + y[0] * dy[1] - b * dy[2] - y[2] * dp[2];
      return 0;
    }
    case ORC_RHS_LOTKA: {
      const double a = p[0], b = p[1], c = p[2], dd = p[3];
      const double x = y[0], w = y[1];
      du[0] = (a - b * w) * dy[0] - b * x * dy[1] + x * dp[0] - x * w * dp[1];
      du[1] = c * w * dy[0] + (c * x - dd) * dy[1] + x * w * dp[2] - w * dp[3];
      return 0;
    }
    default:
      return -1;
  }
}

/* ---- one step of the RK map with a frozen dt ----------------------------- */
/* Same operations as an accepted attempt of the forward solve, zero
 * coefficients skipped (they only matter for non-finite stage values).
 * fused = 1 contracts every "v += K * c" into one fused multiply-add, as the
 * CUDA reverse kernel's replay does.  Stage inputs are returned in Y[i][d]. */
static void step_map_x(const orc_tableau* tb, int32_t rhs, int32_t dim, const double* p, double t,
                       double dt, const double* y, double* y_next,
                       double Y[ORC_MAX_STAGES][ORC_MAX_DIM], double K[ORC_MAX_STAGES][ORC_MAX_DIM], int fused) {
  double f[ORC_MAX_DIM];
  for (int i = 0; i < tb->s; ++i) {
    for (int d = 0; d < dim; ++d) Y[i][d] = y[d];
    for (int j = 0; j < tb->s; ++j) {
      if (tb->m[i][j] == 0.0) continue;
      for (int d = 0; d < dim; ++d)
        Y[i][d] = fused ? fma(K[j][d], tb->m[i][j], Y[i][d]) : Y[i][d] + (K[j][d] * tb->m[i][j]);
    }
    const double st = t + (tb->c[i] * dt);
    oracle_rhs(rhs, dim, st, Y[i], p, NULL, f);
    for (int d = 0; d < dim; ++d) K[i][d] = f[d] * dt;
  }
  for (int d = 0; d < dim; ++d) y_next[d] = y[d];
  for (int j = 0; j < tb->s; ++j) {
    if (tb->b[j] == 0.0) continue;
    for (int d = 0; d < dim; ++d)
      y_next[d] = fused ? fma(K[j][d], tb->b[j], y_next[d]) : y_next[d] + (K[j][d] * tb->b[j]);
  }
}

static void step_map(const orc_tableau* tb, int32_t rhs, int32_t dim, const double* p, double t,
                     double dt, const double* y, double* y_next,
                     double Y[ORC_MAX_STAGES][ORC_MAX_DIM], double K[ORC_MAX_STAGES][ORC_MAX_DIM]) {
  step_map_x(tb, rhs, dim, p, t, dt, y, y_next, Y, K, 0);
}

static double loss_of(const double* y, const double* target, int32_t dim) {
  double L = 0.0;
  for (int d = 0; d < dim; ++d) {
    const double e = y[d] - target[d];
    L = L + (e * e);
  }
  return L;
}

typedef struct {
  int32_t status;
  int64_t n;
  double* dt;
  double* t;
  double* y;  /* [n][dim] start states */
  double yT[ORC_MAX_DIM];
} fwd_log;

static int32_t forward_logged(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim, const double* p,
                              double t0, double t_end, const double* y0, fwd_log* lg) {
  const int64_t cap = (cfg->max_attempts > 0) ? cfg->max_attempts : 10000000;
  const int64_t alloc = cap < 1000000 ? cap : 1000000;
  lg->dt = (double*)malloc(sizeof(double) * alloc);
  lg->t = (double*)malloc(sizeof(double) * alloc);
  lg->y = (double*)malloc(sizeof(double) * alloc * dim);
  double tout;
  int64_t acc, rej;
  lg->status = orc_rk_solve_core(cfg, rhs, dim, p, NULL, t0, t_end, y0, lg->yT, &tout, &acc, &rej,
                                 NULL, NULL, 0, lg->dt, lg->t, lg->y, alloc);
  lg->n = acc < alloc ? acc : alloc;
  if (acc > alloc) lg->status = ORC_MAX_ATTEMPTS_EXCEEDED;
  return lg->status;
}

static void fwd_free(fwd_log* lg) {
  free(lg->dt);
  free(lg->t);
  free(lg->y);
}

int32_t oracle_rk_adjoint_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                              int32_t n_params, const double* p, double t0,
                              double t_end, const double* y0,
                              const double* target, double* loss,
                              double* dl_dy0, double* dl_dp, int32_t checkpoint_every) {
  const int E = checkpoint_every > 0 ? checkpoint_every : 32;
  if (E > 32) return -1;
  if (cfg->layout == ORC_LAYOUT_AS_COMPILED || dim > ORC_MAX_DIM || n_params > ORC_MAX_P) return -1;
  orc_tableau tb;
  orc_tableau_build(cfg->method, cfg->layout, &tb);
  fwd_log lg;
  const int32_t st = forward_logged(cfg, rhs, dim, p, t0, t_end, y0, &lg);
  if (st != ORC_OK) {
    for (int d = 0; d < dim; ++d) dl_dy0[d] = NAN;
    for (int k = 0; k < n_params; ++k) dl_dp[k] = NAN;
    *loss = NAN;
    fwd_free(&lg);
    return st;
  }
  *loss = loss_of(lg.yT, target, dim);
  double lam[ORC_MAX_DIM], mu[ORC_MAX_P];
  for (int d = 0; d < dim; ++d) lam[d] = 2.0 * (lg.yT[d] - target[d]);
  for (int k = 0; k < n_params; ++k) mu[k] = 0.0;

  /* Segments of E accepted steps, last first: replay the segment from its
   * checkpoint (the forward pass's own state at the segment start) with the
   * fused step map, keeping every step's stage inputs, then sweep it in
   * reverse. */
  static __thread double Yseg[32][ORC_MAX_STAGES][ORC_MAX_DIM];
  double Y[ORC_MAX_STAGES][ORC_MAX_DIM], K[ORC_MAX_STAGES][ORC_MAX_DIM];
  double Kb[ORC_MAX_STAGES][ORC_MAX_DIM], yb[ORC_MAX_DIM], v[ORC_MAX_DIM], ub[ORC_MAX_DIM];
  double ycur[ORC_MAX_DIM], ynext[ORC_MAX_DIM];
  for (int64_t seg = (lg.n + E - 1) / E - 1; seg >= 0; --seg) {
    const int64_t k0 = seg * E;
    const int64_t m = (lg.n - k0) < E ? (lg.n - k0) : E;
    memcpy(ycur, lg.y + (size_t)k0 * dim, sizeof(double) * dim);
    double tcur = lg.t[k0];
    for (int64_t j = 0; j < m; ++j) {
      memset(K, 0, sizeof(K));
      step_map_x(&tb, rhs, dim, p, tcur, lg.dt[k0 + j], ycur, ynext, Yseg[j], K, 1);
      memcpy(ycur, ynext, sizeof(double) * dim);
      tcur = tcur + lg.dt[k0 + j];
    }
    for (int64_t j = m - 1; j >= 0; --j) {
    const int64_t n = k0 + j;
    const double dt = lg.dt[n];
    memcpy(Y, Yseg[j], sizeof(Y));
    for (int i = 0; i < tb.s; ++i)
      for (int d = 0; d < dim; ++d) Kb[i][d] = lam[d] * tb.b[i];
    for (int d = 0; d < dim; ++d) yb[d] = lam[d];
    for (int i = tb.s - 1; i >= 0; --i) {
      for (int d = 0; d < dim; ++d) v[d] = Kb[i][d] * dt;
      rhs_vjp(rhs, dim, Y[i], p, v, ub, mu);
      for (int d = 0; d < dim; ++d) yb[d] = yb[d] + ub[d];
      for (int j = 0; j < i; ++j) {
        if (tb.m[i][j] == 0.0) continue;
        for (int d = 0; d < dim; ++d) Kb[j][d] = fma(ub[d], tb.m[i][j], Kb[j][d]);
      }
    }
    for (int d = 0; d < dim; ++d) lam[d] = yb[d];
    }
  }
  for (int d = 0; d < dim; ++d) dl_dy0[d] = lam[d];
  for (int k = 0; k < n_params; ++k) dl_dp[k] = mu[k];
  fwd_free(&lg);
  return ORC_OK;
}

static double replay_loss(const orc_tableau* tb, const fwd_log* lg, int32_t rhs, int32_t dim,
                          const double* p, const double* y0, const double* target) {
  double y[ORC_MAX_DIM], yn[ORC_MAX_DIM];
  double Y[ORC_MAX_STAGES][ORC_MAX_DIM], K[ORC_MAX_STAGES][ORC_MAX_DIM];
  memcpy(y, y0, sizeof(double) * dim);
  memset(K, 0, sizeof(K));
  for (int64_t n = 0; n < lg->n; ++n) {
    step_map(tb, rhs, dim, p, lg->t[n], lg->dt[n], y, yn, Y, K);
    memcpy(y, yn, sizeof(double) * dim);
  }
  return loss_of(y, target, dim);
}

int32_t oracle_rk_frozen_fd_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                                int32_t n_params, const double* p, double t0,
                                double t_end, const double* y0,
                                const double* target, double h, double* dl_dy0,
                                double* dl_dp) {
  if (cfg->layout == ORC_LAYOUT_AS_COMPILED || dim > ORC_MAX_DIM || n_params > ORC_MAX_P) return -1;
  orc_tableau tb;
  orc_tableau_build(cfg->method, cfg->layout, &tb);
  fwd_log lg;
  const int32_t st = forward_logged(cfg, rhs, dim, p, t0, t_end, y0, &lg);
  if (st != ORC_OK) {
    fwd_free(&lg);
    return st;
  }
  double yp[ORC_MAX_DIM], pp[ORC_MAX_P];
  for (int d = 0; d < dim; ++d) {
    memcpy(yp, y0, sizeof(double) * dim);
    yp[d] = y0[d] + h;
    const double lp = replay_loss(&tb, &lg, rhs, dim, p, yp, target);
    yp[d] = y0[d] - h;
    const double lm = replay_loss(&tb, &lg, rhs, dim, p, yp, target);
    dl_dy0[d] = (lp - lm) / (2.0 * h);
  }
  for (int k = 0; k < n_params; ++k) {
    memcpy(pp, p, sizeof(double) * n_params);
    pp[k] = p[k] + h;
    const double lp = replay_loss(&tb, &lg, rhs, dim, pp, y0, target);
    pp[k] = p[k] - h;
    const double lm = replay_loss(&tb, &lg, rhs, dim, pp, y0, target);
    dl_dp[k] = (lp - lm) / (2.0 * h);
  }
  fwd_free(&lg);
  return ORC_OK;
}

int32_t oracle_rk_fwdsens_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                              int32_t n_params, const double* p, double t0,
                              double t_end, const double* y0,
                              const double* target, double* dl_dy0, double* dl_dp) {
  if (cfg->layout == ORC_LAYOUT_AS_COMPILED || dim > ORC_MAX_DIM || n_params > ORC_MAX_P) return -1;
  orc_tableau tb;
  orc_tableau_build(cfg->method, cfg->layout, &tb);
  fwd_log lg;
  const int32_t st = forward_logged(cfg, rhs, dim, p, t0, t_end, y0, &lg);
  if (st != ORC_OK) {
    fwd_free(&lg);
    return st;
  }
  const int nd = dim + n_params;
  double Y[ORC_MAX_STAGES][ORC_MAX_DIM], K[ORC_MAX_STAGES][ORC_MAX_DIM], yn[ORC_MAX_DIM];
  for (int k = 0; k < nd; ++k) {
    double y[ORC_MAX_DIM], dy[ORC_MAX_DIM], dp[ORC_MAX_P];
    memcpy(y, y0, sizeof(double) * dim);
    memset(dy, 0, sizeof(dy));
    memset(dp, 0, sizeof(dp));
    if (k < dim) dy[k] = 1.0;
    else dp[k - dim] = 1.0;
    memset(K, 0, sizeof(K));
    for (int64_t n = 0; n < lg.n; ++n) {
      const double dt = lg.dt[n];
      step_map(&tb, rhs, dim, p, lg.t[n], dt, y, yn, Y, K);
      double dK[ORC_MAX_STAGES][ORC_MAX_DIM], dY[ORC_MAX_DIM], du[ORC_MAX_DIM];
      for (int i = 0; i < tb.s; ++i) {
        for (int d = 0; d < dim; ++d) dY[d] = dy[d];
        for (int j = 0; j < i; ++j)
          for (int d = 0; d < dim; ++d) dY[d] += tb.m[i][j] * dK[j][d];
        rhs_jvp(rhs, dim, Y[i], p, dY, dp, du);
        for (int d = 0; d < dim; ++d) dK[i][d] = dt * du[d];
      }
      for (int i = 0; i < tb.s; ++i)
        for (int d = 0; d < dim; ++d) dy[d] += tb.b[i] * dK[i][d];
      memcpy(y, yn, sizeof(double) * dim);
    }
    double g = 0.0;
    for (int d = 0; d < dim; ++d) g += 2.0 * (lg.yT[d] - target[d]) * dy[d];
    if (k < dim) dl_dy0[k] = g;
    else dl_dp[k - dim] = g;
  }
  fwd_free(&lg);
  return ORC_OK;
}
