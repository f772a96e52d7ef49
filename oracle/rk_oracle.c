/*
 * CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restatement of the explicit embedded Runge-Kutta solvers of bacon-sci
 * 0.16.2: src/ivp/rk.rs (RungeKutta::solve :249-343, RungeKuttaSolver::step
 * :361-423, RKCoefficients45 :430-526, RK23Coefficients :563-621) driven the
 * way src/ivp.rs:214-238 (IVPIterator::next) drives them.
 *
 * Arithmetic is kept in the reference's operation order and without
 * contraction (compile with -ffp-contract=off): every `v += K_j * a` of
 * nalgebra is one rounded product followed by one rounded sum, zero
 * coefficients included.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>


/* ------------------------------------------------------------------------ */
/* Right-hand sides.  Formulas are written with explicit parentheses; the
 * CUDA engine evaluates the same expressions in the same order.            */
void oracle_rhs(int32_t rhs, int32_t dim, double t, const double* y,
                const double* p, const double* shared, double* f) {
  switch (rhs) {
    case ORC_RHS_EXP:
      for (int d = 0; d < dim; ++d) f[d] = y[d];
      break;
    case ORC_RHS_DECAY:
      for (int d = 0; d < dim; ++d) f[d] = -y[d];
      break;
    case ORC_RHS_QUADRATIC:
      for (int d = 0; d < dim; ++d) f[d] = -2.0 * t;
      break;
    case ORC_RHS_SINE:
      for (int d = 0; d < dim; ++d) f[d] = cos(t);
      break;
    case ORC_RHS_HARMONIC:
      f[0] = y[1];
      f[1] = -y[0];
      break;
    case ORC_RHS_VDP: {
      const double mu = p[0];
      f[0] = y[1];
      f[1] = ((mu * (1.0 - (y[0] * y[0]))) * y[1]) - y[0];
      break;
    }
    case ORC_RHS_LORENZ: {
      const double sigma = p[0], rho = p[1], beta = p[2];
      f[0] = sigma * (y[1] - y[0]);
      f[1] = (y[0] * (rho - y[2])) - y[1];
      f[2] = (y[0] * y[1]) - (beta * y[2]);
      break;
    }
    case ORC_RHS_LOTKA: {
      const double a = p[0], b = p[1], c = p[2], dd = p[3];
      f[0] = (a * y[0]) - ((b * y[0]) * y[1]);
      f[1] = ((c * y[0]) * y[1]) - (dd * y[1]);
      break;
    }
    case ORC_RHS_ROBERTSON: {
      const double k1 = p[0], k2 = p[1], k3 = p[2];
      const double r1 = k1 * y[0];
      const double r2 = (k2 * y[1]) * y[1];
      const double r3 = (k3 * y[1]) * y[2];
      f[0] = r3 - r1;
      f[1] = (r1 - r2) - r3;
      f[2] = r2;
      break;
    }
    case ORC_RHS_CHAIN: {
      /* n = dim/2 masses; y = (x_0..x_{n-1}, v_0..v_{n-1}).  p holds, per
       * spring i (0..n-1, spring i joins mass i-1 and mass i, mass -1 being
       * a wall): k_i at p[i]; damping c at p[n]; all masses 1. */
      const int n = dim / 2;
      const double c = p[n];
      for (int i = 0; i < n; ++i) f[i] = y[n + i];
      for (int i = 0; i < n; ++i) {
        const double xl = (i == 0) ? 0.0 : y[i - 1];
        const double xr = (i + 1 < n) ? y[i + 1] : 0.0;
        const double kl = p[i];
        const double kr = (i + 1 < n) ? p[i + 1] : 0.0;
        const double force = (kl * (xl - y[i])) + (kr * (xr - y[i]));
        f[n + i] = force - (c * y[n + i]);
      }
      break;
    }
    case ORC_RHS_LINEAR: {
      for (int r = 0; r < dim; ++r) {
        double acc = 0.0;
        for (int k = 0; k < dim; ++k) acc = acc + (shared[(size_t)r * dim + k] * y[k]);
        f[r] = acc;
      }
      break;
    }
    default:
      for (int d = 0; d < dim; ++d) f[d] = NAN;
  }
}

/* ------------------------------------------------------------------------ */
/* x^(1/4) as a fixed sequence of IEEE-754 operations (sqrt, mul, sub, fma),
 * so that the CPU and the GPU produce the same bits.  It starts from
 * sqrt(sqrt(x)) (within one ulp) and applies one ulp-step correction decided
 * by the residual x - r^4, which is evaluated in double-double.  The result
 * is the correctly rounded fourth root except in cases where the root lies
 * within ~2^-50 ulp of a rounding midpoint. */
static inline uint64_t orc_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double orc_from_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

static double qrt_fix(double x, double r) {
  const double p_hi = r * r;
  const double p_lo = fma(r, r, -p_hi);
  const double q_hi = p_hi * p_hi;
  double q_lo = fma(p_hi, p_hi, -q_hi);
  q_lo = fma(2.0 * p_hi, p_lo, q_lo);
  const double res = (x - q_hi) - q_lo;
  const uint64_t rb = orc_bits(r);
  const uint64_t e = (rb >> 52) & 0x7ffu;
  const double half_ulp = orc_from_bits((e - 53u) << 52);
  const double thr_up = (4.0 * half_ulp) * (p_hi * r);
  const double thr_dn = ((rb & 0x000fffffffffffffull) == 0) ? (0.5 * thr_up) : thr_up;
  if (res > thr_up) return orc_from_bits(rb + 1u);
  if (res < -thr_dn) return orc_from_bits(rb - 1u);
  return r;
}

double oracle_qrt(double x) {
  if (!(x > 0.0)) return (x == 0.0) ? 0.0 : NAN;
  if (x == INFINITY) return INFINITY;
  double s = 1.0;
  if (x > 0x1p400) { x = x * 0x1p-800; s = 0x1p200; }
  else if (x < 0x1p-400) { x = x * 0x1p800; s = 0x1p-200; }
  /* sqrt(sqrt(x)) is within one ulp of x^(1/4), so one correction suffices. */
  const double r = qrt_fix(x, sqrt(sqrt(x)));
  return r * s;
}

/* ------------------------------------------------------------------------ */
/* nalgebra 0.32 Matrix::norm = sqrt(norm_squared); norm_squared sums
 * dotc(col, col).  dotc special-cases static 2-, 3- and 4-vectors and
 * otherwise accumulates in eight lanes (blas.rs `dotx`). */
double oracle_norm(const double* x, int32_t n, int32_t dyn_dim) {
  double s;
  if (!dyn_dim && n == 2) {
    s = (x[0] * x[0]) + (x[1] * x[1]);
  } else if (!dyn_dim && n == 3) {
    s = ((x[0] * x[0]) + (x[1] * x[1])) + (x[2] * x[2]);
  } else if (!dyn_dim && n == 4) {
    double a = x[0] * x[0], b = x[1] * x[1];
    const double c = x[2] * x[2], d = x[3] * x[3];
    a = a + c;
    b = b + d;
    s = a + b;
  } else {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int i = 0;
    while (n - i >= 8) {
      for (int l = 0; l < 8; ++l) acc[l] = acc[l] + (x[i + l] * x[i + l]);
      i += 8;
    }
    double res = 0.0;
    res = res + (acc[0] + acc[4]);
    res = res + (acc[1] + acc[5]);
    res = res + (acc[2] + acc[6]);
    res = res + (acc[3] + acc[7]);
    for (int k = i; k < n; ++k) res = res + (x[k] * x[k]);
    s = 0.0 + res;
  }
  return sqrt(s);
}

/* ------------------------------------------------------------------------ */
/* Tableaux, built coefficient by coefficient the way the reference computes
 * them (src/ivp/rk.rs:435-525 and :568-620). */
#include "oracle_internal.h"

void orc_tableau_build(int method, int layout, orc_tableau* tb) {
  double a[ORC_MAX_STAGES][ORC_MAX_STAGES];
  memset(tb, 0, sizeof(*tb));
  memset(a, 0, sizeof(a));
  if (method == ORC_RK45) {
    tb->s = 6;
    const double c[6] = {0.0, 1.0 / 4.0, 3.0 / 8.0, 12.0 / 13.0, 1.0, 1.0 / 2.0};
    memcpy(tb->c, c, sizeof(c));
    a[1][0] = 1.0 / 4.0;
    a[2][0] = 3.0 / 32.0;
    a[2][1] = 9.0 / 32.0;
    a[3][0] = 1932.0 / 2197.0;
    a[3][1] = -7200.0 / 2197.0;
    a[3][2] = 7296.0 / 2197.0;
    a[4][0] = 439.0 / 216.0;
    a[4][1] = -8.0;
    a[4][2] = 3680.0 / 513.0;
    a[4][3] = -845.0 / 4104.0;
    a[5][0] = -8.0 / 27.0;
    a[5][1] = 2.0;
    a[5][2] = -3544.0 / 2565.0;
    /* The reference literal is 1859/4014 (rk.rs:499); Fehlberg's coefficient,
     * which makes row 5 sum to c_5 = 1/2, is 1859/4104. */
    a[5][3] = (layout == ORC_LAYOUT_FEHLBERG) ? (1859.0 / 4104.0) : (1859.0 / 4014.0);
    a[5][4] = -11.0 / 40.0;
    const double b[6] = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -(1.0 / 5.0), 0.0};
    const double e[6] = {1.0 / 360.0, 0.0, -128.0 / 4275.0, -2197.0 / 75240.0, 1.0 / 50.0, 2.0 / 55.0};
    memcpy(tb->b, b, sizeof(b));
    memcpy(tb->e, e, sizeof(e));
  } else {
    tb->s = 4;
    const double c[4] = {0.0, 1.0 / 2.0, 3.0 / 4.0, 1.0};
    memcpy(tb->c, c, sizeof(c));
    a[1][0] = 1.0 / 2.0;
    a[2][1] = 3.0 / 4.0;
    a[3][0] = 2.0 / 9.0;
    a[3][1] = 1.0 / 3.0;
    a[3][2] = 4.0 / 9.0;
    const double b[4] = {2.0 / 9.0, 1.0 / 3.0, 4.0 / 9.0, 0.0};
    const double e[4] = {-5.0 / 72.0, 1.0 / 12.0, 1.0 / 9.0, -(1.0 / 8.0)};
    memcpy(tb->b, b, sizeof(b));
    memcpy(tb->e, e, sizeof(e));
  }
  for (int i = 0; i < tb->s; ++i)
    for (int j = 0; j < tb->s; ++j)
      tb->m[i][j] = (layout == ORC_LAYOUT_AS_COMPILED) ? a[j][i] : a[i][j];
}

/* ------------------------------------------------------------------------ */


int32_t orc_rk_solve_core(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                          const double* p, const double* shared, double t0, double t_end,
                          const double* y0, double* y_out, double* t_out, int64_t* accepted,
                          int64_t* rejected, double* traj_t, double* traj_y, int64_t traj_cap,
                          double* dt_log, double* t_log, double* y_log, int64_t log_cap) {
  orc_tableau tb;
  orc_tableau_build(cfg->method, cfg->layout, &tb);
  const int s = tb.s;
  double y[ORC_MAX_DIM], scratch[ORC_MAX_DIM], f[ORC_MAX_DIM];
  double K[ORC_MAX_STAGES][ORC_MAX_DIM];
  memset(K, 0, sizeof(K)); /* half_steps start as zeros (rk.rs:323-327) */
  memcpy(y, y0, sizeof(double) * dim);

  const double tol = cfg->tol, dt_min = cfg->dt_min, dt_max = cfg->dt_max;
  const double one_tenth = 1.0 / 10.0, four = 4.0, one_fourth = 1.0 / 4.0;
  const double point_eighty_four = 100.0 / 100.0; /* rk.rs:266-268 */
  double t = t0, end = t_end;
  double dt = (dt_max + dt_min) * (1.0 / 2.0); /* rk.rs:315 */

  double last_t = t0;
  int64_t acc = 0, rej = 0, attempts = 0;
  int32_t status = ORC_OK;
  memcpy(y_out, y0, sizeof(double) * dim);
  if (t0 >= t_end) { /* with_ending_time / with_initial_time (rk.rs:212-234) */
    *t_out = t0;
    *accepted = 0;
    *rejected = 0;
    return ORC_TIME_END_OOB;
  }

  for (;;) {
    /* ---- RungeKuttaSolver::step (rk.rs:361-423) ---- */
    if (t >= end) { status = ORC_OK; break; }
    if (cfg->max_attempts > 0 && attempts >= cfg->max_attempts) {
      status = ORC_MAX_ATTEMPTS_EXCEEDED;
      break;
    }
    ++attempts;
    if (t + dt >= end) dt = end - t;

    for (int i = 0; i < s; ++i) {
      for (int d = 0; d < dim; ++d) scratch[d] = y[d];
      for (int j = 0; j < s; ++j)
        for (int d = 0; d < dim; ++d) scratch[d] = scratch[d] + (K[j][d] * tb.m[i][j]);
      const double step_time = t + (tb.c[i] * dt);
      oracle_rhs(rhs, dim, step_time, scratch, p, shared, f);
      for (int d = 0; d < dim; ++d) K[i][d] = f[d] * dt;
    }

    for (int d = 0; d < dim; ++d) scratch[d] = K[0][d] * tb.e[0];
    for (int j = 1; j < s; ++j)
      for (int d = 0; d < dim; ++d) scratch[d] = scratch[d] + (K[j][d] * tb.e[j]);
    const double error = oracle_norm(scratch, dim, cfg->dyn_dim) / dt;

    const int ok = (error <= tol);
    const double dt_used = dt, t_prev = t;
    double y_prev[ORC_MAX_DIM];
    if (dt_log) memcpy(y_prev, y, sizeof(double) * dim);
    if (ok) {
      t = t + dt;
      for (int j = 0; j < s; ++j)
        for (int d = 0; d < dim; ++d) y[d] = y[d] + (K[j][d] * tb.b[j]);
    }

    const double ratio = tol / error;
    const double root = (cfg->pow_mode == ORC_POW_LIBM) ? pow(ratio, one_fourth) : oracle_qrt(ratio);
    const double delta = point_eighty_four * root;
    if (delta <= one_tenth) dt = dt * one_tenth;
    else if (delta >= four) dt = dt * four;
    else dt = dt * delta;
    if (dt > dt_max) dt = dt_max;

    if (dt < dt_min && t < end) { status = ORC_MINIMUM_TIME_DELTA_EXCEEDED; break; }

    if (ok) {
      if (dt_log && acc < log_cap) {
        /* the step just accepted started at (t - dt_used, y_prev) */
        dt_log[acc] = dt_used;
        t_log[acc] = t_prev;
        memcpy(y_log + (size_t)acc * dim, y_prev, sizeof(double) * dim);
      }
      if (traj_t && acc < traj_cap) {
        traj_t[acc] = t;
        memcpy(traj_y + (size_t)acc * dim, y, sizeof(double) * dim);
      }
      ++acc;
      last_t = t;
      memcpy(y_out, y, sizeof(double) * dim);
    } else {
      ++rej;
    }
  }
  *t_out = last_t;
  *accepted = acc;
  *rejected = rej;
  return status;
}

int32_t oracle_rk_solve_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                            const double* p, const double* shared, double t0,
                            double t_end, const double* y0, double* y_out,
                            double* t_out, int64_t* accepted, int64_t* rejected,
                            double* traj_t, double* traj_y, int64_t traj_cap) {
  return orc_rk_solve_core(cfg, rhs, dim, p, shared, t0, t_end, y0, y_out, t_out, accepted,
                           rejected, traj_t, traj_y, traj_cap, NULL, NULL, NULL, 0);
}

/* ------------------------------------------------------------------------ */
typedef struct {
  const oracle_rk_cfg* cfg;
  int32_t rhs, dim, n_params;
  int64_t n;
  const double *y0, *params, *shared, *t0, *t_end;
  double *y_out, *t_out;
  int64_t *accepted, *rejected;
  int32_t* status;
  atomic_llong next;
} batch_job;

static void* batch_worker(void* arg) {
  batch_job* job = (batch_job*)arg;
  const int64_t chunk = 16;
  double yi[ORC_MAX_DIM], yo[ORC_MAX_DIM], pi[64];
  for (;;) {
    const int64_t start = atomic_fetch_add(&job->next, chunk);
    if (start >= job->n) break;
    const int64_t stop = (start + chunk < job->n) ? start + chunk : job->n;
    for (int64_t i = start; i < stop; ++i) {
      for (int d = 0; d < job->dim; ++d) yi[d] = job->y0[(size_t)d * job->n + i];
      for (int k = 0; k < job->n_params; ++k) pi[k] = job->params[(size_t)k * job->n + i];
      double to;
      int64_t a, r;
      const int32_t st = oracle_rk_solve_one(job->cfg, job->rhs, job->dim, pi, job->shared,
                                             job->t0[i], job->t_end[i], yi, yo, &to, &a, &r,
                                             NULL, NULL, 0);
      for (int d = 0; d < job->dim; ++d) job->y_out[(size_t)d * job->n + i] = yo[d];
      job->t_out[i] = to;
      job->accepted[i] = a;
      job->rejected[i] = r;
      job->status[i] = st;
    }
  }
  return NULL;
}

double oracle_rk_solve_batch(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                             int64_t n, int32_t n_params, const double* y0,
                             const double* params, const double* shared,
                             const double* t0, const double* t_end,
                             double* y_out, double* t_out, int64_t* accepted,
                             int64_t* rejected, int32_t* status,
                             int32_t threads) {
  batch_job job;
  job.cfg = cfg;
  job.rhs = rhs;
  job.dim = dim;
  job.n_params = n_params;
  job.n = n;
  job.y0 = y0;
  job.params = params;
  job.shared = shared;
  job.t0 = t0;
  job.t_end = t_end;
  job.y_out = y_out;
  job.t_out = t_out;
  job.accepted = accepted;
  job.rejected = rejected;
  job.status = status;
  atomic_init(&job.next, 0);
  if (threads < 1) threads = 1;
  if (threads > 1024) threads = 1024;
  struct timespec a, b;
  clock_gettime(CLOCK_MONOTONIC, &a);
  pthread_t tid[1024];
  for (int k = 1; k < threads; ++k) pthread_create(&tid[k], NULL, batch_worker, &job);
  batch_worker(&job);
  for (int k = 1; k < threads; ++k) pthread_join(tid[k], NULL);
  clock_gettime(CLOCK_MONOTONIC, &b);
  return (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
}

/* ------------------------------------------------------------------------ */
/* Analytic Jacobians J[r*dim + c] = d f_r / d y_c of the registry right-hand
 * sides, in a fixed evaluation order (the CUDA engine mirrors it). */
int oracle_rhs_jacobian(int32_t rhs, int32_t dim, double t, const double* y, const double* p,
                        const double* shared, double* J) {
  (void)t;
  for (int i = 0; i < dim * dim; ++i) J[i] = 0.0;
  switch (rhs) {
    case ORC_RHS_EXP:
      for (int d = 0; d < dim; ++d) J[d * dim + d] = 1.0;
      return 0;
    case ORC_RHS_DECAY:
      for (int d = 0; d < dim; ++d) J[d * dim + d] = -1.0;
      return 0;
    case ORC_RHS_QUADRATIC:
    case ORC_RHS_SINE:
      return 0;
    case ORC_RHS_HARMONIC:
      J[1] = 1.0;
      J[2] = -1.0;
      return 0;
    case ORC_RHS_VDP: {
      const double mu = p[0];
      J[1] = 1.0;
      J[2] = (((-2.0 * mu) * y[0]) * y[1]) - 1.0;
      J[3] = mu * (1.0 - (y[0] * y[0]));
      return 0;
    }
    case ORC_RHS_LORENZ:
      J[0] = -p[0];
      J[1] = p[0];
      J[3] = p[1] - y[2];
      J[4] = -1.0;
      J[5] = -y[0];
      J[6] = y[1];
      J[7] = y[0];
      J[8] = -p[2];
      return 0;
    case ORC_RHS_LOTKA:
      J[0] = p[0] - (p[1] * y[1]);
      J[1] = -(p[1] * y[0]);
      J[2] = p[2] * y[1];
      J[3] = (p[2] * y[0]) - p[3];
      return 0;
    case ORC_RHS_ROBERTSON: {
      const double k1 = p[0], k2 = p[1], k3 = p[2];
      J[0] = -k1;
      J[1] = k3 * y[2];
      J[2] = k3 * y[1];
      J[3] = k1;
      J[4] = ((-2.0 * k2) * y[1]) - (k3 * y[2]);
      J[5] = -(k3 * y[1]);
      J[7] = (2.0 * k2) * y[1];
      return 0;
    }
    case ORC_RHS_CHAIN: {
      const int n = dim / 2;
      const double c = p[n];
      for (int i = 0; i < n; ++i) {
        J[i * dim + n + i] = 1.0;
        const double kl = p[i];
        const double kr = (i + 1 < n) ? p[i + 1] : 0.0;
        J[(n + i) * dim + i] = -(kl + kr);
        if (i > 0) J[(n + i) * dim + i - 1] = kl;
        if (i + 1 < n) J[(n + i) * dim + i + 1] = kr;
        J[(n + i) * dim + n + i] = -c;
      }
      return 0;
    }
    case ORC_RHS_LINEAR:
      for (int i = 0; i < dim * dim; ++i) J[i] = shared[i];
      return 0;
    default:
      return -1;
  }
}
