/* CPU restatement (test infrastructure only) of the reference's Adams
 * predictor-corrector solvers and of its Euler solver:
 *
 *   AdamsSolver::runge_kutta   src/ivp/adams.rs:344-395  (RK4 bootstrap)
 *   AdamsSolver::step          src/ivp/adams.rs:411-565  (PECE, yield machine)
 *   AdamsCoefficients5 / 3     src/ivp/adams.rs:572-603, :636-659
 *   Adams::solve               src/ivp/adams.rs:252-334  (dt0 = (max+min)/2)
 *   EulerSolver::step          src/ivp.rs:318-339        (yields the state
 *                                                         before each step)
 *   IVPIterator::next          src/ivp.rs:214-238
 *
 * Every vector operation is written out per component in nalgebra's order
 * (`a + b * c` is a rounded product then a rounded sum; the RK4 combination
 * is ((k1 + 2 k2) + 2 k3) + k4, then times 1/6).  The step factor
 * (tol / (2 err))^(1/O) is libm pow in the reference; ORC_POW_QRT selects the
 * engine's deterministic root (oracle_rootn), ORC_POW_LIBM pow itself.
 * Outputs follow the RK restatement: y_out / t_out = the last yielded item,
 * accepted = items yielded, rejected = step() calls that returned Redo. */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "oracle.h"
#include "oracle_internal.h"

static inline uint64_t ad_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double ad_from_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

/* One ulp-step correction of r ~ (z (1 + adj/z))^(1/n), z in [1, 2^n), r in
 * [1, 2): the residual z + adj - r^n in double-double against n r^(n-1)
 * times half an ulp (the first-order distance to the rounding midpoints), as
 * oracle_qrt does for n = 4. */
static double rootn_fix(double z, double r, int n, double adj) {
  const double r2 = r * r;
  const double r2lo = fma(r, r, -r2);
  double hi, lo, deriv;
  if (n == 3) {
    hi = r2 * r;
    lo = fma(r2lo, r, fma(r2, r, -hi));
    deriv = 3.0 * r2;
  } else {
    const double r4 = r2 * r2;
    const double r4lo = fma(2.0 * r2, r2lo, fma(r2, r2, -r4));
    hi = r4 * r;
    lo = fma(r4lo, r, fma(r4, r, -hi));
    deriv = 5.0 * r4;
  }
  const double res = ((z - hi) - lo) + adj;
  const uint64_t rb = ad_bits(r);
  const uint64_t e = (rb >> 52) & 0x7ffu;
  const double half_ulp = ad_from_bits((e - 53u) << 52);
  const double thr_up = half_ulp * deriv;
  const double thr_dn = ((rb & 0x000fffffffffffffull) == 0) ? (0.5 * thr_up) : thr_up;
  if (res > thr_up) return ad_from_bits(rb + 1u);
  if (res < -thr_dn) return ad_from_bits(rb - 1u);
  return r;
}

/* x^RN(1/n) for n = 3 or 5 -- what the reference's x.powf(n.recip())
 * computes: the exponent is the rounded 1/n, 1/n + delta with
 * delta = +2^-54/5 (n = 5) or -2^-54/3 (n = 3), so the value is the true
 * root times x^delta = 1 + delta ln x.  A fixed sequence of IEEE-754
 * operations (the GPU runs the same one): exponent split x = 2^(nq) z with
 * z in [1, 2^n), a log-linear first guess from the bit pattern, five Newton
 * steps and an ulp-step correction give the true root; ln x from the
 * exponent and a short atanh series (relative error < 1e-5, ample for a term
 * c = delta ln x below 2e-14) moves it by the factor 1 + c, and a second
 * ulp-step correction, on the residual of the radicand z (1 + n c), rounds
 * the result.  Correctly rounded except within ~2^-50 ulp of a midpoint;
 * 0 -> 0, inf -> inf, negative or NaN -> NaN (as pow). */
double oracle_rootn(double x, int n) {
  if (!(x > 0.0)) return (x == 0.0) ? 0.0 : NAN;
  if (x == INFINITY) return INFINITY;
  double s = 1.0;
  int shift = 0;  /* x was multiplied by 2^shift */
  if (x < 0x1p-1000) {  /* subnormal range: scale by 2^(n m) first */
    x = x * (n == 3 ? 0x1p900 : 0x1p1000);
    s = (n == 3) ? 0x1p-300 : 0x1p-200;
    shift = (n == 3) ? 900 : 1000;
  }
  const uint64_t b = ad_bits(x);
  const int e = (int)(b >> 52) - 1023;
  int q = e / n, rem = e % n;
  if (rem < 0) {
    rem += n;
    q -= 1;
  }
  const double z = ad_from_bits((b & 0x000fffffffffffffull) | ((uint64_t)(1023 + rem) << 52));
  double y = ad_from_bits(0x3ff0000000000000ull + (ad_bits(z) - 0x3ff0000000000000ull) / (uint64_t)n);
  for (int it = 0; it < 5; ++it) {
    double ym1 = y;
    for (int k = 2; k < n; ++k) ym1 = ym1 * y;
    const double yn = ym1 * y;
    y = y - (yn - z) / ((double)n * ym1);
  }
  y = rootn_fix(z, y, n, 0.0);
  /* ln x = (e - shift) ln 2 + ln m, m = the mantissa in [1, 2):
   * ln m = 2 atanh(u), u = (m - 1) / (m + 1) in [0, 1/3] */
  const double m = ad_from_bits((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  const double u = (m - 1.0) / (m + 1.0);
  const double u2 = u * u;
  const double lnm = (2.0 * u) * (1.0 + (u2 * ((1.0 / 3.0) + (u2 * ((1.0 / 5.0) + (u2 * (1.0 / 7.0)))))));
  const double lnx = ((double)(e - shift) * 0.6931471805599453) + lnm;
  const double delta = (n == 3) ? -0x1p-54 / 3.0 : 0x1p-54 / 5.0;
  const double c = delta * lnx;
  /* the target is the root of z (1 + n c): move to within an ulp of it, then
   * decide the last ulp with the residual of that radicand */
  y = fma(y, c, y);
  y = rootn_fix(z, y, n, z * ((double)n * c));
  return (y * ad_from_bits((uint64_t)(1023 + q) << 52)) * s;
}

/* ------------------------------------------------------------------------ */
enum { AD_ITEM, AD_REDO, AD_DONE, AD_FAIL };
#define AD_MAXO 5

typedef struct {
  int O, dim, rhs, dyn;
  const double *p, *shared;
  double dt_max, dt_min, time, end, tol, dt;
  double state[ORC_MAX_DIM], save[ORC_MAX_DIM];
  double pc[AD_MAXO], cc[AD_MAXO], ec;
  double one_tenth, one_sixth, half, two, four, order;
  /* deques: prev_values (t, y) and prev_derivatives, front at index 0 */
  double pv_t[AD_MAXO + 1], pv_y[AD_MAXO + 1][ORC_MAX_DIM];
  int npv;
  double pd[AD_MAXO + 1][ORC_MAX_DIM];
  int npd;
  int yield_memory;
  int pow_mode;
} ad_state;

static void pv_pop_front(ad_state* s);
static void pd_pop_front(ad_state* s);

/* The deques hold O + 1 entries: the PECE step reads at most O - 1, and
 * repeated end-clamped RK4 steps (t + (end - t) rounding below end) only
 * need back() and non-emptiness, so a push onto a full deque drops its
 * front (the GPU kernel keeps the same bound). */
static void pv_push(ad_state* s, double t, const double* y) {
  if (s->npv == s->O + 1) pv_pop_front(s);
  s->pv_t[s->npv] = t;
  memcpy(s->pv_y[s->npv], y, sizeof(double) * s->dim);
  s->npv++;
}
static void pv_pop_front(ad_state* s) {
  for (int i = 1; i < s->npv; ++i) {
    s->pv_t[i - 1] = s->pv_t[i];
    memcpy(s->pv_y[i - 1], s->pv_y[i], sizeof(double) * s->dim);
  }
  s->npv--;
}
static void pd_push(ad_state* s, const double* f) {
  if (s->npd == s->O + 1) pd_pop_front(s);
  memcpy(s->pd[s->npd], f, sizeof(double) * s->dim);
  s->npd++;
}
static void pd_pop_front(ad_state* s) {
  for (int i = 1; i < s->npd; ++i) memcpy(s->pd[i - 1], s->pd[i], sizeof(double) * s->dim);
  s->npd--;
}

static void ad_f(const ad_state* s, double t, const double* y, double* f) {
  oracle_rhs(s->rhs, s->dim, t, y, s->p, s->shared, f);
}

/* AdamsSolver::runge_kutta (src/ivp/adams.rs:344-395) */
static void ad_runge_kutta(ad_state* s, int iterations) {
  const int D = s->dim;
  double k1[ORC_MAX_DIM], k2[ORC_MAX_DIM], k3[ORC_MAX_DIM], k4[ORC_MAX_DIM], it[ORC_MAX_DIM], f[ORC_MAX_DIM];
  for (int i = 0; i < iterations; ++i) {
    ad_f(s, s->time, s->state, f);
    for (int d = 0; d < D; ++d) k1[d] = f[d] * s->dt;
    for (int d = 0; d < D; ++d) it[d] = s->state[d] + (k1[d] * s->half);
    ad_f(s, s->time + (s->half * s->dt), it, f);
    for (int d = 0; d < D; ++d) k2[d] = f[d] * s->dt;
    for (int d = 0; d < D; ++d) it[d] = s->state[d] + (k2[d] * s->half);
    ad_f(s, s->time + (s->half * s->dt), it, f);
    for (int d = 0; d < D; ++d) k3[d] = f[d] * s->dt;
    for (int d = 0; d < D; ++d) it[d] = s->state[d] + k3[d];
    ad_f(s, s->time + s->dt, it, f);
    for (int d = 0; d < D; ++d) k4[d] = f[d] * s->dt;
    if (i != 0) {
      ad_f(s, s->time, s->state, f);
      pd_push(s, f);
      pv_push(s, s->time, s->state);
    }
    for (int d = 0; d < D; ++d) {
      const double comb = ((k1[d] + (k2[d] * s->two)) + (k3[d] * s->two)) + k4[d];
      s->state[d] = s->state[d] + (comb * s->one_sixth);
    }
    s->time = s->time + s->dt;
  }
  ad_f(s, s->time, s->state, f);
  pd_push(s, f);
  pv_push(s, s->time, s->state);
}

static double ad_root(const ad_state* s, double x) {
  return (s->pow_mode == ORC_POW_LIBM) ? pow(x, 1.0 / s->order) : oracle_rootn(x, s->O);
}

/* AdamsSolver::step (src/ivp/adams.rs:411-565).  Returns AD_ITEM with the
 * item in (*it, iy), AD_REDO, AD_DONE or AD_FAIL (*fail = code). */
static int ad_step(ad_state* s, double* it, double* iy, int* fail) {
  const int O = s->O, D = s->dim;
  if (s->yield_memory > 0 && s->yield_memory < O) {
    const int get_item = O - s->yield_memory - 1;
    s->yield_memory -= 1;
    if (s->yield_memory == 0) s->yield_memory = O + 1;
    *it = s->pv_t[get_item];
    memcpy(iy, s->pv_y[get_item], sizeof(double) * D);
    return AD_ITEM;
  }
  if (s->yield_memory == O + 1) {
    s->yield_memory = 0;
    pv_push(s, s->time, s->state);
    pv_pop_front(s);
    *it = s->time;
    memcpy(iy, s->state, sizeof(double) * D);
    return AD_ITEM;
  }
  if (s->time >= s->end) return AD_DONE;
  if (s->time + s->dt >= s->end) {
    s->dt = s->end - s->time;
    ad_runge_kutta(s, 1);
    *it = s->time;
    memcpy(iy, s->pv_y[s->npv - 1], sizeof(double) * D);
    return AD_ITEM;
  }
  if (s->npv == 0) {
    memcpy(s->save, s->state, sizeof(double) * D);
    if (s->time + (s->dt * (s->order - 1.0)) >= s->end) s->dt = (s->end - s->time) / (s->order - 1.0);
    ad_runge_kutta(s, O - 1);
    s->yield_memory = O;
    return AD_REDO;
  }
  double scratch[ORC_MAX_DIM], pred[ORC_MAX_DIM], corr[ORC_MAX_DIM], impl[ORC_MAX_DIM], diff[ORC_MAX_DIM];
  for (int d = 0; d < D; ++d) scratch[d] = s->pd[0][d] * s->pc[O - 2];
  for (int i = 1; i < O - 1; ++i) {
    const double c = s->pc[O - i - 2];
    for (int d = 0; d < D; ++d) scratch[d] = scratch[d] + (s->pd[i][d] * c);
  }
  for (int d = 0; d < D; ++d) pred[d] = s->state[d] + (scratch[d] * s->dt);
  ad_f(s, s->time + s->dt, pred, impl);
  for (int d = 0; d < D; ++d) scratch[d] = impl[d] * s->cc[0];
  for (int i = 0; i < O - 1; ++i) {
    const double c = s->cc[O - i - 1];
    for (int d = 0; d < D; ++d) scratch[d] = scratch[d] + (s->pd[i][d] * c);
  }
  for (int d = 0; d < D; ++d) corr[d] = s->state[d] + (scratch[d] * s->dt);
  for (int d = 0; d < D; ++d) diff[d] = corr[d] - pred[d];
  const double error = (s->ec / s->dt) * oracle_norm(diff, D, s->dyn);
  if (error <= s->tol) {
    memcpy(s->state, corr, sizeof(double) * D);
    s->time = s->time + s->dt;
    if (s->yield_memory == O) {
      s->yield_memory -= 1;
      return AD_REDO;
    }
    pd_push(s, impl);
    pv_push(s, s->time, s->state);
    pv_pop_front(s);
    pd_pop_front(s);
    if (error < (s->one_tenth * s->tol)) {
      const double q = ad_root(s, s->tol / (s->two * error));
      if (q > s->four) s->dt = s->dt * s->four;
      else s->dt = s->dt * q;
      if (s->dt > s->dt_max) s->dt = s->dt_max;
      s->npv = 0;
      s->npd = 0;
    }
    *it = s->time;
    memcpy(iy, s->state, sizeof(double) * D);
    return AD_ITEM;
  }
  if (s->yield_memory == O) {
    s->time = s->time - (s->dt * (s->order - 1.0));
    memcpy(s->state, s->save, sizeof(double) * D);
  }
  const double q = ad_root(s, s->tol / (s->two * error));
  if (q < s->one_tenth) s->dt = s->dt * s->one_tenth;
  else s->dt = s->dt * q;
  if (s->dt < s->dt_min) {
    *fail = ORC_MINIMUM_TIME_DELTA_EXCEEDED;
    return AD_FAIL;
  }
  s->npv = 0;
  s->npd = 0;
  return AD_REDO;
}

int32_t oracle_adams_solve_one(const oracle_adams_cfg* cfg, int32_t rhs, int32_t dim, const double* p,
                               const double* shared, double t0, double t_end, const double* y0,
                               double* y_out, double* t_out, int64_t* accepted, int64_t* rejected,
                               double* traj_t, double* traj_y, int64_t traj_cap) {
  static __thread ad_state s;
  if (dim < 1 || dim > ORC_MAX_DIM || (cfg->order != 3 && cfg->order != 5)) return ORC_MAX_ATTEMPTS_EXCEEDED + 2;
  memset(&s, 0, sizeof(s));
  s.O = cfg->order;
  s.dim = dim;
  s.rhs = rhs;
  s.dyn = cfg->dyn_dim;
  s.p = p;
  s.shared = shared;
  s.pow_mode = cfg->pow_mode;
  s.two = 2.0;
  s.half = 1.0 / 2.0;
  s.one_sixth = 1.0 / 6.0;
  s.one_tenth = 1.0 / 10.0;
  s.four = s.two * s.two;
  s.order = (double)cfg->order;
  if (cfg->order == 5) {
    const double tf = 24.0, sh = 720.0;
    const double pc[5] = {55.0 / tf, -59.0 / tf, 37.0 / tf, -9.0 / tf, 0.0};
    const double cc[5] = {251.0 / sh, 646.0 / sh, -264.0 / sh, 106.0 / sh, -19.0 / sh};
    memcpy(s.pc, pc, sizeof(pc));
    memcpy(s.cc, cc, sizeof(cc));
  } else {
    const double pc[3] = {1.0 + (1.0 / 2.0), -(1.0 / 2.0), 0.0};
    const double cc[3] = {5.0 / 12.0, 2.0 / 3.0, -(1.0 / 12.0)};
    memcpy(s.pc, pc, sizeof(pc));
    memcpy(s.cc, cc, sizeof(cc));
  }
  s.ec = 19.0 / 270.0;  /* both orders (src/ivp/adams.rs:600-602, :656-658) */
  s.dt_max = cfg->dt_max;
  s.dt_min = cfg->dt_min;
  s.time = t0;
  s.end = t_end;
  s.tol = cfg->tol;
  s.dt = (cfg->dt_max + cfg->dt_min) * s.half;
  memcpy(s.state, y0, sizeof(double) * dim);
  memcpy(y_out, y0, sizeof(double) * dim);
  *t_out = t0;
  *accepted = 0;
  *rejected = 0;
  if (t0 >= t_end) return ORC_TIME_END_OOB;
  double it, iy[ORC_MAX_DIM];
  int64_t calls = 0;
  for (;;) {
    if (cfg->max_attempts > 0 && calls >= cfg->max_attempts) return ORC_MAX_ATTEMPTS_EXCEEDED;
    ++calls;
    int fail = 0;
    const int r = ad_step(&s, &it, iy, &fail);
    if (r == AD_DONE) return ORC_OK;
    if (r == AD_FAIL) return fail;
    if (r == AD_REDO) {
      (*rejected)++;
      continue;
    }
    if (traj_t && *accepted < traj_cap) {
      traj_t[*accepted] = it;
      memcpy(traj_y + (size_t)(*accepted) * dim, iy, sizeof(double) * dim);
    }
    (*accepted)++;
    *t_out = it;
    memcpy(y_out, iy, sizeof(double) * dim);
  }
}

/* EulerSolver::step (src/ivp.rs:318-339) under the iterator: every step
 * yields the (t, y) it started from, so the state reached at t_end is never
 * yielded; y_out is the last yielded item.  dt is the builder's value. */
int32_t oracle_euler_solve_one(int32_t rhs, int32_t dim, const double* p, const double* shared, double dt,
                               int64_t max_steps, double t0, double t_end, const double* y0, double* y_out,
                               double* t_out, int64_t* accepted, double* traj_t, double* traj_y,
                               int64_t traj_cap) {
  double y[ORC_MAX_DIM], f[ORC_MAX_DIM];
  if (dim < 1 || dim > ORC_MAX_DIM) return ORC_MAX_ATTEMPTS_EXCEEDED + 2;
  memcpy(y, y0, sizeof(double) * dim);
  memcpy(y_out, y0, sizeof(double) * dim);
  *t_out = t0;
  *accepted = 0;
  if (t0 >= t_end) return ORC_TIME_END_OOB;
  double t = t0;
  int64_t steps = 0;
  for (;;) {
    if (t >= t_end) return ORC_OK;
    if (max_steps > 0 && steps >= max_steps) return ORC_MAX_ATTEMPTS_EXCEEDED;
    ++steps;
    if (t + dt >= t_end) dt = t_end - t;
    oracle_rhs(rhs, dim, t, y, p, shared, f);
    if (traj_t && *accepted < traj_cap) {
      traj_t[*accepted] = t;
      memcpy(traj_y + (size_t)(*accepted) * dim, y, sizeof(double) * dim);
    }
    (*accepted)++;
    *t_out = t;
    memcpy(y_out, y, sizeof(double) * dim);
    for (int d = 0; d < dim; ++d) y[d] = y[d] + (f[d] * dt);
    t = t + dt;
  }
}
