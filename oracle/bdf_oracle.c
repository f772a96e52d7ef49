/*
 * CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * BDF solvers.
 *
 * ORC_BDF_AS_COMPILED restates src/ivp/bdf.rs (bacon-sci 0.16.2) step by step:
 *   BDF::solve                 :257-331   dt0 = (max+min)/2, order = O (7 for BDF6)
 *   BDFSolver::runge_kutta     :346-387   RK4 bootstrap, history pushes
 *   BDFSolver::jac_finite_diff :390-411   column = (G(x+dt e) + G(x-dt e)) / (2 dt)
 *   BDFSolver::secant          :414-475   explicit inverse (nalgebra LU
 *                                          try_inverse), Broyden updates, <= 998
 *   BDFSolver::step            :495-634   yield machine, accept/double/halve
 *   BDF6Coefficients / BDF2Coefficients  :641-673, :708-730
 * with every quirk kept (the + in the finite difference, f at t_n, the lower
 * residual built with the higher-order history weights, the time update
 * t -= dt - order on a rejected bootstrap).  nalgebra 0.32's LU (partial
 * pivoting, first maximum of |a|, multiplication by the reciprocal pivot),
 * its triangular solves and its gemv accumulation order are restated from
 * its published algorithms, and so are the full-pivot LU and Householder QR
 * that secant falls back to (bdf.rs:433-443) when the partial-pivot LU has an
 * exactly zero pivot.  The "+" finite difference makes the Jacobian's columns
 * nearly equal, so on multi-dimensional systems that happens (Lotka-Volterra,
 * Lorenz).
 *
 * ORC_BDF_CORRECTED is this engine's stiff BDF (no reference counterpart to
 * follow beyond the structure above): orders 1..6 ramped up after every
 * restart, f at t_{n+1}, a true Newton iteration with the analytic Jacobian
 * (one partial-pivot LU per solve; for a right-hand side affine in y the
 * first update solves the linear system, so the solve ends there, as
 * ARKODE's linear-problem option does), and the reference's error estimate and
 * control — ||y_high - y_low||_2 <= tol, double dt below tol/10, halve on a
 * rejection — where y_low is the order-(q-1) solution with its own
 * coefficients.  After a doubling the history is re-sampled exactly (every
 * second point); after a halving it is interpolated (Lagrange through the
 * stored points).  The CUDA kernel executes the same operation sequence.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"
#include "oracle_internal.h"

#define BDF_MAX_O 8
#define BDF_MAX_HIST 24

typedef double dmat[ORC_MAX_BDF_DIM][ORC_MAX_BDF_DIM];

/* ---- shared helpers -------------------------------------------------------- */
static double bdf_norm(const double* x, int n, int dyn) { return oracle_norm(x, n, dyn); }

/* nalgebra gemv y = M v: column axpys, y = v_0*M[:,0] first, then
 * y = (v_j * M[:,j]) + y. */
static void gemv_cols(const dmat M, const double* v, int n, double* y) {
  for (int i = 0; i < n; ++i) y[i] = v[0] * M[i][0];
  for (int j = 1; j < n; ++j)
    for (int i = 0; i < n; ++i) y[i] = (v[j] * M[i][j]) + y[i];
}

/* nalgebra LU::new (partial pivoting) then try_inverse; returns 0 when a
 * pivot is exactly zero (no inverse). */
static int lu_try_inverse(const dmat A, int n, dmat inv) {
  static __thread dmat a;
  int perm_i[ORC_MAX_BDF_DIM], perm_p[ORC_MAX_BDF_DIM], np = 0;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) a[r][c] = A[r][c];
  for (int i = 0; i < n; ++i) {
    int piv = i;
    double best = fabs(a[i][i]);
    for (int r = i + 1; r < n; ++r)
      if (fabs(a[r][i]) > best) { best = fabs(a[r][i]); piv = r; }
    const double diag = a[piv][i];
    if (diag == 0.0) continue;
    if (piv != i) {
      perm_i[np] = i;
      perm_p[np] = piv;
      ++np;
      for (int c = 0; c <= i; ++c) { const double t = a[i][c]; a[i][c] = a[piv][c]; a[piv][c] = t; }
      for (int c = i + 1; c < n; ++c) { const double t = a[i][c]; a[i][c] = a[piv][c]; a[piv][c] = t; }
    }
    const double inv_diag = 1.0 / diag;
    for (int r = i + 1; r < n; ++r) a[r][i] = a[r][i] * inv_diag;
    for (int c = i + 1; c < n; ++c) {
      const double alpha = -a[i][c];
      for (int r = i + 1; r < n; ++r) a[r][c] = (alpha * a[r][i]) + a[r][c];
    }
  }
  /* out = P * I, then L (unit) and U solves column by column */
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) inv[r][c] = (r == c) ? 1.0 : 0.0;
  for (int k = 0; k < np; ++k)
    for (int c = 0; c < n; ++c) { const double t = inv[perm_i[k]][c]; inv[perm_i[k]][c] = inv[perm_p[k]][c]; inv[perm_p[k]][c] = t; }
  for (int k = 0; k < n; ++k) {
    for (int i = 0; i < n - 1; ++i) {
      const double coeff = inv[i][k] / 1.0;
      const double mc = -coeff;
      for (int r = i + 1; r < n; ++r) inv[r][k] = (mc * a[r][i]) + inv[r][k];
    }
  }
  for (int k = 0; k < n; ++k) {
    for (int i = n - 1; i >= 0; --i) {
      const double diag = a[i][i];
      if (diag == 0.0) return 0;
      const double coeff = inv[i][k] / diag;
      inv[i][k] = coeff;
      const double mc = -coeff;
      for (int r = 0; r < i; ++r) inv[r][k] = (mc * a[r][i]) + inv[r][k];
    }
  }
  return 1;
}

/* nalgebra's dot product of two vectors of run-time length (blas.rs `dotx`,
 * the general path: eight accumulators over whole blocks of eight, folded
 * pairwise into res, then the remaining products added in order).  x and y
 * are columns of row-major n x n matrices starting at row r0: element k is
 * x[(r0 + k) * ORC_MAX_BDF_DIM]. */
static double dotx_col(const double* x, const double* y, int len) {
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int i = 0;
  while (len - i >= 8) {
    for (int l = 0; l < 8; ++l) acc[l] = acc[l] + (x[(i + l) * ORC_MAX_BDF_DIM] * y[(i + l) * ORC_MAX_BDF_DIM]);
    i += 8;
  }
  double res = 0.0;
  res = res + (acc[0] + acc[4]);
  res = res + (acc[1] + acc[5]);
  res = res + (acc[2] + acc[6]);
  res = res + (acc[3] + acc[7]);
  for (int k = i; k < len; ++k) res = res + (x[k * ORC_MAX_BDF_DIM] * y[k * ORC_MAX_BDF_DIM]);
  return res;
}

/* Rust's f64::signum: 1 for +0 and positives, -1 for -0 and negatives. */
static double rs_signum(double x) { return isnan(x) ? x : (signbit(x) ? -1.0 : 1.0); }

/* nalgebra FullPivLU::new (the largest |a| of the remaining block, first in
 * column-major order, swapped into place by a column and a row swap, then a
 * Gauss step), then try_inverse: row permutation, unit-lower and upper
 * solves, inverse column permutation.  Returns 0 when the last diagonal
 * entry is exactly zero (is_invertible). */
static int full_piv_lu_try_inverse(const dmat A, int n, dmat inv) {
  static __thread dmat a;
  int pi[ORC_MAX_BDF_DIM], pp[ORC_MAX_BDF_DIM], qi[ORC_MAX_BDF_DIM], qp[ORC_MAX_BDF_DIM], np = 0, nq = 0;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) a[r][c] = A[r][c];
  for (int i = 0; i < n; ++i) {
    int pr = i, pc = i;
    double best = fabs(a[i][i]);
    for (int c = i; c < n; ++c)
      for (int r = i; r < n; ++r)
        if (fabs(a[r][c]) > best) {
          best = fabs(a[r][c]);
          pr = r;
          pc = c;
        }
    const double diag = a[pr][pc];
    if (diag == 0.0) break; /* the rest of the matrix is zero */
    if (pc != i) {
      for (int r = 0; r < n; ++r) { const double t = a[r][i]; a[r][i] = a[r][pc]; a[r][pc] = t; }
      qi[nq] = i;
      qp[nq] = pc;
      ++nq;
    }
    if (pr != i) {
      pi[np] = i;
      pp[np] = pr;
      ++np;
      for (int c = 0; c < n; ++c) { const double t = a[i][c]; a[i][c] = a[pr][c]; a[pr][c] = t; }
    }
    const double inv_diag = 1.0 / diag;
    for (int r = i + 1; r < n; ++r) a[r][i] = a[r][i] * inv_diag;
    for (int c = i + 1; c < n; ++c) {
      const double alpha = -a[i][c];
      for (int r = i + 1; r < n; ++r) a[r][c] = (alpha * a[r][i]) + a[r][c];
    }
  }
  if (a[n - 1][n - 1] == 0.0) return 0;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) inv[r][c] = (r == c) ? 1.0 : 0.0;
  for (int k = 0; k < np; ++k)
    for (int c = 0; c < n; ++c) { const double t = inv[pi[k]][c]; inv[pi[k]][c] = inv[pp[k]][c]; inv[pp[k]][c] = t; }
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < n - 1; ++i) {
      const double mc = -(inv[i][k] / 1.0);
      for (int r = i + 1; r < n; ++r) inv[r][k] = (mc * a[r][i]) + inv[r][k];
    }
  for (int k = 0; k < n; ++k)
    for (int i = n - 1; i >= 0; --i) {
      const double diag = a[i][i];
      if (diag == 0.0) break; /* the solve's own result is ignored by try_inverse */
      const double coeff = inv[i][k] / diag;
      inv[i][k] = coeff;
      const double mc = -coeff;
      for (int r = 0; r < i; ++r) inv[r][k] = (mc * a[r][i]) + inv[r][k];
    }
  for (int k = nq - 1; k >= 0; --k)
    for (int c = 0; c < n; ++c) { const double t = inv[qi[k]][c]; inv[qi[k]][c] = inv[qp[k]][c]; inv[qp[k]][c] = t; }
  return 1;
}

/* nalgebra QR::new (Householder reflections, householder.rs
 * clear_column_unchecked / reflection_axis_mut) then try_inverse (Q^T by the
 * stored reflections, then the upper solve with R's diagonal).  Returns 0
 * when a diagonal entry of R is exactly zero. */
static int qr_try_inverse(const dmat A, int n, dmat inv) {
  static __thread dmat a;
  double diag[ORC_MAX_BDF_DIM];
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) a[r][c] = A[r][c];
  for (int i = 0; i < n; ++i) {
    const int len = n - i;
    const double sq = 0.0 + dotx_col(&a[i][i], &a[i][i], len);
    const double nrm = sqrt(sq);
    const double x0 = a[i][i];
    const double modulus = (x0 >= 0.0) ? x0 : -x0;
    const double sgn = (x0 >= 0.0) ? 1.0 : -1.0;
    const double signed_norm = sgn * nrm;
    const double factor = (sq + (modulus * nrm)) * 2.0;
    a[i][i] = a[i][i] + signed_norm;
    if (factor != 0.0) {
      const double sf = sqrt(factor);
      for (int r = i; r < n; ++r) a[r][i] = a[r][i] / sf;
      diag[i] = -signed_norm;
      const double sign = rs_signum(diag[i]);
      const double m_two = sign * -2.0;
      for (int c = i + 1; c < n; ++c) {
        const double f = (dotx_col(&a[i][i], &a[i][c], len) - 0.0) * m_two;
        for (int r = i; r < n; ++r) a[r][c] = (f * a[r][i]) + (sign * a[r][c]);
      }
    } else {
      diag[i] = signed_norm;
    }
  }
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) inv[r][c] = (r == c) ? 1.0 : 0.0;
  for (int i = 0; i < n; ++i) {
    const int len = n - i;
    const double sign = rs_signum(diag[i]);
    const double m_two = sign * -2.0;
    for (int c = 0; c < n; ++c) {
      const double f = (dotx_col(&a[i][i], &inv[i][c], len) - 0.0) * m_two;
      for (int r = i; r < n; ++r) inv[r][c] = (f * a[r][i]) + (sign * inv[r][c]);
    }
  }
  for (int k = 0; k < n; ++k)
    for (int i = n - 1; i >= 0; --i) {
      if (diag[i] == 0.0) return 0;
      const double coeff = inv[i][k] / diag[i];
      inv[i][k] = coeff;
      const double mc = -coeff;
      for (int r = 0; r < i; ++r) inv[r][k] = (mc * a[r][i]) + inv[r][k];
    }
  return 1;
}

/* ---- as_compiled: restatement of src/ivp/bdf.rs ------------------------------ */
typedef struct {
  const oracle_bdf_cfg* cfg;
  int32_t rhs, dim;
  const double* p;
  const double* shared;
  int O;
  double hc[BDF_MAX_O], lc[BDF_MAX_O];
  double dt_max, dt_min, time, end, tol, dt, order;
  double state[ORC_MAX_BDF_DIM], save[ORC_MAX_BDF_DIM], scratch[ORC_MAX_BDF_DIM];
  /* prev_values deque */
  double ht[BDF_MAX_HIST];
  double hy[BDF_MAX_HIST][ORC_MAX_BDF_DIM];
  int hfront, hlen;
  int ym; /* yield_memory */
} bdf_ref;

static int dq_push(bdf_ref* s, double t, const double* y) {
  if (s->hlen >= BDF_MAX_HIST) return 0;
  const int k = (s->hfront + s->hlen) % BDF_MAX_HIST;
  s->ht[k] = t;
  memcpy(s->hy[k], y, sizeof(double) * s->dim);
  s->hlen++;
  return 1;
}
static void dq_pop_front(bdf_ref* s) {
  if (s->hlen > 0) { s->hfront = (s->hfront + 1) % BDF_MAX_HIST; s->hlen--; }
}
static int dq_idx(const bdf_ref* s, int i) { return (s->hfront + i) % BDF_MAX_HIST; }

static void rhs_f(bdf_ref* s, double t, const double* y, double* f) {
  oracle_rhs(s->rhs, s->dim, t, y, s->p, s->shared, f);
}

/* bdf.rs:346-387 */
static int ref_runge_kutta(bdf_ref* s, int iterations) {
  const int n = s->dim;
  double k1[ORC_MAX_BDF_DIM], k2[ORC_MAX_BDF_DIM], k3[ORC_MAX_BDF_DIM], k4[ORC_MAX_BDF_DIM], it[ORC_MAX_BDF_DIM], f[ORC_MAX_BDF_DIM];
  for (int i = 0; i < iterations; ++i) {
    rhs_f(s, s->time, s->state, f);
    for (int d = 0; d < n; ++d) k1[d] = f[d] * s->dt;
    for (int d = 0; d < n; ++d) it[d] = s->state[d] + (k1[d] * 0.5);
    rhs_f(s, s->time + (0.5 * s->dt), it, f);
    for (int d = 0; d < n; ++d) k2[d] = f[d] * s->dt;
    for (int d = 0; d < n; ++d) it[d] = s->state[d] + (k2[d] * 0.5);
    rhs_f(s, s->time + (0.5 * s->dt), it, f);
    for (int d = 0; d < n; ++d) k3[d] = f[d] * s->dt;
    for (int d = 0; d < n; ++d) it[d] = s->state[d] + k3[d];
    rhs_f(s, s->time + s->dt, it, f);
    for (int d = 0; d < n; ++d) k4[d] = f[d] * s->dt;
    if (i != 0 && !dq_push(s, s->time, s->state)) return 0;
    for (int d = 0; d < n; ++d) {
      const double inc = (((k1[d] + (k2[d] * 2.0)) + (k3[d] * 2.0)) + k4[d]) * (1.0 / 6.0);
      s->state[d] = s->state[d] + inc;
    }
    s->time = s->time + s->dt;
  }
  return dq_push(s, s->time, s->state);
}

/* bdf.rs:548-575: G(y) = ((-f(t, y)) * dt) * c0 + sum_ind prev[O-ind] * h[ind] + y */
static void ref_residual(bdf_ref* s, int lower, const double* y, double* out) {
  const int n = s->dim;
  double f[ORC_MAX_BDF_DIM];
  rhs_f(s, s->time, y, f);
  const double c0 = lower ? s->lc[0] : s->hc[0];
  for (int d = 0; d < n; ++d) s->scratch[d] = ((-f[d]) * s->dt) * c0;
  for (int ind = 1; ind < s->O; ++ind) {
    const int k = dq_idx(s, s->O - ind);
    for (int d = 0; d < n; ++d) s->scratch[d] = s->scratch[d] + (s->hy[k][d] * s->hc[ind]);
  }
  for (int d = 0; d < n; ++d) out[d] = s->scratch[d] + y[d];
}

/* bdf.rs:414-475 */
static int32_t ref_secant(bdf_ref* s, int lower, double* result) {
  const int n = s->dim;
  static __thread dmat jac, inv, minv;
  double guess[ORC_MAX_BDF_DIM], deriv[ORC_MAX_BDF_DIM], dlast[ORC_MAX_BDF_DIM], above[ORC_MAX_BDF_DIM], below[ORC_MAX_BDF_DIM];
  double shift[ORC_MAX_BDF_DIM], diff[ORC_MAX_BDF_DIM], adj[ORC_MAX_BDF_DIM], u[ORC_MAX_BDF_DIM], w[ORC_MAX_BDF_DIM];
  memcpy(guess, s->state, sizeof(double) * n);
  ref_residual(s, lower, guess, deriv);
  /* jac_finite_diff (bdf.rs:390-411), guess modified in place */
  const double denom = 1.0 / (2.0 * s->dt);
  for (int c = 0; c < n; ++c) {
    guess[c] = guess[c] + s->dt;
    ref_residual(s, lower, guess, above);
    guess[c] = guess[c] - (2.0 * s->dt);
    ref_residual(s, lower, guess, below);
    guess[c] = guess[c] + s->dt;
    for (int r = 0; r < n; ++r) jac[r][c] = (above[r] + below[r]) * denom;
  }
  /* lu().try_inverse(), else full_piv_lu().try_inverse(), else
   * qr().try_inverse(), else SingularMatrix (bdf.rs:429-443) */
  if (!lu_try_inverse(jac, n, inv) && !full_piv_lu_try_inverse(jac, n, inv) && !qr_try_inverse(jac, n, inv))
    return ORC_SINGULAR_MATRIX;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) minv[r][c] = -inv[r][c];
  gemv_cols(minv, deriv, n, shift);
  for (int d = 0; d < n; ++d) guess[d] = guess[d] + shift[d];
  const int max_iter = s->cfg->max_iter > 0 ? s->cfg->max_iter : 1000;
  for (int it = 2; it < max_iter; ++it) {
    memcpy(dlast, deriv, sizeof(double) * n);
    ref_residual(s, lower, guess, deriv);
    for (int d = 0; d < n; ++d) diff[d] = deriv[d] - dlast[d];
    gemv_cols(minv, diff, n, adj);
    /* p = ((-s^T) * adj)[0] */
    double p = adj[0] * (-shift[0]);
    for (int j = 1; j < n; ++j) p = (adj[j] * (-shift[j])) + p;
    /* u = s^T * inv */
    for (int c = 0; c < n; ++c) {
      double acc = inv[0][c] * shift[0];
      for (int j = 1; j < n; ++j) acc = (inv[j][c] * shift[j]) + acc;
      u[c] = acc;
    }
    for (int d = 0; d < n; ++d) w[d] = shift[d] + adj[d];
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) {
        inv[r][c] = inv[r][c] + ((u[c] * w[r]) / p);
        minv[r][c] = -inv[r][c];
      }
    gemv_cols(minv, deriv, n, shift);
    for (int d = 0; d < n; ++d) guess[d] = guess[d] + shift[d];
    if (bdf_norm(shift, n, s->cfg->dyn_dim) <= s->tol) {
      memcpy(result, guess, sizeof(double) * n);
      return ORC_OK;
    }
  }
  return ORC_MAXIMUM_ITERATIONS_EXCEEDED;
}

enum { ST_ITEM = 0, ST_REDO = 1, ST_DONE = 2, ST_FAIL = 3 };

static int ref_step(bdf_ref* s, double* it_t, double* it_y, int32_t* fail) {
  const int n = s->dim, O = s->O;
  if (s->ym > 0 && s->ym <= O) {
    const int get = O - s->ym;
    s->ym -= 1;
    if (s->ym == 0) s->ym = O + 2;
    const int k = dq_idx(s, get);
    *it_t = s->ht[k];
    memcpy(it_y, s->hy[k], sizeof(double) * n);
    return ST_ITEM;
  }
  if (s->ym == O + 2) {
    s->ym = 0;
    if (!dq_push(s, s->time, s->state)) { *fail = ORC_MAX_ATTEMPTS_EXCEEDED; return ST_FAIL; }
    dq_pop_front(s);
    *it_t = s->time;
    memcpy(it_y, s->state, sizeof(double) * n);
    return ST_ITEM;
  }
  if (s->time >= s->end) return ST_DONE;
  if (s->time + s->dt >= s->end) {
    s->dt = s->end - s->time;
    if (!ref_runge_kutta(s, 1)) { *fail = ORC_MAX_ATTEMPTS_EXCEEDED; return ST_FAIL; }
    const int k = dq_idx(s, s->hlen - 1);
    *it_t = s->time;
    memcpy(it_y, s->hy[k], sizeof(double) * n);
    return ST_ITEM;
  }
  if (s->hlen == 0) {
    memcpy(s->save, s->state, sizeof(double) * n);
    if (s->time + (s->dt * s->order) >= s->end) s->dt = (s->end - s->time) / s->order;
    if (!ref_runge_kutta(s, O)) { *fail = ORC_MAX_ATTEMPTS_EXCEEDED; return ST_FAIL; }
    s->ym = O + 1;
    return ST_REDO;
  }
  double high[ORC_MAX_BDF_DIM], low[ORC_MAX_BDF_DIM], diff[ORC_MAX_BDF_DIM];
  int32_t st = ref_secant(s, 0, high);
  if (st != ORC_OK) { *fail = st; return ST_FAIL; }
  st = ref_secant(s, 1, low);
  if (st != ORC_OK) { *fail = st; return ST_FAIL; }
  for (int d = 0; d < n; ++d) diff[d] = high[d] - low[d];
  const double error = bdf_norm(diff, n, s->cfg->dyn_dim);
  if (error <= s->tol) {
    memcpy(s->state, high, sizeof(double) * n);
    s->time = s->time + s->dt;
    if (s->ym == O + 1) { s->ym -= 1; return ST_REDO; }
    if (!dq_push(s, s->time, s->state)) { *fail = ORC_MAX_ATTEMPTS_EXCEEDED; return ST_FAIL; }
    dq_pop_front(s);
    if (error < (0.1 * s->tol)) {
      s->dt = s->dt * 2.0;
      if (s->dt > s->dt_max) s->dt = s->dt_max;
      s->hlen = 0;
      s->hfront = 0;
    }
    *it_t = s->time;
    memcpy(it_y, s->state, sizeof(double) * n);
    return ST_ITEM;
  }
  if (s->ym == O + 1) {
    s->time = s->time - (s->dt - s->order);
    memcpy(s->state, s->save, sizeof(double) * n);
  }
  s->dt = s->dt * 0.5;
  if (s->dt < s->dt_min) { *fail = ORC_MINIMUM_TIME_DELTA_EXCEEDED; return ST_FAIL; }
  s->hlen = 0;
  s->hfront = 0;
  return ST_REDO;
}

static void bdf_coefficients(int method, int* O, double* hc, double* lc) {
  if (method == ORC_BDF6) {
    *O = 7;
    const double h[7] = {60.0 / 147.0, -360.0 / 147.0, 450.0 / 147.0, -400.0 / 147.0,
                         225.0 / 147.0, -72.0 / 147.0, 10.0 / 147.0};
    const double l[7] = {60.0 / 137.0, -300.0 / 137.0, 300.0 / 137.0, -200.0 / 137.0,
                         75.0 / 137.0, -12.0 / 137.0, 0.0};
    memcpy(hc, h, sizeof(h));
    memcpy(lc, l, sizeof(l));
  } else {
    *O = 3;
    const double h[3] = {2.0 / 3.0, -4.0 / 3.0, 1.0 / 3.0};
    const double l[3] = {1.0, -1.0, 0.0};
    memcpy(hc, h, sizeof(h));
    memcpy(lc, l, sizeof(l));
  }
}

static int32_t bdf_as_compiled(const oracle_bdf_cfg* cfg, int32_t rhs, int32_t dim, const double* p,
                               const double* shared, double t0, double t_end, const double* y0,
                               double* y_out, double* t_out, int64_t* accepted, int64_t* rejected,
                               double* traj_t, double* traj_y, int64_t traj_cap) {
  static __thread bdf_ref s;
  memset(&s, 0, sizeof(s));
  s.cfg = cfg;
  s.rhs = rhs;
  s.dim = dim;
  s.p = p;
  s.shared = shared;
  bdf_coefficients(cfg->method, &s.O, s.hc, s.lc);
  s.dt_max = cfg->dt_max;
  s.dt_min = cfg->dt_min;
  if (s.dt_min > s.dt_max) s.dt_min = s.dt_max;
  s.time = t0;
  s.end = t_end;
  s.tol = cfg->tol;
  s.dt = (s.dt_max + s.dt_min) * (1.0 / 2.0);
  s.order = (double)s.O;
  memcpy(s.state, y0, sizeof(double) * dim);
  memcpy(y_out, y0, sizeof(double) * dim);
  *t_out = t0;
  *accepted = 0;
  *rejected = 0;
  if (t0 >= t_end) return ORC_TIME_END_OOB;
  int64_t calls = 0;
  double it_t, it_y[ORC_MAX_BDF_DIM];
  for (;;) {
    if (cfg->max_steps > 0 && calls >= cfg->max_steps) return ORC_MAX_ATTEMPTS_EXCEEDED;
    ++calls;
    int32_t fail = ORC_OK;
    const int r = ref_step(&s, &it_t, it_y, &fail);
    if (r == ST_DONE) return ORC_OK;
    if (r == ST_FAIL) return fail;
    if (r == ST_REDO) { (*rejected)++; continue; }
    if (traj_t && *accepted < traj_cap) {
      traj_t[*accepted] = it_t;
      memcpy(traj_y + (size_t)(*accepted) * dim, it_y, sizeof(double) * dim);
    }
    (*accepted)++;
    *t_out = it_t;
    memcpy(y_out, it_y, sizeof(double) * dim);
  }
}

/* ---- corrected: the engine's stiff BDF ------------------------------------------ */
/* BDF-q in the form y_{n+1} + sum_{j=1..q} a_{q,j} y_{n+1-j} = dt * b_q f_{n+1}. */
static const double kBdfB[7] = {0.0, 1.0, 2.0 / 3.0, 6.0 / 11.0, 12.0 / 25.0, 60.0 / 137.0, 60.0 / 147.0};
static const double kBdfA[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {-1.0, 0, 0, 0, 0, 0},
    {-4.0 / 3.0, 1.0 / 3.0, 0, 0, 0, 0},
    {-18.0 / 11.0, 9.0 / 11.0, -2.0 / 11.0, 0, 0, 0},
    {-48.0 / 25.0, 36.0 / 25.0, -16.0 / 25.0, 3.0 / 25.0, 0, 0},
    {-300.0 / 137.0, 300.0 / 137.0, -200.0 / 137.0, 75.0 / 137.0, -12.0 / 137.0, 0},
    {-360.0 / 147.0, 450.0 / 147.0, -400.0 / 147.0, 225.0 / 147.0, -72.0 / 147.0, 10.0 / 147.0}};

int oracle_rhs_jacobian(int32_t rhs, int32_t dim, double t, const double* y, const double* p,
                        const double* shared, double* J /* row-major dim x dim */);

/* The linear solves go by blocks of 32 rows.  After the LU, each diagonal
 * block of L (unit lower) and of the row-scaled U (unit upper) is replaced by
 * its inverse, strict parts in place (the unit diagonals stay implicit), so
 * that a block's solve is one product with a right-hand side that is already
 * complete rather than a chain of dependent updates.  Column c of an inverse
 * is the solve of the unit vector e_c, every update taken for every column in
 * the same order (updates by a zero leave a value unchanged, so this equals
 * the solve restricted to its non-zero part, and NaN spreads the same way). */
enum { kSolveBlock = 32 };

static void block_inverses(int n, dmat M) {
  double T[kSolveBlock][kSolveBlock], x[kSolveBlock];
  for (int s = 0; s < n; s += kSolveBlock) {
    const int nb = (n - s < kSolveBlock) ? n - s : kSolveBlock;
    for (int c = 0; c < nb; ++c) { /* L_bb^-1 e_c: forward, unit diagonal */
      for (int j = 0; j < nb; ++j) x[j] = (j == c) ? 1.0 : 0.0;
      for (int k = 0; k + 1 < nb; ++k)
        for (int j = k + 1; j < nb; ++j) x[j] = fma(-M[s + j][s + k], x[k], x[j]);
      for (int j = c + 1; j < nb; ++j) T[j][c] = x[j];
    }
    for (int c = 0; c < nb; ++c) { /* U_bb^-1 e_c: backward, unit diagonal */
      for (int j = 0; j < nb; ++j) x[j] = (j == c) ? 1.0 : 0.0;
      for (int k = nb - 1; k > 0; --k)
        for (int j = 0; j < k; ++j) x[j] = fma(-M[s + j][s + k], x[k], x[j]);
      for (int j = 0; j < c; ++j) T[j][c] = x[j];
    }
    for (int j = 0; j < nb; ++j)
      for (int c = 0; c < nb; ++c)
        if (j != c) M[s + j][s + c] = T[j][c];
  }
}

/* Work counters of the corrected BDF on the calling thread, for the
 * algorithmic-flop count of the benchmark's stiff roofline: Newton solves,
 * Newton iterations, factorisations a solver needs at the least (every solve
 * for a right-hand side whose Jacobian depends on y; one per distinct h*b_q
 * value of a solve for the linear chains, whose Jacobian is constant), and
 * the elimination's FMAs: executed (zero updates skipped) and dense. */
static __thread int64_t g_work[5];

/* Factors M in place for the corrected solve: the LU, the row-scaled U and
 * the inverted diagonal blocks.  Returns 0 on an exactly zero pivot. */
static int corrected_factor(int n, dmat M, int* piv, double* rinv) {
  /* LU with partial pivoting (first maximum), row swaps on the whole row.  The
   * elimination and both substitutions update with one fused multiply-add
   * (fma is correctly rounded, so every platform and the GPU agree): half the
   * operations of separate products and differences, and one rounding less. */
  for (int i = 0; i < n; ++i) {
    int pr = i;
    double best = fabs(M[i][i]);
    for (int r = i + 1; r < n; ++r)
      if (fabs(M[r][i]) > best) { best = fabs(M[r][i]); pr = r; }
    piv[i] = pr;
    if (pr != i)
      for (int k = 0; k < n; ++k) { const double t = M[i][k]; M[i][k] = M[pr][k]; M[pr][k] = t; }
    if (M[i][i] == 0.0) return 0;
    const double inv = 1.0 / M[i][i];
    rinv[i] = inv;
    for (int r = i + 1; r < n; ++r) {
      const double l = M[r][i] * inv;
      M[r][i] = l;
      /* An update with an exactly zero multiplier or pivot-row entry is
       * skipped: it would only change the sign of a zero element.  The
       * factors of the chains stay sparse (I - hb J of a banded J), so most
       * updates are skipped. */
      g_work[4] += n - 1 - i;
      if (l == 0.0) continue;
      for (int k = i + 1; k < n; ++k)
        if (M[i][k] != 0.0) {
          M[r][k] = fma(-l, M[i][k], M[r][k]);
          g_work[3]++;
        }
    }
  }
  /* the rows of U scaled by their pivot reciprocal: the back substitution
   * then runs on a unit upper factor, with no product on its critical path */
  for (int r = 0; r < n; ++r)
    for (int k = r + 1; k < n; ++k) M[r][k] = M[r][k] * rinv[r];
  block_inverses(n, M);
  return 1;
}

/* Solves (the factored M) x = v in place in dx. */
static void corrected_solve(int n, dmat M, const int* piv, const double* rinv, double* dx) {
  for (int i = 0; i < n; ++i)
    if (piv[i] != i) { const double t = dx[i]; dx[i] = dx[piv[i]]; dx[piv[i]] = t; }
  /* forward, block by block: the updates from earlier blocks in pivot
   * order, then the product with the block's inverse, x_j = r_j +
   * sum_{k<j} Linv[j][k] r_k in ascending k */
  for (int s = 0; s < n; s += kSolveBlock) {
    const int e = (s + kSolveBlock < n) ? s + kSolveBlock : n;
    for (int r = s; r < e; ++r)
      for (int k = 0; k < s; ++k) dx[r] = fma(-M[r][k], dx[k], dx[r]);
    double rb[kSolveBlock];
    for (int j = s; j < e; ++j) rb[j - s] = dx[j];
    for (int j = s; j < e; ++j) {
      double acc = rb[j - s];
      for (int k = s; k < j; ++k) acc = fma(M[j][k], rb[k - s], acc);
      dx[j] = acc;
    }
  }
  /* back, on the row-scaled upper factor: the right-hand side takes the
   * pivot reciprocals first (the elimination's own, no division); per block
   * from the last, the updates from later blocks in descending pivot order,
   * then x_j = r_j + sum_{k>j} Uinv[j][k] r_k in descending k */
  for (int r = 0; r < n; ++r) dx[r] = dx[r] * rinv[r];
  for (int s = ((n - 1) / kSolveBlock) * kSolveBlock; s >= 0; s -= kSolveBlock) {
    const int e = (s + kSolveBlock < n) ? s + kSolveBlock : n;
    for (int r = s; r < e; ++r)
      for (int k = n - 1; k >= e; --k) dx[r] = fma(-M[r][k], dx[k], dx[r]);
    double rb[kSolveBlock];
    for (int j = s; j < e; ++j) rb[j - s] = dx[j];
    for (int j = s; j < e; ++j) {
      double acc = rb[j - s];
      for (int k = e - 1; k > j; --k) acc = fma(M[j][k], rb[k - s], acc);
      dx[j] = acc;
    }
  }
}

#define BDF_SEEN_MAX 4096
static __thread double g_seen_hb[BDF_SEEN_MAX];
static __thread int g_seen_n;

void oracle_bdf_work(int64_t* out5, int reset) {
  if (out5) memcpy(out5, g_work, sizeof(g_work));
  if (reset) {
    memset(g_work, 0, sizeof(g_work));
    g_seen_n = 0;
  }
}

static void count_factorisation(int32_t rhs, double hb) {
  if (rhs == ORC_RHS_CHAIN) {
    for (int i = 0; i < g_seen_n; ++i)
      if (g_seen_hb[i] == hb) return;
    if (g_seen_n < BDF_SEEN_MAX) g_seen_hb[g_seen_n++] = hb;
  }
  g_work[2]++;
}

/* Right-hand sides affine in y (f = J y + g(t), J constant): with their exact
 * Jacobian G is linear, so the first Newton update lands on the solution up
 * to the rounding of one LU solve. */
static int rhs_affine(int32_t rhs) {
  return rhs == ORC_RHS_EXP || rhs == ORC_RHS_DECAY || rhs == ORC_RHS_QUADRATIC || rhs == ORC_RHS_SINE ||
         rhs == ORC_RHS_HARMONIC || rhs == ORC_RHS_CHAIN || rhs == ORC_RHS_LINEAR;
}

/* Solve G(y) = y - dt*b*f(t1, y) + sum_j a_j H[j-1] = 0 by Newton with the
 * Jacobian at the initial guess (one LU).  Returns 1 on convergence: after
 * the first update for an affine f (unless it is NaN), else once the update's
 * norm is at most 1e-3 tol. */
static int corrected_newton(const oracle_bdf_cfg* cfg, int32_t rhs, int n, const double* p,
                            const double* shared, double t1, double dt, int q,
                            double H[][ORC_MAX_BDF_DIM], const double* guess0, double* y) {
  static __thread double J[ORC_MAX_BDF_DIM * ORC_MAX_BDF_DIM];
  static __thread dmat M;
  double c[ORC_MAX_BDF_DIM], f[ORC_MAX_BDF_DIM], g[ORC_MAX_BDF_DIM], dx[ORC_MAX_BDF_DIM];
  double rinv[ORC_MAX_BDF_DIM]; /* 1 / U[i][i], the elimination's own reciprocal */
  int piv[ORC_MAX_BDF_DIM];
  const double hb = dt * kBdfB[q];
  /* constant part c = sum_j a_j H[j-1] */
  for (int d = 0; d < n; ++d) c[d] = 0.0;
  for (int j = 1; j <= q; ++j)
    for (int d = 0; d < n; ++d) c[d] = c[d] + (kBdfA[q][j - 1] * H[j - 1][d]);
  memcpy(y, guess0, sizeof(double) * n);
  oracle_rhs_jacobian(rhs, n, t1, y, p, shared, J);
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < n; ++k) M[r][k] = ((r == k) ? 1.0 : 0.0) - (hb * J[r * n + k]);
  g_work[0]++;
  count_factorisation(rhs, hb);
  if (!corrected_factor(n, M, piv, rinv)) return 0;
  const int max_newton = cfg->max_iter > 0 ? cfg->max_iter : 8;
  for (int it = 0; it < max_newton; ++it) {
    g_work[1]++;
    oracle_rhs(rhs, n, t1, y, p, shared, f);
    for (int d = 0; d < n; ++d) g[d] = (y[d] - (hb * f[d])) + c[d];
    /* solve M dx = -g */
    for (int d = 0; d < n; ++d) dx[d] = -g[d];
    corrected_solve(n, M, piv, rinv, dx);
    double dn = 0.0;
    for (int d = 0; d < n; ++d) {
      y[d] = y[d] + dx[d];
      dn = dn + (dx[d] * dx[d]);
    }
    if (!(dn == dn)) return 0;
    if (rhs_affine(rhs)) return 1;
    if (sqrt(dn) <= 1e-3 * cfg->tol) return 1;
  }
  return 0;
}

/* Lagrange weights of the nodes s_i = -i (i = 0..q) at the point s. */
static void lagrange_weights(int q, double s, double* w) {
  for (int i = 0; i <= q; ++i) {
    double num = 1.0, den = 1.0;
    for (int k = 0; k <= q; ++k) {
      if (k == i) continue;
      num = num * (s - (double)(-k));
      den = den * ((double)(-i) - (double)(-k));
    }
    w[i] = num / den;
  }
}

static int32_t bdf_corrected(const oracle_bdf_cfg* cfg, int32_t rhs, int32_t dim, const double* p,
                             const double* shared, double t0, double t_end, const double* y0,
                             double* y_out, double* t_out, int64_t* accepted, int64_t* rejected,
                             double* traj_t, double* traj_y, int64_t traj_cap) {
  const int n = dim;
  const int qmax = (cfg->method == ORC_BDF6) ? 6 : 2;
  static __thread double H[7][ORC_MAX_BDF_DIM], Hn[7][ORC_MAX_BDF_DIM];
  double pred[ORC_MAX_BDF_DIM], yh[ORC_MAX_BDF_DIM], yl[ORC_MAX_BDF_DIM], diff[ORC_MAX_BDF_DIM], w[8];
  double dt_min = cfg->dt_min, dt_max = cfg->dt_max;
  if (dt_min > dt_max) dt_min = dt_max;
  double t = t0, dt = (dt_max + dt_min) * 0.5;
  int k = 1; /* history points H[0..k-1], H[0] = y_n */
  memcpy(H[0], y0, sizeof(double) * n);
  memcpy(y_out, y0, sizeof(double) * n);
  *t_out = t0;
  *accepted = 0;
  *rejected = 0;
  if (t0 >= t_end) return ORC_TIME_END_OOB;
  int64_t steps = 0;
  while (t < t_end) {
    if (cfg->max_steps > 0 && steps >= cfg->max_steps) return ORC_MAX_ATTEMPTS_EXCEEDED;
    ++steps;
    double h = dt;
    if (t + h >= t_end) h = t_end - t;
    const int q = (k < qmax) ? k : qmax;
    /* The last step may be shorter than dt: interpolate the history onto
     * spacing h (points inside the stored window). */
    double (*HH)[ORC_MAX_BDF_DIM] = H;
    if (h != dt && k > 1) {
      const double ratio = h / dt;
      for (int j = 0; j < k; ++j) {
        lagrange_weights(k - 1, -ratio * (double)j, w);
        for (int d = 0; d < n; ++d) {
          double s = 0.0;
          for (int i = 0; i < k; ++i) s = s + (w[i] * H[i][d]);
          Hn[j][d] = s;
        }
      }
      HH = Hn;
    }
    /* predictor: extrapolation through the history points */
    lagrange_weights(k - 1, 1.0, w);
    for (int d = 0; d < n; ++d) {
      double s = 0.0;
      for (int i = 0; i < k; ++i) s = s + (w[i] * HH[i][d]);
      pred[d] = s;
    }
    const double t1 = t + h;
    int ok = corrected_newton(cfg, rhs, n, p, shared, t1, h, q, HH, pred, yh);
    double error;
    if (ok && q >= 2) {
      /* the reference's estimate: high-order minus lower-order solution */
      ok = corrected_newton(cfg, rhs, n, p, shared, t1, h, q - 1, HH, yh, yl);
      for (int d = 0; d < n; ++d) diff[d] = yh[d] - yl[d];
      error = oracle_norm(diff, n, cfg->dyn_dim);
    } else {
      /* order 1: half the gap between backward and forward Euler ~ h^2 y''/2 */
      double f0[ORC_MAX_BDF_DIM];
      oracle_rhs(rhs, n, t, H[0], p, shared, f0);
      for (int d = 0; d < n; ++d) diff[d] = 0.5 * (yh[d] - (H[0][d] + (h * f0[d])));
      error = oracle_norm(diff, n, cfg->dyn_dim);
    }
    if (ok && error <= cfg->tol) {
      /* accept: shift history */
      const int kk = (k < 7) ? k + 1 : 7;
      for (int i = kk - 1; i >= 1; --i) memcpy(H[i], H[i - 1], sizeof(double) * n);
      memcpy(H[0], yh, sizeof(double) * n);
      k = kk;
      t = t1;
      if (traj_t && *accepted < traj_cap) {
        traj_t[*accepted] = t;
        memcpy(traj_y + (size_t)(*accepted) * n, yh, sizeof(double) * n);
      }
      (*accepted)++;
      *t_out = t;
      memcpy(y_out, yh, sizeof(double) * n);
      if (h != dt) continue; /* end-clamped step: keep dt */
      if (error < 0.1 * cfg->tol && k == qmax + 1 && dt * 2.0 <= dt_max) {
        /* doubling: every second history point lies on the new grid */
        const int nk = (k + 1) / 2;
        for (int i = 1; i < nk; ++i) memcpy(H[i], H[2 * i], sizeof(double) * n);
        k = nk;
        dt = dt * 2.0;
      }
      continue;
    }
    (*rejected)++;
    /* halving: interpolate the history onto the finer grid */
    const double nd = dt * 0.5;
    if (nd < dt_min) return ORC_MINIMUM_TIME_DELTA_EXCEEDED;
    if (k > 1) {
      for (int j = 0; j < k; ++j) {
        lagrange_weights(k - 1, -0.5 * (double)j, w);
        for (int d = 0; d < n; ++d) {
          double s = 0.0;
          for (int i = 0; i < k; ++i) s = s + (w[i] * H[i][d]);
          Hn[j][d] = s;
        }
      }
      for (int j = 0; j < k; ++j) memcpy(H[j], Hn[j], sizeof(double) * n);
    }
    dt = nd;
  }
  return ORC_OK;
}

int32_t oracle_bdf_solve_one(const oracle_bdf_cfg* cfg, int32_t rhs, int32_t dim,
                             const double* p, const double* shared, double t0,
                             double t_end, const double* y0, double* y_out,
                             double* t_out, int64_t* accepted, int64_t* rejected,
                             double* traj_t, double* traj_y, int64_t traj_cap) {
  if (dim < 1 || dim > ORC_MAX_BDF_DIM) return ORC_MAX_ATTEMPTS_EXCEEDED + 2; /* invalid */
  if (cfg->mode == ORC_BDF_AS_COMPILED)
    return bdf_as_compiled(cfg, rhs, dim, p, shared, t0, t_end, y0, y_out, t_out, accepted, rejected,
                           traj_t, traj_y, traj_cap);
  return bdf_corrected(cfg, rhs, dim, p, shared, t0, t_end, y0, y_out, t_out, accepted, rejected,
                       traj_t, traj_y, traj_cap);
}

/* The corrected BDF's linear solve on its own (a test hook): A (row-major,
 * n x n, n <= 128) x = b.  Returns 1, or 0 on an exactly zero pivot. */
int oracle_corrected_linsolve(int32_t n, const double* A, const double* b, double* x) {
  static __thread dmat M;
  int piv[ORC_MAX_BDF_DIM];
  double rinv[ORC_MAX_BDF_DIM];
  if (n < 1 || n > ORC_MAX_BDF_DIM) return 0;
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < n; ++k) M[r][k] = A[r * n + k];
  if (!corrected_factor(n, M, piv, rinv)) return 0;
  for (int r = 0; r < n; ++r) x[r] = b[r];
  corrected_solve(n, M, piv, rinv, x);
  return 1;
}

/* The inverse secant takes (a test hook): A row-major n x n.  Returns 1 for
 * the partial-pivot LU, 2 for the full-pivot LU fallback, 3 for the QR
 * fallback, 0 when all three fail (SingularMatrix). */
int oracle_bdf_secant_inverse(int32_t n, const double* A, double* inv) {
  static __thread dmat M, R;
  if (n < 1 || n > ORC_MAX_BDF_DIM) return -1;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) M[r][c] = A[r * n + c];
  int which = 0;
  if (lu_try_inverse(M, n, R)) which = 1;
  else if (full_piv_lu_try_inverse(M, n, R)) which = 2;
  else if (qr_try_inverse(M, n, R)) which = 3;
  if (which)
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) inv[r * n + c] = R[r][c];
  return which;
}

