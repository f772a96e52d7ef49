/*
 * CPU ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the bacon-sci 0.16.2 IVP solvers (Rust crate
 * aftix/bacon) used to check the CUDA engine.  Only the test suite, the smoke
 * check and the CPU-baseline leg of the benchmark may load this library; the
 * product path never does.
 *
 * Parity status: the reference cannot be compiled here (it is Rust, and no
 * Rust toolchain is available), and its own tests pin no numeric values
 * beyond loose closed-form checks on right-hand sides that ignore y
 * (src/ivp/rk.rs:682-758).  The restatement is pinned against those
 * closed-form checks and against the published Fehlberg / Bogacki-Shampine
 * tableaux, but bit-level fidelity to the compiled reference is
 * "parity unpinned".
 *
 * Followed reference code (paths inside the aftix/bacon project):
 *   src/ivp.rs:214-238        IVPIterator::next (Redo / Done / Failure)
 *   src/ivp/rk.rs:249-343     RungeKutta::solve (constants, tableaux, dt0)
 *   src/ivp/rk.rs:361-423     RungeKuttaSolver::step (one attempt)
 *   src/ivp/rk.rs:430-526     RKCoefficients45
 *   src/ivp/rk.rs:563-621     RK23Coefficients
 *   src/ivp/bdf.rs:346-673    BDF runge_kutta / jac_finite_diff / secant / step
 */
#ifndef BACON_ORACLE_H
#define BACON_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: 0 = the iterator ended with Done; otherwise the IVPError
 * variant index in declaration order (src/ivp.rs:50-76) plus extensions.
 * Identical numbering to include/bacon_gb300.h. */
enum {
  ORC_OK = 0,
  ORC_MISSING_PARAMETERS = 1,
  ORC_USER_ERROR = 2,
  ORC_TOLERANCE_OOB = 3,
  ORC_TIME_DELTA_OOB = 4,
  ORC_TIME_END_OOB = 5,
  ORC_TIME_START_OOB = 6,
  ORC_FROM_PRIMITIVE_FAILURE = 7,
  ORC_MINIMUM_TIME_DELTA_EXCEEDED = 8,
  ORC_MAXIMUM_ITERATIONS_EXCEEDED = 9,
  ORC_SINGULAR_MATRIX = 10,
  ORC_DYNAMIC_ON_STATIC = 11,
  ORC_STATIC_ON_DYNAMIC = 12,
  ORC_MAX_ATTEMPTS_EXCEEDED = 13
};

/* Right-hand sides (same ids as BACON_RHS_* in include/bacon_gb300.h). */
enum {
  ORC_RHS_EXP = 0,        /* y' = y                          (src/ivp/bdf.rs:769) */
  ORC_RHS_DECAY = 1,      /* y' = -y                         (src/ivp/bdf.rs:781) */
  ORC_RHS_QUADRATIC = 2,  /* y' = -2 t                       (src/ivp/rk.rs:664) */
  ORC_RHS_SINE = 3,       /* y' = cos t                      (src/ivp/rk.rs:668) */
  ORC_RHS_HARMONIC = 4,   /* y0' = y1, y1' = -y0             (src/ivp.rs:527) */
  ORC_RHS_VDP = 5,        /* Van der Pol, p = (mu) */
  ORC_RHS_LORENZ = 6,     /* Lorenz-63, p = (sigma, rho, beta) */
  ORC_RHS_LOTKA = 7,      /* Lotka-Volterra, p = (a, b, c, d) */
  ORC_RHS_ROBERTSON = 8,  /* Robertson kinetics, p = (k1, k2, k3) */
  ORC_RHS_CHAIN = 9,      /* damped spring-mass chain, see oracle_rhs */
  ORC_RHS_LINEAR = 10     /* y' = A y with one shared dense A */
};

enum { ORC_RK45 = 0, ORC_RK23 = 1 };
/* Tableau variants.  as_compiled: the Butcher matrix as nalgebra's
 * column-major from_vec builds it (src/ivp/rk.rs:459, read with row_iter at
 * :370).  as_written: the matrix as the source literal is laid out, row by
 * row.  Both keep the literal 1859/4014 of rk.rs:499.  fehlberg: as_written
 * with that entry replaced by Fehlberg's 1859/4104 (the only variant whose
 * embedded error estimate is O(dt^5)).  RK23 has no such entry; its
 * fehlberg variant equals as_written. */
enum { ORC_LAYOUT_AS_COMPILED = 0, ORC_LAYOUT_AS_WRITTEN = 1, ORC_LAYOUT_FEHLBERG = 2 };
/* How (tol/err)^(1/4) is evaluated (src/ivp/rk.rs:400-401).  LIBM calls the
 * platform pow(), which is what Rust's f64::powf lowers to; QRT is the
 * deterministic IEEE-operation sequence the CUDA engine also executes. */
enum { ORC_POW_QRT = 0, ORC_POW_LIBM = 1 };

typedef struct {
  int32_t method;        /* ORC_RK45 / ORC_RK23 */
  int32_t layout;        /* ORC_LAYOUT_* */
  int32_t pow_mode;      /* ORC_POW_* */
  int32_t dyn_dim;       /* 1: nalgebra Dyn vector (norm summation order) */
  int64_t max_attempts;  /* extension: cap on step() attempts, 0 = none */
  double tol, dt_min, dt_max;
} oracle_rk_cfg;

/* Evaluate one right-hand side: f = rhs(t, y; p).  `shared` is the dense
 * matrix of ORC_RHS_LINEAR (row-major dim x dim), else unused. */
void oracle_rhs(int32_t rhs, int32_t dim, double t, const double* y,
                const double* p, const double* shared, double* f);

/* (x)^(1/4) as the CUDA engine computes it (see oracle_qrt in rk_oracle.c). */
double oracle_qrt(double x);

/* The vector norm of nalgebra 0.32 (norm_squared then sqrt). */
double oracle_norm(const double* x, int32_t n, int32_t dyn_dim);

/* Solve one system.  Returns the terminal status.  Outputs describe the path
 * the reference iterator yields: (t_out, y_out) is its last item (t0, y0 if
 * it yields none), `accepted` its length, `rejected` the number of Redo
 * results.  If traj_t is non-NULL the first traj_cap items are stored
 * (traj_y row-major [k][dim]). */
int32_t oracle_rk_solve_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                            const double* p, const double* shared, double t0,
                            double t_end, const double* y0, double* y_out,
                            double* t_out, int64_t* accepted, int64_t* rejected,
                            double* traj_t, double* traj_y, int64_t traj_cap);

/* Batched wrapper over oracle_rk_solve_one, SoA layout: y0[d*n+i],
 * params[k*n+i], y_out[d*n+i].  Systems are distributed over `threads`
 * POSIX threads with dynamic chunking.  Returns wall seconds. */
double oracle_rk_solve_batch(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                             int64_t n, int32_t n_params, const double* y0,
                             const double* params, const double* shared,
                             const double* t0, const double* t_end,
                             double* y_out, double* t_out, int64_t* accepted,
                             int64_t* rejected, int32_t* status,
                             int32_t threads);

/* ---- BDF (src/ivp/bdf.rs) ------------------------------------------------ */
enum { ORC_BDF6 = 0, ORC_BDF2 = 1 };
/* as_compiled: every quirk of src/ivp/bdf.rs kept (the + sign in the finite
 * difference, Broyden updates of an explicit inverse, f at t_n, lower residual
 * with higher-order history weights, the time jump on rejected bootstrap).
 * corrected: the fixed-leading-coefficient BDF pair the reference intends,
 * with a true Newton iteration (see bdf_oracle.c). */
enum { ORC_BDF_AS_COMPILED = 0, ORC_BDF_CORRECTED = 1 };

typedef struct {
  int32_t method;        /* ORC_BDF6 / ORC_BDF2 */
  int32_t mode;          /* ORC_BDF_* */
  int32_t dyn_dim;
  int32_t max_iter;      /* corrector iterations (reference: 1000) */
  int64_t max_steps;     /* extension: cap on step() calls, 0 = none */
  double tol, dt_min, dt_max;
} oracle_bdf_cfg;

/* Analytic Jacobian of a registry right-hand side, row-major dim x dim. */
int oracle_rhs_jacobian(int32_t rhs, int32_t dim, double t, const double* y, const double* p,
                        const double* shared, double* J);

int32_t oracle_bdf_solve_one(const oracle_bdf_cfg* cfg, int32_t rhs, int32_t dim,
                             const double* p, const double* shared, double t0,
                             double t_end, const double* y0, double* y_out,
                             double* t_out, int64_t* accepted, int64_t* rejected,
                             double* traj_t, double* traj_y, int64_t traj_cap);

/* The corrected BDF's linear solve on its own (a test hook): A (row-major,
 * n x n, n <= 128) x = b.  Returns 1, or 0 on an exactly zero pivot. */
int oracle_corrected_linsolve(int32_t n, const double* A, const double* b, double* x);
/* Work of the corrected BDF on the calling thread since the last reset:
 * out5 = {Newton solves, Newton iterations, factorisations needed at the
 * least (one per distinct h*b_q of a solve for the constant-Jacobian chains,
 * one per Newton solve otherwise), elimination FMAs executed (updates by an
 * exactly zero entry skipped), elimination FMAs of the dense LU}.  reset != 0
 * zeroes the counters. */
void oracle_bdf_work(int64_t* out5, int reset);
/* The inverse the as-compiled BDF's secant takes for a row-major n x n
 * matrix A: 1 partial-pivot LU, 2 full-pivot LU, 3 QR (src/ivp/bdf.rs:429-443),
 * 0 when all fail (SingularMatrix).  Test hook. */
int oracle_bdf_secant_inverse(int32_t n, const double* A, double* inv);

/* ---- Adams predictor-corrector and Euler (src/ivp/adams.rs, src/ivp.rs) -- */
typedef struct {
  int32_t order;         /* 5 (Adams5) or 3 (Adams3) */
  int32_t pow_mode;      /* ORC_POW_QRT: oracle_rootn; ORC_POW_LIBM: pow */
  int32_t dyn_dim;       /* 1: nalgebra Dyn vector (norm summation order) */
  int32_t reserved;
  int64_t max_attempts;  /* extension: cap on step() calls, 0 = none */
  double tol, dt_min, dt_max;
} oracle_adams_cfg;

/* x^(1/n), n = 3 or 5, as a fixed sequence of IEEE operations. */
double oracle_rootn(double x, int n);

int32_t oracle_adams_solve_one(const oracle_adams_cfg* cfg, int32_t rhs, int32_t dim,
                               const double* p, const double* shared, double t0,
                               double t_end, const double* y0, double* y_out,
                               double* t_out, int64_t* accepted, int64_t* rejected,
                               double* traj_t, double* traj_y, int64_t traj_cap);

int32_t oracle_euler_solve_one(int32_t rhs, int32_t dim, const double* p, const double* shared,
                               double dt, int64_t max_steps, double t0, double t_end,
                               const double* y0, double* y_out, double* t_out,
                               int64_t* accepted, double* traj_t, double* traj_y,
                               int64_t traj_cap);

/* ---- gradients (no reference counterpart; oracle for the adjoint) ------- */
/* Discrete adjoint of the accepted-step sequence of a forward solve (step
 * sizes frozen), loss = sum_d (y_T[d] - target[d])^2.  Fills dL/dy0[dim] and
 * dL/dp[n_params] and the loss.  Returns the forward status (-1 for the
 * as_compiled reading, which has no one-step map). */
int32_t oracle_rk_adjoint_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                              int32_t n_params, const double* p, double t0,
                              double t_end, const double* y0,
                              const double* target, double* loss,
                              double* dl_dy0, double* dl_dp, int32_t checkpoint_every);

/* Forward (tangent-linear) sensitivities of the same loss through the same
 * frozen step sequence; agrees with the adjoint up to rounding. */
int32_t oracle_rk_fwdsens_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                              int32_t n_params, const double* p, double t0,
                              double t_end, const double* y0,
                              const double* target, double* dl_dy0, double* dl_dp);

/* Same loss differentiated by replaying the forward run's accepted dt sequence
 * with perturbed inputs (frozen steps), central differences with step h. */
int32_t oracle_rk_frozen_fd_one(const oracle_rk_cfg* cfg, int32_t rhs, int32_t dim,
                                int32_t n_params, const double* p, double t0,
                                double t_end, const double* y0,
                                const double* target, double h, double* dl_dy0,
                                double* dl_dp);

#ifdef __cplusplus
}
#endif
#endif
