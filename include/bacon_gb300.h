/*
 * bacon_gb300 — C ABI of the GB300 (sm_103a) batched initial-value-problem
 * engine.  It replaces, for batches of independent systems, the solver API of
 * the Rust crate bacon-sci 0.16.2 (aftix/bacon):
 *
 *   IVPSolver builder trait            src/ivp.rs:134-190
 *   RungeKutta builder impl            src/ivp/rk.rs:118-344
 *   RungeKuttaSolver::step             src/ivp/rk.rs:361-423
 *   IVPIterator::next / collect_vec    src/ivp.rs:192-239
 *   BDF builder / BDFSolver::step      src/ivp/bdf.rs:124-332, :495-634
 *   Adams builder / AdamsSolver::step  src/ivp/adams.rs:134-334, :344-565
 *   Euler builder / EulerSolver::step  src/ivp.rs:240-485
 *   IVPError                           src/ivp.rs:50-76
 *
 * All entry points are plain C: pointers, sizes and status codes.  Every
 * function returns a bacon_status; bacon_last_error() gives a message for the
 * calling thread's last failure.  Calls on one bacon_ctx must not overlap
 * (the reference solvers are single-threaded objects, src/ivp.rs:102-125);
 * separate contexts may be used from separate threads.
 */
#ifndef BACON_GB300_H
#define BACON_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
/* 1..12 are the IVPError variants in declaration order (src/ivp.rs:50-76).
 * 13.. are extensions of the batched engine. */
typedef enum {
  BACON_OK = 0,
  BACON_MISSING_PARAMETERS = 1,
  BACON_USER_ERROR = 2,
  BACON_TOLERANCE_OOB = 3,
  BACON_TIME_DELTA_OOB = 4,
  BACON_TIME_END_OOB = 5,
  BACON_TIME_START_OOB = 6,
  BACON_FROM_PRIMITIVE_FAILURE = 7,
  BACON_MINIMUM_TIME_DELTA_EXCEEDED = 8,
  BACON_MAXIMUM_ITERATIONS_EXCEEDED = 9,
  BACON_SINGULAR_MATRIX = 10,
  BACON_DYNAMIC_ON_STATIC = 11,
  BACON_STATIC_ON_DYNAMIC = 12,
  /* A system reached the attempt cap.  The reference has no cap and loops
   * forever on a NaN error (rk.rs:392-421); the engine stops instead. */
  BACON_MAX_ATTEMPTS_EXCEEDED = 13,
  BACON_CUDA_ERROR = 14,
  BACON_INVALID_ARGUMENT = 15,
  BACON_UNSUPPORTED = 16,
  /* A system took more accepted steps than a fixed buffer holds: the
   * adjoint's step log, or a trajectory slab. */
  BACON_CAPACITY_EXCEEDED = 17
} bacon_status;

/* ---- right-hand sides --------------------------------------------------- */
/* The reference takes an arbitrary Rust closure (src/ivp.rs:34-48).  Device
 * code cannot call host closures, so the engine carries a registry of device
 * right-hand sides, each with per-system parameters (SoA). */
typedef enum {
  BACON_RHS_EXP = 0,        /* y' = y              any dim, 0 params       */
  BACON_RHS_DECAY = 1,      /* y' = -y             any dim, 0 params       */
  BACON_RHS_QUADRATIC = 2,  /* y' = -2 t           any dim, 0 params       */
  BACON_RHS_SINE = 3,       /* y' = cos t          any dim, 0 params       */
  BACON_RHS_HARMONIC = 4,   /* (y1, -y0)           dim 2,   0 params       */
  BACON_RHS_VDP = 5,        /* Van der Pol         dim 2,   (mu)           */
  BACON_RHS_LORENZ = 6,     /* Lorenz-63           dim 3,   (sigma,rho,beta) */
  BACON_RHS_LOTKA = 7,      /* Lotka-Volterra      dim 2,   (a,b,c,d)      */
  BACON_RHS_ROBERTSON = 8,  /* Robertson kinetics  dim 3,   (k1,k2,k3)     */
  BACON_RHS_CHAIN = 9,      /* spring-mass chain   dim 2n,  (k_0..k_{n-1}, c) */
  BACON_RHS_LINEAR = 10,    /* y' = A y, one shared dense A                */
  BACON_RHS_USER = 11       /* compiled by the caller: bacon_rk_solve_user */
} bacon_rhs;

/* ---- methods and variants ---------------------------------------------- */
typedef enum { BACON_RK45 = 0, BACON_RK23 = 1 } bacon_rk_method;

/* Butcher-matrix variants of the reference tableaux.
 * AS_COMPILED: nalgebra's from_vec fills column-major (src/ivp/rk.rs:459,
 *   :580) and the step reads row_iter (:370), so stage i uses column i of the
 *   literal — stage values from the previous attempt.
 * AS_WRITTEN: the literal read row by row.
 * FEHLBERG: AS_WRITTEN with the literal 1859/4014 (rk.rs:499) replaced by
 *   Fehlberg's 1859/4104.  For RK23 it equals AS_WRITTEN. */
typedef enum {
  BACON_LAYOUT_AS_COMPILED = 0,
  BACON_LAYOUT_AS_WRITTEN = 1,
  BACON_LAYOUT_FEHLBERG = 2
} bacon_layout;

/* FP64_EXACT: every product and sum separately rounded in the reference's
 *   order (bit-identical to the CPU restatement).  FP64_FMA: same algorithm,
 *   products and sums contracted into fused multiply-adds.  FP32_COMP: stages
 *   in single precision with compensated (error-free) accumulation of y and of
 *   the error vector; error norm and step control in FP64. */
typedef enum {
  BACON_FP64_EXACT = 0,
  BACON_FP64_FMA = 1,
  BACON_FP32_COMP = 2,
  /* BACON_RHS_LINEAR only: the products A^k y an attempt needs, as GEMMs on
   * the tcgen05 tensor cores: bf16 integer slices of A and of the vectors
   * (5 x 8 bits, Ozaki splitting) with FP32 accumulation, exact on the
   * three leading diagonals, combined in FP64; relative error ~ 2^-39. */
  BACON_TC_SPLIT = 3
} bacon_precision;

typedef enum { BACON_MEM_DEVICE = 0, BACON_MEM_HOST = 1 } bacon_memory;

/* ---- context ----------------------------------------------------------- */
typedef struct bacon_ctx bacon_ctx;

/* Create a context on CUDA device `device`: a stream, the scratch buffers of
 * the work queue, the autotune cache and the CUDA-graph cache. */
int bacon_ctx_create(int device, bacon_ctx** out);
int bacon_ctx_destroy(bacon_ctx* ctx);
/* Message of the calling thread's last failed call ("" if none). */
const char* bacon_last_error(void);
/* Number of kernels the context launched since creation (diagnostics). */
int64_t bacon_ctx_kernel_launches(const bacon_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or events after the engine's. */
int bacon_ctx_stream(const bacon_ctx* ctx, void** stream);
/* Device time in milliseconds of the last solve's main integration kernel,
 * from CUDA events recorded around it on the context's stream. */
int bacon_ctx_last_kernel_ms(const bacon_ctx* ctx, double* ms);
/* Test hook, no counterpart in the reference: makes the context's next
 * solves take a failure path on purpose, so that tests can check how it is
 * reported.  BACON_FAULT_TC_WITHHOLD: the tensor-core stage GEMM
 * (BACON_TC_SPLIT) never signals that its accumulators are ready, so its
 * epilogue's bounded wait runs out after ~10 ms; the solve returns
 * BACON_CUDA_ERROR and the context stays usable.  BACON_FAULT_NONE turns it
 * off.  Nothing faults or hangs the GPU. */
typedef enum { BACON_FAULT_NONE = 0, BACON_FAULT_TC_WITHHOLD = 1 } bacon_fault;
int bacon_ctx_set_fault_injection(bacon_ctx* ctx, int kind);

/* ---- batch description -------------------------------------------------- */
/* One solve of n independent systems of dimension `dim`.  All arrays are SoA
 * (component-major): y0[d*n + i], params[k*n + i].  t0 / t_end may be NULL, in
 * which case the scalars apply to every system (the reference builder takes
 * scalars, src/ivp/rk.rs:212-234; per-system arrays are the batched
 * extension for uneven end times). */
typedef struct {
  int64_t n;
  int32_t dim;
  int32_t rhs;            /* bacon_rhs */
  int32_t n_params;
  int32_t dyn_dim;        /* 1: systems are nalgebra Dyn vectors (norm order) */
  const double* y0;       /* [dim][n] */
  const double* params;   /* [n_params][n] or NULL */
  const double* t0;       /* [n] or NULL */
  const double* t_end;    /* [n] or NULL */
  const double* shared;   /* BACON_RHS_LINEAR: row-major dim x dim, else NULL */
  double t0_scalar;
  double t_end_scalar;
  double tol;             /* with_tolerance        (rk.rs:168-174) */
  double dt_min;          /* with_minimum_dt       (rk.rs:197-210) */
  double dt_max;          /* with_maximum_dt       (rk.rs:179-192) */
} bacon_problem;

typedef struct {
  int32_t method;         /* bacon_rk_method */
  int32_t layout;         /* bacon_layout */
  int32_t precision;      /* bacon_precision */
  int32_t memory;         /* bacon_memory: where every array lives */
  int64_t max_attempts;   /* cap on attempts per system, 0 = 10,000,000 */
  int32_t block;          /* threads per block, 0 = autotuned */
  int32_t blocks_per_sm;  /* persistent CTAs per SM, 0 = autotuned */
  int32_t use_graph;      /* 1: launch through a cached CUDA graph */
  /* Work order of the persistent kernel: 0 = longest span first when the
   * systems have per-system start or end times, index order otherwise;
   * 1 = index order; 2 = longest span first. */
  int32_t schedule;
  /* Systems a warp integrates at a time, 1..32 (the others of its lanes
   * idle); 0 = 32, or the autotuned count.  Fewer than 32 pays only for a
   * batch too small to fill the GPU, by cutting divergence within warps. */
  int32_t systems_per_warp;
  int32_t reserved;
} bacon_rk_options;

/* Outputs, same memory kind as the inputs.  (t_final, y_final) is the last
 * item the reference iterator would yield ((t0, y0) if none); `accepted` is
 * the number of items it yields, `rejected` the number of Redo results
 * (src/ivp.rs:227-237); status is 0 when the iterator ended with Done, else
 * the error it returned.  traj_t/traj_y (optional, NULL to skip) receive the
 * yielded items per system: traj_t[i*cap + k], traj_y[(i*cap + k)*dim + d];
 * a system with more than traj_cap items ends with BACON_CAPACITY_EXCEEDED
 * when the next one would not fit (see bacon_rk_solve_dense for a packed
 * stream sized to the steps each system takes). */
typedef struct {
  double* y_final;        /* [dim][n] */
  double* t_final;        /* [n] */
  int32_t* accepted;      /* [n] */
  int32_t* rejected;      /* [n] */
  int32_t* status;        /* [n] */
  double* traj_t;         /* [n][traj_cap] or NULL */
  double* traj_y;         /* [n][traj_cap][dim] or NULL */
  int32_t traj_cap;
  int32_t reserved;
} bacon_rk_result;

/* Batched RungeKutta45 / RungeKutta23 solve (persistent kernel).  Returns
 * BACON_OK if every system ended with Done, otherwise the status of the
 * lowest-index system that failed (per-system codes are in result->status),
 * or an argument / CUDA error.  Replaces RungeKutta::solve + collect_vec
 * (src/ivp/rk.rs:249-343, src/ivp.rs:209-211) for each system. */
int bacon_rk_solve(bacon_ctx* ctx, const bacon_problem* problem,
                   const bacon_rk_options* options, bacon_rk_result* result);

/* Autotuner: runs bacon_rk_solve on this batch with each candidate launch
 * shape (threads per block x persistent CTAs per SM), times the integration
 * kernel with CUDA events, and caches the fastest in the context for this
 * kernel and batch size (rounded to a power of two).  Later solves that leave
 * block and blocks_per_sm at 0 use it; without tuning an occupancy model
 * applies.  The result arrays receive the last candidate's (identical)
 * outputs. */
int bacon_rk_autotune(bacon_ctx* ctx, const bacon_problem* problem,
                      const bacon_rk_options* options, bacon_rk_result* result,
                      int32_t* best_block, int32_t* best_blocks_per_sm);

/* What the autotuner chose for a batch, and what it measured.  The
 * persistent kernels keep a system on one lane: the FP64 pipe charges a warp
 * instruction the same time however few lanes are active, so splitting a
 * system across lanes multiplies its FP64 time.  The choices are the
 * register budget (kernel variant), the launch shape and, for a batch too
 * small to fill the GPU, the systems per warp (32, 16 or 8). */
typedef struct {
  int32_t variant;          /* 0: default kernel; 1, 2: register-capped variants */
  int32_t max_registers;    /* the variant's budget per thread, 0 = the compiler's */
  int32_t systems_per_warp; /* lanes per warp that take systems */
  int32_t block;            /* threads per block */
  int32_t blocks_per_sm;    /* persistent CTAs per SM */
  int32_t candidates;       /* (variant, shape) pairs timed */
  double best_ms;           /* integration-kernel time of the choice */
  double default_ms;        /* same without tuning (occupancy model, variant 0) */
} bacon_tune_result;

/* bacon_rk_autotune over register budgets as well as launch shapes: times
 * the default kernel and, where compiled (RKF45 fehlberg reading, Van der
 * Pol / Lorenz-63 / Lotka-Volterra, FP64_EXACT and FP32_COMP), the variants
 * capped at 80 and 64 registers per thread, each at several shapes, and
 * caches the fastest (variant, shape) in the context for this kernel and
 * batch size.  Results of every variant are bit-identical. */
int bacon_rk_autotune_ex(bacon_ctx* ctx, const bacon_problem* problem, const bacon_rk_options* options,
                         bacon_rk_result* result, bacon_tune_result* tuned);
/* Stores a tuning (variant, block, blocks_per_sm of `tuned`) in the context's
 * cache for this kernel and batch size, as the autotuner would: a choice
 * kept from an earlier run applies without timing again. */
int bacon_rk_set_tuned(bacon_ctx* ctx, const bacon_problem* problem, const bacon_rk_options* options,
                       const bacon_tune_result* tuned);

/* The same solve with the plain one-launch-per-attempt GPU baseline (state,
 * t and dt in HBM, host loop until every system is done).  Same results. */
int bacon_rk_solve_plain(bacon_ctx* ctx, const bacon_problem* problem,
                         const bacon_rk_options* options,
                         bacon_rk_result* result);

/* ---- right-hand sides compiled by the caller ------------------------------ */
/* The reference's derivative is any Rust closure (src/ivp.rs:34-48).  The
 * registry above covers the benchmark's systems; any other right-hand side
 * is compiled by the caller into the same persistent kernel: a device functor
 * (dimension, parameter count, eval) in a .cu file that includes
 * include/bacon_gb300_rhs.cuh, which defines a launcher with
 * BACON_DEFINE_RK_LAUNCHER.  The engine does everything around the launch
 * (staging, longest-first order, counters, results, status) and calls the
 * launcher on its stream with the kernel's arguments.
 *
 * bacon_rk_kernel_args is the persistent kernel's argument block, field for
 * field (bacon_gb300/csrc/rk_kernel.cuh RkArgs); the launcher passes it on
 * unchanged. */
typedef struct {
  int64_t n;
  const double* y0;
  const double* params;
  const double* t0;
  const double* t_end;
  double t0_s, t_end_s;
  double tol, dt_min, dt_max;
  int64_t max_attempts;
  double* y_out;
  double* t_out;
  int32_t* accepted;
  int32_t* rejected;
  int32_t* status;
  double* traj_t;
  double* traj_y;
  int32_t traj_cap;
  const int64_t* traj_off;
  unsigned long long* queue;
  unsigned long long* first_fail;
  const uint32_t* order;
  double* dt_log;
  double* ckpt;
  int32_t ckpt_every;
  int32_t max_steps;
  int32_t ckpt_slots;
  int32_t lanes;
} bacon_rk_kernel_args;

/* Launches the caller's kernel for (method, layout, precision) with `grid`
 * CTAs of `block` threads on `stream` (a cudaStream_t).  Returns BACON_OK,
 * BACON_UNSUPPORTED when that combination was not compiled, or
 * BACON_CUDA_ERROR. */
typedef int (*bacon_rk_launch_fn)(const bacon_rk_kernel_args* args, int32_t method, int32_t layout,
                                  int32_t precision, int32_t grid, int32_t block, void* stream, void* user);

/* bacon_rk_solve for problem->rhs == BACON_RHS_USER: problem->dim and
 * n_params describe the caller's functor; its kernel runs through `launch`
 * (`user` is passed through).  options->block / blocks_per_sm set the launch
 * shape (0: 128 threads, 2 CTAs per SM).  Same results, statuses and
 * trajectory slabs as bacon_rk_solve. */
int bacon_rk_solve_user(bacon_ctx* ctx, const bacon_problem* problem, const bacon_rk_options* options,
                        bacon_rk_result* result, bacon_rk_launch_fn launch, void* user);

/* ---- BDF (src/ivp/bdf.rs) ------------------------------------------------ */
typedef enum { BACON_BDF6 = 0, BACON_BDF2 = 1 } bacon_bdf_method;
/* AS_COMPILED: the reference's BDFSolver::step (bdf.rs:495-634) with every
 *   quirk of 0.16.2 kept (RK4 bootstrap, yield machine, f at t_n, the "+"
 *   finite-difference Jacobian, Broyden updates of an explicit LU inverse, the
 *   lower residual with the higher-order history weights, t -= dt - order on
 *   a rejected bootstrap).  On the reference's own test problems it yields no
 *   items; on Robertson it stops with MaximumIterationsExceeded.
 * CORRECTED: the engine's stiff BDF: orders 1..6 ramped up implicitly, f at
 *   t_{n+1}, Newton with the analytic Jacobian and partial-pivot LU, the
 *   reference's error estimate ||y_q - y_{q-1}|| and dt control. */
typedef enum { BACON_BDF_AS_COMPILED = 0, BACON_BDF_CORRECTED = 1 } bacon_bdf_mode;

typedef struct {
  int32_t method;         /* bacon_bdf_method */
  int32_t mode;           /* bacon_bdf_mode */
  int32_t memory;         /* bacon_memory */
  int32_t max_iter;       /* corrector iterations; 0 = 1000 (as_compiled, the
                             reference's bound, bdf.rs:449) or 8 (corrected) */
  int64_t max_steps;      /* cap on step() calls per system, 0 = 10,000,000 */
  int32_t block;          /* 0 = 128 */
  int32_t blocks_per_sm;  /* 0 = occupancy model */
} bacon_bdf_options;

/* Batched BDF6 / BDF2 solve of systems with dim <= 8 (one system per
 * thread).  Same result semantics as bacon_rk_solve (rejected = Redo count). */
int bacon_bdf_solve(bacon_ctx* ctx, const bacon_problem* problem,
                    const bacon_bdf_options* options, bacon_rk_result* result);

/* ---- Adams predictor-corrector and Euler (src/ivp/adams.rs, src/ivp.rs) -- */
typedef struct {
  int32_t order;          /* 5 (Adams5) or 3 (Adams3); ignored by Euler */
  int32_t memory;         /* bacon_memory */
  int64_t max_attempts;   /* cap on step() calls per system, 0 = 10,000,000 */
  int32_t block;          /* 0 = 128 */
  int32_t blocks_per_sm;  /* 0 = occupancy model */
  /* Systems per warp, 1..32 (0 = model).  Each lane runs its system's
   * steps in order and the lanes of a warp are in different phases of the
   * reference's step, so a warp iteration costs the union of its lanes'
   * paths.  Fewer systems per warp shorten that union; more fill the FP64
   * pipe.  The model takes 32 when the batch fills the GPU and fewer for
   * small batches. */
  int32_t systems_per_warp;
  int32_t reserved;
} bacon_adams_options;

/* Batched Adams5 / Adams3 (AdamsSolver::step, src/ivp/adams.rs:411-565, with
 * its RK4 bootstrap :344-395 and the iterator of src/ivp.rs:214-238), one
 * system per thread.  dt0 = (dt_max + dt_min) / 2 (adams.rs:310).  The step
 * factor (tol / (2 err))^(1/O) is x^RN(1/O) evaluated by a fixed IEEE
 * operation sequence (correctly rounded except within ~2^-50 ulp of a
 * midpoint).  Same result semantics as bacon_rk_solve: the last yielded item,
 * accepted = items yielded, rejected = Redo count.  RHS: EXP/DECAY (dim 1,
 * 2), QUADRATIC, SINE (dim 1), HARMONIC, VDP, LORENZ, LOTKA. */
int bacon_adams_solve(bacon_ctx* ctx, const bacon_problem* problem,
                      const bacon_adams_options* options, bacon_rk_result* result);

/* Batched Euler (EulerSolver::step, src/ivp.rs:318-339) with the builder's
 * step dt (with_maximum_dt / with_minimum_dt: the first value set, then the
 * mean with each later one, src/ivp.rs:395-423).  The iterator yields the
 * state each step starts from, so the last yielded item is the state at the
 * start of the final step.  problem->tol, dt_min and dt_max are unused. */
int bacon_euler_solve(bacon_ctx* ctx, const bacon_problem* problem, double dt,
                      const bacon_adams_options* options, bacon_rk_result* result);

/* A batch of systems of one right-hand side whose sizes differ.  System i's
 * state is y0[y_offsets[i] .. y_offsets[i+1]) and its parameters
 * params[p_offsets[i] .. p_offsets[i+1]).  In the reference each is its own
 * solver over a DVector state (bdf.rs:257-333 builds one per system), so norms
 * take nalgebra's dynamic-vector order.  Right-hand sides: BACON_RHS_CHAIN
 * (dim 2 m_i for m_i = 1..64 masses, m_i + 1 parameters: k_1..k_{m_i}, c). */
typedef struct {
  int64_t n;
  int32_t rhs;
  int32_t reserved;
  const int64_t* y_offsets; /* [n+1], y_offsets[0] = 0 */
  const int64_t* p_offsets; /* [n+1], p_offsets[0] = 0 */
  const double* y0;         /* [y_offsets[n]] */
  const double* params;     /* [p_offsets[n]] */
  const double* t0;         /* [n] or NULL: t0_scalar */
  const double* t_end;      /* [n] or NULL: t_end_scalar */
  double t0_scalar, t_end_scalar;
  double tol, dt_min, dt_max;
} bacon_ragged_problem;

typedef struct {
  double* y_final;   /* [y_offsets[n]] last yielded state */
  double* t_final;   /* [n] */
  int32_t* accepted; /* [n] */
  int32_t* rejected; /* [n] */
  int32_t* status;   /* [n] */
} bacon_ragged_result;

/* Checks a ragged batch whose offsets are host arrays: rhs CHAIN, offsets
 * from 0, every dim even in 2..128 with dim/2 + 1 parameters, tol > 0, dt
 * bounds > 0.  BACON_OK or BACON_INVALID_ARGUMENT / BACON_UNSUPPORTED. */
int bacon_ragged_validate(const bacon_ragged_problem* problem);

/* One launch of the corrected BDF (BDF6 / BDF2) over a stiff batch of two
 * parts: a uniform batch of small systems (one thread each, as
 * bacon_bdf_solve; uniform rhs ROBERTSON or VDP) and a ragged batch (one warp
 * each, largest first; LU factors in a per-warp device workspace).  Either
 * part may be NULL, not both.  Same memory kind for every array
 * (options->memory).  Results are bit-identical to solving each system alone
 * with the corrected BDF.  Returns BACON_OK or the status of the lowest
 * failing ragged system, else of the lowest failing uniform system. */
int bacon_bdf_solve_mixed(bacon_ctx* ctx, const bacon_problem* uniform,
                          const bacon_ragged_problem* ragged,
                          const bacon_bdf_options* options,
                          bacon_rk_result* uniform_result,
                          bacon_ragged_result* ragged_result);

/* ---- dense output --------------------------------------------------------- */
/* Every item the reference iterator yields, for every system: the batched
 * counterpart of collect_vec (src/ivp.rs:209-238), which returns each
 * accepted (t, y).  The items are packed into one stream with CSR offsets:
 * system i's items, in yield order, are t[k] and y[k*dim .. (k+1)*dim) for k
 * in [offsets[i], offsets[i+1]), so memory follows the steps each system
 * takes, not n times the longest.  Same memory kind as the problem. */
typedef struct {
  int64_t capacity;  /* items t and y can hold (0: only count) */
  double* t;         /* [capacity] */
  double* y;         /* [capacity][dim] */
  int64_t* offsets;  /* [n+1], written by the call */
  int64_t total;     /* out: items of the whole batch, offsets[n] */
} bacon_dense_output;

/* bacon_rk_solve / bacon_bdf_solve / bacon_adams_solve / bacon_euler_solve
 * with dense output.
 * Two passes: the first solve counts each system's items, an exclusive scan
 * of the counts gives the offsets, and a second solve (bit-identical to the
 * first) writes each item to its slot.  If total > capacity the call returns
 * BACON_CAPACITY_EXCEEDED after the first pass with `total`, `offsets` and
 * the per-system results filled and t / y untouched: allocate `total` items
 * and call again.  result->traj_t / traj_y must be NULL.  The fixed per-system
 * slabs of bacon_rk_result (traj_t, traj_cap) remain; a system whose slab is
 * full ends with BACON_CAPACITY_EXCEEDED instead of dropping items.  For
 * BACON_RHS_LINEAR the items come from the lock-step engine's control kernel
 * (every precision, BACON_TC_SPLIT included). */
int bacon_rk_solve_dense(bacon_ctx* ctx, const bacon_problem* problem, const bacon_rk_options* options,
                         bacon_rk_result* result, bacon_dense_output* dense);
int bacon_bdf_solve_dense(bacon_ctx* ctx, const bacon_problem* problem, const bacon_bdf_options* options,
                          bacon_rk_result* result, bacon_dense_output* dense);
int bacon_adams_solve_dense(bacon_ctx* ctx, const bacon_problem* problem, const bacon_adams_options* options,
                            bacon_rk_result* result, bacon_dense_output* dense);
int bacon_euler_solve_dense(bacon_ctx* ctx, const bacon_problem* problem, double dt,
                            const bacon_adams_options* options, bacon_rk_result* result,
                            bacon_dense_output* dense);

/* Dense output of the ragged part of a mixed batch: system i's items are
 * t[offsets[i] .. offsets[i+1]) and its states, dim_i values each, are
 * y[value_offsets[i] .. value_offsets[i+1]) (item k from
 * value_offsets[i] + k * dim_i).  Memory kind as the batch. */
typedef struct {
  int64_t capacity;        /* items t can hold */
  int64_t value_capacity;  /* doubles y can hold */
  double* t;               /* [capacity] */
  double* y;               /* [value_capacity] */
  int64_t* offsets;        /* [n+1], written by the call */
  int64_t* value_offsets;  /* [n+1], written by the call */
  int64_t total;           /* out: items of the ragged part */
  int64_t total_values;    /* out: doubles of the ragged part */
} bacon_ragged_dense_output;

/* bacon_bdf_solve_mixed with dense output, in the same two passes as
 * bacon_rk_solve_dense.  uniform_dense / ragged_dense may be NULL: that
 * part's items are then not recorded.  BACON_CAPACITY_EXCEEDED after the
 * first pass, with the totals and offsets filled, when either part's
 * capacity is short. */
int bacon_bdf_solve_mixed_dense(bacon_ctx* ctx, const bacon_problem* uniform, const bacon_ragged_problem* ragged,
                                const bacon_bdf_options* options, bacon_rk_result* uniform_result,
                                bacon_ragged_result* ragged_result, bacon_dense_output* uniform_dense,
                                bacon_ragged_dense_output* ragged_dense);

/* ---- discrete adjoint ---------------------------------------------------- */
/* Gradient of L_i = sum_d (y_i(T)[d] - target_i[d])^2 for every system i with
 * respect to its initial state and parameters, through the accepted-step
 * sequence of the forward solve (step sizes held fixed: the gradient of the
 * discrete map).  The reference has no gradient entry point; this is the
 * batched `solve_ivp_adjoint`.  The forward pass logs each accepted dt and
 * checkpoints (t, y) every `checkpoint_every` accepted steps; the backward
 * pass replays each segment from its checkpoint and sweeps it in reverse.
 * Same memory kind as the problem.  Tableau layouts AS_WRITTEN / FEHLBERG,
 * FP64_EXACT only. */
typedef struct {
  const double* target;     /* [dim][n] */
  double* loss;             /* [n] */
  double* dl_dy0;           /* [dim][n] */
  double* dl_dp;            /* [n_params][n], NULL when n_params == 0 */
  int32_t checkpoint_every; /* accepted steps per checkpoint, 1..32; 0 = 32 */
  int32_t max_steps;        /* accepted steps logged per system; 0 = 1024 */
} bacon_adjoint;

int bacon_rk_solve_adjoint(bacon_ctx* ctx, const bacon_problem* problem,
                           const bacon_rk_options* options, bacon_rk_result* result,
                           bacon_adjoint* adjoint);
/* Device time in milliseconds of the last adjoint's reverse kernel. */
int bacon_ctx_last_reverse_ms(const bacon_ctx* ctx, double* ms);

/* ---- allocation-free solve ------------------------------------------------ */
/* No counterpart in the reference.  The batched solve of bacon_rk_solve for
 * callers that cannot allocate device memory: a library inside an application
 * whose memory pool has reserved the GPU's memory, a hot loop where an
 * allocation's latency or failure is not acceptable, or plugin code that holds
 * only a stream and device pointers.  It needs no bacon_ctx and calls no
 * cudaMalloc, cudaFree or other allocating routine: its scratch (work
 * counter, lowest-failing-index slot, longest-first order) is one fixed device
 * array of about 4 MiB inside the library, which every GPU that loads the
 * library holds until the process exits.
 *   - options->memory must be BACON_MEM_DEVICE (every array on the device);
 *     use_graph is ignored.
 *   - At most 1,048,576 systems: a larger n returns BACON_CAPACITY_EXCEEDED
 *     before any GPU work.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.  The CUDA runtime loads device code
 *     lazily, so that first call is also what places the array and the
 *     kernel on the device: make it before the caller's memory pool
 *     reserves the GPU's memory.  A call with n == 0 does only this set-up
 *     (for the kernel its options select) and is the cheap way to do it.
 *   - The device address is kept for the life of the process; calls must
 *     not span a cudaDeviceReset.
 *   - All calls share the one array, which keeps the last call's contents;
 *     each call resets what must start at zero.  Calls whose GPU work overlaps
 *     (other host threads or streams) race on it: serialize them.
 *   - `stream` is a cudaStream_t (NULL: the legacy default stream).  The call
 *     returns once the solve has finished; outputs as for bacon_rk_solve.
 *   - Failures are reported through the return code only; bacon_last_error()
 *     is not updated, because composing a message would allocate. */
int bacon_rk_solve_noalloc(const bacon_problem* problem, const bacon_rk_options* options,
                           bacon_rk_result* result, void* stream);

/* Validate a problem the way the reference builder does (rk.rs:168-256):
 * tolerance, dt bounds, start/end order, missing parameters.  No GPU work. */
int bacon_rk_validate(const bacon_problem* problem);

/* ---- builder (mirrors the IVPSolver trait, src/ivp.rs:134-190) ---------- */
typedef struct bacon_builder bacon_builder;

/* kind: 0 = RungeKutta45, 1 = RungeKutta23, 2 = BDF6, 3 = BDF2, 4 = Adams5,
 * 5 = Adams3, 6 = Euler.  bacon_builder_new mirrors IVPSolver::new (static
 * dimension `dim`); bacon_builder_new_dyn mirrors new_dyn(size).  For Euler,
 * with_tolerance is a no-op and with_maximum_dt / with_minimum_dt set one
 * step size (the first value, then the mean with each later one,
 * src/ivp.rs:389-423); bacon_builder_problem then puts that step in dt_min
 * and dt_max. */
int bacon_builder_new(int32_t kind, int32_t dim, bacon_builder** out);
int bacon_builder_new_dyn(int32_t kind, int32_t size, bacon_builder** out);
void bacon_builder_free(bacon_builder* b);
int bacon_builder_with_tolerance(bacon_builder* b, double tol);
int bacon_builder_with_maximum_dt(bacon_builder* b, double max);
int bacon_builder_with_minimum_dt(bacon_builder* b, double min);
int bacon_builder_with_initial_time(bacon_builder* b, double initial);
int bacon_builder_with_ending_time(bacon_builder* b, double ending);
/* Batched initial conditions, SoA [dim][n] (with_initial_conditions_slice
 * for n systems at once). */
int bacon_builder_with_initial_conditions(bacon_builder* b, const double* y0, int64_t n);
/* with_derivative: a registry right-hand side plus per-system parameters. */
int bacon_builder_with_derivative(bacon_builder* b, int32_t rhs, const double* params,
                                  int32_t n_params);
/* Batched extension: per-system end times (host array of n). */
int bacon_builder_with_ending_times(bacon_builder* b, const double* t_end, int64_t n);
/* Fill a bacon_problem from the builder (MissingParameters if incomplete,
 * rk.rs:250-256).  Pointers in the problem alias the builder's host copies. */
int bacon_builder_problem(const bacon_builder* b, bacon_problem* out);

/* ---- diagnostics --------------------------------------------------------- */
/* Measured FP64 fused-multiply-add throughput of the current device in
 * GFLOP/s (2 flops per DFMA), from a register-resident microbenchmark. */
int bacon_measure_fp64_peak(bacon_ctx* ctx, double* gflops);

#ifdef __cplusplus
}
#endif
#endif
