// C ABI of the engine: contexts, the builder mirror, validation, and the
// host side of the batched solves (staging, launch configuration, CUDA-graph
// cache).  See include/bacon_gb300.h for the reference interfaces replaced.
#include "bacon_gb300.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "adams.h"
#include "adams_kernel.cuh"
#include "bdf.h"
#include "linear.cuh"
#include "linear.h"
#include "linear_tc.cuh"
#include "bdf_kernel.cuh"
#include "bdf_ragged.cuh"
#include "order.h"
#include "plain.h"
#include "registry.h"
#include "rk_adjoint.cuh"
#include <nvtx3/nvToolsExt.h>

namespace bacon {
double measure_fp64_fma_gflops(cudaStream_t stream, int num_sms);
}

namespace {
// An NVTX range around each public solve, so a profiler's timeline (or
// `ncu --nvtx --nvtx-include`) can attribute kernels to the call that
// launched them.  NVTX is header-only and costs nothing without a tool.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
}  // namespace

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define BACON_CUDA(expr)                                                                     \
  do {                                                                                       \
    cudaError_t e_ = (expr);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail(BACON_CUDA_ERROR, std::string(#expr) + ": " + cudaGetErrorString(e_));    \
  } while (0)

// Grow-only device allocation owned by a context.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

uint64_t fnv1a(const void* data, size_t len, uint64_t h = 1469598103934665603ull) {
  const unsigned char* b = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < len; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

int expected_dim(int rhs) {
  switch (rhs) {
    case BACON_RHS_HARMONIC:
    case BACON_RHS_VDP:
    case BACON_RHS_LOTKA:
      return 2;
    case BACON_RHS_LORENZ:
    case BACON_RHS_ROBERTSON:
      return 3;
    default:
      return -1;  // any
  }
}

int expected_params(int rhs, int dim) {
  switch (rhs) {
    case BACON_RHS_VDP: return 1;
    case BACON_RHS_LORENZ: return 3;
    case BACON_RHS_LOTKA: return 4;
    case BACON_RHS_ROBERTSON: return 3;
    case BACON_RHS_CHAIN: return dim / 2 + 1;
    default: return 0;
  }
}

}  // namespace

struct bacon_ctx {
  int device = 0;
  int fault_injection = BACON_FAULT_NONE;  // bacon_ctx_set_fault_injection
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  // [0] work counter [1] first failing index [2] live [3] adjoint queue /
  // tensor-core error flag [5] first failing ragged index [8..11] ragged work
  // counters, one per size class
  unsigned long long* d_ctl = nullptr;
  unsigned long long* h_ctl = nullptr;  // pinned mirror
  std::vector<bacon::RkEntry> kernels;
  DevBuf in_y0, in_params, in_t0, in_tend, out_y, out_t, out_acc, out_rej, out_st, out_tt, out_ty;
  DevBuf pl_y, pl_K, pl_t, pl_dt, pl_end, pl_att, pl_acc, pl_rej, pl_st;
  DevBuf ord, ord_scratch;  // longest-first work order and its sort scratch
  struct Graph {
    cudaGraphExec_t exec = nullptr;
  };
  std::unordered_map<uint64_t, Graph> graphs;
  // Autotuned launch per (kernel, batch size): kernel variant, threads per
  // block, persistent CTAs per SM, systems per warp (0: 32).
  struct Tuned {
    int variant, block, bps, lanes;
  };
  std::unordered_map<uint64_t, Tuned> tuned;
  int force_variant = -1;  // set by the autotuner while it times a variant
  int64_t launches = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // around the last main kernel
  bool ev_valid = false;
  cudaEvent_t ev2 = nullptr, ev3 = nullptr;  // around the last adjoint reverse kernel
  bool rev_valid = false;
  std::vector<bacon::AdjEntry> adjoint_kernels;
  std::vector<bacon::BdfEntry> bdf_kernels;
  std::vector<bacon::AdamsEntry> adams_kernels;
  DevBuf adj_dt, adj_ck, adj_tgt, adj_loss, adj_gy, adj_gp;
  DevBuf lin_A, lin_y, lin_K, lin_t, lin_dt, lin_end, lin_att;
  DevBuf tc_sa, tc_ea, tc_sy, tc_ey;
  DevBuf rg_yoff, rg_poff, rg_y0, rg_p, rg_t0, rg_te, rg_yout, rg_tout, rg_acc, rg_rej, rg_st, rg_ord, rg_lu;
  // Packed dense output: while dense_off is set, the solves write every
  // yielded item of system i to [dense_off[i], dense_off[i+1]) of the device
  // streams dense_t / dense_y (the second pass of the *_solve_dense calls).
  const int64_t* dense_off = nullptr;
  double* dense_t = nullptr;
  double* dense_y = nullptr;
  // the same for the ragged part of bacon_bdf_solve_mixed: item offsets and
  // value offsets (items x each system's dimension)
  const int64_t* rg_dense_off = nullptr;
  const int64_t* rg_dense_voff = nullptr;
  double* rg_dense_t = nullptr;
  double* rg_dense_y = nullptr;
  DevBuf dn_off, dn_t, dn_y;
  DevBuf rdn_off, rdn_voff, rdn_t, rdn_y;
};

extern "C" {

const char* bacon_last_error(void) { return g_last_error.c_str(); }

int bacon_ctx_create(int device, bacon_ctx** out) {
  if (!out) return fail(BACON_INVALID_ARGUMENT, "bacon_ctx_create: out is NULL");
  *out = nullptr;
  int count = 0;
  BACON_CUDA(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return fail(BACON_INVALID_ARGUMENT, "bacon_ctx_create: no such device");
  BACON_CUDA(cudaSetDevice(device));
  bacon_ctx* c = new bacon_ctx();
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&c->d_ctl), 16 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&c->h_ctl), 16 * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    delete c;
    return fail(BACON_CUDA_ERROR, std::string("bacon_ctx_create: ") + cudaGetErrorString(e));
  }
  c->kernels = bacon::all_rk_kernels();
  c->adjoint_kernels = bacon::all_adjoint_kernels();
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreate(&c->ev2) != cudaSuccess || cudaEventCreate(&c->ev3) != cudaSuccess) {
    bacon_ctx_destroy(c);
    return fail(BACON_CUDA_ERROR, "bacon_ctx_create: event creation failed");
  }
  *out = c;
  return BACON_OK;
}

int bacon_ctx_destroy(bacon_ctx* c) {
  if (!c) return BACON_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& kv : c->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  for (DevBuf* b : {&c->in_y0, &c->in_params, &c->in_t0, &c->in_tend, &c->out_y, &c->out_t,
                    &c->out_acc, &c->out_rej, &c->out_st, &c->out_tt, &c->out_ty, &c->pl_y, &c->pl_K,
                    &c->pl_t, &c->pl_dt, &c->pl_end, &c->pl_att, &c->pl_acc, &c->pl_rej, &c->pl_st,
                    &c->ord, &c->ord_scratch, &c->adj_dt, &c->adj_ck, &c->adj_tgt, &c->adj_loss,
                    &c->adj_gy, &c->adj_gp, &c->lin_A, &c->lin_y, &c->lin_K, &c->lin_t, &c->lin_dt,
                    &c->lin_end, &c->lin_att, &c->tc_sa, &c->tc_ea, &c->tc_sy, &c->tc_ey, &c->rg_yoff,
                    &c->rg_poff, &c->rg_y0, &c->rg_p, &c->rg_t0, &c->rg_te, &c->rg_yout, &c->rg_tout,
                    &c->rg_acc, &c->rg_rej, &c->rg_st, &c->rg_ord, &c->rg_lu, &c->dn_off, &c->dn_t, &c->dn_y,
                    &c->rdn_off, &c->rdn_voff, &c->rdn_t, &c->rdn_y})
    b->release();
  if (c->ev2) cudaEventDestroy(c->ev2);
  if (c->ev3) cudaEventDestroy(c->ev3);
  if (c->d_ctl) cudaFree(c->d_ctl);
  if (c->h_ctl) cudaFreeHost(c->h_ctl);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return BACON_OK;
}

int64_t bacon_ctx_kernel_launches(const bacon_ctx* c) { return c ? c->launches : 0; }

int bacon_ctx_set_fault_injection(bacon_ctx* c, int kind) {
  if (!c) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  if (kind != BACON_FAULT_NONE && kind != BACON_FAULT_TC_WITHHOLD)
    return fail(BACON_INVALID_ARGUMENT, "unknown fault-injection kind");
  c->fault_injection = kind;
  return BACON_OK;
}

int bacon_ctx_stream(const bacon_ctx* c, void** stream) {
  if (!c || !stream) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  *stream = reinterpret_cast<void*>(c->stream);
  return BACON_OK;
}

int bacon_ctx_last_reverse_ms(const bacon_ctx* c, double* ms) {
  if (!c || !ms) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  if (!c->rev_valid) return fail(BACON_INVALID_ARGUMENT, "no adjoint run yet");
  float f = 0.f;
  BACON_CUDA(cudaEventElapsedTime(&f, c->ev2, c->ev3));
  *ms = f;
  return BACON_OK;
}

int bacon_ctx_last_kernel_ms(const bacon_ctx* c, double* ms) {
  if (!c || !ms) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  if (!c->ev_valid) return fail(BACON_INVALID_ARGUMENT, "no timed kernel yet");
  float f = 0.f;
  BACON_CUDA(cudaEventElapsedTime(&f, c->ev0, c->ev1));
  *ms = f;
  return BACON_OK;
}

// Builder-equivalent checks on a filled problem (src/ivp/rk.rs:168-256).
int bacon_rk_validate(const bacon_problem* p) {
  if (!p) return fail(BACON_INVALID_ARGUMENT, "problem is NULL");
  if (p->n < 0) return fail(BACON_INVALID_ARGUMENT, "n < 0");
  if (p->dim < 1) return fail(BACON_INVALID_ARGUMENT, "dim < 1");
  if (p->n > 0 && !p->y0) return fail(BACON_MISSING_PARAMETERS, "initial conditions missing");
  if (p->tol <= 0.0) return fail(BACON_TOLERANCE_OOB, "tolerance <= 0");
  if (p->dt_max <= 0.0 || p->dt_min <= 0.0) return fail(BACON_TIME_DELTA_OOB, "dt bound <= 0");
  if (!p->t0 && !p->t_end && p->t0_scalar >= p->t_end_scalar)
    return fail(BACON_TIME_END_OOB, "ending time is not after the initial time");
  const int ed = expected_dim(p->rhs);
  if (p->rhs < 0 || p->rhs > BACON_RHS_USER) return fail(BACON_INVALID_ARGUMENT, "unknown rhs");
  if (ed > 0 && p->dim != ed) return fail(BACON_INVALID_ARGUMENT, "dim does not match the rhs");
  if (p->n_params < expected_params(p->rhs, p->dim))
    return fail(BACON_INVALID_ARGUMENT, "too few parameters for the rhs");
  if (p->n > 0 && p->n_params > 0 && !p->params) return fail(BACON_INVALID_ARGUMENT, "params is NULL");
  return BACON_OK;
}

int bacon_measure_fp64_peak(bacon_ctx* c, double* gflops) {
  if (!c || !gflops) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  BACON_CUDA(cudaSetDevice(c->device));
  const double g = bacon::measure_fp64_fma_gflops(c->stream, c->num_sms);
  if (g < 0) return fail(BACON_CUDA_ERROR, "fp64 probe failed");
  c->launches += 4;
  *gflops = g;
  return BACON_OK;
}

}  // extern "C"

namespace {

// Occupancy model for the persistent kernels: the FP64 pipe is saturated by
// two 128-thread CTAs per SM, while every extra resident thread lengthens the
// tail in which lanes run out of systems.  Aim for >= 16 systems per thread
// and at least 256 threads per SM.
// Persistent CTAs per SM: enough threads that every thread still has ~16
// systems (so the longest-first order balances the tail), at least
// min_threads per SM, at most 4 CTAs.  The FP64-bound kernels run at the same
// speed from 256 to 512 threads per SM; the FP32-stage kernel is latency bound
// and asks for 768 (measured on Lorenz 1M: 211 ms at 256 threads, 157 ms at
// 768 or more).
int model_blocks_per_sm(int64_t n, int num_sms, int block, int max_bps, int min_threads = 256) {
  const int64_t threads_for_tail = n / 16;
  int64_t bps = threads_for_tail / (static_cast<int64_t>(num_sms) * block);
  const int64_t floor_bps = (min_threads + block - 1) / block;
  if (bps < floor_bps) bps = floor_bps;
  if (bps > 4) bps = 4;
  if (bps > max_bps) bps = max_bps;
  return static_cast<int>(bps < 1 ? 1 : bps);
}

// Autotune cache key: the kernel and the batch size rounded to a power of two.
uint64_t tune_key(const bacon::RkKey& k, int64_t n) {
  int lg = 0;
  while ((int64_t{1} << lg) < n && lg < 62) ++lg;
  uint64_t h = fnv1a(&k, sizeof(k));
  return fnv1a(&lg, sizeof(lg), h);
}

// Effective dt bounds after the builder's cross-clamping with minimum set
// before maximum (with_minimum_dt then with_maximum_dt, rk.rs:179-210).
void clamp_dt(double& dt_min, double dt_max) {
  if (dt_min > dt_max) dt_min = dt_max;
}

struct Resolved {
  const double *y0, *params, *t0, *t_end;
  double *y_out, *t_out, *traj_t, *traj_y;
  int32_t *acc, *rej, *st;
};

int stage_inputs(bacon_ctx* c, const bacon_problem* p, const bacon_rk_result* r, bool host, Resolved& o) {
  const size_t n = static_cast<size_t>(p->n);
  const size_t yb = n * p->dim * sizeof(double);
  if (!host) {
    o = Resolved{p->y0, p->params, p->t0, p->t_end, r->y_final, r->t_final, r->traj_t, r->traj_y,
                 r->accepted, r->rejected, r->status};
    return BACON_OK;
  }
  BACON_CUDA(c->in_y0.ensure(yb));
  BACON_CUDA(c->out_y.ensure(yb));
  BACON_CUDA(c->out_t.ensure(n * sizeof(double)));
  BACON_CUDA(c->out_acc.ensure(n * sizeof(int32_t)));
  BACON_CUDA(c->out_rej.ensure(n * sizeof(int32_t)));
  BACON_CUDA(c->out_st.ensure(n * sizeof(int32_t)));
  o.y0 = c->in_y0.as<double>();
  o.params = nullptr;
  if (p->n_params > 0 && p->params) {
    BACON_CUDA(c->in_params.ensure(n * p->n_params * sizeof(double)));
    o.params = c->in_params.as<double>();
  }
  o.t0 = nullptr;
  o.t_end = nullptr;
  if (p->t0) {
    BACON_CUDA(c->in_t0.ensure(n * sizeof(double)));
    o.t0 = c->in_t0.as<double>();
  }
  if (p->t_end) {
    BACON_CUDA(c->in_tend.ensure(n * sizeof(double)));
    o.t_end = c->in_tend.as<double>();
  }
  o.y_out = c->out_y.as<double>();
  o.t_out = c->out_t.as<double>();
  o.acc = c->out_acc.as<int32_t>();
  o.rej = c->out_rej.as<int32_t>();
  o.st = c->out_st.as<int32_t>();
  o.traj_t = nullptr;
  o.traj_y = nullptr;
  if (r->traj_t && r->traj_cap > 0) {
    BACON_CUDA(c->out_tt.ensure(n * r->traj_cap * sizeof(double)));
    BACON_CUDA(c->out_ty.ensure(n * r->traj_cap * p->dim * sizeof(double)));
    o.traj_t = c->out_tt.as<double>();
    o.traj_y = c->out_ty.as<double>();
  }
  return BACON_OK;
}

int enqueue_h2d(bacon_ctx* c, const bacon_problem* p, const Resolved& o) {
  const size_t n = static_cast<size_t>(p->n);
  BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(o.y0), p->y0, n * p->dim * sizeof(double),
                             cudaMemcpyHostToDevice, c->stream));
  if (o.params)
    BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(o.params), p->params, n * p->n_params * sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
  if (o.t0)
    BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(o.t0), p->t0, n * sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
  if (o.t_end)
    BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(o.t_end), p->t_end, n * sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
  return BACON_OK;
}

int enqueue_d2h(bacon_ctx* c, const bacon_problem* p, const bacon_rk_result* r, const Resolved& o) {
  const size_t n = static_cast<size_t>(p->n);
  BACON_CUDA(cudaMemcpyAsync(r->y_final, o.y_out, n * p->dim * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  BACON_CUDA(cudaMemcpyAsync(r->t_final, o.t_out, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  BACON_CUDA(cudaMemcpyAsync(r->accepted, o.acc, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  BACON_CUDA(cudaMemcpyAsync(r->rejected, o.rej, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  BACON_CUDA(cudaMemcpyAsync(r->status, o.st, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  if (o.traj_t) {
    BACON_CUDA(cudaMemcpyAsync(r->traj_t, o.traj_t, n * r->traj_cap * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
    BACON_CUDA(cudaMemcpyAsync(r->traj_y, o.traj_y, n * r->traj_cap * p->dim * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
  }
  return BACON_OK;
}

bool is_pinned_or_device(const void* ptr) {
  if (!ptr) return true;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int check_result_ptrs(const bacon_problem* p, const bacon_rk_result* r) {
  if (!r) return fail(BACON_INVALID_ARGUMENT, "result is NULL");
  if (p->n > 0 && (!r->y_final || !r->t_final || !r->accepted || !r->rejected || !r->status))
    return fail(BACON_INVALID_ARGUMENT, "result array is NULL");
  if ((r->traj_t == nullptr) != (r->traj_y == nullptr))
    return fail(BACON_INVALID_ARGUMENT, "traj_t and traj_y must be given together");
  if (r->traj_t && r->traj_cap < 0) return fail(BACON_INVALID_ARGUMENT, "traj_cap < 0");
  return BACON_OK;
}

// Reads the lowest failing index and its status after the solve finished.
int batch_return_code(bacon_ctx* c, const bacon_rk_result* r, bool host, const Resolved& o) {
  const unsigned long long ff = c->h_ctl[1];
  if (ff == ~0ull) return BACON_OK;
  int32_t st = 0;
  if (host) {
    st = r->status[ff];
  } else {
    BACON_CUDA(cudaMemcpy(&st, o.st + ff, sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  return fail(st, "system " + std::to_string(ff) + " ended with status " + std::to_string(st));
}

}  // namespace

namespace {

// Lock-step batched RKF45 for y' = A y with a shared A (linear.cuh): one
// round = one attempt for every running system = S GEMMs + one control
// kernel; the host relaunches the round until no system runs.  The FP64
// modes form the stage values K_i = dt A Y_i; the tensor-core mode forms the
// products v_k = A^k y and the control kernel combines them (LinPoly).
int linear_solve(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt, bacon_rk_result* r) {
  if (!p->shared) return fail(BACON_MISSING_PARAMETERS, "BACON_RHS_LINEAR needs the shared matrix");
  const bool tc = opt->precision == BACON_TC_SPLIT;
  bacon::LinKernels k;
  bacon::LinTcKernels tk;
  // The tensor-core mode computes the products v_k = A^k y (one GEMM each)
  // and combines them in its own control kernel, with FMA contraction: they
  // carry ~2^-39 relative error, far above a contraction's rounding.
  if (!bacon::lin_kernels(opt->method, opt->layout, tc ? 1 : opt->precision, p->dim, k) ||
      (tc && !bacon::lin_tc_kernels(opt->method, opt->layout, p->dim, tk)))
    return fail(BACON_UNSUPPORTED, "linear engine: dim 64/128/256 (128/256 on tensor cores); layouts "
                                   "as_written / fehlberg; precision FP64_EXACT, FP64_FMA or TC_SPLIT");
  if (p->n == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));
  const bool host = opt->memory == BACON_MEM_HOST;
  Resolved o{};
  int rc;
  if ((rc = stage_inputs(c, p, r, host, o)) != BACON_OK) return rc;
  const size_t n = static_cast<size_t>(p->n), D = static_cast<size_t>(p->dim);
  const double* A = p->shared;
  if (host) {
    BACON_CUDA(c->lin_A.ensure(D * D * sizeof(double)));
    BACON_CUDA(cudaMemcpyAsync(c->lin_A.p, p->shared, D * D * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    A = c->lin_A.as<double>();
    if ((rc = enqueue_h2d(c, p, o)) != BACON_OK) return rc;
  }
  BACON_CUDA(c->lin_y.ensure(n * D * sizeof(double)));
  BACON_CUDA(c->lin_K.ensure(static_cast<size_t>(k.stages) * n * D * sizeof(double)));
  BACON_CUDA(c->lin_t.ensure(n * sizeof(double)));
  BACON_CUDA(c->lin_dt.ensure(n * sizeof(double)));
  BACON_CUDA(c->lin_end.ensure(n * sizeof(double)));
  BACON_CUDA(c->lin_att.ensure(n * sizeof(int64_t)));
  double dt_min = p->dt_min;
  clamp_dt(dt_min, p->dt_max);
  bacon::LinArgs st{};
  st.n = p->n;
  st.A = A;
  st.y = c->lin_y.as<double>();
  st.K = c->lin_K.as<double>();
  st.t = c->lin_t.as<double>();
  st.dt = c->lin_dt.as<double>();
  st.end = c->lin_end.as<double>();
  st.attempts = c->lin_att.as<int64_t>();
  st.accepted = o.acc;
  st.rejected = o.rej;
  st.status = o.st;
  st.live = reinterpret_cast<unsigned int*>(c->d_ctl + 2);
  st.tol = p->tol;
  st.dt_min = dt_min;
  st.dt_max = p->dt_max;
  st.max_attempts = opt->max_attempts > 0 ? opt->max_attempts : 10000000;
  st.traj_t = o.traj_t;
  st.traj_y = o.traj_y;
  st.traj_cap = o.traj_t ? r->traj_cap : 0;
  if (c->dense_off) {  // the second pass of bacon_rk_solve_dense
    st.traj_t = c->dense_t;
    st.traj_y = c->dense_y;
    st.traj_off = c->dense_off;
  }
  bacon::LinInitArgs ia{};
  ia.st = st;
  ia.dim = p->dim;
  ia.stages = k.stages;
  ia.y0 = o.y0;
  ia.t0 = o.t0;
  ia.t_end = o.t_end;
  ia.t0_s = p->t0_scalar;
  ia.t_end_s = p->t_end_scalar;
  ia.dt0 = (p->dt_max + dt_min) * 0.5;
  void* iargs[] = {&ia};
  const unsigned ig = static_cast<unsigned>((n * D + 255) / 256);
  BACON_CUDA(cudaLaunchKernel(k.init, dim3(ig), dim3(256), iargs, 0, c->stream));
  unsigned int* h_live = reinterpret_cast<unsigned int*>(c->h_ctl + 2);
  int first = 1;
  void* cargs[] = {&st, &first};
  void* sargs[] = {&st};
  const unsigned cg = static_cast<unsigned>((n * 32 + 255) / 256);
  const unsigned ctl_g = static_cast<unsigned>((n + bacon::kLinCtlSystemsPerBlock - 1) / bacon::kLinCtlSystemsPerBlock);
  const dim3 sg(static_cast<unsigned>((n + 63) / 64), static_cast<unsigned>(D / 64));
  const void* control = tc ? tk.control : k.control;
  BACON_CUDA(cudaMemsetAsync(st.live, 0, sizeof(unsigned int), c->stream));
  BACON_CUDA(cudaLaunchKernel(control, dim3(ctl_g), dim3(bacon::kLinCtlThreads), cargs, 0, c->stream));
  BACON_CUDA(cudaMemcpyAsync(h_live, st.live, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  c->launches += 2;
  first = 0;
  bacon::TcArgs ta{};
  unsigned int* d_err = reinterpret_cast<unsigned int*>(c->d_ctl + 3);
  if (tc) {
    BACON_CUDA(c->tc_sa.ensure(static_cast<size_t>(tk.slices) * D * D * sizeof(__nv_bfloat16)));
    BACON_CUDA(c->tc_ea.ensure(D * sizeof(int32_t)));
    // the stage-input slices are chunk images of 64-system tiles: padded to
    // whole tiles, zeroed once (padding systems are never written)
    const size_t sy_systems = static_cast<size_t>((n + bacon::kTcN - 1) / bacon::kTcN) * bacon::kTcN;
    const size_t sy_bytes = static_cast<size_t>(tk.slices) * sy_systems * D * sizeof(__nv_bfloat16);
    BACON_CUDA(c->tc_sy.ensure(sy_bytes));
    BACON_CUDA(cudaMemsetAsync(c->tc_sy.p, 0, sy_bytes, c->stream));
    BACON_CUDA(c->tc_ey.ensure(n * sizeof(int32_t)));
    BACON_CUDA(cudaFuncSetAttribute(tk.gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, tk.smem_bytes));
    BACON_CUDA(cudaFuncSetAttribute(tk.gemm_last, cudaFuncAttributeMaxDynamicSharedMemorySize, tk.smem_bytes));
    ta.st = st;
    ta.sa = c->tc_sa.as<__nv_bfloat16>();
    ta.ea = c->tc_ea.as<int32_t>();
    ta.sy = c->tc_sy.as<__nv_bfloat16>();
    ta.ey = c->tc_ey.as<int32_t>();
    ta.error_flag = d_err;
    // about one second at the SM clock; the fault-injection hook withholds
    // the accumulator hand-off and shortens the waits to ~10 ms
    ta.withhold_tmem_full = c->fault_injection == BACON_FAULT_TC_WITHHOLD ? 1 : 0;
    ta.wait_limit = ta.withhold_tmem_full ? 20000000ll : 2000000000ll;
    BACON_CUDA(cudaMemsetAsync(c->d_ctl + 3, 0, sizeof(unsigned long long), c->stream));
    const double* Ap = A;
    __nv_bfloat16* sa = c->tc_sa.as<__nv_bfloat16>();
    int32_t* ea = c->tc_ea.as<int32_t>();
    void* aargs[] = {&Ap, &sa, &ea};
    BACON_CUDA(cudaLaunchKernel(tk.slice_a, dim3(static_cast<unsigned>((D * 32 + 255) / 256)), dim3(256), aargs, 0,
                                c->stream));
    c->launches += 1;
  }
  __nv_bfloat16* sy = c->tc_sy.as<__nv_bfloat16>();
  int32_t* ey = c->tc_ey.as<int32_t>();
  // persistent stage GEMM: one CTA per SM over (systems / 64) x (D / 128) tiles
  const long long tc_tiles = ((n + bacon::kTcN - 1) / bacon::kTcN) * (D / bacon::kTcM);
  const dim3 tg(static_cast<unsigned>(tc_tiles < c->num_sms ? tc_tiles : c->num_sms));
  // One round: the S products (or stage GEMMs), the live-counter reset, the
  // control kernel and the copies the host reads.  It is captured once as a
  // CUDA graph and relaunched until no system runs, one launch per round.
  auto enqueue_round = [&]() -> int {
    for (int s = 0; s < k.stages; ++s) {
      if (tc) {
        // v_{s+1} = A v_s into K[s], v_0 = y
        ta.stage = s;
        const double* x = s == 0 ? st.y : st.K + static_cast<size_t>(s - 1) * n * D;
        void* slargs[] = {&ta, &x, &sy, &ey};
        BACON_CUDA(cudaLaunchKernel(tk.slice_vec, dim3(cg), dim3(256), slargs, 0, c->stream));
        void* gargs[] = {&ta};
        BACON_CUDA(cudaLaunchKernel(s + 1 == k.stages ? tk.gemm_last : tk.gemm, tg,
                                    dim3(static_cast<unsigned>(tk.gemm_threads)), gargs,
                                    static_cast<size_t>(tk.smem_bytes), c->stream));
      } else {
        BACON_CUDA(cudaLaunchKernel(k.stage[s], sg, dim3(256), sargs, 0, c->stream));
      }
    }
    BACON_CUDA(cudaMemsetAsync(st.live, 0, sizeof(unsigned int), c->stream));
    BACON_CUDA(cudaLaunchKernel(control, dim3(ctl_g), dim3(bacon::kLinCtlThreads), cargs, 0, c->stream));
    BACON_CUDA(cudaMemcpyAsync(h_live, st.live, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    if (tc)  // a tensor-core stage that gave up a bounded wait ends the solve
      BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 3, c->d_ctl + 3, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 c->stream));
    return BACON_OK;
  };
  struct RoundGraph {
    cudaGraphExec_t exec = nullptr;
    ~RoundGraph() {
      if (exec) cudaGraphExecDestroy(exec);
    }
  } round;
  BACON_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  const int erc = enqueue_round();
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
  if (erc != BACON_OK) {
    if (graph) cudaGraphDestroy(graph);
    return erc;
  }
  if (ce != cudaSuccess) return fail(BACON_CUDA_ERROR, std::string("round graph capture: ") + cudaGetErrorString(ce));
  const cudaError_t ie = cudaGraphInstantiate(&round.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess)
    return fail(BACON_CUDA_ERROR, std::string("round graph instantiate: ") + cudaGetErrorString(ie));
  const int per_round = (tc ? 2 * k.stages : k.stages) + 1;  // kernels in one round
  BACON_CUDA(cudaEventRecord(c->ev0, c->stream));
  while (*h_live > 0) {
    BACON_CUDA(cudaGraphLaunch(round.exec, c->stream));
    BACON_CUDA(cudaStreamSynchronize(c->stream));
    c->launches += per_round;
    if (tc && c->h_ctl[3] != 0) return fail(BACON_CUDA_ERROR, "tensor-core stage: a bounded mbarrier wait gave up");
  }
  BACON_CUDA(cudaEventRecord(c->ev1, c->stream));
  c->ev_valid = true;
  int dim = p->dim;
  double* yo = o.y_out;
  void* oargs[] = {&st, &dim, &yo};
  BACON_CUDA(cudaLaunchKernel(k.output, dim3(ig), dim3(256), oargs, 0, c->stream));
  BACON_CUDA(cudaMemcpyAsync(o.t_out, st.t, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  c->launches += 1;
  if (host && (rc = enqueue_d2h(c, p, r, o)) != BACON_OK) return rc;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  BACON_CUDA(cudaGetLastError());
  if (tc) {
    unsigned int herr = 0;
    BACON_CUDA(cudaMemcpy(&herr, d_err, sizeof(herr), cudaMemcpyDeviceToHost));
    if (herr) return fail(BACON_CUDA_ERROR, "tensor-core stage: a bounded mbarrier wait gave up");
  }
  std::vector<int32_t> hs;
  const int32_t* sp = r->status;
  if (!host) {
    hs.resize(n);
    BACON_CUDA(cudaMemcpy(hs.data(), o.st, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    sp = hs.data();
  }
  for (size_t i = 0; i < n; ++i)
    if (sp[i] != 0) return fail(sp[i], "system " + std::to_string(i) + " ended with status " + std::to_string(sp[i]));
  return BACON_OK;
}

}  // namespace

extern "C" int bacon_rk_solve(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                              bacon_rk_result* r) {
  NvtxRange nvtx_range("bacon_rk_solve");
  if (c && opt && p && p->rhs == BACON_RHS_LINEAR) {
    int rc0 = bacon_rk_validate(p);
    if (rc0 != BACON_OK) return rc0;
    if ((rc0 = check_result_ptrs(p, r)) != BACON_OK) return rc0;
    return linear_solve(c, p, opt, r);
  }
  if (!c || !opt) return fail(BACON_INVALID_ARGUMENT, "NULL context or options");
  int rc = bacon_rk_validate(p);
  if (rc != BACON_OK) return rc;
  if ((rc = check_result_ptrs(p, r)) != BACON_OK) return rc;
  if (opt->method != BACON_RK45 && opt->method != BACON_RK23)
    return fail(BACON_INVALID_ARGUMENT, "unknown method");
  if (opt->layout < 0 || opt->layout > 2) return fail(BACON_INVALID_ARGUMENT, "unknown layout");
  if (opt->precision < 0 || opt->precision > 2) return fail(BACON_INVALID_ARGUMENT, "unknown precision");
  if (p->dyn_dim && p->dim == 4) return fail(BACON_UNSUPPORTED, "dynamic 4-vectors are not compiled");
  const int layout = (opt->method == BACON_RK23 && opt->layout == BACON_LAYOUT_FEHLBERG) ? 1 : opt->layout;
  const bacon::RkKey key{opt->method, layout, opt->precision, p->rhs, p->dim};
  const void* fn = nullptr;
  for (const auto& e : c->kernels)
    if (e.key == key && e.variant == 0) fn = e.fn;
  if (!fn) return fail(BACON_UNSUPPORTED, "no compiled kernel for this (method, layout, precision, rhs, dim)");
  if (p->n == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));

  const bool host = opt->memory == BACON_MEM_HOST;
  Resolved o{};
  if ((rc = stage_inputs(c, p, r, host, o)) != BACON_OK) return rc;

  double dt_min = p->dt_min;
  clamp_dt(dt_min, p->dt_max);
  bacon::RkArgs a{};
  a.n = p->n;
  a.y0 = o.y0;
  a.params = o.params;
  a.t0 = o.t0;
  a.t_end = o.t_end;
  a.t0_s = p->t0_scalar;
  a.t_end_s = p->t_end_scalar;
  a.tol = p->tol;
  a.dt_min = dt_min;
  a.dt_max = p->dt_max;
  a.max_attempts = opt->max_attempts > 0 ? opt->max_attempts : 10000000;
  a.y_out = o.y_out;
  a.t_out = o.t_out;
  a.accepted = o.acc;
  a.rejected = o.rej;
  a.status = o.st;
  a.traj_t = o.traj_t;
  a.traj_y = o.traj_y;
  a.traj_cap = (o.traj_t ? r->traj_cap : 0);
  if (c->dense_off) {
    a.traj_t = c->dense_t;
    a.traj_y = c->dense_y;
    a.traj_off = c->dense_off;
  }
  a.queue = c->d_ctl;
  a.first_fail = c->d_ctl + 1;
  a.order = nullptr;

  // Longest-first order when spans differ between systems (or on request).
  const bool per_system_times = (p->t0 != nullptr) || (p->t_end != nullptr);
  const bool lpt = (opt->schedule == 2 || (opt->schedule == 0 && per_system_times)) && p->n < (1ll << 32);
  bacon::OrderArgs oa{};
  if (lpt) {
    BACON_CUDA(c->ord.ensure(static_cast<size_t>(p->n) * sizeof(uint32_t)));
    BACON_CUDA(c->ord_scratch.ensure(sizeof(bacon::OrderScratch)));
    oa = bacon::OrderArgs{p->n, o.t0, o.t_end, p->t0_scalar, p->t_end_scalar,
                          c->ord_scratch.as<bacon::OrderScratch>(), c->ord.as<uint32_t>()};
    a.order = oa.order;
  }

  // Launch shape: explicit options, else the autotuned shape for this kernel
  // and batch size (bacon_rk_autotune), else the occupancy model.
  int block = opt->block > 0 ? opt->block : 0;
  int bps = opt->blocks_per_sm > 0 ? opt->blocks_per_sm : 0;
  if (opt->systems_per_warp < 0 || opt->systems_per_warp > 32)
    return fail(BACON_INVALID_ARGUMENT, "systems_per_warp must be 0..32");
  int lanes = opt->systems_per_warp == 32 ? 0 : opt->systems_per_warp;
  const uint64_t tkey = tune_key(key, p->n);
  int variant = c->force_variant;
  if (block == 0 && bps == 0 && variant < 0 && lanes == 0) {
    auto it = c->tuned.find(tkey);
    if (it != c->tuned.end()) {
      variant = it->second.variant;
      block = it->second.block;
      bps = it->second.bps;
      lanes = it->second.lanes;
    }
  }
  a.lanes = lanes;
  if (variant > 0) {
    const void* vfn = nullptr;
    for (const auto& e : c->kernels)
      if (e.key == key && e.variant == variant) vfn = e.fn;
    if (!vfn) return fail(BACON_UNSUPPORTED, "no such kernel variant for this key");
    fn = vfn;
  }
  const bool ff = opt->precision == BACON_FP32_COMP;
  // systems per warp below 32: one-warp blocks, as many as the batch needs
  const int spw = lanes > 0 ? lanes : 32;
  if (block == 0) block = lanes > 0 ? 32 : bacon::default_block(p->n, c->num_sms, ff ? 256 : 128);
  if (block % 32 != 0 || block > 256) return fail(BACON_INVALID_ARGUMENT, "block must be a multiple of 32, <= 256");
  int max_bps = 0;
  BACON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_bps, fn, block, 0));
  if (max_bps < 1) return fail(BACON_CUDA_ERROR, "kernel cannot be resident");
  if (bps == 0) bps = model_blocks_per_sm(p->n, c->num_sms, block, max_bps, ff ? 768 : 256);
  if (bps > max_bps) bps = max_bps;
  long long grid = static_cast<long long>(c->num_sms) * bps;
  const long long per_block = static_cast<long long>(block / 32) * spw;  // systems a block holds at a time
  const long long need = (p->n + per_block - 1) / per_block;
  if (grid > need) grid = need;

  void* args[] = {&a};
  bool use_graph = opt->use_graph != 0;
  if (use_graph && host) {
    for (const void* q : {static_cast<const void*>(p->y0), static_cast<const void*>(p->params),
                          static_cast<const void*>(p->t0), static_cast<const void*>(p->t_end),
                          static_cast<const void*>(r->y_final), static_cast<const void*>(r->t_final),
                          static_cast<const void*>(r->accepted), static_cast<const void*>(r->rejected),
                          static_cast<const void*>(r->status), static_cast<const void*>(r->traj_t),
                          static_cast<const void*>(r->traj_y)})
      if (!is_pinned_or_device(q)) use_graph = false;
  }

  bool capturing = false;
  auto enqueue_all = [&]() -> int {
    int e;
    if (host && (e = enqueue_h2d(c, p, o)) != BACON_OK) return e;
    if (lpt) BACON_CUDA(bacon::enqueue_lpt_order(oa, c->num_sms, c->stream));
    BACON_CUDA(cudaMemsetAsync(c->d_ctl, 0, sizeof(unsigned long long), c->stream));
    BACON_CUDA(cudaMemsetAsync(c->d_ctl + 1, 0xff, sizeof(unsigned long long), c->stream));
    BACON_CUDA(cudaEventRecordWithFlags(c->ev0, c->stream, capturing ? cudaEventRecordExternal : 0));
    BACON_CUDA(cudaLaunchKernel(fn, dim3(static_cast<unsigned>(grid)), dim3(block), args, 0, c->stream));
    BACON_CUDA(cudaEventRecordWithFlags(c->ev1, c->stream, capturing ? cudaEventRecordExternal : 0));
    if (host && (e = enqueue_d2h(c, p, r, o)) != BACON_OK) return e;
    BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 1, c->d_ctl + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c->stream));
    return BACON_OK;
  };

  if (use_graph) {
    uint64_t h = fnv1a(&a, sizeof(a));
    h = fnv1a(&key, sizeof(key), h);
    h = fnv1a(&fn, sizeof(fn), h);  // the kernel variant
    h = fnv1a(&grid, sizeof(grid), h);
    h = fnv1a(&block, sizeof(block), h);
    const void* hp[] = {p->y0, p->params, p->t0, p->t_end, r->y_final, r->t_final, r->accepted,
                        r->rejected, r->status, r->traj_t, r->traj_y};
    h = fnv1a(hp, sizeof(hp), h);
    h = fnv1a(&host, sizeof(host), h);
    auto it = c->graphs.find(h);
    if (it == c->graphs.end()) {
      BACON_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      capturing = true;
      const int e = enqueue_all();
      capturing = false;
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (e != BACON_OK) {
        if (g) cudaGraphDestroy(g);
        return e;
      }
      if (ce != cudaSuccess) return fail(BACON_CUDA_ERROR, std::string("graph capture: ") + cudaGetErrorString(ce));
      cudaGraphExec_t ex = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return fail(BACON_CUDA_ERROR, std::string("graph instantiate: ") + cudaGetErrorString(ie));
      it = c->graphs.emplace(h, bacon_ctx::Graph{ex}).first;
    }
    BACON_CUDA(cudaGraphLaunch(it->second.exec, c->stream));
  } else {
    if ((rc = enqueue_all()) != BACON_OK) return rc;
  }
  c->launches += lpt ? 5 : 1;
  c->ev_valid = true;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  BACON_CUDA(cudaGetLastError());
  return batch_return_code(c, r, host, o);
}

// The caller's right-hand side: the engine's staging, order and result
// handling around a kernel the caller compiled (include/bacon_gb300_rhs.cuh).
static_assert(sizeof(bacon_rk_kernel_args) == sizeof(bacon::RkArgs), "kernel argument block layout");
static_assert(offsetof(bacon_rk_kernel_args, traj_off) == offsetof(bacon::RkArgs, traj_off), "layout");
static_assert(offsetof(bacon_rk_kernel_args, order) == offsetof(bacon::RkArgs, order), "layout");
static_assert(offsetof(bacon_rk_kernel_args, ckpt_slots) == offsetof(bacon::RkArgs, ckpt_slots), "layout");
static_assert(offsetof(bacon_rk_kernel_args, lanes) == offsetof(bacon::RkArgs, lanes), "layout");

extern "C" int bacon_rk_solve_user(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                                   bacon_rk_result* r, bacon_rk_launch_fn launch, void* user) {
  NvtxRange nvtx_range("bacon_rk_solve_user");
  if (!c || !opt || !launch) return fail(BACON_INVALID_ARGUMENT, "NULL context, options or launcher");
  int rc = bacon_rk_validate(p);
  if (rc != BACON_OK) return rc;
  if (p->rhs != BACON_RHS_USER) return fail(BACON_INVALID_ARGUMENT, "bacon_rk_solve_user takes BACON_RHS_USER");
  if ((rc = check_result_ptrs(p, r)) != BACON_OK) return rc;
  if (opt->method != BACON_RK45 && opt->method != BACON_RK23) return fail(BACON_INVALID_ARGUMENT, "unknown method");
  if (opt->layout < 0 || opt->layout > 2) return fail(BACON_INVALID_ARGUMENT, "unknown layout");
  if (opt->precision < 0 || opt->precision > 2) return fail(BACON_INVALID_ARGUMENT, "unknown precision");
  if (p->n == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));
  const bool host = opt->memory == BACON_MEM_HOST;
  Resolved o{};
  if ((rc = stage_inputs(c, p, r, host, o)) != BACON_OK) return rc;
  double dt_min = p->dt_min;
  clamp_dt(dt_min, p->dt_max);
  bacon::RkArgs a{};
  a.n = p->n;
  a.y0 = o.y0;
  a.params = o.params;
  a.t0 = o.t0;
  a.t_end = o.t_end;
  a.t0_s = p->t0_scalar;
  a.t_end_s = p->t_end_scalar;
  a.tol = p->tol;
  a.dt_min = dt_min;
  a.dt_max = p->dt_max;
  a.max_attempts = opt->max_attempts > 0 ? opt->max_attempts : 10000000;
  a.y_out = o.y_out;
  a.t_out = o.t_out;
  a.accepted = o.acc;
  a.rejected = o.rej;
  a.status = o.st;
  a.traj_t = o.traj_t;
  a.traj_y = o.traj_y;
  a.traj_cap = (o.traj_t ? r->traj_cap : 0);
  a.queue = c->d_ctl;
  a.first_fail = c->d_ctl + 1;
  const bool per_system_times = (p->t0 != nullptr) || (p->t_end != nullptr);
  const bool lpt = (opt->schedule == 2 || (opt->schedule == 0 && per_system_times)) && p->n < (1ll << 32);
  bacon::OrderArgs oa{};
  if (lpt) {
    BACON_CUDA(c->ord.ensure(static_cast<size_t>(p->n) * sizeof(uint32_t)));
    BACON_CUDA(c->ord_scratch.ensure(sizeof(bacon::OrderScratch)));
    oa = bacon::OrderArgs{p->n, o.t0, o.t_end, p->t0_scalar, p->t_end_scalar,
                          c->ord_scratch.as<bacon::OrderScratch>(), c->ord.as<uint32_t>()};
    a.order = oa.order;
  }
  if (opt->systems_per_warp < 0 || opt->systems_per_warp > 32)
    return fail(BACON_INVALID_ARGUMENT, "systems_per_warp must be 0..32");
  a.lanes = opt->systems_per_warp == 32 ? 0 : opt->systems_per_warp;
  const int spw = a.lanes > 0 ? a.lanes : 32;
  const int block = opt->block > 0 ? opt->block : (a.lanes > 0 ? 32 : bacon::default_block(p->n, c->num_sms, 128));
  if (block % 32 != 0 || block > 256) return fail(BACON_INVALID_ARGUMENT, "block must be a multiple of 32, <= 256");
  const int bps = opt->blocks_per_sm > 0 ? opt->blocks_per_sm : (a.lanes > 0 ? 8 : 2);
  long long grid = static_cast<long long>(c->num_sms) * bps;
  const long long per_block = static_cast<long long>(block / 32) * spw;  // systems a block holds at a time
  const long long need = (p->n + per_block - 1) / per_block;
  if (grid > need) grid = need;
  if (host && (rc = enqueue_h2d(c, p, o)) != BACON_OK) return rc;
  if (lpt) BACON_CUDA(bacon::enqueue_lpt_order(oa, c->num_sms, c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl, 0, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 1, 0xff, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaEventRecord(c->ev0, c->stream));
  bacon_rk_kernel_args ka;
  std::memcpy(&ka, &a, sizeof(ka));
  const int lrc = launch(&ka, opt->method, opt->layout, opt->precision, static_cast<int32_t>(grid), block,
                         reinterpret_cast<void*>(c->stream), user);
  if (lrc != BACON_OK) {
    cudaStreamSynchronize(c->stream);
    return fail(lrc, "the caller's launcher failed for this (method, layout, precision)");
  }
  BACON_CUDA(cudaEventRecord(c->ev1, c->stream));
  if (host && (rc = enqueue_d2h(c, p, r, o)) != BACON_OK) return rc;
  BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 1, c->d_ctl + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
  c->launches += lpt ? 5 : 1;
  c->ev_valid = true;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  BACON_CUDA(cudaGetLastError());
  return batch_return_code(c, r, host, o);
}

extern "C" int bacon_rk_solve_plain(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                                    bacon_rk_result* r) {
  NvtxRange nvtx_range("bacon_rk_solve_plain");
  if (!c || !opt) return fail(BACON_INVALID_ARGUMENT, "NULL context or options");
  int rc = bacon_rk_validate(p);
  if (rc != BACON_OK) return rc;
  if ((rc = check_result_ptrs(p, r)) != BACON_OK) return rc;
  if (opt->precision != BACON_FP64_EXACT) return fail(BACON_UNSUPPORTED, "the plain baseline is FP64 exact only");
  if (r->traj_t) return fail(BACON_UNSUPPORTED, "the plain baseline records no trajectory");
  if (p->dyn_dim && p->dim == 4) return fail(BACON_UNSUPPORTED, "dynamic 4-vectors are not compiled");
  const void* fn = bacon::plain_kernel(p->rhs, p->dim);
  if (!fn) return fail(BACON_UNSUPPORTED, "no plain kernel for this (rhs, dim)");
  if (p->n == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));
  const bool host = opt->memory == BACON_MEM_HOST;
  Resolved o{};
  if ((rc = stage_inputs(c, p, r, host, o)) != BACON_OK) return rc;
  if (host && (rc = enqueue_h2d(c, p, o)) != BACON_OK) return rc;

  bacon::PlainTables tb{};
  bacon::plain_tables(opt->method, (opt->method == BACON_RK23 && opt->layout == 2) ? 1 : opt->layout, tb);
  BACON_CUDA(bacon::plain_upload_tables(tb, c->stream));
  const size_t n = static_cast<size_t>(p->n);
  const int S = tb.stages;
  BACON_CUDA(c->pl_K.ensure(n * S * p->dim * sizeof(double)));
  BACON_CUDA(c->pl_dt.ensure(n * sizeof(double)));
  BACON_CUDA(c->pl_end.ensure(n * sizeof(double)));
  BACON_CUDA(c->pl_att.ensure(n * sizeof(int64_t)));

  double dt_min = p->dt_min;
  clamp_dt(dt_min, p->dt_max);
  bacon::PlainArgs st{};
  st.n = p->n;
  st.stages = S;
  st.dim = p->dim;
  st.y = o.y_out;  // the state array doubles as the output
  st.K = c->pl_K.as<double>();
  st.t = o.t_out;
  st.dt = c->pl_dt.as<double>();
  st.end = c->pl_end.as<double>();
  st.attempts = c->pl_att.as<int64_t>();
  st.accepted = o.acc;
  st.rejected = o.rej;
  st.status = o.st;
  st.params = o.params;
  st.live = reinterpret_cast<unsigned int*>(c->d_ctl + 2);
  st.tol = p->tol;
  st.dt_min = dt_min;
  st.dt_max = p->dt_max;
  st.max_attempts = opt->max_attempts > 0 ? opt->max_attempts : 10000000;

  bacon::PlainInitArgs ia{};
  ia.n = p->n;
  ia.dim = p->dim;
  ia.stages = S;
  ia.y0 = o.y0;
  ia.t0 = o.t0;
  ia.t_end = o.t_end;
  ia.t0_s = p->t0_scalar;
  ia.t_end_s = p->t_end_scalar;
  ia.dt0 = (p->dt_max + dt_min) * 0.5;
  ia.st = st;
  const int block = opt->block > 0 ? opt->block : 256;
  const unsigned grid = static_cast<unsigned>((p->n + block - 1) / block);
  void* iargs[] = {&ia};
  BACON_CUDA(cudaLaunchKernel(bacon::plain_init_kernel(), dim3(grid), dim3(block), iargs, 0, c->stream));
  c->launches += 1;
  void* sargs[] = {&st};
  unsigned int* h_live = reinterpret_cast<unsigned int*>(c->h_ctl + 2);
  for (;;) {
    BACON_CUDA(cudaMemsetAsync(st.live, 0, sizeof(unsigned int), c->stream));
    BACON_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(block), sargs, 0, c->stream));
    c->launches += 1;
    BACON_CUDA(cudaMemcpyAsync(h_live, st.live, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    BACON_CUDA(cudaStreamSynchronize(c->stream));
    if (*h_live == 0) break;
  }
  BACON_CUDA(cudaGetLastError());
  if (host && (rc = enqueue_d2h(c, p, r, o)) != BACON_OK) return rc;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  // Lowest failing index: scan the statuses on the host.
  std::vector<int32_t> hs;
  const int32_t* sp = r->status;
  if (!host) {
    hs.resize(n);
    BACON_CUDA(cudaMemcpy(hs.data(), o.st, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    sp = hs.data();
  }
  for (size_t i = 0; i < n; ++i)
    if (sp[i] != 0) return fail(sp[i], "system " + std::to_string(i) + " ended with status " + std::to_string(sp[i]));
  return BACON_OK;
}

// ---------------------------------------------------------------------------
// Batched BDF (one system per thread, dim <= 8).
extern "C" int bacon_bdf_solve(bacon_ctx* c, const bacon_problem* p, const bacon_bdf_options* opt,
                               bacon_rk_result* r) {
  NvtxRange nvtx_range("bacon_bdf_solve");
  if (!c || !opt) return fail(BACON_INVALID_ARGUMENT, "NULL context or options");
  int rc = bacon_rk_validate(p);
  if (rc != BACON_OK) return rc;
  if ((rc = check_result_ptrs(p, r)) != BACON_OK) return rc;
  if (opt->method != BACON_BDF6 && opt->method != BACON_BDF2) return fail(BACON_INVALID_ARGUMENT, "unknown method");
  if (opt->mode != BACON_BDF_AS_COMPILED && opt->mode != BACON_BDF_CORRECTED)
    return fail(BACON_INVALID_ARGUMENT, "unknown mode");
  if (c->bdf_kernels.empty()) c->bdf_kernels = bacon::all_bdf_kernels();
  const int want_method = (opt->mode == BACON_BDF_CORRECTED) ? 0 : opt->method;
  const void* fn = nullptr;
  for (const auto& e : c->bdf_kernels)
    if (e.mode == opt->mode && e.method == want_method && e.rhs == p->rhs && e.dim == p->dim) fn = e.fn;
  if (!fn) return fail(BACON_UNSUPPORTED, "no BDF kernel for this (mode, method, rhs, dim)");
  if (p->n == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));
  const bool host = opt->memory == BACON_MEM_HOST;
  Resolved o{};
  if ((rc = stage_inputs(c, p, r, host, o)) != BACON_OK) return rc;
  bacon::BdfArgs a{};
  a.n = p->n;
  a.y0 = o.y0;
  a.params = o.params;
  a.t0 = o.t0;
  a.t_end = o.t_end;
  a.t0_s = p->t0_scalar;
  a.t_end_s = p->t_end_scalar;
  a.tol = p->tol;
  a.dt_min = p->dt_min;
  a.dt_max = p->dt_max;
  a.max_steps = opt->max_steps > 0 ? opt->max_steps : 10000000;
  a.max_iter = opt->max_iter > 0 ? opt->max_iter : (opt->mode == BACON_BDF_CORRECTED ? 8 : 1000);
  a.qmax = (opt->method == BACON_BDF6) ? 6 : 2;
  a.y_out = o.y_out;
  a.t_out = o.t_out;
  a.accepted = o.acc;
  a.rejected = o.rej;
  a.status = o.st;
  a.traj_t = o.traj_t;
  a.traj_y = o.traj_y;
  a.traj_cap = o.traj_t ? r->traj_cap : 0;
  if (c->dense_off) {
    a.traj_t = c->dense_t;
    a.traj_y = c->dense_y;
    a.traj_off = c->dense_off;
  }
  a.queue = c->d_ctl;
  a.first_fail = c->d_ctl + 1;
  int dyn = p->dyn_dim ? 1 : 0;
  const int block = opt->block > 0 ? opt->block : bacon::default_block(p->n, c->num_sms, 128);
  if (block % 32 != 0 || block > 128) return fail(BACON_INVALID_ARGUMENT, "block must be a multiple of 32, <= 128");
  int max_bps = 0;
  BACON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_bps, fn, block, 0));
  if (max_bps < 1) return fail(BACON_CUDA_ERROR, "kernel cannot be resident");
  int bps = opt->blocks_per_sm > 0 ? opt->blocks_per_sm : model_blocks_per_sm(p->n, c->num_sms, block, max_bps);
  if (bps > max_bps) bps = max_bps;
  long long grid = static_cast<long long>(c->num_sms) * bps;
  const long long need = (p->n + block - 1) / block;
  if (grid > need) grid = need;
  if (host && (rc = enqueue_h2d(c, p, o)) != BACON_OK) return rc;
  BACON_CUDA(cudaMemsetAsync(c->d_ctl, 0, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 1, 0xff, sizeof(unsigned long long), c->stream));
  void* args[] = {&a, &dyn};
  BACON_CUDA(cudaEventRecord(c->ev0, c->stream));
  BACON_CUDA(cudaLaunchKernel(fn, dim3(static_cast<unsigned>(grid)), dim3(block), args, 0, c->stream));
  BACON_CUDA(cudaEventRecord(c->ev1, c->stream));
  if (host && (rc = enqueue_d2h(c, p, r, o)) != BACON_OK) return rc;
  BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 1, c->d_ctl + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
  c->launches += 1;
  c->ev_valid = true;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  BACON_CUDA(cudaGetLastError());
  return batch_return_code(c, r, host, o);
}

// ---------------------------------------------------------------------------
// Adams predictor-corrector and Euler: one system per thread.
namespace {

int adams_like_solve(bacon_ctx* c, const bacon_problem* p, int order, double euler_dt,
                     const bacon_adams_options* opt, bacon_rk_result* r) {
  int rc;
  if ((rc = check_result_ptrs(p, r)) != BACON_OK) return rc;
  if (c->adams_kernels.empty()) c->adams_kernels = bacon::all_adams_kernels();
  const void* fn = nullptr;
  for (const auto& e : c->adams_kernels)
    if (e.order == order && e.rhs == p->rhs && e.dim == p->dim) fn = e.fn;
  if (!fn) return fail(BACON_UNSUPPORTED, "no Adams/Euler kernel for this (rhs, dim)");
  if (p->n == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));
  const bool host = opt->memory == BACON_MEM_HOST;
  Resolved o{};
  if ((rc = stage_inputs(c, p, r, host, o)) != BACON_OK) return rc;
  bacon::AdamsArgs a{};
  a.n = p->n;
  a.y0 = o.y0;
  a.params = o.params;
  a.t0 = o.t0;
  a.t_end = o.t_end;
  a.t0_s = p->t0_scalar;
  a.t_end_s = p->t_end_scalar;
  a.tol = p->tol;
  a.dt_min = p->dt_min;
  a.dt_max = p->dt_max;
  a.euler_dt = euler_dt;
  a.max_attempts = opt->max_attempts > 0 ? opt->max_attempts : 10000000;
  a.y_out = o.y_out;
  a.t_out = o.t_out;
  a.accepted = o.acc;
  a.rejected = o.rej;
  a.status = o.st;
  a.traj_t = o.traj_t;
  a.traj_y = o.traj_y;
  a.traj_cap = o.traj_t ? r->traj_cap : 0;
  if (c->dense_off) {
    a.traj_t = c->dense_t;
    a.traj_y = c->dense_y;
    a.traj_off = c->dense_off;
  }
  a.dyn_dim = p->dyn_dim ? 1 : 0;
  a.queue = c->d_ctl;
  a.first_fail = c->d_ctl + 1;
  // One thread runs each system's steps in order, so a batch smaller than
  // the GPU's thread slots is latency bound: each dependent FP64 operation
  // costs ~64 cycles, and warps that share an SM also share its FP64 pipe.
  // The lanes of a warp are in different phases of the reference's step, so
  // a warp iteration costs the union of their paths: a small batch runs
  // fewer systems per warp (more warps, shorter unions), down to ~4 warps per
  // SM, which is where four latency-bound warps fill one SM's FP64 pipe.
  int lanes = opt->systems_per_warp;
  if (lanes < 0 || lanes > 32) return fail(BACON_INVALID_ARGUMENT, "systems_per_warp must be 0..32");
  if (lanes == 0) {
    const int64_t per_warp = p->n / (static_cast<int64_t>(c->num_sms) * 4);
    lanes = 32;
    while (lanes > 1 && lanes / 2 >= per_warp) lanes /= 2;
  }
  a.lanes = lanes;
  int block = opt->block > 0 ? opt->block : (lanes < 32 ? 32 : 128);
  if (opt->block <= 0 && opt->blocks_per_sm <= 0 && lanes == 32) {
    const int64_t warps = (p->n + lanes - 1) / lanes;
    const int64_t per_sm = (warps + c->num_sms - 1) / c->num_sms * 32;
    if (per_sm < 128) block = static_cast<int>(per_sm <= 32 ? 32 : (per_sm + 31) / 32 * 32);
  }
  if (block % 32 != 0 || block > 128) return fail(BACON_INVALID_ARGUMENT, "block must be a multiple of 32, <= 128");
  int max_bps = 0;
  BACON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_bps, fn, block, 0));
  if (max_bps < 1) return fail(BACON_CUDA_ERROR, "kernel cannot be resident");
  // Step counts differ by orders of magnitude between systems and the launch
  // lasts as long as the slowest, so every system starts at once when the
  // occupancy allows (no second round behind a slow first one).
  int bps = opt->blocks_per_sm > 0 ? opt->blocks_per_sm : max_bps;
  if (bps > max_bps) bps = max_bps;
  long long grid = static_cast<long long>(c->num_sms) * bps;
  const long long warps_needed = (p->n + lanes - 1) / lanes;
  const long long need = (warps_needed * 32 + block - 1) / block;
  if (grid > need) grid = need;
  if (host && (rc = enqueue_h2d(c, p, o)) != BACON_OK) return rc;
  BACON_CUDA(cudaMemsetAsync(c->d_ctl, 0, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 1, 0xff, sizeof(unsigned long long), c->stream));
  void* args[] = {&a};
  BACON_CUDA(cudaEventRecord(c->ev0, c->stream));
  BACON_CUDA(cudaLaunchKernel(fn, dim3(static_cast<unsigned>(grid)), dim3(block), args, 0, c->stream));
  BACON_CUDA(cudaEventRecord(c->ev1, c->stream));
  if (host && (rc = enqueue_d2h(c, p, r, o)) != BACON_OK) return rc;
  BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 1, c->d_ctl + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
  c->launches += 1;
  c->ev_valid = true;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  BACON_CUDA(cudaGetLastError());
  return batch_return_code(c, r, host, o);
}

}  // namespace

extern "C" int bacon_adams_solve(bacon_ctx* c, const bacon_problem* p, const bacon_adams_options* opt,
                                 bacon_rk_result* r) {
  NvtxRange nvtx_range("bacon_adams_solve");
  if (!c || !opt) return fail(BACON_INVALID_ARGUMENT, "NULL context or options");
  int rc = bacon_rk_validate(p);
  if (rc != BACON_OK) return rc;
  if (opt->order != 5 && opt->order != 3) return fail(BACON_INVALID_ARGUMENT, "order must be 5 or 3");
  return adams_like_solve(c, p, opt->order, 0.0, opt, r);
}

extern "C" int bacon_euler_solve(bacon_ctx* c, const bacon_problem* p, double dt, const bacon_adams_options* opt,
                                 bacon_rk_result* r) {
  NvtxRange nvtx_range("bacon_euler_solve");
  if (!c || !opt) return fail(BACON_INVALID_ARGUMENT, "NULL context or options");
  if (!p) return fail(BACON_INVALID_ARGUMENT, "problem is NULL");
  if (!(dt > 0.0)) return fail(BACON_TIME_DELTA_OOB, "dt <= 0");
  // Euler ignores the tolerance and the dt bounds (src/ivp.rs:390-393):
  // validate the rest with placeholders for them.
  bacon_problem q = *p;
  q.tol = 1.0;
  q.dt_min = q.dt_max = dt;
  int rc = bacon_rk_validate(&q);
  if (rc != BACON_OK) return rc;
  return adams_like_solve(c, &q, 1, dt, opt, r);
}

// ---------------------------------------------------------------------------
// Mixed stiff batch: ragged systems (a warp each) and a uniform batch of
// small systems (a thread each) in one launch of bdf_mixed_kernel.
namespace {

int validate_ragged(const bacon_ragged_problem* g, const std::vector<int64_t>& yo, const std::vector<int64_t>& po,
                    int& max_dim) {
  if (g->rhs != BACON_RHS_CHAIN) return fail(BACON_UNSUPPORTED, "ragged batches support rhs CHAIN");
  if (!(g->tol > 0.0)) return fail(BACON_INVALID_ARGUMENT, "ragged tol must be > 0");
  if (!(g->dt_min > 0.0) || !(g->dt_max > 0.0)) return fail(BACON_INVALID_ARGUMENT, "ragged dt bounds must be > 0");
  if (yo[0] != 0 || po[0] != 0) return fail(BACON_INVALID_ARGUMENT, "ragged offsets must start at 0");
  max_dim = 0;
  for (int64_t i = 0; i < g->n; ++i) {
    const int64_t d = yo[i + 1] - yo[i];
    if (d < 2 || d > bacon::kRagMaxDim || d % 2 != 0)
      return fail(BACON_INVALID_ARGUMENT, "ragged system " + std::to_string(i) + ": dim must be even, 2..128");
    if (po[i + 1] - po[i] != d / 2 + 1)
      return fail(BACON_INVALID_ARGUMENT, "ragged system " + std::to_string(i) + ": chain takes dim/2 + 1 params");
    if (d > max_dim) max_dim = static_cast<int>(d);
  }
  return BACON_OK;
}

}  // namespace

extern "C" int bacon_ragged_validate(const bacon_ragged_problem* g) {
  if (!g) return fail(BACON_INVALID_ARGUMENT, "ragged problem is NULL");
  if (g->n < 0) return fail(BACON_INVALID_ARGUMENT, "ragged n < 0");
  if (g->n == 0) return BACON_OK;
  if (!g->y_offsets || !g->p_offsets) return fail(BACON_INVALID_ARGUMENT, "ragged offsets are NULL");
  std::vector<int64_t> yo(g->y_offsets, g->y_offsets + g->n + 1), po(g->p_offsets, g->p_offsets + g->n + 1);
  int ld = 0;
  return validate_ragged(g, yo, po, ld);
}

extern "C" int bacon_bdf_solve_mixed(bacon_ctx* c, const bacon_problem* up, const bacon_ragged_problem* g,
                                     const bacon_bdf_options* opt, bacon_rk_result* ur, bacon_ragged_result* gr) {
  NvtxRange nvtx_range("bacon_bdf_solve_mixed");
  if (!c || !opt) return fail(BACON_INVALID_ARGUMENT, "NULL context or options");
  if (!up && !g) return fail(BACON_INVALID_ARGUMENT, "both parts are NULL");
  if (opt->method != BACON_BDF6 && opt->method != BACON_BDF2) return fail(BACON_INVALID_ARGUMENT, "unknown method");
  if (opt->mode != BACON_BDF_CORRECTED) return fail(BACON_UNSUPPORTED, "the mixed batch runs the corrected BDF");
  const bool host = opt->memory == BACON_MEM_HOST;
  int rc;
  if (up) {
    if ((rc = bacon_rk_validate(up)) != BACON_OK) return rc;
    if ((rc = check_result_ptrs(up, ur)) != BACON_OK) return rc;
    if (ur->traj_t) return fail(BACON_UNSUPPORTED, "the mixed batch records no trajectory");
  }
  if (g && g->n < 0) return fail(BACON_INVALID_ARGUMENT, "ragged n < 0");
  const int64_t gn = g ? g->n : 0;
  if (gn > 0) {
    if (!gr || !gr->y_final || !gr->t_final || !gr->accepted || !gr->rejected || !gr->status)
      return fail(BACON_INVALID_ARGUMENT, "ragged result array is NULL");
    if (!g->y_offsets || !g->p_offsets || !g->y0 || !g->params)
      return fail(BACON_INVALID_ARGUMENT, "ragged input array is NULL");
    if (gn >= (int64_t(1) << 32)) return fail(BACON_INVALID_ARGUMENT, "ragged n must be < 2^32");
  }
  const void* fn = bacon::bdf_mixed_kernel_for(up && up->n > 0 ? up->rhs : -1, up ? up->dim : 0);
  if (!fn) return fail(BACON_UNSUPPORTED, "no mixed kernel for this uniform (rhs, dim): ROBERTSON or VDP");
  const int64_t un = up ? up->n : 0;

  // ragged offsets on the host: validation, the largest dimension, the order
  std::vector<int64_t> yo, po;
  int ld = 2;
  if (gn > 0) {
    yo.resize(gn + 1);
    po.resize(gn + 1);
    if (host) {
      std::memcpy(yo.data(), g->y_offsets, (gn + 1) * sizeof(int64_t));
      std::memcpy(po.data(), g->p_offsets, (gn + 1) * sizeof(int64_t));
    } else {
      BACON_CUDA(cudaSetDevice(c->device));
      BACON_CUDA(cudaMemcpy(yo.data(), g->y_offsets, (gn + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
      BACON_CUDA(cudaMemcpy(po.data(), g->p_offsets, (gn + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
    }
    if ((rc = validate_ragged(g, yo, po, ld)) != BACON_OK) return rc;
  }
  if (un == 0 && gn == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));
  // work order: size classes in kernel phase order, largest dim first within
  // a class (longest-first scheduling)
  std::vector<uint32_t> order(gn);
  for (int64_t i = 0; i < gn; ++i) order[i] = static_cast<uint32_t>(i);
  auto dim_of = [&](uint32_t i) { return static_cast<int>(yo[i + 1] - yo[i]); };
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    const int ca = bacon::rag_class_of(dim_of(a)), cb = bacon::rag_class_of(dim_of(b));
    return ca != cb ? ca < cb : dim_of(a) > dim_of(b);
  });
  int64_t class_n[bacon::kRagClasses] = {0, 0, 0, 0};
  unsigned class_mask = 0;
  for (int64_t i = 0; i < gn; ++i) {
    const int cl = bacon::rag_class_of(dim_of(static_cast<uint32_t>(i)));
    ++class_n[cl];
    class_mask |= 1u << cl;
  }

  // launch shape: one CTA of 8 warps per SM (its shared memory fills the SM)
  const int block = bacon::kRagWarps * 32;
  const size_t smem = bacon::rag_cta_smem_bytes(class_mask);
  BACON_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int max_bps = 0;
  BACON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_bps, fn, block, smem));
  if (max_bps < 1) return fail(BACON_CUDA_ERROR, "mixed kernel cannot be resident");
  int bps = opt->blocks_per_sm > 0 ? opt->blocks_per_sm : max_bps;
  if (bps > max_bps) bps = max_bps;
  long long grid = static_cast<long long>(c->num_sms) * bps;
  const long long need = gn + (un + block - 1) / block;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;

  // uniform part
  Resolved uo{};
  bacon::BdfArgs a{};
  int dyn = 0;
  if (un > 0) {
    if ((rc = stage_inputs(c, up, ur, host, uo)) != BACON_OK) return rc;
    a.n = un;
    a.y0 = uo.y0;
    a.params = uo.params;
    a.t0 = uo.t0;
    a.t_end = uo.t_end;
    a.t0_s = up->t0_scalar;
    a.t_end_s = up->t_end_scalar;
    a.tol = up->tol;
    a.dt_min = up->dt_min;
    a.dt_max = up->dt_max;
    a.y_out = uo.y_out;
    a.t_out = uo.t_out;
    a.accepted = uo.acc;
    a.rejected = uo.rej;
    a.status = uo.st;
    if (c->dense_off) {  // the second pass of bacon_bdf_solve_mixed_dense
      a.traj_t = c->dense_t;
      a.traj_y = c->dense_y;
      a.traj_off = c->dense_off;
    }
    dyn = up->dyn_dim ? 1 : 0;
  }
  a.max_steps = opt->max_steps > 0 ? opt->max_steps : 10000000;
  a.max_iter = opt->max_iter > 0 ? opt->max_iter : 8;
  a.qmax = (opt->method == BACON_BDF6) ? 6 : 2;
  a.queue = c->d_ctl;
  a.first_fail = c->d_ctl + 1;

  // ragged part
  bacon::RaggedArgs rg{};
  rg.n = gn;
  rg.max_steps = a.max_steps;
  rg.max_iter = a.max_iter;
  rg.qmax = a.qmax;
  rg.queues = c->d_ctl + 8;
  rg.first_fail = c->d_ctl + 5;
  rg.error_flag = reinterpret_cast<unsigned int*>(c->d_ctl + 6);
  rg.traj_t = c->rg_dense_t;
  rg.traj_y = c->rg_dense_y;
  rg.traj_off = c->rg_dense_off;
  rg.traj_voff = c->rg_dense_voff;
  for (int cl = 0, start = 0; cl < bacon::kRagClasses; start += static_cast<int>(class_n[cl]), ++cl) {
    rg.class_start[cl] = start;
    rg.class_n[cl] = class_n[cl];
  }
  const size_t ytot = gn > 0 ? static_cast<size_t>(yo[gn]) : 0;
  const size_t ptot = gn > 0 ? static_cast<size_t>(po[gn]) : 0;
  if (gn > 0) {
    rg.t0_s = g->t0_scalar;
    rg.t_end_s = g->t_end_scalar;
    rg.tol = g->tol;
    rg.dt_min = g->dt_min;
    rg.dt_max = g->dt_max;
    const size_t nn = static_cast<size_t>(gn);
    BACON_CUDA(c->rg_ord.ensure(nn * sizeof(uint32_t)));
    rg.order = c->rg_ord.as<uint32_t>();
    BACON_CUDA(c->rg_lu.ensure(static_cast<size_t>(grid) * bacon::rag_gcache_cta_doubles() * sizeof(double)));
    rg.gcache = c->rg_lu.as<double>();
    if (host) {
      BACON_CUDA(c->rg_yoff.ensure((nn + 1) * sizeof(int64_t)));
      BACON_CUDA(c->rg_poff.ensure((nn + 1) * sizeof(int64_t)));
      BACON_CUDA(c->rg_y0.ensure(ytot * sizeof(double)));
      BACON_CUDA(c->rg_p.ensure(ptot * sizeof(double)));
      BACON_CUDA(c->rg_yout.ensure(ytot * sizeof(double)));
      BACON_CUDA(c->rg_tout.ensure(nn * sizeof(double)));
      BACON_CUDA(c->rg_acc.ensure(nn * sizeof(int32_t)));
      BACON_CUDA(c->rg_rej.ensure(nn * sizeof(int32_t)));
      BACON_CUDA(c->rg_st.ensure(nn * sizeof(int32_t)));
      rg.y_off = c->rg_yoff.as<int64_t>();
      rg.p_off = c->rg_poff.as<int64_t>();
      rg.y0 = c->rg_y0.as<double>();
      rg.params = c->rg_p.as<double>();
      rg.t0 = nullptr;
      rg.t_end = nullptr;
      if (g->t0) {
        BACON_CUDA(c->rg_t0.ensure(nn * sizeof(double)));
        rg.t0 = c->rg_t0.as<double>();
      }
      if (g->t_end) {
        BACON_CUDA(c->rg_te.ensure(nn * sizeof(double)));
        rg.t_end = c->rg_te.as<double>();
      }
      rg.y_out = c->rg_yout.as<double>();
      rg.t_out = c->rg_tout.as<double>();
      rg.accepted = c->rg_acc.as<int32_t>();
      rg.rejected = c->rg_rej.as<int32_t>();
      rg.status = c->rg_st.as<int32_t>();
    } else {
      rg.y_off = g->y_offsets;
      rg.p_off = g->p_offsets;
      rg.y0 = g->y0;
      rg.params = g->params;
      rg.t0 = g->t0;
      rg.t_end = g->t_end;
      rg.y_out = gr->y_final;
      rg.t_out = gr->t_final;
      rg.accepted = gr->accepted;
      rg.rejected = gr->rejected;
      rg.status = gr->status;
    }
  }

  // copies in, counters, the launch, copies out
  if (host && un > 0 && (rc = enqueue_h2d(c, up, uo)) != BACON_OK) return rc;
  if (gn > 0) {
    const size_t nn = static_cast<size_t>(gn);
    BACON_CUDA(cudaMemcpyAsync(const_cast<uint32_t*>(rg.order), order.data(), nn * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, c->stream));
    if (host) {
      BACON_CUDA(cudaMemcpyAsync(const_cast<int64_t*>(rg.y_off), yo.data(), (nn + 1) * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, c->stream));
      BACON_CUDA(cudaMemcpyAsync(const_cast<int64_t*>(rg.p_off), po.data(), (nn + 1) * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, c->stream));
      BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(rg.y0), g->y0, ytot * sizeof(double), cudaMemcpyHostToDevice,
                                 c->stream));
      BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(rg.params), g->params, ptot * sizeof(double),
                                 cudaMemcpyHostToDevice, c->stream));
      if (rg.t0)
        BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(rg.t0), g->t0, nn * sizeof(double), cudaMemcpyHostToDevice,
                                   c->stream));
      if (rg.t_end)
        BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(rg.t_end), g->t_end, nn * sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream));
    }
  }
  BACON_CUDA(cudaMemsetAsync(c->d_ctl, 0, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 1, 0xff, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 8, 0, bacon::kRagClasses * sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 5, 0xff, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 6, 0, sizeof(unsigned long long), c->stream));
  void* args[] = {&a, &dyn, &rg};
  BACON_CUDA(cudaEventRecord(c->ev0, c->stream));
  BACON_CUDA(cudaLaunchKernel(fn, dim3(static_cast<unsigned>(grid)), dim3(block), args, smem, c->stream));
  BACON_CUDA(cudaEventRecord(c->ev1, c->stream));
  if (host && un > 0 && (rc = enqueue_d2h(c, up, ur, uo)) != BACON_OK) return rc;
  if (host && gn > 0) {
    const size_t nn = static_cast<size_t>(gn);
    BACON_CUDA(cudaMemcpyAsync(gr->y_final, rg.y_out, ytot * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BACON_CUDA(cudaMemcpyAsync(gr->t_final, rg.t_out, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BACON_CUDA(cudaMemcpyAsync(gr->accepted, rg.accepted, nn * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    BACON_CUDA(cudaMemcpyAsync(gr->rejected, rg.rejected, nn * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    BACON_CUDA(cudaMemcpyAsync(gr->status, rg.status, nn * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  }
  BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 1, c->d_ctl + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
  BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 5, c->d_ctl + 5, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
  c->launches += 1;
  c->ev_valid = true;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  BACON_CUDA(cudaGetLastError());
  if (c->h_ctl[6] != 0) return fail(BACON_CUDA_ERROR, "ragged BDF: a bounded wait on a factor copy gave up");
  const unsigned long long gf = c->h_ctl[5];
  if (gn > 0 && gf != ~0ull) {
    int32_t st = 0;
    if (host) st = gr->status[gf];
    else BACON_CUDA(cudaMemcpy(&st, rg.status + gf, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return fail(st, "ragged system " + std::to_string(gf) + " ended with status " + std::to_string(st));
  }
  if (un > 0) return batch_return_code(c, ur, host, uo);
  return BACON_OK;
}

// ---------------------------------------------------------------------------
// Dense output: every item the reference iterator yields, packed into one
// (t, y) stream with CSR offsets (src/ivp.rs:209-238, collect_vec per
// system).  Two passes: the first solve counts each system's items, a scan of
// the counts gives the offsets, and the second solve, bit-identical to the
// first, writes each item straight to its slot.
namespace {

struct DenseGuard {  // clears the context's dense overrides on every exit
  bacon_ctx* c;
  ~DenseGuard() {
    c->dense_off = nullptr;
    c->dense_t = nullptr;
    c->dense_y = nullptr;
    c->rg_dense_off = nullptr;
    c->rg_dense_voff = nullptr;
    c->rg_dense_t = nullptr;
    c->rg_dense_y = nullptr;
  }
};

// Copies n values between the caller's memory (host or device, as `host`
// says) and a host vector.
template <class T>
int caller_to_host(bacon_ctx* c, bool host, T* dst, const T* src, size_t n) {
  if (n == 0) return BACON_OK;
  if (host) {
    std::memcpy(dst, src, n * sizeof(T));
    return BACON_OK;
  }
  BACON_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  return BACON_OK;
}
template <class T>
int host_to_caller(bacon_ctx* c, bool host, T* dst, const T* src, size_t n) {
  if (n == 0) return BACON_OK;
  if (host) {
    std::memcpy(dst, src, n * sizeof(T));
    return BACON_OK;
  }
  BACON_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  return BACON_OK;
}

template <class Solve>
int dense_two_pass(bacon_ctx* c, const bacon_problem* p, int memory, bacon_rk_result* r, bacon_dense_output* dz,
                   Solve solve) {
  if (!c || !p || !r || !dz) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  if (r->traj_t || r->traj_y) return fail(BACON_INVALID_ARGUMENT, "dense output replaces traj_t / traj_y: pass NULL");
  if (dz->capacity < 0) return fail(BACON_INVALID_ARGUMENT, "capacity < 0");
  if (p->n > 0 && !dz->offsets) return fail(BACON_INVALID_ARGUMENT, "offsets is NULL");
  if (dz->capacity > 0 && (!dz->t || !dz->y)) return fail(BACON_INVALID_ARGUMENT, "t or y is NULL");
  const bool host = memory == BACON_MEM_HOST;
  // Pass 1: the solve alone, for the per-system item counts.
  int rc = solve();
  if (rc == BACON_CUDA_ERROR || rc == BACON_INVALID_ARGUMENT || rc == BACON_UNSUPPORTED) return rc;
  const std::string pass1_msg = g_last_error;
  const size_t n = static_cast<size_t>(p->n);
  std::vector<int32_t> counts(n);
  if (n > 0) {
    if (host) {
      std::memcpy(counts.data(), r->accepted, n * sizeof(int32_t));
    } else {
      BACON_CUDA(cudaMemcpyAsync(counts.data(), r->accepted, n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
      BACON_CUDA(cudaStreamSynchronize(c->stream));
    }
  }
  std::vector<int64_t> off(n + 1);
  off[0] = 0;
  for (size_t i = 0; i < n; ++i) off[i + 1] = off[i] + counts[i];
  dz->total = off[n];
  if (n > 0) {
    if (host) {
      std::memcpy(dz->offsets, off.data(), (n + 1) * sizeof(int64_t));
    } else {
      BACON_CUDA(cudaMemcpyAsync(dz->offsets, off.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                                 c->stream));
      BACON_CUDA(cudaStreamSynchronize(c->stream));
    }
  }
  if (off[n] > dz->capacity)
    return fail(BACON_CAPACITY_EXCEEDED, "dense output needs " + std::to_string(off[n]) + " items, capacity is " +
                                             std::to_string(dz->capacity));
  if (off[n] == 0) {
    g_last_error = pass1_msg;
    return rc;
  }
  // Pass 2: the same solve, writing every item to its packed slot.
  const size_t total = static_cast<size_t>(off[n]);
  DenseGuard guard{c};
  if (host) {
    BACON_CUDA(c->dn_off.ensure((n + 1) * sizeof(int64_t)));
    BACON_CUDA(c->dn_t.ensure(total * sizeof(double)));
    BACON_CUDA(c->dn_y.ensure(total * p->dim * sizeof(double)));
    BACON_CUDA(cudaMemcpyAsync(c->dn_off.p, off.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                               c->stream));
    c->dense_off = c->dn_off.as<int64_t>();
    c->dense_t = c->dn_t.as<double>();
    c->dense_y = c->dn_y.as<double>();
  } else {
    c->dense_off = dz->offsets;
    c->dense_t = dz->t;
    c->dense_y = dz->y;
  }
  const int rc2 = solve();
  if (rc2 == BACON_CUDA_ERROR || rc2 == BACON_INVALID_ARGUMENT || rc2 == BACON_UNSUPPORTED) return rc2;
  if (rc2 != rc) return fail(BACON_CUDA_ERROR, "dense output: the second pass ended differently from the first");
  if (host) {
    BACON_CUDA(cudaMemcpyAsync(dz->t, c->dense_t, total * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BACON_CUDA(cudaMemcpyAsync(dz->y, c->dense_y, total * p->dim * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
    BACON_CUDA(cudaStreamSynchronize(c->stream));
  }
  return rc2;
}

}  // namespace

extern "C" int bacon_rk_solve_dense(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                                    bacon_rk_result* r, bacon_dense_output* dense) {
  NvtxRange nvtx_range("bacon_rk_solve_dense");
  if (!opt || !p) return fail(BACON_INVALID_ARGUMENT, "NULL problem or options");
  return dense_two_pass(c, p, opt->memory, r, dense, [&]() { return bacon_rk_solve(c, p, opt, r); });
}

extern "C" int bacon_bdf_solve_mixed_dense(bacon_ctx* c, const bacon_problem* up, const bacon_ragged_problem* g,
                                           const bacon_bdf_options* opt, bacon_rk_result* ur, bacon_ragged_result* gr,
                                           bacon_dense_output* ud, bacon_ragged_dense_output* gd) {
  NvtxRange nvtx_range("bacon_bdf_solve_mixed_dense");
  if (!c || !opt) return fail(BACON_INVALID_ARGUMENT, "NULL context or options");
  const bool host = opt->memory == BACON_MEM_HOST;
  const int64_t un = up ? up->n : 0, gn = g ? g->n : 0;
  if (!up) ud = nullptr;
  if (!g) gd = nullptr;
  if (ud) {
    if (ud->capacity < 0) return fail(BACON_INVALID_ARGUMENT, "capacity < 0");
    if (un > 0 && !ud->offsets) return fail(BACON_INVALID_ARGUMENT, "offsets is NULL");
    if (ud->capacity > 0 && (!ud->t || !ud->y)) return fail(BACON_INVALID_ARGUMENT, "t or y is NULL");
  }
  if (gd) {
    if (gd->capacity < 0 || gd->value_capacity < 0) return fail(BACON_INVALID_ARGUMENT, "capacity < 0");
    if (gn > 0 && (!gd->offsets || !gd->value_offsets)) return fail(BACON_INVALID_ARGUMENT, "offsets is NULL");
    if ((gd->capacity > 0 && !gd->t) || (gd->value_capacity > 0 && !gd->y))
      return fail(BACON_INVALID_ARGUMENT, "t or y is NULL");
  }
  // Pass 1: the solve alone, for the per-system item counts.
  int rc = bacon_bdf_solve_mixed(c, up, g, opt, ur, gr);
  if (rc == BACON_CUDA_ERROR || rc == BACON_INVALID_ARGUMENT || rc == BACON_UNSUPPORTED) return rc;
  const std::string pass1_msg = g_last_error;
  int rc0;
  std::vector<int64_t> uoff, goff, gvoff;
  if (ud) {
    std::vector<int32_t> cnt(static_cast<size_t>(un));
    if ((rc0 = caller_to_host(c, host, cnt.data(), ur->accepted, cnt.size())) != BACON_OK) return rc0;
    uoff.assign(static_cast<size_t>(un) + 1, 0);
    for (int64_t i = 0; i < un; ++i) uoff[i + 1] = uoff[i] + cnt[i];
    ud->total = uoff[un];
    if (un > 0 && (rc0 = host_to_caller(c, host, ud->offsets, uoff.data(), uoff.size())) != BACON_OK) return rc0;
  }
  if (gd) {
    std::vector<int32_t> cnt(static_cast<size_t>(gn));
    std::vector<int64_t> yo(static_cast<size_t>(gn) + 1);
    if ((rc0 = caller_to_host(c, host, cnt.data(), gr->accepted, cnt.size())) != BACON_OK) return rc0;
    if ((rc0 = caller_to_host(c, host, yo.data(), g->y_offsets, yo.size())) != BACON_OK) return rc0;
    goff.assign(static_cast<size_t>(gn) + 1, 0);
    gvoff.assign(static_cast<size_t>(gn) + 1, 0);
    for (int64_t i = 0; i < gn; ++i) {
      goff[i + 1] = goff[i] + cnt[i];
      gvoff[i + 1] = gvoff[i] + static_cast<int64_t>(cnt[i]) * (yo[i + 1] - yo[i]);
    }
    gd->total = goff[gn];
    gd->total_values = gvoff[gn];
    if (gn > 0) {
      if ((rc0 = host_to_caller(c, host, gd->offsets, goff.data(), goff.size())) != BACON_OK) return rc0;
      if ((rc0 = host_to_caller(c, host, gd->value_offsets, gvoff.data(), gvoff.size())) != BACON_OK) return rc0;
    }
  }
  if (ud && ud->total > ud->capacity)
    return fail(BACON_CAPACITY_EXCEEDED, "dense output of the uniform part needs " + std::to_string(ud->total) +
                                             " items, capacity is " + std::to_string(ud->capacity));
  if (gd && (gd->total > gd->capacity || gd->total_values > gd->value_capacity))
    return fail(BACON_CAPACITY_EXCEEDED, "dense output of the ragged part needs " + std::to_string(gd->total) +
                                             " items and " + std::to_string(gd->total_values) + " values");
  const int64_t utot = ud ? ud->total : 0, gtot = gd ? gd->total : 0, gvtot = gd ? gd->total_values : 0;
  if (utot == 0 && gtot == 0) {
    g_last_error = pass1_msg;
    return rc;
  }
  // Pass 2: the same solve, writing every item to its packed slot.
  DenseGuard guard{c};
  const int dim = up ? up->dim : 0;
  if (utot > 0) {
    if (host) {
      BACON_CUDA(c->dn_off.ensure(uoff.size() * sizeof(int64_t)));
      BACON_CUDA(c->dn_t.ensure(static_cast<size_t>(utot) * sizeof(double)));
      BACON_CUDA(c->dn_y.ensure(static_cast<size_t>(utot) * dim * sizeof(double)));
      BACON_CUDA(cudaMemcpyAsync(c->dn_off.p, uoff.data(), uoff.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                                 c->stream));
      c->dense_off = c->dn_off.as<int64_t>();
      c->dense_t = c->dn_t.as<double>();
      c->dense_y = c->dn_y.as<double>();
    } else {
      c->dense_off = ud->offsets;
      c->dense_t = ud->t;
      c->dense_y = ud->y;
    }
  }
  if (gtot > 0) {
    if (host) {
      BACON_CUDA(c->rdn_off.ensure(goff.size() * sizeof(int64_t)));
      BACON_CUDA(c->rdn_voff.ensure(gvoff.size() * sizeof(int64_t)));
      BACON_CUDA(c->rdn_t.ensure(static_cast<size_t>(gtot) * sizeof(double)));
      BACON_CUDA(c->rdn_y.ensure(static_cast<size_t>(gvtot) * sizeof(double)));
      BACON_CUDA(cudaMemcpyAsync(c->rdn_off.p, goff.data(), goff.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                                 c->stream));
      BACON_CUDA(cudaMemcpyAsync(c->rdn_voff.p, gvoff.data(), gvoff.size() * sizeof(int64_t),
                                 cudaMemcpyHostToDevice, c->stream));
      c->rg_dense_off = c->rdn_off.as<int64_t>();
      c->rg_dense_voff = c->rdn_voff.as<int64_t>();
      c->rg_dense_t = c->rdn_t.as<double>();
      c->rg_dense_y = c->rdn_y.as<double>();
    } else {
      c->rg_dense_off = gd->offsets;
      c->rg_dense_voff = gd->value_offsets;
      c->rg_dense_t = gd->t;
      c->rg_dense_y = gd->y;
    }
  }
  const int rc2 = bacon_bdf_solve_mixed(c, up, g, opt, ur, gr);
  if (rc2 == BACON_CUDA_ERROR || rc2 == BACON_INVALID_ARGUMENT || rc2 == BACON_UNSUPPORTED) return rc2;
  if (rc2 != rc) return fail(BACON_CUDA_ERROR, "dense output: the second pass ended differently from the first");
  if (host) {
    if (utot > 0) {
      BACON_CUDA(cudaMemcpyAsync(ud->t, c->dense_t, utot * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      BACON_CUDA(cudaMemcpyAsync(ud->y, c->dense_y, utot * dim * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    if (gtot > 0) {
      BACON_CUDA(cudaMemcpyAsync(gd->t, c->rg_dense_t, gtot * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
      BACON_CUDA(cudaMemcpyAsync(gd->y, c->rg_dense_y, gvtot * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    BACON_CUDA(cudaStreamSynchronize(c->stream));
  }
  return rc2;
}

extern "C" int bacon_bdf_solve_dense(bacon_ctx* c, const bacon_problem* p, const bacon_bdf_options* opt,
                                     bacon_rk_result* r, bacon_dense_output* dense) {
  NvtxRange nvtx_range("bacon_bdf_solve_dense");
  if (!opt || !p) return fail(BACON_INVALID_ARGUMENT, "NULL problem or options");
  return dense_two_pass(c, p, opt->memory, r, dense, [&]() { return bacon_bdf_solve(c, p, opt, r); });
}

extern "C" int bacon_adams_solve_dense(bacon_ctx* c, const bacon_problem* p, const bacon_adams_options* opt,
                                       bacon_rk_result* r, bacon_dense_output* dense) {
  NvtxRange nvtx_range("bacon_adams_solve_dense");
  if (!opt || !p) return fail(BACON_INVALID_ARGUMENT, "NULL problem or options");
  return dense_two_pass(c, p, opt->memory, r, dense, [&]() { return bacon_adams_solve(c, p, opt, r); });
}

extern "C" int bacon_euler_solve_dense(bacon_ctx* c, const bacon_problem* p, double dt,
                                       const bacon_adams_options* opt, bacon_rk_result* r,
                                       bacon_dense_output* dense) {
  NvtxRange nvtx_range("bacon_euler_solve_dense");
  if (!opt || !p) return fail(BACON_INVALID_ARGUMENT, "NULL problem or options");
  return dense_two_pass(c, p, opt->memory, r, dense, [&]() { return bacon_euler_solve(c, p, dt, opt, r); });
}

// ---------------------------------------------------------------------------
// Autotuner: times the persistent kernel on the caller's own batch for a set
// of launch shapes and caches the fastest for this kernel and batch size.
extern "C" int bacon_rk_autotune_ex(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                                    bacon_rk_result* r, bacon_tune_result* out) {
  NvtxRange nvtx_range("bacon_rk_autotune");
  if (!c || !opt || !p) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  if (p->rhs == BACON_RHS_LINEAR) return fail(BACON_UNSUPPORTED, "the linear engine has no persistent kernel");
  // Launch shapes (threads per block, CTAs per SM) per register budget: the
  // default kernel over the whole range, the capped ones at the occupancies
  // their budgets open up.
  static const int kShapes[][2] = {{32, 4}, {64, 2}, {128, 1}, {128, 2}, {128, 3}, {128, 4}, {256, 1}, {256, 2}};
  static const int kCappedShapes[][2] = {{128, 4}, {256, 2}, {256, 3}, {256, 4}};
  const int layout = (opt->method == BACON_RK23 && opt->layout == BACON_LAYOUT_FEHLBERG) ? 1 : opt->layout;
  const bacon::RkKey key{opt->method, layout, opt->precision, p->rhs, p->dim};
  std::vector<int> variants{0};
  for (const auto& e : c->kernels)
    if (e.key == key && e.variant > 0) variants.push_back(e.variant);
  bacon_rk_options o = *opt;
  o.use_graph = 0;
  double best_ms = 1e300, default_ms = 0.0;
  int bv = 0, bb = 0, bs = 0, count = 0;
  struct Restore {
    bacon_ctx* c;
    ~Restore() { c->force_variant = -1; }
  } restore{c};
  // The untuned default first (occupancy model, variant 0).
  c->force_variant = 0;
  o.block = 0;
  o.blocks_per_sm = 0;
  int rc = bacon_rk_solve(c, p, &o, r);
  if (rc == BACON_CUDA_ERROR || rc == BACON_INVALID_ARGUMENT || rc == BACON_UNSUPPORTED) return rc;
  if (bacon_ctx_last_kernel_ms(c, &default_ms) != BACON_OK) return BACON_CUDA_ERROR;
  for (int v : variants) {
    c->force_variant = v;
    const void* vfn = nullptr;
    for (const auto& e : c->kernels)
      if (e.key == key && e.variant == v) vfn = e.fn;
    const auto* shapes = v == 0 ? kShapes : kCappedShapes;
    const int ns = v == 0 ? static_cast<int>(sizeof(kShapes) / sizeof(kShapes[0]))
                          : static_cast<int>(sizeof(kCappedShapes) / sizeof(kCappedShapes[0]));
    std::vector<std::pair<int, int>> timed;
    for (int k = 0; k < ns; ++k) {
      // the shape as launched: CTAs per SM capped by this variant's occupancy,
      // and a shape that caps onto one already timed is not timed again
      int bps = shapes[k][1];
      if (vfn) {
        int max_bps = 0;
        BACON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_bps, vfn, shapes[k][0], 0));
        if (max_bps >= 1 && bps > max_bps) bps = max_bps;
      }
      const std::pair<int, int> shape{shapes[k][0], bps};
      if (std::find(timed.begin(), timed.end(), shape) != timed.end()) continue;
      timed.push_back(shape);
      o.block = shapes[k][0];
      o.blocks_per_sm = bps;
      rc = bacon_rk_solve(c, p, &o, r);
      if (rc == BACON_CUDA_ERROR || rc == BACON_INVALID_ARGUMENT || rc == BACON_UNSUPPORTED) return rc;
      double ms = 0.0;
      if (bacon_ctx_last_kernel_ms(c, &ms) != BACON_OK) return BACON_CUDA_ERROR;
      ++count;
      if (ms < best_ms) {
        best_ms = ms;
        bv = v;
        bb = shapes[k][0];
        bs = bps;
      }
    }
  }
  // Systems per warp below 32, for a batch too small to give every SM four
  // warps of 32 (default kernel, one-warp blocks): less divergence within a
  // warp where the FP64 pipe has room for more warps.
  int bl = 0;
  if (p->n <= static_cast<int64_t>(c->num_sms) * 32 * 4) {
    c->force_variant = 0;
    for (int lanes : {16, 8}) {
      o.block = 32;
      o.blocks_per_sm = 0;
      o.systems_per_warp = lanes;
      rc = bacon_rk_solve(c, p, &o, r);
      if (rc == BACON_CUDA_ERROR || rc == BACON_INVALID_ARGUMENT || rc == BACON_UNSUPPORTED) return rc;
      double ms = 0.0;
      if (bacon_ctx_last_kernel_ms(c, &ms) != BACON_OK) return BACON_CUDA_ERROR;
      ++count;
      if (ms < best_ms) {
        best_ms = ms;
        bv = 0;
        bb = 32;
        bs = 0;  // as many one-warp blocks as the batch needs, up to the occupancy
        bl = lanes;
      }
    }
    o.systems_per_warp = 0;
  }
  c->tuned[tune_key(key, p->n)] = bacon_ctx::Tuned{bv, bb, bs, bl};
  if (out) {
    out->variant = bv;
    out->max_registers = bacon::variant_max_registers(bv);
    out->systems_per_warp = bl > 0 ? bl : 32;
    out->block = bb;
    out->blocks_per_sm = bs;
    out->candidates = count;
    out->best_ms = best_ms;
    out->default_ms = default_ms;
  }
  return BACON_OK;
}

extern "C" int bacon_rk_set_tuned(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                                  const bacon_tune_result* t) {
  if (!c || !opt || !p || !t) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  if (t->block % 32 != 0 || t->block < 32 || t->block > 256 || t->blocks_per_sm < 0)
    return fail(BACON_INVALID_ARGUMENT, "block must be a multiple of 32 in 32..256, blocks_per_sm >= 0");
  const int layout = (opt->method == BACON_RK23 && opt->layout == BACON_LAYOUT_FEHLBERG) ? 1 : opt->layout;
  const bacon::RkKey key{opt->method, layout, opt->precision, p->rhs, p->dim};
  bool found = false;
  for (const auto& e : c->kernels)
    if (e.key == key && e.variant == t->variant) found = true;
  if (!found) return fail(BACON_UNSUPPORTED, "no such kernel variant for this (method, layout, precision, rhs, dim)");
  if (t->systems_per_warp < 0 || t->systems_per_warp > 32)
    return fail(BACON_INVALID_ARGUMENT, "systems_per_warp must be 0..32");
  const int lanes = t->systems_per_warp == 32 ? 0 : t->systems_per_warp;
  c->tuned[tune_key(key, p->n)] = bacon_ctx::Tuned{t->variant, t->block, t->blocks_per_sm, lanes};
  return BACON_OK;
}

extern "C" int bacon_rk_autotune(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                                 bacon_rk_result* r, int32_t* best_block, int32_t* best_blocks_per_sm) {
  bacon_tune_result t{};
  const int rc = bacon_rk_autotune_ex(c, p, opt, r, &t);
  if (rc != BACON_OK) return rc;
  if (best_block) *best_block = t.block;
  if (best_blocks_per_sm) *best_blocks_per_sm = t.blocks_per_sm;
  return BACON_OK;
}

// ---------------------------------------------------------------------------
// Discrete adjoint: recording forward pass, then the reverse kernel.
extern "C" int bacon_rk_solve_adjoint(bacon_ctx* c, const bacon_problem* p, const bacon_rk_options* opt,
                                      bacon_rk_result* r, bacon_adjoint* adj) {
  NvtxRange nvtx_range("bacon_rk_solve_adjoint");
  if (!c || !opt || !adj) return fail(BACON_INVALID_ARGUMENT, "NULL context, options or adjoint");
  int rc = bacon_rk_validate(p);
  if (rc != BACON_OK) return rc;
  if ((rc = check_result_ptrs(p, r)) != BACON_OK) return rc;
  if (r->traj_t) return fail(BACON_UNSUPPORTED, "the adjoint records no trajectory");
  if (opt->precision != BACON_FP64_EXACT) return fail(BACON_UNSUPPORTED, "the adjoint runs in FP64_EXACT");
  if (opt->layout == BACON_LAYOUT_AS_COMPILED)
    return fail(BACON_UNSUPPORTED, "the as_compiled matrix reuses stages across attempts: no one-step map");
  if (p->dyn_dim && p->dim == 4) return fail(BACON_UNSUPPORTED, "dynamic 4-vectors are not compiled");
  if (p->n > 0 && (!adj->target || !adj->loss || !adj->dl_dy0 || (p->n_params > 0 && !adj->dl_dp)))
    return fail(BACON_INVALID_ARGUMENT, "adjoint array is NULL");
  const int every = adj->checkpoint_every > 0 ? adj->checkpoint_every : 32;
  const int max_steps = adj->max_steps > 0 ? adj->max_steps : 1024;
  if (every > 32) return fail(BACON_INVALID_ARGUMENT, "checkpoint_every must be in 1..32");
  const int layout = (opt->method == BACON_RK23) ? 1 : opt->layout;
  const bacon::RkKey key{opt->method, layout, 0, p->rhs, p->dim};
  const bacon::AdjEntry* ent = nullptr;
  for (const auto& e : c->adjoint_kernels)
    if (e.key == key) ent = &e;
  if (!ent) return fail(BACON_UNSUPPORTED, "no adjoint kernel for this (method, layout, rhs, dim)");
  if (p->n == 0) return BACON_OK;
  BACON_CUDA(cudaSetDevice(c->device));
  const bool host = opt->memory == BACON_MEM_HOST;
  Resolved o{};
  if ((rc = stage_inputs(c, p, r, host, o)) != BACON_OK) return rc;
  const size_t n = static_cast<size_t>(p->n);
  const int slots = (max_steps + every - 1) / every;
  BACON_CUDA(c->adj_dt.ensure(n * max_steps * sizeof(double)));
  BACON_CUDA(c->adj_ck.ensure(n * slots * (p->dim + 1) * sizeof(double)));
  const double* tgt = adj->target;
  double *loss = adj->loss, *gy = adj->dl_dy0, *gp = adj->dl_dp;
  if (host) {
    BACON_CUDA(c->adj_tgt.ensure(n * p->dim * sizeof(double)));
    BACON_CUDA(c->adj_loss.ensure(n * sizeof(double)));
    BACON_CUDA(c->adj_gy.ensure(n * p->dim * sizeof(double)));
    BACON_CUDA(c->adj_gp.ensure(n * (p->n_params > 0 ? p->n_params : 1) * sizeof(double)));
    tgt = c->adj_tgt.as<double>();
    loss = c->adj_loss.as<double>();
    gy = c->adj_gy.as<double>();
    gp = c->adj_gp.as<double>();
  }

  double dt_min = p->dt_min;
  clamp_dt(dt_min, p->dt_max);
  bacon::RkArgs a{};
  a.n = p->n;
  a.y0 = o.y0;
  a.params = o.params;
  a.t0 = o.t0;
  a.t_end = o.t_end;
  a.t0_s = p->t0_scalar;
  a.t_end_s = p->t_end_scalar;
  a.tol = p->tol;
  a.dt_min = dt_min;
  a.dt_max = p->dt_max;
  a.max_attempts = opt->max_attempts > 0 ? opt->max_attempts : 10000000;
  a.y_out = o.y_out;
  a.t_out = o.t_out;
  a.accepted = o.acc;
  a.rejected = o.rej;
  a.status = o.st;
  a.queue = c->d_ctl;
  a.first_fail = c->d_ctl + 1;
  a.dt_log = c->adj_dt.as<double>();
  a.ckpt = c->adj_ck.as<double>();
  a.ckpt_every = every;
  a.max_steps = max_steps;
  a.ckpt_slots = slots;
  const bool per_system_times = (p->t0 != nullptr) || (p->t_end != nullptr);
  const bool lpt = (opt->schedule == 2 || (opt->schedule == 0 && per_system_times)) && p->n < (1ll << 32);
  bacon::OrderArgs oa{};
  if (lpt) {
    BACON_CUDA(c->ord.ensure(n * sizeof(uint32_t)));
    BACON_CUDA(c->ord_scratch.ensure(sizeof(bacon::OrderScratch)));
    oa = bacon::OrderArgs{p->n, o.t0, o.t_end, p->t0_scalar, p->t_end_scalar,
                          c->ord_scratch.as<bacon::OrderScratch>(), c->ord.as<uint32_t>()};
    a.order = oa.order;
  }
  bacon::AdjArgs b{};
  b.n = p->n;
  b.params = o.params;
  b.y_final = o.y_out;
  b.accepted = o.acc;
  b.status = o.st;
  b.dt_log = a.dt_log;
  b.ckpt = a.ckpt;
  b.target = tgt;
  b.loss = loss;
  b.dl_dy0 = gy;
  b.dl_dp = gp;
  b.max_steps = max_steps;
  b.ckpt_slots = slots;
  b.ckpt_every = every;
  b.queue = c->d_ctl + 3;
  // The reverse pass replays each system's accepted steps: hand the systems
  // out most steps first (the counts are known once the forward pass ends).
  bacon::OrderArgs rev_oa{};
  const bool rev_lpt = p->n < (1ll << 32);
  if (rev_lpt) {
    BACON_CUDA(c->ord.ensure(n * sizeof(uint32_t)));
    BACON_CUDA(c->ord_scratch.ensure(sizeof(bacon::OrderScratch)));
    rev_oa = bacon::OrderArgs{p->n, nullptr, nullptr, 0.0, 0.0, c->ord_scratch.as<bacon::OrderScratch>(),
                              c->ord.as<uint32_t>(), o.acc};
    b.order = rev_oa.order;
  }

  const int block = opt->block > 0 ? opt->block : bacon::default_block(p->n, c->num_sms, 128);
  if (block % 32 != 0 || block > 256) return fail(BACON_INVALID_ARGUMENT, "block must be a multiple of 32, <= 256");
  int fwd_bps = 0, rev_bps = 0;
  BACON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fwd_bps, ent->fwd, block, 0));
  BACON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rev_bps, ent->rev, 128, 0));
  if (fwd_bps < 1 || rev_bps < 1) return fail(BACON_CUDA_ERROR, "adjoint kernels cannot be resident");
  // The recording pass is the forward solve plus its step log: the same
  // occupancy model as bacon_rk_solve.
  int bps = opt->blocks_per_sm > 0 ? opt->blocks_per_sm : model_blocks_per_sm(p->n, c->num_sms, block, fwd_bps);
  if (bps > fwd_bps) bps = fwd_bps;
  const long long need = (p->n + block - 1) / block;
  long long fgrid = static_cast<long long>(c->num_sms) * bps;
  if (fgrid > need) fgrid = need;
  long long rgrid = static_cast<long long>(c->num_sms) * (rev_bps < 2 ? rev_bps : 2);
  const long long rneed = (p->n + 127) / 128;
  if (rgrid > rneed) rgrid = rneed;

  if (host) {
    if ((rc = enqueue_h2d(c, p, o)) != BACON_OK) return rc;
    BACON_CUDA(cudaMemcpyAsync(const_cast<double*>(tgt), adj->target, n * p->dim * sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
  }
  if (lpt) BACON_CUDA(bacon::enqueue_lpt_order(oa, c->num_sms, c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl, 0, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 1, 0xff, sizeof(unsigned long long), c->stream));
  BACON_CUDA(cudaMemsetAsync(c->d_ctl + 3, 0, sizeof(unsigned long long), c->stream));
  void* fargs[] = {&a};
  void* rargs[] = {&b};
  BACON_CUDA(cudaEventRecord(c->ev0, c->stream));
  BACON_CUDA(cudaLaunchKernel(ent->fwd, dim3(static_cast<unsigned>(fgrid)), dim3(block), fargs, 0, c->stream));
  BACON_CUDA(cudaEventRecord(c->ev1, c->stream));
  BACON_CUDA(cudaEventRecord(c->ev2, c->stream));
  if (rev_lpt) BACON_CUDA(bacon::enqueue_lpt_order(rev_oa, c->num_sms, c->stream));
  BACON_CUDA(cudaLaunchKernel(ent->rev, dim3(static_cast<unsigned>(rgrid)), dim3(128), rargs, 0, c->stream));
  BACON_CUDA(cudaEventRecord(c->ev3, c->stream));
  if (host) {
    if ((rc = enqueue_d2h(c, p, r, o)) != BACON_OK) return rc;
    BACON_CUDA(cudaMemcpyAsync(adj->loss, loss, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BACON_CUDA(cudaMemcpyAsync(adj->dl_dy0, gy, n * p->dim * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (p->n_params > 0)
      BACON_CUDA(cudaMemcpyAsync(adj->dl_dp, gp, n * p->n_params * sizeof(double), cudaMemcpyDeviceToHost,
                                 c->stream));
  }
  BACON_CUDA(cudaMemcpyAsync(c->h_ctl + 1, c->d_ctl + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
  c->launches += (lpt ? 6 : 2) + (rev_lpt ? 4 : 0);
  c->ev_valid = true;
  c->rev_valid = true;
  BACON_CUDA(cudaStreamSynchronize(c->stream));
  BACON_CUDA(cudaGetLastError());
  return batch_return_code(c, r, host, o);
}

// ---------------------------------------------------------------------------
// Builder mirror of the IVPSolver trait (src/ivp.rs:134-190,
// src/ivp/rk.rs:136-247, src/ivp/bdf.rs:144-255).
struct bacon_builder {
  int32_t kind = 0;
  int32_t dim = 0;
  bool dyn = false;
  bool has_dt_max = false, has_dt_min = false, has_t0 = false, has_end = false, has_tol = false;
  double dt_max = 0, dt_min = 0, t0 = 0, t_end = 0, tol = 0;
  bool has_euler_dt = false;  // Euler (kind 6): one step size
  double euler_dt = 0;
  std::vector<double> y0;
  int64_t n = 0;
  bool has_y0 = false;
  int32_t rhs = -1;
  std::vector<double> params;
  int32_t n_params = 0;
  std::vector<double> t_ends;
};

extern "C" {

int bacon_builder_new(int32_t kind, int32_t dim, bacon_builder** out) {
  if (!out) return fail(BACON_INVALID_ARGUMENT, "out is NULL");
  if (kind < 0 || kind > 6 || dim < 1) return fail(BACON_INVALID_ARGUMENT, "bad kind or dim");
  *out = new bacon_builder();
  (*out)->kind = kind;
  (*out)->dim = dim;
  return BACON_OK;
}

int bacon_builder_new_dyn(int32_t kind, int32_t size, bacon_builder** out) {
  const int rc = bacon_builder_new(kind, size, out);
  if (rc == BACON_OK) (*out)->dyn = true;
  return rc;
}

void bacon_builder_free(bacon_builder* b) { delete b; }

int bacon_builder_with_tolerance(bacon_builder* b, double tol) {
  if (!b) return fail(BACON_INVALID_ARGUMENT, "builder is NULL");
  if (b->kind == 6) return BACON_OK;  // Euler: a no-op (src/ivp.rs:390-393)
  if (tol <= 0.0) return fail(BACON_TOLERANCE_OOB, "the provided tolerance was out-of-bounds");
  b->tol = tol;
  b->has_tol = true;
  return BACON_OK;
}

// Euler keeps one step: the first value set, then the mean with each later
// one (src/ivp.rs:395-423).
static int euler_set_dt(bacon_builder* b, double v) {
  b->euler_dt = b->has_euler_dt ? (b->euler_dt + v) / 2.0 : v;
  b->has_euler_dt = true;
  return BACON_OK;
}

int bacon_builder_with_maximum_dt(bacon_builder* b, double max) {
  if (!b) return fail(BACON_INVALID_ARGUMENT, "builder is NULL");
  if (max <= 0.0) return fail(BACON_TIME_DELTA_OOB, "the provided time delta was out-of-bounds");
  if (b->kind == 6) return euler_set_dt(b, max);
  b->dt_max = max;
  b->has_dt_max = true;
  if (b->has_dt_min && b->dt_min > max) b->dt_min = max;
  return BACON_OK;
}

int bacon_builder_with_minimum_dt(bacon_builder* b, double min) {
  if (!b) return fail(BACON_INVALID_ARGUMENT, "builder is NULL");
  if (min <= 0.0) return fail(BACON_TIME_DELTA_OOB, "the provided time delta was out-of-bounds");
  if (b->kind == 6) return euler_set_dt(b, min);
  b->dt_min = min;
  b->has_dt_min = true;
  if (b->has_dt_max && b->dt_max < min) b->dt_max = min;
  return BACON_OK;
}

int bacon_builder_with_initial_time(bacon_builder* b, double initial) {
  if (!b) return fail(BACON_INVALID_ARGUMENT, "builder is NULL");
  b->t0 = initial;
  b->has_t0 = true;
  if (b->has_end && b->t_end <= initial)
    return fail(BACON_TIME_START_OOB, "the provided starting time was after the provided ending time");
  for (double e : b->t_ends)
    if (e <= initial) return fail(BACON_TIME_START_OOB, "the provided starting time was after an ending time");
  return BACON_OK;
}

int bacon_builder_with_ending_time(bacon_builder* b, double ending) {
  if (!b) return fail(BACON_INVALID_ARGUMENT, "builder is NULL");
  b->t_end = ending;
  b->has_end = true;
  b->t_ends.clear();
  if (b->has_t0 && b->t0 >= ending)
    return fail(BACON_TIME_END_OOB, "the provided ending time was before the provided starting time");
  return BACON_OK;
}

int bacon_builder_with_ending_times(bacon_builder* b, const double* t_end, int64_t n) {
  if (!b || (!t_end && n > 0) || n < 0) return fail(BACON_INVALID_ARGUMENT, "bad arguments");
  b->t_ends.assign(t_end, t_end + n);
  b->has_end = true;
  if (b->has_t0)
    for (int64_t i = 0; i < n; ++i)
      if (b->t0 >= t_end[i])
        return fail(BACON_TIME_END_OOB, "ending time of system " + std::to_string(i) + " is not after the start");
  return BACON_OK;
}

int bacon_builder_with_initial_conditions(bacon_builder* b, const double* y0, int64_t n) {
  if (!b || (!y0 && n > 0) || n < 0) return fail(BACON_INVALID_ARGUMENT, "bad arguments");
  b->y0.assign(y0, y0 + static_cast<size_t>(n) * b->dim);
  b->n = n;
  b->has_y0 = true;
  return BACON_OK;
}

int bacon_builder_with_derivative(bacon_builder* b, int32_t rhs, const double* params, int32_t n_params) {
  if (!b || n_params < 0 || (n_params > 0 && !params)) return fail(BACON_INVALID_ARGUMENT, "bad arguments");
  if (rhs < 0 || rhs > BACON_RHS_LINEAR) return fail(BACON_INVALID_ARGUMENT, "unknown rhs");
  b->rhs = rhs;
  b->n_params = n_params;
  b->params.clear();
  if (n_params > 0) {
    if (!b->has_y0) return fail(BACON_INVALID_ARGUMENT, "set initial conditions before per-system parameters");
    b->params.assign(params, params + static_cast<size_t>(n_params) * b->n);
  }
  return BACON_OK;
}

int bacon_builder_problem(const bacon_builder* b, bacon_problem* out) {
  if (!b || !out) return fail(BACON_INVALID_ARGUMENT, "NULL argument");
  // rk.rs:250-256 / bdf.rs:258-264 / adams.rs:253-259: every parameter must
  // have been set; Euler needs no tolerance and one step size (ivp.rs:444-452).
  const bool euler = b->kind == 6;
  const bool have_dt = euler ? b->has_euler_dt : (b->has_dt_max && b->has_dt_min && b->has_tol);
  if (!have_dt || !b->has_t0 || !b->has_end || !b->has_y0 || b->rhs < 0)
    return fail(BACON_MISSING_PARAMETERS, "the solver does not have all required parameters set");
  if (!b->t_ends.empty() && static_cast<int64_t>(b->t_ends.size()) != b->n)
    return fail(BACON_INVALID_ARGUMENT, "ending times and initial conditions disagree in length");
  std::memset(out, 0, sizeof(*out));
  out->n = b->n;
  out->dim = b->dim;
  out->rhs = b->rhs;
  out->n_params = b->n_params;
  out->dyn_dim = b->dyn ? 1 : 0;
  out->y0 = b->y0.data();
  out->params = b->n_params > 0 ? b->params.data() : nullptr;
  out->t0 = nullptr;
  out->t_end = b->t_ends.empty() ? nullptr : b->t_ends.data();
  out->t0_scalar = b->t0;
  out->t_end_scalar = b->t_ends.empty() ? b->t_end : 0.0;
  if (!b->t_ends.empty()) out->t_end_scalar = b->t0 + 1.0;  // unused: per-system ends given
  out->tol = euler ? 1.0 : b->tol;
  out->dt_min = euler ? b->euler_dt : b->dt_min;
  out->dt_max = euler ? b->euler_dt : b->dt_max;
  return BACON_OK;
}

}  // extern "C"
