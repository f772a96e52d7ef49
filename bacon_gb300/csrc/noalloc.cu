// Allocation-free batched Runge-Kutta solve (bacon_rk_solve_noalloc).
//
// Some callers cannot allocate device memory: a library embedded in an
// application whose memory pool has reserved the GPU's memory, a hot loop
// where an allocation's latency or failure is not acceptable, or plugin code
// that is handed nothing but a stream and device pointers.  This entry point
// runs the same persistent kernel as bacon_rk_solve without a context and
// without cudaMalloc, cudaFree or any other allocating call.  The scratch the
// kernel needs (work counter, lowest-failing-index slot, longest-first order
// and its sort counters) lives in one fixed device array in this file.  Every
// GPU that loads the library holds that array (about 4 MiB) until the process
// exits.  The CUDA runtime loads device code lazily, so the array and the
// kernels are placed on a device by the first call there; a call with n == 0
// does only that, for the kernel its options select.  Make that call before
// the caller's memory pool reserves the GPU's memory.
// The device address found then is kept for the life of the process: calls
// must not span a cudaDeviceReset, which rebuilds the context and may move
// the array.
#include "bacon_gb300.h"

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "order.h"
#include "registry.h"
#include "rk_kernel.cuh"

namespace {

// Largest batch the fixed scratch can order: one 32-bit index per system.
constexpr int64_t kNoallocMaxSystems = int64_t{1} << 20;

// Byte offsets of the scratch parts inside the array.
constexpr size_t kQueueOff = 0;        // unsigned long long work counter
constexpr size_t kFirstFailOff = 8;    // unsigned long long lowest failing index
constexpr size_t kOrderScratchOff = 256;
constexpr size_t kOrderOff = kOrderScratchOff + ((sizeof(bacon::OrderScratch) + 255) / 256) * 256;
constexpr size_t kScratchBytes = kOrderOff + sizeof(uint32_t) * kNoallocMaxSystems;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Kernel table, built when the library is loaded so that the entry point
// itself never allocates.
const std::vector<bacon::RkEntry> g_kernels = bacon::all_rk_kernels();

// Device address of the scratch array on the current device, looked up once
// per device (the host-side name of a __device__ array is not an address the
// GPU can use).
cudaError_t scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

int expected_dim(int rhs) {
  switch (rhs) {
    case BACON_RHS_HARMONIC:
    case BACON_RHS_VDP:
    case BACON_RHS_LOTKA: return 2;
    case BACON_RHS_LORENZ:
    case BACON_RHS_ROBERTSON: return 3;
    default: return -1;
  }
}

int expected_params(int rhs) {
  switch (rhs) {
    case BACON_RHS_VDP: return 1;
    case BACON_RHS_LORENZ: return 3;
    case BACON_RHS_LOTKA: return 4;
    case BACON_RHS_ROBERTSON: return 3;
    default: return 0;
  }
}

}  // namespace

extern "C" int bacon_rk_solve_noalloc(const bacon_problem* p, const bacon_rk_options* opt,
                                      bacon_rk_result* r, void* stream) {
  if (!p || !opt || !r) return BACON_INVALID_ARGUMENT;
  if (opt->memory != BACON_MEM_DEVICE) return BACON_INVALID_ARGUMENT;
  // The builder's checks (src/ivp/rk.rs:168-256), without composing messages.
  if (p->n < 0 || p->dim < 1) return BACON_INVALID_ARGUMENT;
  if (p->n > kNoallocMaxSystems) return BACON_CAPACITY_EXCEEDED;
  if (p->n > 0 && !p->y0) return BACON_MISSING_PARAMETERS;
  if (p->tol <= 0.0) return BACON_TOLERANCE_OOB;
  if (p->dt_max <= 0.0 || p->dt_min <= 0.0) return BACON_TIME_DELTA_OOB;
  if (!p->t0 && !p->t_end && p->t0_scalar >= p->t_end_scalar) return BACON_TIME_END_OOB;
  if (p->rhs < 0 || p->rhs > BACON_RHS_LINEAR) return BACON_INVALID_ARGUMENT;
  const int ed = expected_dim(p->rhs);
  if (ed > 0 && p->dim != ed) return BACON_INVALID_ARGUMENT;
  if (p->n_params < expected_params(p->rhs)) return BACON_INVALID_ARGUMENT;
  if (p->n > 0 && p->n_params > 0 && !p->params) return BACON_INVALID_ARGUMENT;
  if (p->n > 0 && (!r->y_final || !r->t_final || !r->accepted || !r->rejected || !r->status))
    return BACON_INVALID_ARGUMENT;
  if ((r->traj_t == nullptr) != (r->traj_y == nullptr) || (r->traj_t && r->traj_cap < 0))
    return BACON_INVALID_ARGUMENT;
  if (opt->method != BACON_RK45 && opt->method != BACON_RK23) return BACON_INVALID_ARGUMENT;
  if (opt->layout < 0 || opt->layout > 2 || opt->precision < 0 || opt->precision > 2)
    return BACON_INVALID_ARGUMENT;
  if (p->dyn_dim && p->dim == 4) return BACON_UNSUPPORTED;
  const int layout = (opt->method == BACON_RK23 && opt->layout == BACON_LAYOUT_FEHLBERG) ? 1 : opt->layout;
  const bacon::RkKey key{opt->method, layout, opt->precision, p->rhs, p->dim};
  const void* fn = nullptr;
  for (const auto& e : g_kernels)
    if (e.key == key && e.variant == 0) fn = e.fn;
  if (!fn) return BACON_UNSUPPORTED;

  // The address lookup places the scratch array on the current device (CUDA
  // loads device code lazily), so it comes before the n == 0 return: a
  // zero-size call is the warm-up that places the array and the kernels.
  unsigned char* scratch = nullptr;
  if (scratch_for_current_device(&scratch) != cudaSuccess) return BACON_CUDA_ERROR;
  if (p->n == 0) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess || bacon::preload_lpt_order_kernels() != cudaSuccess)
      return BACON_CUDA_ERROR;
    return BACON_OK;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, num_sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return BACON_CUDA_ERROR;

  double dt_min = p->dt_min;
  if (dt_min > p->dt_max) dt_min = p->dt_max;  // with_minimum_dt, then with_maximum_dt
  bacon::RkArgs a{};
  a.n = p->n;
  a.y0 = p->y0;
  a.params = p->params;
  a.t0 = p->t0;
  a.t_end = p->t_end;
  a.t0_s = p->t0_scalar;
  a.t_end_s = p->t_end_scalar;
  a.tol = p->tol;
  a.dt_min = dt_min;
  a.dt_max = p->dt_max;
  a.max_attempts = opt->max_attempts > 0 ? opt->max_attempts : 10000000;
  a.y_out = r->y_final;
  a.t_out = r->t_final;
  a.accepted = r->accepted;
  a.rejected = r->rejected;
  a.status = r->status;
  a.traj_t = r->traj_t;
  a.traj_y = r->traj_y;
  a.traj_cap = r->traj_t ? r->traj_cap : 0;
  a.queue = reinterpret_cast<unsigned long long*>(scratch + kQueueOff);
  a.first_fail = reinterpret_cast<unsigned long long*>(scratch + kFirstFailOff);
  a.order = nullptr;
  const bool per_system_times = (p->t0 != nullptr) || (p->t_end != nullptr);
  const bool lpt = opt->schedule == 2 || (opt->schedule == 0 && per_system_times);
  bacon::OrderArgs oa{};
  if (lpt) {
    oa = bacon::OrderArgs{p->n, p->t0, p->t_end, p->t0_scalar, p->t_end_scalar,
                          reinterpret_cast<bacon::OrderScratch*>(scratch + kOrderScratchOff),
                          reinterpret_cast<uint32_t*>(scratch + kOrderOff)};
    a.order = oa.order;
  }

  if (opt->systems_per_warp < 0 || opt->systems_per_warp > 32) return BACON_INVALID_ARGUMENT;
  a.lanes = opt->systems_per_warp == 32 ? 0 : opt->systems_per_warp;
  const int spw = a.lanes > 0 ? a.lanes : 32;
  const int block =
      opt->block > 0 ? opt->block : (a.lanes > 0 ? 32 : bacon::default_block(p->n, num_sms, 128));
  if (block % 32 != 0 || block > 256) return BACON_INVALID_ARGUMENT;
  int max_bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_bps, fn, block, 0) != cudaSuccess || max_bps < 1)
    return BACON_CUDA_ERROR;
  int bps = opt->blocks_per_sm > 0 ? opt->blocks_per_sm : max_bps;
  if (bps > max_bps) bps = max_bps;
  long long grid = static_cast<long long>(num_sms) * bps;
  const long long per_block = static_cast<long long>(block / 32) * spw;  // systems a block holds at a time
  const long long need = (p->n + per_block - 1) / per_block;
  if (grid > need) grid = need;

  // The array keeps the previous call's contents: reset the counters.
  if (lpt && bacon::enqueue_lpt_order(oa, num_sms, s) != cudaSuccess) return BACON_CUDA_ERROR;
  if (cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), s) != cudaSuccess ||
      cudaMemsetAsync(a.first_fail, 0xff, sizeof(unsigned long long), s) != cudaSuccess)
    return BACON_CUDA_ERROR;
  void* args[] = {&a};
  if (cudaLaunchKernel(fn, dim3(static_cast<unsigned>(grid)), dim3(block), args, 0, s) != cudaSuccess)
    return BACON_CUDA_ERROR;
  unsigned long long first_fail = 0;
  if (cudaMemcpyAsync(&first_fail, a.first_fail, sizeof(first_fail), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return BACON_CUDA_ERROR;
  if (first_fail == ~0ull) return BACON_OK;
  int32_t st = 0;
  if (cudaMemcpyAsync(&st, r->status + first_fail, sizeof(st), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return BACON_CUDA_ERROR;
  return st;
}
