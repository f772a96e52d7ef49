// Longest-first (LPT) work order for the persistent kernels.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace bacon {

constexpr int kOrderBuckets = 1024;

struct OrderScratch {
  unsigned long long minmax[2];           // bit patterns of the min / max span
  unsigned int offset[kOrderBuckets];     // bucket counts, then write cursors
};

struct OrderArgs {
  int64_t n;
  const double* t0;     // [n] or null
  const double* t_end;  // [n] or null
  double t0_s, t_end_s;
  OrderScratch* scratch;
  uint32_t* order;      // [n] output permutation, longest span first
  // When set, system i's span is weight[i] (a work count known beforehand,
  // such as the accepted steps a reverse pass replays) instead of t_end - t0.
  const int32_t* weight = nullptr;
};

// Enqueues the four kernels that fill a.order.  Needs n < 2^32.
cudaError_t enqueue_lpt_order(const OrderArgs& a, int num_sms, cudaStream_t s);

// Loads the order kernels' device code onto the current device now rather
// than at their first launch.
cudaError_t preload_lpt_order_kernels();

}  // namespace bacon
