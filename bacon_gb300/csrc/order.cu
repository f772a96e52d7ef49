// Longest-first work order for the persistent kernels.
//
// Systems with uneven integration spans (t_end - t0) finish at uneven times;
// handing the longest ones out first (LPT scheduling) keeps every lane busy
// until the queue drains.  The order is a counting sort of the spans into
// kOrderBuckets buckets, longest bucket first, built on the device in four
// short kernels: span min/max, histogram, scan, scatter.  Order within a
// bucket depends on atomic timing; the per-system results do not, since every
// system is integrated independently.
#include <cstdint>

#include "order.h"

namespace bacon {

namespace {

__device__ __forceinline__ double span_of(const OrderArgs& a, int64_t i) {
  if (a.weight) {
    const int32_t w = a.weight[i];
    return w > 0 ? static_cast<double>(w) : 0.0;
  }
  const double t0 = a.t0 ? a.t0[i] : a.t0_s;
  const double te = a.t_end ? a.t_end[i] : a.t_end_s;
  const double s = te - t0;
  return (s > 0.0) ? s : 0.0;  // NaN and negative spans sort as the shortest
}

// Positive doubles order like their bit patterns.
__global__ void span_minmax_kernel(OrderArgs a) {
  unsigned long long lo = ~0ull, hi = 0ull;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(span_of(a, i)));
    lo = b < lo ? b : lo;
    hi = b > hi ? b : hi;
  }
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long l2 = __shfl_down_sync(0xffffffffu, lo, off);
    const unsigned long long h2 = __shfl_down_sync(0xffffffffu, hi, off);
    lo = l2 < lo ? l2 : lo;
    hi = h2 > hi ? h2 : hi;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(a.scratch->minmax + 0, lo);
    atomicMax(a.scratch->minmax + 1, hi);
  }
}

__device__ __forceinline__ int bucket_of(const OrderArgs& a, int64_t i) {
  const double lo = __longlong_as_double(static_cast<long long>(a.scratch->minmax[0]));
  const double hi = __longlong_as_double(static_cast<long long>(a.scratch->minmax[1]));
  const double s = span_of(a, i);
  const double w = hi - lo;
  int b = (w > 0.0) ? static_cast<int>((hi - s) / w * (kOrderBuckets - 1)) : 0;  // longest -> 0
  b = b < 0 ? 0 : (b >= kOrderBuckets ? kOrderBuckets - 1 : b);
  return b;
}

__global__ void span_histogram_kernel(OrderArgs a) {
  __shared__ unsigned int h[kOrderBuckets];
  for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x) h[k] = 0u;
  __syncthreads();
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    atomicAdd(&h[bucket_of(a, i)], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x)
    if (h[k]) atomicAdd(&a.scratch->offset[k], h[k]);
}

// Exclusive scan of the bucket counts, one block of kOrderBuckets threads.
__global__ void span_scan_kernel(OrderArgs a) {
  __shared__ unsigned int s[kOrderBuckets];
  const int k = threadIdx.x;
  s[k] = a.scratch->offset[k];
  __syncthreads();
  for (int off = 1; off < kOrderBuckets; off <<= 1) {
    const unsigned int v = (k >= off) ? s[k - off] : 0u;
    __syncthreads();
    s[k] += v;
    __syncthreads();
  }
  a.scratch->offset[k] = (k == 0) ? 0u : s[k - 1];
}

__global__ void span_scatter_kernel(OrderArgs a) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const unsigned int pos = atomicAdd(&a.scratch->offset[bucket_of(a, i)], 1u);
    a.order[pos] = static_cast<uint32_t>(i);
  }
}

}  // namespace

cudaError_t enqueue_lpt_order(const OrderArgs& a, int num_sms, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(a.scratch->offset, 0, sizeof(a.scratch->offset), s);
  if (e != cudaSuccess) return e;
  // minmax[0] starts at all ones (minimum), minmax[1] at zero (maximum).
  e = cudaMemsetAsync(a.scratch->minmax, 0xff, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.scratch->minmax + 1, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const int block = 256;
  const int grid = num_sms * 4;
  span_minmax_kernel<<<grid, block, 0, s>>>(a);
  span_histogram_kernel<<<grid, block, 0, s>>>(a);
  span_scan_kernel<<<1, kOrderBuckets, 0, s>>>(a);
  span_scatter_kernel<<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

// Forces the four kernels' device code onto the current device (the CUDA
// runtime loads kernels lazily, at their first launch or query).
cudaError_t preload_lpt_order_kernels() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, span_minmax_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, span_histogram_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, span_scan_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, span_scatter_kernel);
  return e;
}

}  // namespace bacon
