// FP64 fused-multiply-add throughput probe.  The roofline of the FP64
// integrators is the FP64 pipe, whose peak the driver's peak file does not
// record, so the engine measures it on the device it runs on.
#include <cstdint>

#include <cuda_runtime.h>

namespace bacon {

// Each thread runs 8 independent FMA chains in registers; nothing touches
// memory except one store per thread so the work is not optimised away.
__global__ void __launch_bounds__(256) fp64_fma_probe_kernel(double* sink, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      x0 = __fma_rn(x0, a, b);
      x1 = __fma_rn(x1, a, b);
      x2 = __fma_rn(x2, a, b);
      x3 = __fma_rn(x3, a, b);
      x4 = __fma_rn(x4, a, b);
      x5 = __fma_rn(x5, a, b);
      x6 = __fma_rn(x6, a, b);
      x7 = __fma_rn(x7, a, b);
    }
  }
  const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1234.5678) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Returns GFLOP/s (2 flops per FMA) or a negative value on CUDA failure.
double measure_fp64_fma_gflops(cudaStream_t stream, int num_sms) {
  const int block = 256;
  const int grid = num_sms * 4;
  const int iters = 4096;
  double* sink = nullptr;
  if (cudaMallocAsync(reinterpret_cast<void**>(&sink), sizeof(double) * grid * block, stream) != cudaSuccess)
    return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, stream);
    fp64_fma_probe_kernel<<<grid, block, 0, stream>>>(sink, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      best = -1.0;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 32.0 * static_cast<double>(iters) * grid * block;
    const double g = flops / (ms * 1e-3) * 1e-9;
    if (rep > 0 && g > best) best = g;  // first run is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(sink, stream);
  cudaStreamSynchronize(stream);
  return best;
}

}  // namespace bacon
