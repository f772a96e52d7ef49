// Host interface of the linear (shared-A) RKF45 engine.
#pragma once

#include <cstdint>

namespace bacon {

struct LinArgs;

struct LinKernels {
  const void* init = nullptr;     // __global__ void(LinInitArgs)
  const void* stage[6] = {};      // __global__ void(LinArgs)
  const void* control = nullptr;  // __global__ void(LinArgs, int first)
  const void* output = nullptr;   // __global__ void(LinArgs, int dim, double* y_out)
  int stages = 0;
};

// Kernels for (method, layout, precision) and dim in {64, 128, 256}.  The
// as_compiled reading is not offered (its stage values mix attempts).
bool lin_kernels(int method, int layout, int precision, int dim, LinKernels& k);

// Tensor-core (split-precision) variant.  An attempt needs the products
// v_k = A^k y, k = 1..S (the stage values are polynomials in dt A applied to
// y): per product a slicing kernel for v_{k-1} and the tcgen05 GEMM, then
// the control kernel that combines them with each system's dt; plus the
// one-off slicing of A.  dim in {128, 256}.
struct LinTcKernels {
  const void* slice_a = nullptr;   // __global__ void(const double* A, bf16* sa, int32_t* ea)
  const void* slice_vec = nullptr; // __global__ void(TcArgs, const double* x, bf16* sy, int32_t* ey)
  const void* control = nullptr;   // __global__ void(LinArgs, int first)
  const void* gemm = nullptr;      // __global__ void(TcArgs)
  const void* gemm_last = nullptr; // the GEMM for v_S (reduced precision when only the error uses it)
  int last_pairs = 0;              // slice products of that GEMM
  int smem_bytes = 0;
  int gemm_threads = 0;
  int slices = 0;
};
bool lin_tc_kernels(int method, int layout, int dim, LinTcKernels& k);

}  // namespace bacon
