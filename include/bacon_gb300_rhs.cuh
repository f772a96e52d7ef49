/*
 * Right-hand sides compiled by the caller, for bacon_rk_solve_user.
 *
 * The reference takes any Rust closure as the derivative (src/ivp.rs:34-48).
 * A GPU kernel cannot call back into host code, so a right-hand side outside
 * the engine's registry is compiled into the same persistent Runge-Kutta
 * kernel by the caller.  Write a functor with the registry's shape:
 *
 *   struct MyRhs {
 *     static constexpr int DIM = 2, NP = 1;      // state size, parameters
 *     static constexpr bool kUsesT = false;      // true if f depends on t
 *     template <class Ops, class V>
 *     __device__ static void eval(double t, const V (&y)[DIM], const V* p, V (&f)[DIM]) {
 *       f[0] = y[1];
 *       f[1] = Ops::sub(Ops::mul(p[0], y[0]), y[1]);   // Ops: the arithmetic policy
 *     }
 *   };
 *   BACON_DEFINE_RK_LAUNCHER(my_rhs_launch, MyRhs)
 *
 * compile the file with
 *   nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 --expt-relaxed-constexpr \
 *        -Xcompiler -fPIC -shared -I include -I bacon_gb300/csrc my_rhs.cu -o libmy_rhs.so
 * and pass my_rhs_launch to bacon_rk_solve_user with problem->rhs =
 * BACON_RHS_USER, dim = DIM and n_params >= NP.  Use Ops::mul / add / sub /
 * div for every operation whose rounding the exact mode must fix; the FP32
 * stage mode (precision 2) additionally needs kUsesT == false and an eval
 * that accepts float-float values (V), as the registry's functors do.
 * Compiled combinations: RK45 and RK23, every tableau reading, FP64_EXACT
 * and FP64_FMA.
 */
#pragma once

#include <cuda_runtime.h>

#include "bacon_gb300.h"
#include "rk_kernel.cuh"

namespace bacon_user {

template <class Rhs, int M, int L>
const void* rk_kernel_for(int32_t precision) {
  using Lit = typename std::conditional<M == 0, bacon::Rkf45Literal, bacon::Bs23Literal>::type;
  using T = bacon::Tableau<Lit, L>;
  if (precision == BACON_FP64_EXACT)
    return reinterpret_cast<const void*>(&bacon::rk_persistent_kernel<T, Rhs, bacon::ExactOps>);
  if (precision == BACON_FP64_FMA)
    return reinterpret_cast<const void*>(&bacon::rk_persistent_kernel<T, Rhs, bacon::FmaOps>);
  return nullptr;
}

// Launches the caller's persistent kernel for (method, layout, precision).
template <class Rhs>
int launch_rk(const bacon_rk_kernel_args* args, int32_t method, int32_t layout, int32_t precision, int32_t grid,
              int32_t block, void* stream) {
  static_assert(sizeof(bacon::RkArgs) == sizeof(bacon_rk_kernel_args), "kernel argument block layout");
  const void* fn = nullptr;
  if (method == BACON_RK45) {
    if (layout == 0) fn = rk_kernel_for<Rhs, 0, 0>(precision);
    else if (layout == 1) fn = rk_kernel_for<Rhs, 0, 1>(precision);
    else if (layout == 2) fn = rk_kernel_for<Rhs, 0, 2>(precision);
  } else if (method == BACON_RK23) {
    if (layout == 0) fn = rk_kernel_for<Rhs, 1, 0>(precision);
    else if (layout == 1 || layout == 2) fn = rk_kernel_for<Rhs, 1, 1>(precision);
  }
  if (!fn) return BACON_UNSUPPORTED;
  bacon::RkArgs a;
  static_assert(std::is_trivially_copyable<bacon::RkArgs>::value, "plain data");
  memcpy(&a, args, sizeof(a));
  void* kargs[] = {&a};
  const cudaError_t e = cudaLaunchKernel(fn, dim3(static_cast<unsigned>(grid)), dim3(static_cast<unsigned>(block)),
                                         kargs, 0, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? BACON_OK : BACON_CUDA_ERROR;
}

}  // namespace bacon_user

/* Defines `extern "C" int NAME(...)`, a bacon_rk_launch_fn for functor RHS. */
#define BACON_DEFINE_RK_LAUNCHER(NAME, RHS)                                                              \
  extern "C" int NAME(const bacon_rk_kernel_args* args, int32_t method, int32_t layout, int32_t precision, \
                      int32_t grid, int32_t block, void* stream, void* user) {                             \
    (void)user;                                                                                            \
    return bacon_user::launch_rk<RHS>(args, method, layout, precision, grid, block, stream);                \
  }
