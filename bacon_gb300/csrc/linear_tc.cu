// Instantiations of the tensor-core (split-precision) engine for the linear
// right-hand side: the GEMM, the slicing kernels and the control kernel that
// combines the products A^k y.
#include <cuda_bf16.h>

#include "linear.h"
#include "linear_tc.cuh"

namespace bacon {

namespace {
template <class Tab, int D>
void fill_tc(LinTcKernels& k) {
  k.slice_a = reinterpret_cast<const void*>(&lin_tc_slice_a_kernel<D>);
  k.slice_vec = reinterpret_cast<const void*>(&lin_tc_slice_vec_kernel<D>);
  k.control = reinterpret_cast<const void*>(&lin_control_kernel<FmaOps, Tab, D, true>);
  k.gemm = reinterpret_cast<const void*>(&lin_tc_stage_kernel<D>);
  // The last product enters only the error estimate when the update's
  // polynomial has no term of degree S (fehlberg, as_written, BS23 alike):
  // its leading two diagonals (~2^-15) suffice there.
  if constexpr (LinPoly<Tab>::kCoef.beta[Tab::S] == 0.0) {
    k.gemm_last = reinterpret_cast<const void*>(&lin_tc_stage_kernel<D, 2>);
    k.last_pairs = 3;
  } else {
    k.gemm_last = k.gemm;
    k.last_pairs = kTcSlices * (kTcSlices + 1) / 2;
  }
  k.smem_bytes = 2 * kTcBufBytes;
  k.gemm_threads = kTcThreads;
  k.slices = kTcSlices;
}

template <int D>
bool pick(int method, int layout, LinTcKernels& k) {
  if (method == 0) {
    if (layout == 1) fill_tc<Tableau<Rkf45Literal, kAsWritten>, D>(k);
    else if (layout == 2) fill_tc<Tableau<Rkf45Literal, kFehlberg>, D>(k);
    else return false;
  } else {
    if (layout == 1 || layout == 2) fill_tc<Tableau<Bs23Literal, kAsWritten>, D>(k);
    else return false;
  }
  return true;
}
}  // namespace

bool lin_tc_kernels(int method, int layout, int dim, LinTcKernels& k) {
  if (dim == 128) return pick<128>(method, layout, k);
  if (dim == 256) return pick<256>(method, layout, k);
  return false;
}

}  // namespace bacon
