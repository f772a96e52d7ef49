// Instantiations of the linear (shared-A) RKF45 engine: FP64 exact and FMA
// stage GEMMs, the control kernel, and the layout kernels.
#include "linear.h"
#include "linear.cuh"

namespace bacon {

namespace {

// Solver construction per system (rk.rs:249-343): state from y0 (SoA in,
// per-system contiguous out), dt = (dt_max + dt_min) / 2, K = 0.
__global__ void lin_init_kernel(LinInitArgs a) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = a.st.n;
  const int D = a.dim;
  if (i < n * D) {
    const int64_t sys = i / D;
    const int d = static_cast<int>(i % D);
    a.st.y[i] = a.y0[static_cast<int64_t>(d) * n + sys];
    for (int s = 0; s < a.stages; ++s) a.st.K[static_cast<int64_t>(s) * n * D + i] = 0.0;
  }
  if (i < n) {
    a.st.t[i] = a.t0 ? a.t0[i] : a.t0_s;
    a.st.end[i] = a.t_end ? a.t_end[i] : a.t_end_s;
    a.st.dt[i] = a.dt0;
    a.st.attempts[i] = 0;
    a.st.accepted[i] = 0;
    a.st.rejected[i] = 0;
    a.st.status[i] = kLinRunning;
  }
}

__global__ void lin_output_kernel(LinArgs st, int dim, double* y_out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = st.n;
  if (i >= n * dim) return;
  const int64_t sys = i / dim;
  const int d = static_cast<int>(i % dim);
  y_out[static_cast<int64_t>(d) * n + sys] = st.y[i];
}

template <class Ops, class Tab, int D>
void fill(LinKernels& k) {
  k.stage[0] = reinterpret_cast<const void*>(&lin_stage_kernel<Ops, Tab, D, 0>);
  k.stage[1] = reinterpret_cast<const void*>(&lin_stage_kernel<Ops, Tab, D, 1>);
  k.stage[2] = reinterpret_cast<const void*>(&lin_stage_kernel<Ops, Tab, D, 2>);
  k.stage[3] = reinterpret_cast<const void*>(&lin_stage_kernel<Ops, Tab, D, 3>);
  if constexpr (Tab::S > 4) {
    k.stage[4] = reinterpret_cast<const void*>(&lin_stage_kernel<Ops, Tab, D, 4>);
    k.stage[5] = reinterpret_cast<const void*>(&lin_stage_kernel<Ops, Tab, D, 5>);
  }
  k.stages = Tab::S;
  k.control = reinterpret_cast<const void*>(&lin_control_kernel<Ops, Tab, D>);
}

template <class Ops, int D>
bool pick_layout(int method, int layout, LinKernels& k) {
  if (method == 0) {
    if (layout == 1) fill<Ops, Tableau<Rkf45Literal, kAsWritten>, D>(k);
    else if (layout == 2) fill<Ops, Tableau<Rkf45Literal, kFehlberg>, D>(k);
    else return false;
  } else {
    if (layout == 1 || layout == 2) fill<Ops, Tableau<Bs23Literal, kAsWritten>, D>(k);
    else return false;
  }
  return true;
}

}  // namespace

bool lin_kernels(int method, int layout, int precision, int dim, LinKernels& k) {
  k.init = reinterpret_cast<const void*>(&lin_init_kernel);
  k.output = reinterpret_cast<const void*>(&lin_output_kernel);
  if (precision == 0) {
    if (dim == 64) return pick_layout<ExactOps, 64>(method, layout, k);
    if (dim == 128) return pick_layout<ExactOps, 128>(method, layout, k);
    if (dim == 256) return pick_layout<ExactOps, 256>(method, layout, k);
  } else if (precision == 1) {
    if (dim == 64) return pick_layout<FmaOps, 64>(method, layout, k);
    if (dim == 128) return pick_layout<FmaOps, 128>(method, layout, k);
    if (dim == 256) return pick_layout<FmaOps, 256>(method, layout, k);
  }
  return false;
}

}  // namespace bacon
