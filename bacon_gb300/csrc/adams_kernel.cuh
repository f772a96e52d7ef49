// Persistent batched Adams predictor-corrector (Adams5 / Adams3) and Euler
// kernels: one thread per system, all solver state in registers, systems
// pulled from a work counter with warp-aggregated atomics (as the RK engine).
//
// Adams: each loop iteration is one call of the reference's
// AdamsSolver::step (src/ivp/adams.rs:411-565) under IVPIterator::next
// (src/ivp.rs:214-238): the RK4 bootstrap of O-1 steps
// (AdamsSolver::runge_kutta, :344-395), the "yield memory" that re-emits the
// bootstrap states after the first accepted PECE step, the derivative history
// that then lacks that step's derivative, the end-clamped single RK4 step, the
// PECE step with error (19/270) / dt * ||corrector - predictor||, the factor
// (tol / (2 err))^(1/O) (rootn) and the history cleared on every dt change.
// Euler: EulerSolver::step (src/ivp.rs:318-339), which yields the state each
// step starts from.  Outputs as the RK engine: the last yielded item,
// accepted = items yielded, rejected = step() calls that returned Redo.
#pragma once

#include "bdf_kernel.cuh"

namespace bacon {

struct AdamsArgs {
  int64_t n;
  const double* y0;      // [D][n]
  const double* params;  // [P][n]
  const double* t0;      // [n] or null
  const double* t_end;   // [n] or null
  double t0_s, t_end_s;
  double tol, dt_min, dt_max;
  double euler_dt;       // Euler: the builder's step
  int64_t max_attempts;  // cap on step() calls per system
  double* y_out;
  double* t_out;
  int32_t* accepted;
  int32_t* rejected;
  int32_t* status;
  double* traj_t;
  double* traj_y;
  int32_t traj_cap;
  int32_t dyn_dim;
  const int64_t* traj_off;  // [n+1] packed offsets, or null: slabs of traj_cap
  int32_t lanes;            // systems per warp: lanes 0..lanes-1 of each warp take systems
  unsigned long long* queue;
  unsigned long long* first_fail;
};

// Predictor and corrector coefficients (AdamsCoefficients5 / 3,
// src/ivp/adams.rs:572-603, :636-659), with the reference's expressions.
template <int O>
struct AdamsCoef;
template <>
struct AdamsCoef<5> {
  __device__ __forceinline__ static constexpr double pc(int i) {
    return i == 0 ? 55.0 / 24.0 : i == 1 ? -59.0 / 24.0 : i == 2 ? 37.0 / 24.0 : i == 3 ? -9.0 / 24.0 : 0.0;
  }
  __device__ __forceinline__ static constexpr double cc(int i) {
    return i == 0 ? 251.0 / 720.0 : i == 1 ? 646.0 / 720.0 : i == 2 ? -264.0 / 720.0 : i == 3 ? 106.0 / 720.0
                                                                                               : -19.0 / 720.0;
  }
};
template <>
struct AdamsCoef<3> {
  __device__ __forceinline__ static constexpr double pc(int i) {
    return i == 0 ? 1.0 + (1.0 / 2.0) : i == 1 ? -(1.0 / 2.0) : 0.0;
  }
  __device__ __forceinline__ static constexpr double cc(int i) {
    return i == 0 ? 5.0 / 12.0 : i == 1 ? 2.0 / 3.0 : -(1.0 / 12.0);
  }
};

// Pulls the next system index for this thread (warp-aggregated atomic);
// false when the batch is exhausted.
__device__ __forceinline__ bool next_system(unsigned long long* queue, int64_t n, int64_t& idx) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned mask = __activemask();
  const int leader = __ffs(mask) - 1;
  unsigned long long ticket = 0;
  if (static_cast<int>(lane) == leader) ticket = atomicAdd(queue, static_cast<unsigned long long>(__popc(mask)));
  ticket = __shfl_sync(mask, ticket, leader) + __popc(mask & ((1u << lane) - 1u));
  idx = static_cast<int64_t>(ticket);
  return idx < n;
}

// Adams state of one system.  The deques prev_values / prev_derivatives are
// arrays with the front at index 0; every index is a compile-time constant
// (shifts and predicated writes), so they stay in registers.  They hold O + 1
// entries: the PECE step reads at most O - 1, and repeated end-clamped RK4
// steps (t + (end - t) rounding below end) only need back() and
// non-emptiness, so a push onto a full deque drops its front.
template <int O, int D>
struct AdamsState {
  static constexpr int kCap = O + 1;
  double time, end, dt, tol, dt_min, dt_max;
  double state[D], save[D];
  double pv_t[kCap], pv_y[kCap][D];
  double pd[kCap][D];
  int npv, npd, yield_memory;
  // A step() call whose RK4 run is in progress: rk_left RK4 steps remain,
  // rk_i is the next one's index, rk_kind 1 = the start-up run (the call
  // returns Redo), 2 = the end-clamped single step (it yields an item).
  int rk_left, rk_i, rk_kind;
};

template <int O, int D>
__device__ __forceinline__ void ad_pv_pop_front(AdamsState<O, D>& s);
template <int O, int D>
__device__ __forceinline__ void ad_pd_pop_front(AdamsState<O, D>& s);

template <int O, int D>
__device__ __forceinline__ void ad_pv_push(AdamsState<O, D>& s, double t, const double (&y)[D]) {
  if (s.npv == AdamsState<O, D>::kCap) ad_pv_pop_front(s);
#pragma unroll
  for (int i = 0; i < AdamsState<O, D>::kCap; ++i)
    if (i == s.npv) {
      s.pv_t[i] = t;
#pragma unroll
      for (int d = 0; d < D; ++d) s.pv_y[i][d] = y[d];
    }
  s.npv++;
}
template <int O, int D>
__device__ __forceinline__ void ad_pv_pop_front(AdamsState<O, D>& s) {
#pragma unroll
  for (int i = 1; i < AdamsState<O, D>::kCap; ++i) {
    s.pv_t[i - 1] = s.pv_t[i];
#pragma unroll
    for (int d = 0; d < D; ++d) s.pv_y[i - 1][d] = s.pv_y[i][d];
  }
  s.npv--;
}
template <int O, int D>
__device__ __forceinline__ void ad_pd_push(AdamsState<O, D>& s, const double (&f)[D]) {
  if (s.npd == AdamsState<O, D>::kCap) ad_pd_pop_front(s);
#pragma unroll
  for (int i = 0; i < AdamsState<O, D>::kCap; ++i)
    if (i == s.npd)
#pragma unroll
      for (int d = 0; d < D; ++d) s.pd[i][d] = f[d];
  s.npd++;
}
template <int O, int D>
__device__ __forceinline__ void ad_pd_pop_front(AdamsState<O, D>& s) {
#pragma unroll
  for (int i = 1; i < AdamsState<O, D>::kCap; ++i)
#pragma unroll
    for (int d = 0; d < D; ++d) s.pd[i - 1][d] = s.pd[i][d];
  s.npd--;
}

// Entry i (< L) of prev_values, i known only at run time: a chain of selects
// over the compile-time positions.  (A predicated copy inside a loop lets the
// compiler turn the deques into indexed local memory, on every step's path.)
template <int L, int O, int D>
__device__ __forceinline__ void ad_pv_select(const AdamsState<O, D>& s, int i, double& t, double (&y)[D]) {
  t = s.pv_t[0];
#pragma unroll
  for (int d = 0; d < D; ++d) y[d] = s.pv_y[0][d];
#pragma unroll
  for (int k = 1; k < L; ++k) {
    const bool hit = (k == i);
    t = hit ? s.pv_t[k] : t;
#pragma unroll
    for (int d = 0; d < D; ++d) y[d] = hit ? s.pv_y[k][d] : y[d];
  }
}

// AdamsSolver::runge_kutta (src/ivp/adams.rs:344-395), one RK4 step at a
// time: step i of a run (the history pushes of the reference's loop happen
// from i = 1 on), then, after the last, the closing evaluation and pushes.
// A run of O - 1 steps costs ~20 right-hand-side evaluations against ~1 for a
// PECE step, so the kernel advances a run by one RK4 step per loop iteration:
// the lanes of a warp that are in a PECE step then wait for one RK4 step of
// a neighbour, not for its whole run.  The operations and their order are the
// reference's.
template <int O, class Rhs>
__device__ __forceinline__ void ad_rk4_step(AdamsState<O, Rhs::DIM>& s, const double* p, int i) {
  using X = ExactOps;
  constexpr int D = Rhs::DIM;
  double k1[D], k2[D], k3[D], k4[D], it[D], f[D];
  Rhs::template eval<X>(s.time, s.state, p, f);
#pragma unroll
  for (int d = 0; d < D; ++d) k1[d] = X::mul(f[d], s.dt);
#pragma unroll
  for (int d = 0; d < D; ++d) it[d] = X::add(s.state[d], X::mul(k1[d], 0.5));
  Rhs::template eval<X>(X::add(s.time, X::mul(0.5, s.dt)), it, p, f);
#pragma unroll
  for (int d = 0; d < D; ++d) k2[d] = X::mul(f[d], s.dt);
#pragma unroll
  for (int d = 0; d < D; ++d) it[d] = X::add(s.state[d], X::mul(k2[d], 0.5));
  Rhs::template eval<X>(X::add(s.time, X::mul(0.5, s.dt)), it, p, f);
#pragma unroll
  for (int d = 0; d < D; ++d) k3[d] = X::mul(f[d], s.dt);
#pragma unroll
  for (int d = 0; d < D; ++d) it[d] = X::add(s.state[d], k3[d]);
  Rhs::template eval<X>(X::add(s.time, s.dt), it, p, f);
#pragma unroll
  for (int d = 0; d < D; ++d) k4[d] = X::mul(f[d], s.dt);
  if (i != 0) {
    Rhs::template eval<X>(s.time, s.state, p, f);
    ad_pd_push(s, f);
    ad_pv_push(s, s.time, s.state);
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double comb = X::add(X::add(X::add(k1[d], X::mul(k2[d], 2.0)), X::mul(k3[d], 2.0)), k4[d]);
    s.state[d] = X::add(s.state[d], X::mul(comb, 1.0 / 6.0));
  }
  s.time = X::add(s.time, s.dt);
}

template <int O, class Rhs>
__device__ __forceinline__ void ad_rk4_close(AdamsState<O, Rhs::DIM>& s, const double* p) {
  double f[Rhs::DIM];
  Rhs::template eval<ExactOps>(s.time, s.state, p, f);
  ad_pd_push(s, f);
  ad_pv_push(s, s.time, s.state);
}

enum : int { kAdItem = 0, kAdRedo = 1, kAdDone = 2, kAdFail = 3, kAdPending = 4 };

// AdamsSolver::step (src/ivp/adams.rs:411-565).
template <int O, class Rhs>
__device__ __forceinline__ int ad_step(AdamsState<O, Rhs::DIM>& s, const double* p, bool dyn, double& it,
                                       double (&iy)[Rhs::DIM], int32_t& fail) {
  using X = ExactOps;
  using C = AdamsCoef<O>;
  constexpr int D = Rhs::DIM;
  constexpr double order = static_cast<double>(O);
  if (s.yield_memory > 0 && s.yield_memory < O) {
    const int get_item = O - s.yield_memory - 1;
    s.yield_memory -= 1;
    if (s.yield_memory == 0) s.yield_memory = O + 1;
    ad_pv_select<O>(s, get_item, it, iy);
    return kAdItem;
  }
  if (s.yield_memory == O + 1) {
    s.yield_memory = 0;
    ad_pv_push(s, s.time, s.state);
    ad_pv_pop_front(s);
    it = s.time;
#pragma unroll
    for (int d = 0; d < D; ++d) iy[d] = s.state[d];
    return kAdItem;
  }
  if (s.time >= s.end) return kAdDone;
  if (X::add(s.time, s.dt) >= s.end) {
    s.dt = X::sub(s.end, s.time);
    s.rk_kind = 2;  // one RK4 step, then yield the last history value
    s.rk_i = 0;
    s.rk_left = 1;
    return kAdPending;
  }
  if (s.npv == 0) {
#pragma unroll
    for (int d = 0; d < D; ++d) s.save[d] = s.state[d];
    if (X::add(s.time, X::mul(s.dt, order - 1.0)) >= s.end) s.dt = X::div(X::sub(s.end, s.time), order - 1.0);
    s.rk_kind = 1;  // the start-up run of O - 1 RK4 steps, then Redo
    s.rk_i = 0;
    s.rk_left = O - 1;
    return kAdPending;
  }
  double scratch[D], pred[D], corr[D], impl[D], diff[D];
#pragma unroll
  for (int d = 0; d < D; ++d) scratch[d] = X::mul(s.pd[0][d], C::pc(O - 2));
#pragma unroll
  for (int i = 1; i < O - 1; ++i)
#pragma unroll
    for (int d = 0; d < D; ++d) scratch[d] = X::add(scratch[d], X::mul(s.pd[i][d], C::pc(O - i - 2)));
#pragma unroll
  for (int d = 0; d < D; ++d) pred[d] = X::add(s.state[d], X::mul(scratch[d], s.dt));
  Rhs::template eval<X>(X::add(s.time, s.dt), pred, p, impl);
#pragma unroll
  for (int d = 0; d < D; ++d) scratch[d] = X::mul(impl[d], C::cc(0));
#pragma unroll
  for (int i = 0; i < O - 1; ++i)
#pragma unroll
    for (int d = 0; d < D; ++d) scratch[d] = X::add(scratch[d], X::mul(s.pd[i][d], C::cc(O - i - 1)));
#pragma unroll
  for (int d = 0; d < D; ++d) corr[d] = X::add(s.state[d], X::mul(scratch[d], s.dt));
#pragma unroll
  for (int d = 0; d < D; ++d) diff[d] = X::sub(corr[d], pred[d]);
  const double error = X::mul(X::div(19.0 / 270.0, s.dt), bdf_norm(diff, dyn));
  if (error <= s.tol) {
#pragma unroll
    for (int d = 0; d < D; ++d) s.state[d] = corr[d];
    s.time = X::add(s.time, s.dt);
    if (s.yield_memory == O) {
      s.yield_memory -= 1;
      return kAdRedo;
    }
    ad_pd_push(s, impl);
    ad_pv_push(s, s.time, s.state);
    ad_pv_pop_front(s);
    ad_pd_pop_front(s);
    if (error < X::mul(0.1, s.tol)) {
      const double q = rootn<O>(X::div(s.tol, X::mul(2.0, error)));
      if (q > 4.0) s.dt = X::mul(s.dt, 4.0);
      else s.dt = X::mul(s.dt, q);
      if (s.dt > s.dt_max) s.dt = s.dt_max;
      s.npv = 0;
      s.npd = 0;
    }
    it = s.time;
#pragma unroll
    for (int d = 0; d < D; ++d) iy[d] = s.state[d];
    return kAdItem;
  }
  if (s.yield_memory == O) {
    s.time = X::sub(s.time, X::mul(s.dt, order - 1.0));
#pragma unroll
    for (int d = 0; d < D; ++d) s.state[d] = s.save[d];
  }
  const double q = rootn<O>(X::div(s.tol, X::mul(2.0, error)));
  if (q < 0.1) s.dt = X::mul(s.dt, 0.1);
  else s.dt = X::mul(s.dt, q);
  if (s.dt < s.dt_min) {
    fail = kStMinDt;
    return kAdFail;
  }
  s.npv = 0;
  s.npd = 0;
  return kAdRedo;
}

// Advances a step() call's RK4 run by one step; when the run is complete,
// finishes the call as the reference's step() does after runge_kutta
// returns: Redo for the start-up run, the last history value for the
// end-clamped step.
template <int O, class Rhs>
__device__ __forceinline__ int ad_continue(AdamsState<O, Rhs::DIM>& s, const double* p, double& it,
                                           double (&iy)[Rhs::DIM]) {
  ad_rk4_step<O, Rhs>(s, p, s.rk_i);
  s.rk_i += 1;
  s.rk_left -= 1;
  if (s.rk_left > 0) return kAdPending;
  ad_rk4_close<O, Rhs>(s, p);
  if (s.rk_kind == 1) {
    s.yield_memory = O;
    return kAdRedo;
  }
  double back_t;
  ad_pv_select<AdamsState<O, Rhs::DIM>::kCap>(s, s.npv - 1, back_t, iy);
  it = s.time;
  return kAdItem;
}

template <int O, class Rhs>
__global__ void __launch_bounds__(128) adams_persistent_kernel(const AdamsArgs a) {
  constexpr int D = Rhs::DIM;
  constexpr int P = Rhs::NP > 0 ? Rhs::NP : 1;
  const int64_t n = a.n;
  if (static_cast<int>(threadIdx.x & 31u) >= a.lanes) return;  // idle lane (no block-wide sync below)
  const bool dyn = a.dyn_dim != 0;
  int64_t idx;
  while (next_system(a.queue, n, idx)) {
    double p[P];
#pragma unroll
    for (int k = 0; k < Rhs::NP; ++k) p[k] = a.params[k * n + idx];
    AdamsState<O, D> s;
    s.time = a.t0 ? a.t0[idx] : a.t0_s;
    s.end = a.t_end ? a.t_end[idx] : a.t_end_s;
    s.tol = a.tol;
    s.dt_min = a.dt_min;
    s.dt_max = a.dt_max;
    s.dt = ExactOps::mul(ExactOps::add(a.dt_max, a.dt_min), 0.5);
    s.npv = s.npd = s.yield_memory = 0;
    s.rk_left = s.rk_i = s.rk_kind = 0;
    double last_y[D], last_t = s.time;
#pragma unroll
    for (int d = 0; d < D; ++d) s.state[d] = last_y[d] = a.y0[d * n + idx];
    int32_t acc = 0, rej = 0, status = kStOk;
    if (s.time >= s.end) {
      status = kStTimeEndOob;
    } else {
      int64_t calls = 0;
      for (;;) {
        double it, iy[D];
        int32_t fail = 0;
        int r;
        if (s.rk_left > 0) {
          r = ad_continue<O, Rhs>(s, p, it, iy);  // the call in progress
        } else {
          if (calls >= a.max_attempts) {
            status = kStMaxAttempts;
            break;
          }
          ++calls;
          r = ad_step<O, Rhs>(s, p, dyn, it, iy, fail);
        }
        if (r == kAdPending) continue;
        if (r == kAdDone) break;
        if (r == kAdFail) {
          status = fail;
          break;
        }
        if (r == kAdRedo) {
          ++rej;
          continue;
        }
        if (a.traj_t != nullptr) {
          const int64_t slot = traj_slot(a.traj_off, a.traj_cap, idx, acc);
          if (slot < 0) {
            status = kStCapacity;  // the trajectory buffer is full: the item is not yielded
            break;
          }
          a.traj_t[slot] = it;
#pragma unroll
          for (int d = 0; d < D; ++d) a.traj_y[slot * D + d] = iy[d];
        }
        ++acc;
        last_t = it;
#pragma unroll
        for (int d = 0; d < D; ++d) last_y[d] = iy[d];
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) a.y_out[d * n + idx] = last_y[d];
    a.t_out[idx] = last_t;
    a.accepted[idx] = acc;
    a.rejected[idx] = rej;
    a.status[idx] = status;
    if (status != kStOk) atomicMin(a.first_fail, static_cast<unsigned long long>(idx));
  }
}

// EulerSolver::step under the iterator (src/ivp.rs:318-339, :214-238).
template <class Rhs>
__global__ void __launch_bounds__(128) euler_persistent_kernel(const AdamsArgs a) {
  using X = ExactOps;
  constexpr int D = Rhs::DIM;
  constexpr int P = Rhs::NP > 0 ? Rhs::NP : 1;
  const int64_t n = a.n;
  if (static_cast<int>(threadIdx.x & 31u) >= a.lanes) return;  // idle lane (no block-wide sync below)
  int64_t idx;
  while (next_system(a.queue, n, idx)) {
    double p[P], y[D], f[D], last_y[D];
#pragma unroll
    for (int k = 0; k < Rhs::NP; ++k) p[k] = a.params[k * n + idx];
#pragma unroll
    for (int d = 0; d < D; ++d) y[d] = last_y[d] = a.y0[d * n + idx];
    double t = a.t0 ? a.t0[idx] : a.t0_s;
    const double end = a.t_end ? a.t_end[idx] : a.t_end_s;
    double dt = a.euler_dt, last_t = t;
    int32_t acc = 0, status = kStOk;
    if (t >= end) {
      status = kStTimeEndOob;
    } else {
      int64_t steps = 0;
      while (t < end) {
        if (steps >= a.max_attempts) {
          status = kStMaxAttempts;
          break;
        }
        ++steps;
        if (X::add(t, dt) >= end) dt = X::sub(end, t);
        Rhs::template eval<X>(t, y, p, f);
        if (a.traj_t != nullptr) {
          const int64_t slot = traj_slot(a.traj_off, a.traj_cap, idx, acc);
          if (slot < 0) {
            status = kStCapacity;  // the trajectory buffer is full: the item is not yielded
            break;
          }
          a.traj_t[slot] = t;
#pragma unroll
          for (int d = 0; d < D; ++d) a.traj_y[slot * D + d] = y[d];
        }
        ++acc;
        last_t = t;
#pragma unroll
        for (int d = 0; d < D; ++d) last_y[d] = y[d];
#pragma unroll
        for (int d = 0; d < D; ++d) y[d] = X::add(y[d], X::mul(f[d], dt));
        t = X::add(t, dt);
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) a.y_out[d * n + idx] = last_y[d];
    a.t_out[idx] = last_t;
    a.accepted[idx] = acc;
    a.rejected[idx] = 0;
    a.status[idx] = status;
    if (status != kStOk) atomicMin(a.first_fail, static_cast<unsigned long long>(idx));
  }
}

}  // namespace bacon
