// Persistent batched embedded Runge-Kutta kernel (RKF45 / Bogacki-Shampine).
//
// One thread owns one system at a time; all of its solver state (y, the
// stage values K, t, dt, counters) lives in registers for the whole solve.
// A persistent grid pulls system indices from a global work counter with
// warp-aggregated atomics, so systems with uneven end times balance across
// the GPU.  Each loop iteration is one call of the reference's
// RungeKuttaSolver::step (src/ivp/rk.rs:361-423), and the loop replaces the
// IVPIterator that retries Redo and stops on Done / Failure
// (src/ivp.rs:220-238).
#pragma once

#include <cstdint>
#include <type_traits>

#include "device_math.cuh"
#include "rhs.cuh"
#include "tableau.cuh"
#include "traj.cuh"

namespace bacon {

// Status codes shared with include/bacon_gb300.h.
enum : int32_t {
  kStOk = 0,
  kStTimeEndOob = 5,
  kStMinDt = 8,
  kStMaxIter = 9,
  kStSingular = 10,
  kStMaxAttempts = 13,
  kStCapacity = 17,
};

struct RkArgs {
  int64_t n;
  const double* y0;      // [D][n]
  const double* params;  // [P][n]
  const double* t0;      // [n] or null
  const double* t_end;   // [n] or null
  double t0_s, t_end_s;
  double tol, dt_min, dt_max;
  int64_t max_attempts;
  double* y_out;         // [D][n]
  double* t_out;         // [n]
  int32_t* accepted;     // [n]
  int32_t* rejected;     // [n]
  int32_t* status;       // [n]
  double* traj_t;        // [n][cap], the packed stream, or null
  double* traj_y;        // [n][cap][D], the packed stream, or null
  int32_t traj_cap;
  const int64_t* traj_off;  // [n+1] packed offsets, or null: slabs of traj_cap
  unsigned long long* queue;       // work counter, zero at launch
  unsigned long long* first_fail;  // lowest failing index, ~0 at launch
  const uint32_t* order;           // work order (a permutation of [0, n)) or null
  // Adjoint recording (kRecord kernels only): per accepted step k the dt it
  // used, dt_log[i*max_steps + k]; every ckpt_every accepted steps the
  // (t, y) it started from, ckpt[(i*ckpt_slots + k/ckpt_every)*(D+1) + {0, 1+d}].
  double* dt_log;
  double* ckpt;
  int32_t ckpt_every;
  int32_t max_steps;
  int32_t ckpt_slots;
  int32_t lanes;  // systems per warp: lanes 0..lanes-1 take systems (0: all 32)
};

template <int I, int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

// nalgebra 0.32 norm of a static 1..3-vector (blas.rs dotx special cases;
// a 1-vector goes through the general loop: 0 + x*x).
template <class Ops, int D>
__device__ __forceinline__ double static_norm(const double (&v)[D]) {
  static_assert(D >= 1 && D <= 3, "static_norm covers dims 1..3");
  if constexpr (D == 1) {
    return Ops::sqrt(Ops::mul(v[0], v[0]));
  } else if constexpr (D == 2) {
    return Ops::sqrt(Ops::add(Ops::mul(v[0], v[0]), Ops::mul(v[1], v[1])));
  } else {
    return Ops::sqrt(Ops::add(Ops::add(Ops::mul(v[0], v[0]), Ops::mul(v[1], v[1])),
                              Ops::mul(v[2], v[2])));
  }
}

template <int D>
__device__ __forceinline__ void poison_components(double (&v)[D], uint32_t mask) {
  if (mask) {
#pragma unroll
    for (int d = 0; d < D; ++d)
      if ((mask >> d) & 1u) v[d] = __longlong_as_double(0x7ff8000000000000ll);
  }
}

// kMinBlocks sets the register budget through the launch bounds: the compiler
// keeps every thread within 65536 / (256 * kMinBlocks) registers (1: up to
// 255, 3: 80, 4: 64), trading spills for resident warps.  The autotuner times
// the budgets on the caller's batch.
template <class Tab, class Rhs, class Ops, bool kRecord = false, int kMinBlocks = 1>
__global__ void __launch_bounds__(256, kMinBlocks) rk_persistent_kernel(const RkArgs a) {
  constexpr int D = Rhs::DIM;
  constexpr int S = Tab::S;
  constexpr int P = Rhs::NP > 0 ? Rhs::NP : 1;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t n = a.n;
  const double tol = a.tol, dt_min = a.dt_min, dt_max = a.dt_max;
  const double dt0 = Ops::mul(Ops::add(dt_max, dt_min), 0.5);  // rk.rs:315

  double y[D], K[S][D], p[P];
  uint32_t kbad[S];
  double t = 0.0, end = 0.0, dt = 0.0;
  int32_t acc = 0, rej = 0;
  int64_t attempts = 0, idx = 0;
  // lanes beyond a.lanes never take a system; they stay in the loop's
  // warp-wide votes (full masks) and idle
  bool have = false, exhausted = a.lanes > 0 && static_cast<int>(lane) >= a.lanes;

  for (;;) {
    // ---- pull new systems for idle lanes (one atomic per warp) ----
    const bool need = !have && !exhausted;
    const unsigned need_mask = __ballot_sync(0xffffffffu, need);
    if (need_mask) {
      const int leader = __ffs(need_mask) - 1;
      unsigned long long base = 0;
      if (static_cast<int>(lane) == leader)
        base = atomicAdd(a.queue, static_cast<unsigned long long>(__popc(need_mask)));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const int64_t cand = static_cast<int64_t>(base) + __popc(need_mask & lt_mask);
        if (cand < n) {
          idx = a.order ? static_cast<int64_t>(a.order[cand]) : cand;
          have = true;
          t = a.t0 ? a.t0[idx] : a.t0_s;
          end = a.t_end ? a.t_end[idx] : a.t_end_s;
#pragma unroll
          for (int d = 0; d < D; ++d) y[d] = a.y0[d * n + idx];
#pragma unroll
          for (int k = 0; k < Rhs::NP; ++k) p[k] = a.params[k * n + idx];
#pragma unroll
          for (int j = 0; j < S; ++j) {
            kbad[j] = 0u;
#pragma unroll
            for (int d = 0; d < D; ++d) K[j][d] = 0.0;  // rk.rs:323-327
          }
          dt = dt0;
          acc = 0;
          rej = 0;
          attempts = 0;
        } else {
          exhausted = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, !have)) break;
    if (!have) continue;

    // ---- one RungeKuttaSolver::step ----
    int32_t fin = -1;
    if (attempts == 0 && t >= end) {
      fin = kStTimeEndOob;  // with_ending_time rejects end <= start (rk.rs:227-231)
    } else if (t >= end) {
      fin = kStOk;  // rk.rs:362-364
    } else if (attempts >= a.max_attempts) {
      fin = kStMaxAttempts;
    }
    if (fin < 0) {
      ++attempts;
      if (Ops::add(t, dt) >= end) dt = Ops::sub(end, t);  // rk.rs:366-368
      const double dt_used = dt;

      // Stages (rk.rs:370-384): scratch = y + sum_j M[i][j] K_j; K_i = f(.) * dt.
      static_for<0, S>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        double s[D];
#pragma unroll
        for (int d = 0; d < D; ++d) s[d] = y[d];
        uint32_t poison = 0u;
        static_for<0, S>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          constexpr double m = Tab::M(i, j);
          if constexpr (m != 0.0) {
#pragma unroll
            for (int d = 0; d < D; ++d) s[d] = Ops::axpy(s[d], K[j][d], m);
          } else {
            poison |= kbad[j];
          }
        });
        poison_components(s, poison);
        double st = t;
        if constexpr (Rhs::kUsesT) st = Ops::add(t, Ops::mul(Tab::c(i), dt));
        double fv[D];
        Rhs::template eval<Ops>(st, s, p, fv);
#pragma unroll
        for (int d = 0; d < D; ++d) K[i][d] = Ops::mul(fv[d], dt);
        kbad[i] = nonfinite_mask(K[i]);
      });

      // Error estimate (rk.rs:386-390): ||sum_j e_j K_j|| / dt.
      double ev[D];
      uint32_t epoison = 0u;
      if constexpr (Tab::e(0) != 0.0) {
#pragma unroll
        for (int d = 0; d < D; ++d) ev[d] = Ops::mul(K[0][d], Tab::e(0));
      } else {
#pragma unroll
        for (int d = 0; d < D; ++d) ev[d] = 0.0;
        epoison |= kbad[0];
      }
      static_for<1, S>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        if constexpr (Tab::e(j) != 0.0) {
#pragma unroll
          for (int d = 0; d < D; ++d) ev[d] = Ops::axpy(ev[d], K[j][d], Tab::e(j));
        } else {
          epoison |= kbad[j];
        }
      });
      poison_components(ev, epoison);
      const double err = Ops::div(static_norm<Ops>(ev), dt);
      const bool ok = nn_le(err, tol);  // err >= 0 or NaN (integer compare)

      // Accept (rk.rs:392-398).
      double tn = t, yn[D];
      if (ok) {
        tn = Ops::add(t, dt);
#pragma unroll
        for (int d = 0; d < D; ++d) yn[d] = y[d];
        uint32_t bpoison = 0u;
        static_for<0, S>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          if constexpr (Tab::b(j) != 0.0) {
#pragma unroll
            for (int d = 0; d < D; ++d) yn[d] = Ops::axpy(yn[d], K[j][d], Tab::b(j));
          } else {
            bpoison |= kbad[j];
          }
        });
        poison_components(yn, bpoison);
      }

      // Controller (rk.rs:400-416); the safety factor is 100/100 = 1.
      const double delta = qrt(Ops::div(tol, err));
      // delta and dt are >= 0 or NaN: the compares run on the bit patterns
      if (nn_le(delta, 0.1)) dt = Ops::mul(dt, 0.1);
      else if (nn_ge(delta, 4.0)) dt = Ops::mul(dt, 4.0);
      else dt = Ops::mul(dt, delta);
      if (nn_gt(dt, dt_max)) dt = dt_max;

      if (nn_lt(dt, dt_min) && (ok ? tn : t) < end) {
        fin = kStMinDt;  // the accepted state of this attempt is never yielded
      } else if (kRecord && ok && acc >= a.max_steps) {
        fin = kStCapacity;  // the step log is full
      } else if (ok && a.traj_t != nullptr && traj_slot(a.traj_off, a.traj_cap, idx, acc) < 0) {
        fin = kStCapacity;  // the trajectory buffer is full: the item is not yielded
      } else if (ok) {
        if constexpr (kRecord) {
          a.dt_log[idx * a.max_steps + acc] = dt_used;
          if (acc % a.ckpt_every == 0) {
            double* c = a.ckpt + (idx * a.ckpt_slots + acc / a.ckpt_every) * (D + 1);
            c[0] = t;
#pragma unroll
            for (int d = 0; d < D; ++d) c[1 + d] = y[d];
          }
        }
        if (a.traj_t != nullptr) {
          const int64_t slot = traj_slot(a.traj_off, a.traj_cap, idx, acc);
          a.traj_t[slot] = tn;
#pragma unroll
          for (int d = 0; d < D; ++d) a.traj_y[slot * D + d] = yn[d];
        }
        t = tn;
#pragma unroll
        for (int d = 0; d < D; ++d) y[d] = yn[d];
        ++acc;
      } else {
        ++rej;
        // A rejection that leaves dt bitwise unchanged (the factor rounded to
        // exactly 1) with finite stages makes the next attempt identical: the
        // tableau reads only this attempt's stages (every layout but
        // as_compiled), so every attempt up to the cap is rejected the same
        // way and the reference would loop forever.  Jump to the cap with the
        // counts those attempts would leave.
        if constexpr (Tab::kLayout != kAsCompiled) {
          uint32_t bad = 0u;
#pragma unroll
          for (int j = 0; j < S; ++j) bad |= kbad[j];
          if (bad == 0u && dt == dt_used) {
            rej += static_cast<int32_t>(a.max_attempts - attempts);
            attempts = a.max_attempts;
          }
        }
      }
    }

    if (fin >= 0) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.y_out[d * n + idx] = y[d];
      a.t_out[idx] = t;
      a.accepted[idx] = acc;
      a.rejected[idx] = rej;
      a.status[idx] = fin;
      if (fin != kStOk) atomicMin(a.first_fail, static_cast<unsigned long long>(idx));
      have = false;
    }
  }
}

}  // namespace bacon
