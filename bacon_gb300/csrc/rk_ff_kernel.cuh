// Persistent batched Runge-Kutta kernel, FP32-stage mode (BACON_FP32_COMP).
//
// Same work loop and step logic as rk_persistent_kernel, but the stage
// values, the state and the error vector are float-float pairs (ff.cuh)
// computed on the FP32 pipe, i.e. every sum is compensated (error-free
// transformations, the pairwise generalisation of Kahan summation).  The
// controller state stays in FP64: t, dt, the accept test
// ||sum_j e_j K_j||^2 <= (tol * dt)^2 (the reference's err <= tol with
// err = ||.|| / dt, src/ivp/rk.rs:386-392) and the dt update.  Only the
// step-size factor (tol/err)^(1/4), which scales the next dt and decides no
// accept, is evaluated with FP32 special-function instructions.  Results are
// not bit-identical to the reference's FP64 arithmetic (~48-bit stages).
#pragma once

#include "ff.cuh"
#include "rk_kernel.cuh"

namespace bacon {

// log2(num / den) for non-negative num and den over the whole double range,
// from the bit patterns with integer operations only (no FP64 instruction):
// the exponent difference plus log2f of the quotient of the two mantissas,
// each truncated to a float in [1, 2), so the quotient lies in (1/2, 2) and
// nothing under- or overflows however small (tol*dt)^2 gets.  Accurate to
// ~2^-22, ample for a step factor.  den = 0 gives +inf, a NaN den NaN, an
// infinite den or num = 0 -inf (subnormal operands read as 2^-1023 * m).
__device__ __forceinline__ float log2_ratio(double num, double den) {
  const long long bn = __double_as_longlong(num), bd = __double_as_longlong(den);
  constexpr long long kInf = 0x7ff0000000000000ll;
  if (bd > kInf) return __int_as_float(0x7fc00000);
  if (bd == 0) return INFINITY;
  if (bd == kInf || bn == 0) return -INFINITY;
  const int e = static_cast<int>(bn >> 52) - static_cast<int>(bd >> 52);
  const float mn = __int_as_float(0x3f800000 | static_cast<int>((bn >> 29) & 0x7fffff));
  const float md = __int_as_float(0x3f800000 | static_cast<int>((bd >> 29) & 0x7fffff));
  return static_cast<float>(e) + log2f(__fdiv_rn(mn, md));
}

// Largest factor a rejected attempt may keep: 1 - 2^-20.  The reference's
// factor (tol/err)^(1/4) is below 1 whenever err > tol; in FP32 a ratio
// within ~1e-7 of 1 rounds to exactly 1, which would leave dt unchanged and
// repeat the same rejected attempt until max_attempts.
constexpr float kRejectMaxFactor = 0.99999905f;

template <class Tab, class Rhs, int kMinBlocks = 1>
__global__ void __launch_bounds__(256, kMinBlocks) rk_persistent_ff_kernel(const RkArgs a) {
  constexpr int D = Rhs::DIM;
  constexpr int S = Tab::S;
  constexpr int P = Rhs::NP > 0 ? Rhs::NP : 1;
  static_assert(!Rhs::kUsesT, "the FP32-stage kernel covers autonomous right-hand sides");
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t n = a.n;
  const double tol = a.tol, dt_min = a.dt_min, dt_max = a.dt_max;
  const double dt0 = __dmul_rn(__dadd_rn(dt_max, dt_min), 0.5);

  ff y[D], K[S][D], p[P];
  double t = 0.0, end = 0.0, dt = 0.0;
  int32_t acc = 0, rej = 0;
  int64_t attempts = 0, idx = 0;
  bool have = false, exhausted = a.lanes > 0 && static_cast<int>(lane) >= a.lanes;  // as rk_persistent_kernel

  for (;;) {
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
          for (int d = 0; d < D; ++d) y[d] = ff_from_double(a.y0[d * n + idx]);
#pragma unroll
          for (int k = 0; k < Rhs::NP; ++k) p[k] = ff_from_double(a.params[k * n + idx]);
#pragma unroll
          for (int j = 0; j < S; ++j)
#pragma unroll
            for (int d = 0; d < D; ++d) K[j][d] = ff{0.0f, 0.0f};
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

    int32_t fin = -1;
    if (attempts == 0 && t >= end) {
      fin = kStTimeEndOob;
    } else if (t >= end) {
      fin = kStOk;
    } else if (attempts >= a.max_attempts) {
      fin = kStMaxAttempts;
    }
    if (fin < 0) {
      ++attempts;
      if (__dadd_rn(t, dt) >= end) dt = __dsub_rn(end, t);
      const ff dtf = ff_from_double(dt);

      static_for<0, S>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        ff s[D];
#pragma unroll
        for (int d = 0; d < D; ++d) s[d] = y[d];
        static_for<0, S>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          constexpr double m = Tab::M(i, j);
          if constexpr (m != 0.0) {
            constexpr float mf = static_cast<float>(m);
            if constexpr (static_cast<double>(mf) == m) {
#pragma unroll
              for (int d = 0; d < D; ++d) s[d] = ff_mad_f(s[d], K[j][d], mf);
            } else {
              constexpr ff mc = ff_const(m);
#pragma unroll
              for (int d = 0; d < D; ++d) s[d] = ff_mad(s[d], K[j][d], mc);
            }
          }
        });
        ff fv[D];
        Rhs::template eval<FfOps>(t, s, p, fv);
#pragma unroll
        for (int d = 0; d < D; ++d) K[i][d] = ff_mul(fv[d], dtf);
      });

      ff ev[D];
#pragma unroll
      for (int d = 0; d < D; ++d) ev[d] = ff{0.0f, 0.0f};
      static_for<0, S>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        constexpr double e = Tab::e(j);
        if constexpr (e != 0.0) {
          constexpr ff ec = ff_const(e);
#pragma unroll
          for (int d = 0; d < D; ++d) ev[d] = ff_mad(ev[d], K[j][d], ec);
        }
      });
      ff n2f = ff_mul(ev[0], ev[0]);
#pragma unroll
      for (int d = 1; d < D; ++d) n2f = ff_mad(n2f, ev[d], ev[d]);
      const double n2 = ff_to_double(n2f);
      const double tdt = __dmul_rn(tol, dt);
      const double thr = __dmul_rn(tdt, tdt);
      const bool ok = nn_le(n2, thr);  // squares of norms: >= 0 or NaN (integer compare)

      double tn = t;
      ff yn[D];
      if (ok) {
        tn = __dadd_rn(t, dt);
#pragma unroll
        for (int d = 0; d < D; ++d) yn[d] = y[d];
        static_for<0, S>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          constexpr double bj = Tab::b(j);
          if constexpr (bj != 0.0) {
            constexpr ff bc = ff_const(bj);
#pragma unroll
            for (int d = 0; d < D; ++d) yn[d] = ff_mad(yn[d], K[j][d], bc);
          }
        });
      }

      // (tol/err)^(1/4) = (thr / n2)^(1/8) = 2^(log2(thr / n2) / 8); +inf
      // when the error vanishes, NaN for a NaN error (as the reference).
      float delta = exp2f(0.125f * log2_ratio(thr, n2));
      if (!ok && delta > kRejectMaxFactor) delta = kRejectMaxFactor;
      if (delta <= 0.1f) dt = __dmul_rn(dt, 0.1);
      else if (delta >= 4.0f) dt = __dmul_rn(dt, 4.0);
      else dt = __dmul_rn(dt, static_cast<double>(delta));
      if (nn_gt(dt, dt_max)) dt = dt_max;  // dt >= 0 or NaN (integer compare)

      if (nn_lt(dt, dt_min) && (ok ? tn : t) < end) {
        fin = kStMinDt;
      } else if (ok && a.traj_t != nullptr && traj_slot(a.traj_off, a.traj_cap, idx, acc) < 0) {
        fin = kStCapacity;  // the trajectory buffer is full: the item is not yielded
      } else if (ok) {
        if (a.traj_t != nullptr) {
          const int64_t slot = traj_slot(a.traj_off, a.traj_cap, idx, acc);
          a.traj_t[slot] = tn;
#pragma unroll
          for (int d = 0; d < D; ++d) a.traj_y[slot * D + d] = ff_to_double(yn[d]);
        }
        t = tn;
#pragma unroll
        for (int d = 0; d < D; ++d) y[d] = yn[d];
        ++acc;
      } else {
        ++rej;
      }
    }

    if (fin >= 0) {
#pragma unroll
      for (int d = 0; d < D; ++d) a.y_out[d * n + idx] = ff_to_double(y[d]);
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
