// Discrete adjoint of the batched Runge-Kutta solve.
//
// The forward pass is the persistent kernel with kRecord = true: it logs the
// dt of every accepted step and checkpoints (t, y) every C accepted steps.
// The reverse kernel below walks each system's accepted steps backwards one
// segment of C steps at a time: it replays the segment forward from its
// checkpoint with the logged step sizes (stage inputs kept in per-thread
// local memory), then sweeps the segment in reverse through the vector-
// Jacobian products of the stages.  Step sizes are constants of the adjoint
// (the controller is not differentiated), so the result is the gradient of
// the discrete map the forward pass applied, up to rounding: the replay and
// the sweep have no reference counterpart and fuse every multiply-add (one
// rounding instead of two), so a replayed stage input sits within a few ulps
// of the forward pass's, and each segment restarts from the forward pass's
// own checkpointed state.  The replay order is LPT: most accepted steps first.
//
// Loss per system: L = sum_d (y_T[d] - target[d])^2; outputs dL/dy0, dL/dp.
// The reference (bacon-sci) has no gradients; the arithmetic order follows
// the CPU oracle (oracle/adjoint_oracle.c) so results are bit-reproducible.
#pragma once

#include "rk_kernel.cuh"

namespace bacon {

struct AdjArgs {
  int64_t n;
  const double* params;     // [P][n]
  const double* y_final;    // [D][n]  last yielded state of the forward pass
  const int32_t* accepted;  // [n]
  const int32_t* status;    // [n]
  const double* dt_log;     // [n][max_steps]
  const double* ckpt;       // [n][ckpt_slots][D+1]
  const double* target;     // [D][n]
  double* loss;             // [n]
  double* dl_dy0;           // [D][n]
  double* dl_dp;            // [P][n]
  int32_t max_steps;
  int32_t ckpt_slots;
  int32_t ckpt_every;       // segment length, 1..C
  unsigned long long* queue;
  const uint32_t* order;    // work order, most accepted steps first, or null
};

template <class Tab, class Rhs, int C>
__global__ void __launch_bounds__(128) rk_adjoint_reverse_kernel(const AdjArgs a) {
  using Ops = ExactOps;
  constexpr int D = Rhs::DIM;
  constexpr int S = Tab::S;
  constexpr int NP = Rhs::NP;
  constexpr int P = NP > 0 ? NP : 1;
  const int64_t n = a.n;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  double Ybuf[C][S][D];  // stage inputs of the segment being reversed (local memory)
  const int E = a.ckpt_every;

  for (;;) {
    unsigned long long ticket = 0;
    const unsigned mask = __activemask();
    const int leader = __ffs(mask) - 1;
    const unsigned lane = threadIdx.x & 31u;
    if (static_cast<int>(lane) == leader) ticket = atomicAdd(a.queue, static_cast<unsigned long long>(__popc(mask)));
    ticket = __shfl_sync(mask, ticket, leader) + __popc(mask & ((1u << lane) - 1u));
    if (static_cast<int64_t>(ticket) >= n) break;
    const int64_t i = a.order ? static_cast<int64_t>(a.order[ticket]) : static_cast<int64_t>(ticket);

    if (a.status[i] != kStOk) {
      a.loss[i] = nan;
#pragma unroll
      for (int d = 0; d < D; ++d) a.dl_dy0[d * n + i] = nan;
#pragma unroll
      for (int k = 0; k < NP; ++k) a.dl_dp[k * n + i] = nan;
      continue;
    }
    double p[P];
#pragma unroll
    for (int k = 0; k < NP; ++k) p[k] = a.params[k * n + i];
    double lam[D], mu[P];
    double L = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double e = Ops::sub(a.y_final[d * n + i], a.target[d * n + i]);
      L = Ops::add(L, Ops::mul(e, e));
      lam[d] = Ops::mul(2.0, e);
    }
#pragma unroll
    for (int k = 0; k < P; ++k) mu[k] = 0.0;

    const int32_t N = a.accepted[i];
    const double* dts = a.dt_log + i * a.max_steps;
    for (int seg = (N + E - 1) / E - 1; seg >= 0; --seg) {
      const int k0 = seg * E;
      const int m = (N - k0) < E ? (N - k0) : E;
      const double* ck = a.ckpt + (i * a.ckpt_slots + seg) * (D + 1);
      double t = ck[0], y[D];
#pragma unroll
      for (int d = 0; d < D; ++d) y[d] = ck[1 + d];
      // Replay the segment (the accepted attempts of the forward pass).
      for (int j = 0; j < m; ++j) {
        const double dt = dts[k0 + j];
        double K[S][D];
        static_for<0, S>([&](auto ic) {
          constexpr int s = decltype(ic)::value;
          double st[D];
#pragma unroll
          for (int d = 0; d < D; ++d) st[d] = y[d];
          static_for<0, S>([&](auto qc) {
            constexpr int q = decltype(qc)::value;
            constexpr double mm = Tab::M(s, q);
            if constexpr (mm != 0.0) {
#pragma unroll
              for (int d = 0; d < D; ++d) st[d] = __fma_rn(K[q][d], mm, st[d]);
            }
          });
#pragma unroll
          for (int d = 0; d < D; ++d) Ybuf[j][s][d] = st[d];
          double tt = t;
          if constexpr (Rhs::kUsesT) tt = Ops::add(t, Ops::mul(Tab::c(s), dt));
          double fv[D];
          Rhs::template eval<Ops>(tt, st, p, fv);
#pragma unroll
          for (int d = 0; d < D; ++d) K[s][d] = Ops::mul(fv[d], dt);
        });
        static_for<0, S>([&](auto qc) {
          constexpr int q = decltype(qc)::value;
          if constexpr (Tab::b(q) != 0.0) {
#pragma unroll
            for (int d = 0; d < D; ++d) y[d] = __fma_rn(K[q][d], Tab::b(q), y[d]);
          }
        });
        t = Ops::add(t, dt);
      }
      // Reverse sweep.
      for (int j = m - 1; j >= 0; --j) {
        const double dt = dts[k0 + j];
        double Kb[S][D], yb[D];
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
          for (int d = 0; d < D; ++d) Kb[s][d] = Ops::mul(lam[d], Tab::b(s));
#pragma unroll
        for (int d = 0; d < D; ++d) yb[d] = lam[d];
        static_for<0, S>([&](auto rc) {
          constexpr int s = S - 1 - decltype(rc)::value;
          double v[D], ys[D], ub[D];
#pragma unroll
          for (int d = 0; d < D; ++d) {
            v[d] = Ops::mul(Kb[s][d], dt);
            ys[d] = Ybuf[j][s][d];
          }
          Vjp<Rhs>::eval(ys, p, v, ub, mu);
#pragma unroll
          for (int d = 0; d < D; ++d) yb[d] = Ops::add(yb[d], ub[d]);
          static_for<0, s>([&](auto qc) {
            constexpr int q = decltype(qc)::value;
            constexpr double mm = Tab::M(s, q);
            if constexpr (mm != 0.0) {
#pragma unroll
              for (int d = 0; d < D; ++d) Kb[q][d] = __fma_rn(ub[d], mm, Kb[q][d]);
            }
          });
        });
#pragma unroll
        for (int d = 0; d < D; ++d) lam[d] = yb[d];
      }
    }
    a.loss[i] = L;
#pragma unroll
    for (int d = 0; d < D; ++d) a.dl_dy0[d * n + i] = lam[d];
#pragma unroll
    for (int k = 0; k < NP; ++k) a.dl_dp[k * n + i] = mu[k];
  }
}

}  // namespace bacon
