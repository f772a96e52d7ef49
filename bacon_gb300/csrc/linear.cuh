// Batched RKF45 for linear systems y' = A y with one shared dense A.
//
// All systems advance in lock-step rounds; a round is one attempt
// (src/ivp/rk.rs:361-423) for every system still running.  The right-hand
// side of a stage, K_i = dt * A * Y_i with Y_i = y + sum_j M(i,j) K_j, is a
// GEMM over the batch: A (D x D) times the D x n matrix of stage inputs.
// Each system keeps its own t, dt, accept/reject state and status.
//
// Layout in HBM: every per-system vector is contiguous, [n][D] (the GEMM's B
// operand is then K-major), stage values K are [S][n][D], A is row-major.
#pragma once

#include <cstdint>

#include "device_math.cuh"
#include "rk_kernel.cuh"
#include "tableau.cuh"
#include "traj.cuh"

namespace bacon {

constexpr int32_t kLinRunning = -1;

struct LinArgs {
  int64_t n;
  const double* A;     // [D][D] row-major
  double* y;           // [n][D]  last yielded state
  double* K;           // [S][n][D]
  double* t;           // [n]
  double* dt;          // [n]  dt of the attempt in flight (end-clamped)
  double* end;         // [n]
  int64_t* attempts;   // [n]
  int32_t* accepted;   // [n]
  int32_t* rejected;   // [n]
  int32_t* status;     // [n]  kLinRunning while integrating
  unsigned int* live;  // systems running after the control kernel
  double tol, dt_min, dt_max;
  int64_t max_attempts;
  // yielded items (t, y) of every accepted attempt, or NULL: a per-system
  // slab of traj_cap items, or the packed stream with offsets traj_off
  double* traj_t;
  double* traj_y;
  const int64_t* traj_off;
  int32_t traj_cap;
};

// ---------------------------------------------------------------------------
// Stage kernel (FP64 SIMT GEMM): K_i[s][r] = dt_s * sum_k A[r][k] * Y_i[s][k].
// 64 x 64 output tile (rows x systems), 256 threads with 4 x 4 outputs each;
// the B tile is formed from y and the earlier stage values while it is
// loaded.  Sums run over k in increasing order, so with ExactOps each output
// equals the CPU oracle's matvec acc = acc + A[r][k] * y[k] bit for bit.
template <class Ops, class Tab, int D, int STAGE>
__global__ void __launch_bounds__(256) lin_stage_kernel(const LinArgs a) {
  constexpr int TM = 64, TN = 64, TK = 16;
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN + 1];
  const int r0 = blockIdx.y * TM;
  const int64_t s0 = static_cast<int64_t>(blockIdx.x) * TN;
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t n = a.n;

  // Skip tiles whose systems have all finished.
  __shared__ int any_running;
  if (tid == 0) any_running = 0;
  __syncthreads();
  if (tid < TN && s0 + tid < n && a.status[s0 + tid] == kLinRunning) any_running = 1;
  __syncthreads();
  if (!any_running) return;

  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int k0 = 0; k0 < D; k0 += TK) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int idx = tid + e * 256;  // 0..1023
      const int rr = idx / TK, kk = idx % TK;
      As[kk][rr] = a.A[static_cast<int64_t>(r0 + rr) * D + k0 + kk];
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int idx = tid + e * 256;
      const int ss = idx / TK, kk = idx % TK;
      const int64_t sys = s0 + ss;
      double v = 0.0;
      if (sys < n) {
        const int64_t off = sys * D + k0 + kk;
        v = a.y[off];
        static_for<0, Tab::S>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          constexpr double m = Tab::M(STAGE, j);
          if constexpr (m != 0.0) v = Ops::axpy(v, a.K[(static_cast<int64_t>(j) * n) * D + off], m);
        });
      }
      Bs[kk][ss] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      double av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = Ops::axpy(acc[i][j], av[i], bv[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int64_t sys = s0 + tx * 4 + j;
    if (sys >= n || a.status[sys] != kLinRunning) continue;
    const double dts = a.dt[sys];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      a.K[(static_cast<int64_t>(STAGE) * n + sys) * D + r0 + ty * 4 + i] = Ops::mul(acc[i][j], dts);
  }
}

// The tableau's stage polynomials for y' = A y.  With z = dt A the stage
// inputs are Y_i = P_i(z) y, P_0 = 1, P_i = 1 + sum_{j<i} M(i,j) z P_j, and
// the stage values K_j = z P_j(z) y.  So the attempt's update and error
// vector are polynomials in z applied to y,
//     sum_j b_j K_j = sum_{k=1..S} beta_k dt^k A^k y,
//     sum_j e_j K_j = sum_{k=1..S} eps_k  dt^k A^k y,
// and one attempt needs the S products v_k = A^k y = A v_{k-1}, whatever its
// dt.  (For the fehlberg pair beta = 1, 1/2, 1/6, 1/24, 1/104, 0 and
// eps = 0, 0, 0, 0, -1/780, 1/2080, up to the rounding of the quotients; the
// as_written matrix leaves eps_2..eps_4 nonzero.)
// Evaluated at compile time from the same IEEE quotients as the stage
// kernels.
template <class Tab>
struct LinPoly {
  static constexpr int S = Tab::S;
  struct Coef {
    double beta[S + 1];
    double eps[S + 1];
  };
  static constexpr Coef make() {
    double P[S][S] = {};  // P[i][k]: coefficient of z^k in P_i
    for (int i = 0; i < S; ++i) {
      P[i][0] = 1.0;
      for (int j = 0; j < i; ++j)
        for (int k = 0; k + 1 < S; ++k) P[i][k + 1] += Tab::M(i, j) * P[j][k];
    }
    Coef c{};
    for (int j = 0; j < S; ++j)
      for (int k = 0; k < S; ++k) {
        c.beta[k + 1] += Tab::b(j) * P[j][k];
        c.eps[k + 1] += Tab::e(j) * P[j][k];
      }
    // A coefficient below 1e-15 in magnitude is the rounding residue of an
    // exact zero (an order condition of the pair: eps_1..eps_4 of fehlberg
    // come out near 1e-18); the genuine ones are above 1e-4.
    for (int k = 0; k <= S; ++k) {
      if (c.beta[k] < 1e-15 && c.beta[k] > -1e-15) c.beta[k] = 0.0;
      if (c.eps[k] < 1e-15 && c.eps[k] > -1e-15) c.eps[k] = 0.0;
    }
    return c;
  }
  static constexpr Coef kCoef = make();
};

// c[k-1] = beta_k dt^k (update) or eps_k dt^k (error), k = 1..S.
template <class Tab, bool kBeta>
__device__ __forceinline__ void lin_poly_scalars(double dt, double (&c)[Tab::S]) {
  double p = dt;
  static_for<0, Tab::S>([&](auto jc) {
    constexpr int j = decltype(jc)::value;
    constexpr double coef = kBeta ? LinPoly<Tab>::kCoef.beta[j + 1] : LinPoly<Tab>::kCoef.eps[j + 1];
    c[j] = coef * p;
    p = p * dt;
  });
}

// Control kernel: finish the attempt in flight (error estimate, accept,
// controller, dt_min check: rk.rs:386-416), then open the next one (Done /
// attempt cap, end clamp: rk.rs:362-368).  With kPoly the attempt's vectors
// are the products v_k = A^k y in K[k-1] (the tensor-core engine), combined
// through LinPoly with the system's dt; otherwise they are the stage values.
//
// A warp serves kLinCtlGroup = 4 consecutive systems.  The element-wise
// work (error vector, update of y) runs as full-warp passes over one system
// at a time.  The nalgebra norm and the scalar controller run once for all
// four: lanes 8g..8g+7 hold system g's eight norm accumulators (blas.rs
// dotx: strides of 8, combined in its order) and compute its controller.  On
// GB300 an FP64 warp instruction costs the same whatever its active lanes,
// and this kernel is FP64-pipe bound, so the norm with 8 of 32 lanes active
// and the one-lane controller had cost as much as the vector work.
constexpr int kLinCtlGroup = 4;    // systems per warp
constexpr int kLinCtlThreads = 128;
constexpr int kLinCtlSystemsPerBlock = kLinCtlGroup * kLinCtlThreads / 32;

template <class Ops, class Tab, int D, bool kPoly = false>
__global__ void __launch_bounds__(kLinCtlThreads) lin_control_kernel(const LinArgs a, int first) {
  static_assert(D >= 8 && D % 32 == 0, "dimension must be a multiple of 32");
  constexpr int S = Tab::S;
  constexpr int PER = D / 32;
  constexpr int G = kLinCtlGroup;
  static_assert(G == 4, "the warp-level skip below names four systems");
  const unsigned lane = threadIdx.x & 31u;
  const int w = threadIdx.x / 32;
  const int g = static_cast<int>(lane / 8);  // this lane's system in the norm and the controller
  const int r = static_cast<int>(lane % 8);  // its accumulator
  const int64_t n = a.n;
  const int64_t sys0 = (static_cast<int64_t>(blockIdx.x) * kLinCtlThreads + threadIdx.x) / 32 * G;
  if (sys0 >= n) return;  // whole warp
  bool run[G];
#pragma unroll
  for (int k = 0; k < G; ++k) run[k] = sys0 + k < n && a.status[sys0 + k] == kLinRunning;
  if (!(run[0] || run[1] || run[2] || run[3])) return;  // whole warp
  const int64_t sys = sys0 + g;
  const bool mine = g == 0 ? run[0] : g == 1 ? run[1] : g == 2 ? run[2] : run[3];  // no stack frame
  double t = 0.0, dt = 0.0, end = 0.0;
  int64_t att = 0;
  if (mine) {
    t = a.t[sys];
    dt = a.dt[sys];
    end = a.end[sys];
    att = a.attempts[sys];
  }
  int32_t st = kLinRunning;
  int32_t acc_add = 0, rej_add = 0;
  int64_t slot = -1;

  if (!first) {
    __shared__ double ev_s[kLinCtlThreads / 32][G][D];
#pragma unroll
    for (int k = 0; k < G; ++k) {
      if (!run[k]) continue;  // whole warp
      double eh[S];  // kPoly: eps_k dt^k for this system
      if constexpr (kPoly) lin_poly_scalars<Tab, false>(a.dt[sys0 + k], eh);
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int d = lane + 32 * q;
        const int64_t off = (sys0 + k) * D + d;
        double e = 0.0;
        if constexpr (kPoly) {
          static_for<0, S>([&](auto jc) {
            constexpr int j = decltype(jc)::value;
            if constexpr (LinPoly<Tab>::kCoef.eps[j + 1] != 0.0)
              e = Ops::axpy(e, a.K[(static_cast<int64_t>(j) * n) * D + off], eh[j]);
          });
        } else {
          if constexpr (Tab::e(0) != 0.0) e = Ops::mul(a.K[off], Tab::e(0));
          static_for<1, S>([&](auto jc) {
            constexpr int j = decltype(jc)::value;
            if constexpr (Tab::e(j) != 0.0) e = Ops::axpy(e, a.K[(static_cast<int64_t>(j) * n) * D + off], Tab::e(j));
          });
        }
        ev_s[w][k][d] = e;
      }
    }
    __syncwarp();
    // nalgebra norm of system g's error vector; lanes of a stopped system
    // compute on stale values and their result is not used
    const double* ev = ev_s[w][g];
    double accl = 0.0;
#pragma unroll 8
    for (int i = 0; i < D; i += 8) accl = __dadd_rn(accl, __dmul_rn(ev[i + r], ev[i + r]));
    double acc[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) acc[l] = __shfl_sync(0xffffffffu, accl, 8 * g + l);
    double res = 0.0;
    res = __dadd_rn(res, __dadd_rn(acc[0], acc[4]));
    res = __dadd_rn(res, __dadd_rn(acc[1], acc[5]));
    res = __dadd_rn(res, __dadd_rn(acc[2], acc[6]));
    res = __dadd_rn(res, __dadd_rn(acc[3], acc[7]));
    const double err = Ops::div(__dsqrt_rn(__dadd_rn(0.0, res)), dt);
    const bool ok = err <= a.tol;
    const double tn = ok ? Ops::add(t, dt) : t;
    const double delta = qrt(Ops::div(a.tol, err));
    double ndt;
    if (delta <= 0.1) ndt = Ops::mul(dt, 0.1);
    else if (delta >= 4.0) ndt = Ops::mul(dt, 4.0);
    else ndt = Ops::mul(dt, delta);
    if (ndt > a.dt_max) ndt = a.dt_max;
    bool upd = false;
    // the slot of the item this attempt yields if accepted (before the
    // accepted count is updated below)
    if (a.traj_t != nullptr && mine) slot = traj_slot(a.traj_off, a.traj_cap, sys, a.accepted[sys]);
    if (ndt < a.dt_min && tn < end) {
      st = kStMinDt;
    } else if (ok && a.traj_t != nullptr && slot < 0) {
      st = kStCapacity;  // the trajectory is full: the item is not yielded
    } else if (ok) {
      upd = true;
      t = tn;
      acc_add = 1;
    } else {
      rej_add = 1;
      // dt bitwise unchanged by a rejection: the next attempt is this one
      // again, up to the cap (as in rk_persistent_kernel); jump there.
      if (ndt == dt) {
        rej_add += static_cast<int32_t>(a.max_attempts - att);
        att = a.max_attempts;
      }
    }
    dt = ndt;
    // y += sum_j b_j K_j for the accepted systems, a full-warp pass each
    const unsigned upd_mask = __ballot_sync(0xffffffffu, upd && mine);
#pragma unroll
    for (int k = 0; k < G; ++k) {
      if (!((upd_mask >> (8 * k)) & 1u)) continue;  // whole warp
      double bh[S];  // kPoly: beta_k dt^k for this system
      if constexpr (kPoly) lin_poly_scalars<Tab, true>(a.dt[sys0 + k], bh);
      // system k's item slot and new time, from its lanes 8k..8k+7
      const long long slot_k = __shfl_sync(0xffffffffu, static_cast<long long>(slot), 8 * k);
      const double t_k = __shfl_sync(0xffffffffu, t, 8 * k);
      if (a.traj_t != nullptr && lane == 0) a.traj_t[slot_k] = t_k;
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int64_t off = (sys0 + k) * D + lane + 32 * q;
        double v = a.y[off];
        static_for<0, S>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          if constexpr (kPoly) {
            if constexpr (LinPoly<Tab>::kCoef.beta[j + 1] != 0.0)
              v = Ops::axpy(v, a.K[(static_cast<int64_t>(j) * n) * D + off], bh[j]);
          } else {
            if constexpr (Tab::b(j) != 0.0) v = Ops::axpy(v, a.K[(static_cast<int64_t>(j) * n) * D + off], Tab::b(j));
          }
        });
        a.y[off] = v;
        if (a.traj_t != nullptr) a.traj_y[slot_k * D + lane + 32 * q] = v;
      }
    }
  }
  if (st == kLinRunning) {
    if (t >= end) {
      st = (first && att == 0) ? kStTimeEndOob : kStOk;
    } else if (att >= a.max_attempts) {
      st = kStMaxAttempts;
    } else {
      if (Ops::add(t, dt) >= end) dt = Ops::sub(end, t);
    }
  }
  if (mine && r == 0) {
    if (acc_add) a.accepted[sys] += acc_add;
    if (rej_add) a.rejected[sys] += rej_add;
    a.t[sys] = t;
    a.dt[sys] = dt;
    if (st != kLinRunning) {
      a.status[sys] = st;
      a.attempts[sys] = att;
    } else {
      a.attempts[sys] = att + 1;
      atomicAdd(a.live, 1u);
    }
  }
}

}  // namespace bacon

namespace bacon {
struct LinInitArgs {
  LinArgs st;
  int dim;
  int stages;
  const double* y0;     // [D][n] SoA
  const double* t0;
  const double* t_end;
  double t0_s, t_end_s, dt0;
};
}  // namespace bacon
