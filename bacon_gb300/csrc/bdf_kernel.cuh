// Batched implicit BDF kernels (one system per thread, small dimensions).
//
// Corrected mode: the engine's stiff BDF.  Orders 1..qmax (6 for BDF6, 2 for
// BDF2) ramp up after the start, f is evaluated at t_{n+1}, and each step
// solves the order-q and order-(q-1) formulas
//     y + sum_j a_{q,j} y_{n+1-j} = dt * b_q * f(t_{n+1}, y)
// by Newton's method with the analytic Jacobian (one partial-pivot LU per
// solve, factors and pivots in registers).  Error control follows
// src/ivp/bdf.rs:580-633: err = ||y_q - y_{q-1}||_2, accept if err <= tol,
// double dt below tol/10 (here only with a full history, re-sampling every
// second point), halve on rejection (Lagrange re-interpolation of the
// history), MinimumTimeDeltaExceeded below dt_min.  The operation sequence is
// the CPU oracle's (oracle/bdf_oracle.c, bdf_corrected), in exact FP64; the
// LU elimination and both substitutions update with fused multiply-adds
// (correctly rounded, so the oracle's C fma gives the same bits).
#pragma once

#include "rk_kernel.cuh"

namespace bacon {

struct BdfArgs {
  int64_t n;
  const double* y0;      // [D][n]
  const double* params;  // [P][n]
  const double* t0;      // [n] or null
  const double* t_end;   // [n] or null
  double t0_s, t_end_s;
  double tol, dt_min, dt_max;
  int64_t max_steps;
  int32_t max_iter;      // Newton iterations per solve
  int32_t qmax;          // 6 (BDF6) or 2 (BDF2)
  double* y_out;
  double* t_out;
  int32_t* accepted;
  int32_t* rejected;
  int32_t* status;
  double* traj_t;
  double* traj_y;
  int32_t traj_cap;
  const int64_t* traj_off;  // [n+1] packed offsets, or null: slabs of traj_cap
  unsigned long long* queue;
  unsigned long long* first_fail;
};

// BDF-q coefficients (b_q, a_{q,j}), the same quotients as the oracle.
__device__ __forceinline__ double bdf_b(int q) {
  switch (q) {
    case 1: return 1.0;
    case 2: return 2.0 / 3.0;
    case 3: return 6.0 / 11.0;
    case 4: return 12.0 / 25.0;
    case 5: return 60.0 / 137.0;
    default: return 60.0 / 147.0;
  }
}

__device__ __forceinline__ double bdf_a(int q, int j) {  // j = 1..q
  switch (q) {
    case 1: return -1.0;
    case 2: return j == 1 ? -4.0 / 3.0 : 1.0 / 3.0;
    case 3: return j == 1 ? -18.0 / 11.0 : j == 2 ? 9.0 / 11.0 : -2.0 / 11.0;
    case 4: return j == 1 ? -48.0 / 25.0 : j == 2 ? 36.0 / 25.0 : j == 3 ? -16.0 / 25.0 : 3.0 / 25.0;
    case 5:
      return j == 1 ? -300.0 / 137.0 : j == 2 ? 300.0 / 137.0 : j == 3 ? -200.0 / 137.0
             : j == 4 ? 75.0 / 137.0 : -12.0 / 137.0;
    default:
      return j == 1 ? -360.0 / 147.0 : j == 2 ? 450.0 / 147.0 : j == 3 ? -400.0 / 147.0
             : j == 4 ? 225.0 / 147.0 : j == 5 ? -72.0 / 147.0 : 10.0 / 147.0;
  }
}

// Lagrange weights of the nodes s_i = -i (i = 0..q) at s (oracle order).
__device__ __forceinline__ void lagrange_weights(int q, double s, double (&w)[7]) {
  for (int i = 0; i <= q; ++i) {
    double num = 1.0, den = 1.0;
    for (int k = 0; k <= q; ++k) {
      if (k == i) continue;
      num = __dmul_rn(num, __dsub_rn(s, static_cast<double>(-k)));
      den = __dmul_rn(den, __dsub_rn(static_cast<double>(-i), static_cast<double>(-k)));
    }
    w[i] = __ddiv_rn(num, den);
  }
}

// Euclidean norm of a dynamic or static vector, nalgebra order (see
// oracle_norm): static 2/3/4 special cases, else eight lanes.
template <int D>
__device__ __forceinline__ double bdf_norm(const double (&x)[D], bool dyn) {
  using O = ExactOps;
  if (!dyn && D == 2) return O::sqrt(O::add(O::mul(x[0], x[0]), O::mul(x[1 % D], x[1 % D])));
  if (!dyn && D == 3)
    return O::sqrt(O::add(O::add(O::mul(x[0], x[0]), O::mul(x[1 % D], x[1 % D])), O::mul(x[2 % D], x[2 % D])));
  if (!dyn && D == 4) {
    double a = O::mul(x[0], x[0]), b = O::mul(x[1 % D], x[1 % D]);
    const double c = O::mul(x[2 % D], x[2 % D]), d = O::mul(x[3 % D], x[3 % D]);
    a = O::add(a, c);
    b = O::add(b, d);
    return O::sqrt(O::add(a, b));
  }
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int i = 0;
  while (D - i >= 8) {
#pragma unroll
    for (int l = 0; l < 8; ++l) acc[l] = O::add(acc[l], O::mul(x[(i + l) % D], x[(i + l) % D]));
    i += 8;
  }
  double res = 0.0;
  res = O::add(res, O::add(acc[0], acc[4]));
  res = O::add(res, O::add(acc[1], acc[5]));
  res = O::add(res, O::add(acc[2], acc[6]));
  res = O::add(res, O::add(acc[3], acc[7]));
  for (int k = i; k < D; ++k) res = O::add(res, O::mul(x[k], x[k]));
  return O::sqrt(O::add(0.0, res));
}

// x == 0.0 (either sign) on the bit pattern, without an FP64 instruction.
__device__ __forceinline__ bool bits_zero(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) << 1) == 0ull;
}

// Newton solve of G(y) = y - h*b_q*f(t1, y) + sum_j a_{q,j} HH[j-1] = 0.
template <class Rhs, int D>
__device__ __forceinline__ bool bdf_newton(const double* p, double t1, double h, int q, const double (&HH)[7][D],
                                           const double (&guess)[D], double (&y)[D], int max_newton, double tol) {
  using O = ExactOps;
  const double hb = O::mul(h, bdf_b(q));
  double c[D];
#pragma unroll
  for (int d = 0; d < D; ++d) c[d] = 0.0;
  for (int j = 1; j <= q; ++j) {
    const double aj = bdf_a(q, j);
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = O::add(c[d], O::mul(aj, HH[j - 1][d]));
  }
#pragma unroll
  for (int d = 0; d < D; ++d) y[d] = guess[d];
  double M[D][D];
  Jac<Rhs>::template eval<O>(y, p, M);
#pragma unroll
  for (int r = 0; r < D; ++r)
#pragma unroll
    for (int k = 0; k < D; ++k) M[r][k] = O::sub((r == k) ? 1.0 : 0.0, O::mul(hb, M[r][k]));
  int piv[D];
  double rinv[D];  // 1 / U[i][i], the elimination's own reciprocal
#pragma unroll
  for (int i = 0; i < D; ++i) {
    int pr = i;
    double best = fabs(M[i][i]);
#pragma unroll
    for (int r = i + 1; r < D; ++r)
      if (fabs(M[r][i]) > best) {
        best = fabs(M[r][i]);
        pr = r;
      }
    piv[i] = pr;
    if (pr != i) {
#pragma unroll
      for (int k = 0; k < D; ++k) {
        // swap rows i and pr through a select (registers cannot be indexed)
        double a = M[i][k], b = 0.0;
#pragma unroll
        for (int r = i + 1; r < D; ++r)
          if (r == pr) b = M[r][k];
#pragma unroll
        for (int r = i + 1; r < D; ++r)
          if (r == pr) M[r][k] = a;
        M[i][k] = b;
      }
    }
    if (M[i][i] == 0.0) return false;
    const double inv = O::div(1.0, M[i][i]);
    rinv[i] = inv;
#pragma unroll
    for (int r = i + 1; r < D; ++r) {
      const double l = O::mul(M[r][i], inv);
      M[r][i] = l;
      // an exactly zero multiplier or pivot-row entry skips the update (the
      // oracle's rule; the zero tests are integer operations)
#pragma unroll
      for (int k = i + 1; k < D; ++k)
        if (!bits_zero(l) && !bits_zero(M[i][k])) M[r][k] = __fma_rn(-l, M[i][k], M[r][k]);
    }
  }
  // rows of U scaled by their pivot reciprocal (a unit upper factor)
#pragma unroll
  for (int r = 0; r < D; ++r)
#pragma unroll
    for (int k = r + 1; k < D; ++k) M[r][k] = O::mul(M[r][k], rinv[r]);
  // the unit factors replaced by their inverses (strict parts in place; one
  // block of the 32-row blocked solve), column c the solve of e_c with every
  // update taken for every column
  {
    double T[D][D];
#pragma unroll
    for (int cc = 0; cc < D; ++cc) {
      double x[D];
#pragma unroll
      for (int j = 0; j < D; ++j) x[j] = (j == cc) ? 1.0 : 0.0;
#pragma unroll
      for (int k = 0; k + 1 < D; ++k)
#pragma unroll
        for (int j = k + 1; j < D; ++j) x[j] = __fma_rn(-M[j][k], x[k], x[j]);
#pragma unroll
      for (int j = cc + 1; j < D; ++j) T[j][cc] = x[j];
#pragma unroll
      for (int j = 0; j < D; ++j) x[j] = (j == cc) ? 1.0 : 0.0;
#pragma unroll
      for (int k = D - 1; k > 0; --k)
#pragma unroll
        for (int j = 0; j < k; ++j) x[j] = __fma_rn(-M[j][k], x[k], x[j]);
#pragma unroll
      for (int j = 0; j < cc; ++j) T[j][cc] = x[j];
    }
#pragma unroll
    for (int j = 0; j < D; ++j)
#pragma unroll
      for (int cc = 0; cc < D; ++cc)
        if (j != cc) M[j][cc] = T[j][cc];
  }
  const double conv = O::mul(1e-3, tol);
  for (int it = 0; it < max_newton; ++it) {
    double f[D], dx[D];
    Rhs::template eval<O>(t1, y, p, f);
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = -O::add(O::sub(y[d], O::mul(hb, f[d])), c[d]);
#pragma unroll
    for (int i = 0; i < D; ++i) {
      if (piv[i] != i) {
        double a = dx[i], b = 0.0;
#pragma unroll
        for (int r = i + 1; r < D; ++r)
          if (r == piv[i]) b = dx[r];
#pragma unroll
        for (int r = i + 1; r < D; ++r)
          if (r == piv[i]) dx[r] = a;
        dx[i] = b;
      }
    }
    {
      // x = Linv r (ascending k), then the reciprocals, then x = Uinv r
      // (descending k)
      double rb[D];
#pragma unroll
      for (int j = 0; j < D; ++j) rb[j] = dx[j];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double acc = rb[j];
#pragma unroll
        for (int k = 0; k < j; ++k) acc = __fma_rn(M[j][k], rb[k], acc);
        dx[j] = acc;
      }
#pragma unroll
      for (int j = 0; j < D; ++j) rb[j] = O::mul(dx[j], rinv[j]);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double acc = rb[j];
#pragma unroll
        for (int k = D - 1; k > j; --k) acc = __fma_rn(M[j][k], rb[k], acc);
        dx[j] = acc;
      }
    }
    double dn = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      y[d] = O::add(y[d], dx[d]);
      dn = O::add(dn, O::mul(dx[d], dx[d]));
    }
    if (!(dn == dn)) return false;
    if constexpr (Rhs::kAffine) return true;  // the first update solves the linear system
    if (O::sqrt(dn) <= conv) return true;
  }
  return false;
}

// One system of the corrected BDF, integrated by the calling thread alone
// (state in registers and local memory).
template <class Rhs>
__device__ __forceinline__ void bdf_corrected_system(const BdfArgs& a, int64_t idx, bool dyn) {
  using O = ExactOps;
  constexpr int D = Rhs::DIM;
  constexpr int P = Rhs::NP > 0 ? Rhs::NP : 1;
  const int64_t n = a.n;
  double dt_min = a.dt_min;
  const double dt_max = a.dt_max;
  if (dt_min > dt_max) dt_min = dt_max;
  const int qmax = a.qmax;
  double p[P];
#pragma unroll
  for (int k = 0; k < Rhs::NP; ++k) p[k] = a.params[k * n + idx];
  double H[7][D], Hn[7][D];
#pragma unroll
  for (int d = 0; d < D; ++d) H[0][d] = a.y0[d * n + idx];
  double t = a.t0 ? a.t0[idx] : a.t0_s;
  const double t_end = a.t_end ? a.t_end[idx] : a.t_end_s;
  double dt = O::mul(O::add(dt_max, dt_min), 0.5);
  int k = 1;
  int32_t acc = 0, rej = 0, status = kStOk;
  double last_t = t, last_y[D];
#pragma unroll
  for (int d = 0; d < D; ++d) last_y[d] = H[0][d];
  int64_t steps = 0;
  if (t >= t_end) status = kStTimeEndOob;
  while (status == kStOk && t < t_end) {
    if (steps >= a.max_steps) {
      status = kStMaxAttempts;
      break;
    }
    ++steps;
    double h = dt;
    if (O::add(t, h) >= t_end) h = O::sub(t_end, t);
    const int q = (k < qmax) ? k : qmax;
    double w[7];
    double HH[7][D];
    if (h != dt && k > 1) {
      const double ratio = O::div(h, dt);
      for (int j = 0; j < k; ++j) {
        lagrange_weights(k - 1, O::mul(-ratio, static_cast<double>(j)), w);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double s = 0.0;
          for (int i = 0; i < k; ++i) s = O::add(s, O::mul(w[i], H[i][d]));
          HH[j][d] = s;
        }
      }
    } else {
      for (int j = 0; j < k; ++j)
#pragma unroll
        for (int d = 0; d < D; ++d) HH[j][d] = H[j][d];
    }
    double pred[D], yh[D], yl[D], diff[D];
    lagrange_weights(k - 1, 1.0, w);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double s = 0.0;
      for (int i = 0; i < k; ++i) s = O::add(s, O::mul(w[i], HH[i][d]));
      pred[d] = s;
    }
    const double t1 = O::add(t, h);
    bool ok = bdf_newton<Rhs, D>(p, t1, h, q, HH, pred, yh, a.max_iter, a.tol);
    double error;
    if (ok && q >= 2) {
      ok = bdf_newton<Rhs, D>(p, t1, h, q - 1, HH, yh, yl, a.max_iter, a.tol);
#pragma unroll
      for (int d = 0; d < D; ++d) diff[d] = O::sub(yh[d], yl[d]);
      error = bdf_norm(diff, dyn);
    } else {
      double f0[D];
      Rhs::template eval<O>(t, H[0], p, f0);
#pragma unroll
      for (int d = 0; d < D; ++d) diff[d] = O::mul(0.5, O::sub(yh[d], O::add(H[0][d], O::mul(h, f0[d]))));
      error = bdf_norm(diff, dyn);
    }
    if (ok && error <= a.tol && a.traj_t != nullptr && traj_slot(a.traj_off, a.traj_cap, idx, acc) < 0) {
      status = kStCapacity;  // the trajectory buffer is full: the item is not yielded
      break;
    }
    if (ok && error <= a.tol) {
      const int kk = (k < 7) ? k + 1 : 7;
      for (int i = kk - 1; i >= 1; --i)
#pragma unroll
        for (int d = 0; d < D; ++d) H[i][d] = H[i - 1][d];
#pragma unroll
      for (int d = 0; d < D; ++d) H[0][d] = yh[d];
      k = kk;
      t = t1;
      if (a.traj_t != nullptr) {
        const int64_t slot = traj_slot(a.traj_off, a.traj_cap, idx, acc);
        a.traj_t[slot] = t;
#pragma unroll
        for (int d = 0; d < D; ++d) a.traj_y[slot * D + d] = yh[d];
      }
      ++acc;
      last_t = t;
#pragma unroll
      for (int d = 0; d < D; ++d) last_y[d] = yh[d];
      if (h != dt) continue;
      if (error < O::mul(0.1, a.tol) && k == qmax + 1 && O::mul(dt, 2.0) <= dt_max) {
        const int nk = (k + 1) / 2;
        for (int i = 1; i < nk; ++i)
#pragma unroll
          for (int d = 0; d < D; ++d) H[i][d] = H[2 * i][d];
        k = nk;
        dt = O::mul(dt, 2.0);
      }
      continue;
    }
    ++rej;
    const double nd = O::mul(dt, 0.5);
    if (nd < dt_min) {
      status = kStMinDt;
      break;
    }
    if (k > 1) {
      for (int j = 0; j < k; ++j) {
        lagrange_weights(k - 1, O::mul(-0.5, static_cast<double>(j)), w);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double s = 0.0;
          for (int i = 0; i < k; ++i) s = O::add(s, O::mul(w[i], H[i][d]));
          Hn[j][d] = s;
        }
      }
      for (int j = 0; j < k; ++j)
#pragma unroll
        for (int d = 0; d < D; ++d) H[j][d] = Hn[j][d];
    }
    dt = nd;
  }
#pragma unroll
  for (int d = 0; d < D; ++d) a.y_out[d * n + idx] = last_y[d];
  a.t_out[idx] = last_t;
  a.accepted[idx] = acc;
  a.rejected[idx] = rej;
  a.status[idx] = status;
  if (status != kStOk) atomicMin(a.first_fail, static_cast<unsigned long long>(idx));
}

// Every thread pulls systems from the work counter until the batch is done.
template <class Rhs>
__device__ __forceinline__ void bdf_corrected_thread_loop(const BdfArgs& a, bool dyn) {
  const unsigned lane = threadIdx.x & 31u;
  for (;;) {
    unsigned long long ticket = 0;
    const unsigned mask = __activemask();
    const int leader = __ffs(mask) - 1;
    if (static_cast<int>(lane) == leader) ticket = atomicAdd(a.queue, static_cast<unsigned long long>(__popc(mask)));
    ticket = __shfl_sync(mask, ticket, leader) + __popc(mask & ((1u << lane) - 1u));
    const int64_t idx = static_cast<int64_t>(ticket);
    if (idx >= a.n) break;
    bdf_corrected_system<Rhs>(a, idx, dyn);
  }
}

template <class Rhs>
__global__ void __launch_bounds__(128) bdf_corrected_kernel(const BdfArgs a, int dyn_dim) {
  bdf_corrected_thread_loop<Rhs>(a, dyn_dim != 0);
}

// ---------------------------------------------------------------------------
// As-compiled mode: the reference's BDF (src/ivp/bdf.rs:257-673) per system,
// every quirk kept — RK4 bootstrap of O steps, the yield machine, residuals
// with f at t_n and the lower formula built on the higher-order history
// weights, the finite-difference "Jacobian" (G(x+dt e) + G(x-dt e)) / (2 dt),
// an explicit inverse from nalgebra's partial-pivot LU, up to 998 Broyden
// updates, and t -= dt - order on a rejected bootstrap.  O = 7 (BDF6) or 3
// (BDF2).  Mirrors the CPU oracle's restatement operation by operation.
template <int O, int D>
struct BdfRefState {
  static constexpr int kHist = O + 3;  // the deque never exceeds O + 2 entries
  double hc[O], lc[O];
  double dt_max, dt_min, time, end, tol, dt, order;
  double state[D], save[D];
  double ht[kHist];
  double hy[kHist][D];
  int hfront, hlen, ym;
};

template <int O, int D>
__device__ __forceinline__ bool ref_push(BdfRefState<O, D>& s, double t, const double (&y)[D]) {
  if (s.hlen >= BdfRefState<O, D>::kHist) return false;
  const int k = (s.hfront + s.hlen) % BdfRefState<O, D>::kHist;
  s.ht[k] = t;
#pragma unroll
  for (int d = 0; d < D; ++d) s.hy[k][d] = y[d];
  s.hlen++;
  return true;
}

template <int O, int D>
__device__ __forceinline__ int ref_idx(const BdfRefState<O, D>& s, int i) {
  return (s.hfront + i) % BdfRefState<O, D>::kHist;
}

template <class Rhs, int O, int D>
__device__ bool ref_rk4(BdfRefState<O, D>& s, const double* p, int iterations) {
  using Op = ExactOps;
  double k1[D], k2[D], k3[D], k4[D], it[D], f[D];
  for (int i = 0; i < iterations; ++i) {
    Rhs::template eval<Op>(s.time, s.state, p, f);
#pragma unroll
    for (int d = 0; d < D; ++d) k1[d] = Op::mul(f[d], s.dt);
#pragma unroll
    for (int d = 0; d < D; ++d) it[d] = Op::add(s.state[d], Op::mul(k1[d], 0.5));
    Rhs::template eval<Op>(Op::add(s.time, Op::mul(0.5, s.dt)), it, p, f);
#pragma unroll
    for (int d = 0; d < D; ++d) k2[d] = Op::mul(f[d], s.dt);
#pragma unroll
    for (int d = 0; d < D; ++d) it[d] = Op::add(s.state[d], Op::mul(k2[d], 0.5));
    Rhs::template eval<Op>(Op::add(s.time, Op::mul(0.5, s.dt)), it, p, f);
#pragma unroll
    for (int d = 0; d < D; ++d) k3[d] = Op::mul(f[d], s.dt);
#pragma unroll
    for (int d = 0; d < D; ++d) it[d] = Op::add(s.state[d], k3[d]);
    Rhs::template eval<Op>(Op::add(s.time, s.dt), it, p, f);
#pragma unroll
    for (int d = 0; d < D; ++d) k4[d] = Op::mul(f[d], s.dt);
    if (i != 0 && !ref_push(s, s.time, s.state)) return false;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double inc =
          Op::mul(Op::add(Op::add(Op::add(k1[d], Op::mul(k2[d], 2.0)), Op::mul(k3[d], 2.0)), k4[d]), 1.0 / 6.0);
      s.state[d] = Op::add(s.state[d], inc);
    }
    s.time = Op::add(s.time, s.dt);
  }
  return ref_push(s, s.time, s.state);
}

template <class Rhs, int O, int D>
__device__ __forceinline__ void ref_residual(const BdfRefState<O, D>& s, const double* p, bool lower,
                                             const double (&y)[D], double (&out)[D]) {
  using Op = ExactOps;
  double f[D], sc[D];
  Rhs::template eval<Op>(s.time, y, p, f);
  const double c0 = lower ? s.lc[0] : s.hc[0];
#pragma unroll
  for (int d = 0; d < D; ++d) sc[d] = Op::mul(Op::mul(-f[d], s.dt), c0);
  for (int ind = 1; ind < O; ++ind) {
    const int k = ref_idx(s, O - ind);
#pragma unroll
    for (int d = 0; d < D; ++d) sc[d] = Op::add(sc[d], Op::mul(s.hy[k][d], s.hc[ind]));
  }
#pragma unroll
  for (int d = 0; d < D; ++d) out[d] = Op::add(sc[d], y[d]);
}

// nalgebra's dot product of two vectors of run-time length (blas.rs `dotx`,
// general path): the rows r0.. of columns cx and cy of a D x D matrix.
template <int D>
__device__ __forceinline__ double ref_dotx_col(const double (&x)[D][D], int cx, const double (&y)[D][D], int cy,
                                               int r0) {
  using Op = ExactOps;
  const int len = D - r0;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int i = 0;
  while (len - i >= 8) {
    for (int l = 0; l < 8; ++l) acc[l] = Op::add(acc[l], Op::mul(x[r0 + i + l][cx], y[r0 + i + l][cy]));
    i += 8;
  }
  double res = 0.0;
  res = Op::add(res, Op::add(acc[0], acc[4]));
  res = Op::add(res, Op::add(acc[1], acc[5]));
  res = Op::add(res, Op::add(acc[2], acc[6]));
  res = Op::add(res, Op::add(acc[3], acc[7]));
  for (int k = i; k < len; ++k) res = Op::add(res, Op::mul(x[r0 + k][cx], y[r0 + k][cy]));
  return res;
}

// Rust's f64::signum: 1 for +0 and positives, -1 for -0 and negatives.
__device__ __forceinline__ double rs_signum(double x) { return isnan(x) ? x : (signbit(x) ? -1.0 : 1.0); }

// nalgebra FullPivLU::new + try_inverse, secant's first fallback
// (src/ivp/bdf.rs:433-437): the largest |a| of the remaining block, first in
// column-major order, brought to the diagonal by a column and a row swap,
// then a Gauss step; invertible when the last diagonal entry is not zero.
// A cold path, kept out of line.
template <int D>
__device__ __noinline__ bool ref_full_piv_lu_inverse(const double (&A)[D][D], double (&inv)[D][D]) {
  using Op = ExactOps;
  double a[D][D];
  int pi[D], pp[D], qi[D], qp[D], np = 0, nq = 0;
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) a[r][c] = A[r][c];
  for (int i = 0; i < D; ++i) {
    int pr = i, pc = i;
    double best = fabs(a[i][i]);
    for (int c = i; c < D; ++c)
      for (int r = i; r < D; ++r)
        if (fabs(a[r][c]) > best) {
          best = fabs(a[r][c]);
          pr = r;
          pc = c;
        }
    const double diag = a[pr][pc];
    if (diag == 0.0) break;  // the rest of the matrix is zero
    if (pc != i) {
      for (int r = 0; r < D; ++r) {
        const double t = a[r][i];
        a[r][i] = a[r][pc];
        a[r][pc] = t;
      }
      qi[nq] = i;
      qp[nq] = pc;
      ++nq;
    }
    if (pr != i) {
      pi[np] = i;
      pp[np] = pr;
      ++np;
      for (int c = 0; c < D; ++c) {
        const double t = a[i][c];
        a[i][c] = a[pr][c];
        a[pr][c] = t;
      }
    }
    const double inv_diag = Op::div(1.0, diag);
    for (int r = i + 1; r < D; ++r) a[r][i] = Op::mul(a[r][i], inv_diag);
    for (int c = i + 1; c < D; ++c) {
      const double alpha = -a[i][c];
      for (int r = i + 1; r < D; ++r) a[r][c] = Op::add(Op::mul(alpha, a[r][i]), a[r][c]);
    }
  }
  if (a[D - 1][D - 1] == 0.0) return false;
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) inv[r][c] = (r == c) ? 1.0 : 0.0;
  for (int k = 0; k < np; ++k)
    for (int c = 0; c < D; ++c) {
      const double t = inv[pi[k]][c];
      inv[pi[k]][c] = inv[pp[k]][c];
      inv[pp[k]][c] = t;
    }
  for (int k = 0; k < D; ++k)
    for (int i = 0; i < D - 1; ++i) {
      const double mc = -Op::div(inv[i][k], 1.0);
      for (int r = i + 1; r < D; ++r) inv[r][k] = Op::add(Op::mul(mc, a[r][i]), inv[r][k]);
    }
  for (int k = 0; k < D; ++k)
    for (int i = D - 1; i >= 0; --i) {
      const double diag = a[i][i];
      if (diag == 0.0) break;  // try_inverse ignores the solve's own result
      const double coeff = Op::div(inv[i][k], diag);
      inv[i][k] = coeff;
      const double mc = -coeff;
      for (int r = 0; r < i; ++r) inv[r][k] = Op::add(Op::mul(mc, a[r][i]), inv[r][k]);
    }
  for (int k = nq - 1; k >= 0; --k)
    for (int c = 0; c < D; ++c) {
      const double t = inv[qi[k]][c];
      inv[qi[k]][c] = inv[qp[k]][c];
      inv[qp[k]][c] = t;
    }
  return true;
}

// nalgebra QR::new (Householder reflections: householder.rs
// clear_column_unchecked, reflection_axis_mut) + try_inverse (Q^T by the
// stored reflections, then the upper solve on R's diagonal), secant's second
// fallback (src/ivp/bdf.rs:438-440).  False when a diagonal entry of R is 0.
template <int D>
__device__ __noinline__ bool ref_qr_inverse(const double (&A)[D][D], double (&inv)[D][D]) {
  using Op = ExactOps;
  double a[D][D], diag[D];
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) a[r][c] = A[r][c];
  for (int i = 0; i < D; ++i) {
    const double sq = Op::add(0.0, ref_dotx_col(a, i, a, i, i));
    const double nrm = Op::sqrt(sq);
    const double x0 = a[i][i];
    const double modulus = (x0 >= 0.0) ? x0 : -x0;
    const double sgn = (x0 >= 0.0) ? 1.0 : -1.0;
    const double signed_norm = Op::mul(sgn, nrm);
    const double factor = Op::mul(Op::add(sq, Op::mul(modulus, nrm)), 2.0);
    a[i][i] = Op::add(a[i][i], signed_norm);
    if (factor != 0.0) {
      const double sf = Op::sqrt(factor);
      for (int r = i; r < D; ++r) a[r][i] = Op::div(a[r][i], sf);
      diag[i] = -signed_norm;
      const double sign = rs_signum(diag[i]);
      const double m_two = Op::mul(sign, -2.0);
      for (int c = i + 1; c < D; ++c) {
        const double f = Op::mul(Op::sub(ref_dotx_col(a, i, a, c, i), 0.0), m_two);
        for (int r = i; r < D; ++r) a[r][c] = Op::add(Op::mul(f, a[r][i]), Op::mul(sign, a[r][c]));
      }
    } else {
      diag[i] = signed_norm;
    }
  }
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) inv[r][c] = (r == c) ? 1.0 : 0.0;
  for (int i = 0; i < D; ++i) {
    const double sign = rs_signum(diag[i]);
    const double m_two = Op::mul(sign, -2.0);
    for (int c = 0; c < D; ++c) {
      const double f = Op::mul(Op::sub(ref_dotx_col(a, i, inv, c, i), 0.0), m_two);
      for (int r = i; r < D; ++r) inv[r][c] = Op::add(Op::mul(f, a[r][i]), Op::mul(sign, inv[r][c]));
    }
  }
  for (int k = 0; k < D; ++k)
    for (int i = D - 1; i >= 0; --i) {
      if (diag[i] == 0.0) return false;
      const double coeff = Op::div(inv[i][k], diag[i]);
      inv[i][k] = coeff;
      const double mc = -coeff;
      for (int r = 0; r < i; ++r) inv[r][k] = Op::add(Op::mul(mc, a[r][i]), inv[r][k]);
    }
  return true;
}

// nalgebra LU::new + try_inverse (partial pivoting, first maximum).
template <int D>
__device__ bool ref_lu_inverse(const double (&A)[D][D], double (&inv)[D][D]) {
  using Op = ExactOps;
  double a[D][D];
  int pi[D], pp[D], np = 0;
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) a[r][c] = A[r][c];
  for (int i = 0; i < D; ++i) {
    int piv = i;
    double best = fabs(a[i][i]);
    for (int r = i + 1; r < D; ++r)
      if (fabs(a[r][i]) > best) {
        best = fabs(a[r][i]);
        piv = r;
      }
    const double diag = a[piv][i];
    if (diag == 0.0) continue;
    if (piv != i) {
      pi[np] = i;
      pp[np] = piv;
      ++np;
      for (int c = 0; c < D; ++c) {
        const double t = a[i][c];
        a[i][c] = a[piv][c];
        a[piv][c] = t;
      }
    }
    const double inv_diag = Op::div(1.0, diag);
    for (int r = i + 1; r < D; ++r) a[r][i] = Op::mul(a[r][i], inv_diag);
    for (int c = i + 1; c < D; ++c) {
      const double alpha = -a[i][c];
      for (int r = i + 1; r < D; ++r) a[r][c] = Op::add(Op::mul(alpha, a[r][i]), a[r][c]);
    }
  }
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) inv[r][c] = (r == c) ? 1.0 : 0.0;
  for (int k = 0; k < np; ++k)
    for (int c = 0; c < D; ++c) {
      const double t = inv[pi[k]][c];
      inv[pi[k]][c] = inv[pp[k]][c];
      inv[pp[k]][c] = t;
    }
  for (int k = 0; k < D; ++k)
    for (int i = 0; i < D - 1; ++i) {
      const double mc = -Op::div(inv[i][k], 1.0);
      for (int r = i + 1; r < D; ++r) inv[r][k] = Op::add(Op::mul(mc, a[r][i]), inv[r][k]);
    }
  for (int k = 0; k < D; ++k)
    for (int i = D - 1; i >= 0; --i) {
      const double diag = a[i][i];
      if (diag == 0.0) return false;
      const double coeff = Op::div(inv[i][k], diag);
      inv[i][k] = coeff;
      const double mc = -coeff;
      for (int r = 0; r < i; ++r) inv[r][k] = Op::add(Op::mul(mc, a[r][i]), inv[r][k]);
    }
  return true;
}

// nalgebra gemv: y = v_0 M[:,0], then y = (v_j M[:,j]) + y.
template <int D>
__device__ __forceinline__ void ref_gemv(const double (&M)[D][D], const double (&v)[D], double (&y)[D]) {
  using Op = ExactOps;
#pragma unroll
  for (int i = 0; i < D; ++i) y[i] = Op::mul(v[0], M[i][0]);
#pragma unroll
  for (int j = 1; j < D; ++j)
#pragma unroll
    for (int i = 0; i < D; ++i) y[i] = Op::add(Op::mul(v[j], M[i][j]), y[i]);
}

// bdf.rs:414-475.  Returns a status; the root in `result` on success.
template <class Rhs, int O, int D>
__device__ int32_t ref_secant(const BdfRefState<O, D>& s, const double* p, bool lower, int max_iter, bool dyn,
                              double (&result)[D]) {
  using Op = ExactOps;
  double guess[D], deriv[D], above[D], below[D], shift[D];
  double jac[D][D], inv[D][D], minv[D][D];
#pragma unroll
  for (int d = 0; d < D; ++d) guess[d] = s.state[d];
  ref_residual<Rhs>(s, p, lower, guess, deriv);
  const double denom = Op::div(1.0, Op::mul(2.0, s.dt));
  for (int c = 0; c < D; ++c) {
    double gc = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d)
      if (d == c) gc = guess[d];
    gc = Op::add(gc, s.dt);
#pragma unroll
    for (int d = 0; d < D; ++d)
      if (d == c) guess[d] = gc;
    ref_residual<Rhs>(s, p, lower, guess, above);
    gc = Op::sub(gc, Op::mul(2.0, s.dt));
#pragma unroll
    for (int d = 0; d < D; ++d)
      if (d == c) guess[d] = gc;
    ref_residual<Rhs>(s, p, lower, guess, below);
    gc = Op::add(gc, s.dt);
#pragma unroll
    for (int d = 0; d < D; ++d)
      if (d == c) guess[d] = gc;
    for (int r = 0; r < D; ++r) jac[r][c] = Op::mul(Op::add(above[r], below[r]), denom);
  }
  // lu().try_inverse(), else full_piv_lu().try_inverse(), else
  // qr().try_inverse(), else SingularMatrix (src/ivp/bdf.rs:429-443)
  if (!ref_lu_inverse(jac, inv) && !ref_full_piv_lu_inverse(jac, inv) && !ref_qr_inverse(jac, inv))
    return kStSingular;
  for (int r = 0; r < D; ++r)
    for (int c = 0; c < D; ++c) minv[r][c] = -inv[r][c];
  ref_gemv(minv, deriv, shift);
#pragma unroll
  for (int d = 0; d < D; ++d) guess[d] = Op::add(guess[d], shift[d]);
  for (int it = 2; it < max_iter; ++it) {
    double dlast[D], diff[D], adj[D], u[D], w[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dlast[d] = deriv[d];
    ref_residual<Rhs>(s, p, lower, guess, deriv);
#pragma unroll
    for (int d = 0; d < D; ++d) diff[d] = Op::sub(deriv[d], dlast[d]);
    ref_gemv(minv, diff, adj);
    double pp = Op::mul(adj[0], -shift[0]);
#pragma unroll
    for (int j = 1; j < D; ++j) pp = Op::add(Op::mul(adj[j], -shift[j]), pp);
    for (int c = 0; c < D; ++c) {
      double acc = Op::mul(inv[0][c], shift[0]);
      for (int j = 1; j < D; ++j) acc = Op::add(Op::mul(inv[j][c], shift[j]), acc);
      u[c] = acc;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) w[d] = Op::add(shift[d], adj[d]);
    for (int r = 0; r < D; ++r)
      for (int c = 0; c < D; ++c) {
        inv[r][c] = Op::add(inv[r][c], Op::div(Op::mul(u[c], w[r]), pp));
        minv[r][c] = -inv[r][c];
      }
    ref_gemv(minv, deriv, shift);
#pragma unroll
    for (int d = 0; d < D; ++d) guess[d] = Op::add(guess[d], shift[d]);
    if (bdf_norm(shift, dyn) <= s.tol) {
#pragma unroll
      for (int d = 0; d < D; ++d) result[d] = guess[d];
      return kStOk;
    }
  }
  return kStMaxIter;
}

enum : int { kRefItem = 0, kRefRedo = 1, kRefDone = 2, kRefFail = 3 };

template <class Rhs, int O, int D>
__device__ int ref_step(BdfRefState<O, D>& s, const double* p, int max_iter, bool dyn, double& it_t,
                        double (&it_y)[D], int32_t& fail) {
  using Op = ExactOps;
  if (s.ym > 0 && s.ym <= O) {
    const int get = O - s.ym;
    s.ym -= 1;
    if (s.ym == 0) s.ym = O + 2;
    const int k = ref_idx(s, get);
    it_t = s.ht[k];
#pragma unroll
    for (int d = 0; d < D; ++d) it_y[d] = s.hy[k][d];
    return kRefItem;
  }
  if (s.ym == O + 2) {
    s.ym = 0;
    if (!ref_push(s, s.time, s.state)) {
      fail = kStMaxAttempts;
      return kRefFail;
    }
    s.hfront = (s.hfront + 1) % BdfRefState<O, D>::kHist;
    s.hlen--;
    it_t = s.time;
#pragma unroll
    for (int d = 0; d < D; ++d) it_y[d] = s.state[d];
    return kRefItem;
  }
  if (s.time >= s.end) return kRefDone;
  if (Op::add(s.time, s.dt) >= s.end) {
    s.dt = Op::sub(s.end, s.time);
    if (!ref_rk4<Rhs>(s, p, 1)) {
      fail = kStMaxAttempts;
      return kRefFail;
    }
    const int k = ref_idx(s, s.hlen - 1);
    it_t = s.time;
#pragma unroll
    for (int d = 0; d < D; ++d) it_y[d] = s.hy[k][d];
    return kRefItem;
  }
  if (s.hlen == 0) {
#pragma unroll
    for (int d = 0; d < D; ++d) s.save[d] = s.state[d];
    if (Op::add(s.time, Op::mul(s.dt, s.order)) >= s.end) s.dt = Op::div(Op::sub(s.end, s.time), s.order);
    if (!ref_rk4<Rhs>(s, p, O)) {
      fail = kStMaxAttempts;
      return kRefFail;
    }
    s.ym = O + 1;
    return kRefRedo;
  }
  double high[D], low[D], diff[D];
  int32_t st = ref_secant<Rhs>(s, p, false, max_iter, dyn, high);
  if (st != kStOk) {
    fail = st;
    return kRefFail;
  }
  st = ref_secant<Rhs>(s, p, true, max_iter, dyn, low);
  if (st != kStOk) {
    fail = st;
    return kRefFail;
  }
#pragma unroll
  for (int d = 0; d < D; ++d) diff[d] = Op::sub(high[d], low[d]);
  const double error = bdf_norm(diff, dyn);
  if (error <= s.tol) {
#pragma unroll
    for (int d = 0; d < D; ++d) s.state[d] = high[d];
    s.time = Op::add(s.time, s.dt);
    if (s.ym == O + 1) {
      s.ym -= 1;
      return kRefRedo;
    }
    if (!ref_push(s, s.time, s.state)) {
      fail = kStMaxAttempts;
      return kRefFail;
    }
    s.hfront = (s.hfront + 1) % BdfRefState<O, D>::kHist;
    s.hlen--;
    if (error < Op::mul(0.1, s.tol)) {
      s.dt = Op::mul(s.dt, 2.0);
      if (s.dt > s.dt_max) s.dt = s.dt_max;
      s.hlen = 0;
      s.hfront = 0;
    }
    it_t = s.time;
#pragma unroll
    for (int d = 0; d < D; ++d) it_y[d] = s.state[d];
    return kRefItem;
  }
  if (s.ym == O + 1) {
    s.time = Op::sub(s.time, Op::sub(s.dt, s.order));
#pragma unroll
    for (int d = 0; d < D; ++d) s.state[d] = s.save[d];
  }
  s.dt = Op::mul(s.dt, 0.5);
  if (s.dt < s.dt_min) {
    fail = kStMinDt;
    return kRefFail;
  }
  s.hlen = 0;
  s.hfront = 0;
  return kRefRedo;
}

template <class Rhs, int O>
__global__ void __launch_bounds__(128) bdf_as_compiled_kernel(const BdfArgs a, int dyn_dim) {
  using Op = ExactOps;
  constexpr int D = Rhs::DIM;
  constexpr int P = Rhs::NP > 0 ? Rhs::NP : 1;
  const int64_t n = a.n;
  const bool dyn = dyn_dim != 0;
  const unsigned lane = threadIdx.x & 31u;
  for (;;) {
    unsigned long long ticket = 0;
    const unsigned mask = __activemask();
    const int leader = __ffs(mask) - 1;
    if (static_cast<int>(lane) == leader) ticket = atomicAdd(a.queue, static_cast<unsigned long long>(__popc(mask)));
    ticket = __shfl_sync(mask, ticket, leader) + __popc(mask & ((1u << lane) - 1u));
    const int64_t idx = static_cast<int64_t>(ticket);
    if (idx >= n) break;

    double p[P];
#pragma unroll
    for (int k = 0; k < Rhs::NP; ++k) p[k] = a.params[k * n + idx];
    BdfRefState<O, D> s;
    if (O == 7) {
      const double h[7] = {60.0 / 147.0, -360.0 / 147.0, 450.0 / 147.0, -400.0 / 147.0,
                           225.0 / 147.0, -72.0 / 147.0, 10.0 / 147.0};
      const double l[7] = {60.0 / 137.0, -300.0 / 137.0, 300.0 / 137.0, -200.0 / 137.0,
                           75.0 / 137.0, -12.0 / 137.0, 0.0};
#pragma unroll
      for (int i = 0; i < O; ++i) {
        s.hc[i] = h[i % 7];
        s.lc[i] = l[i % 7];
      }
    } else {
      const double h[3] = {2.0 / 3.0, -4.0 / 3.0, 1.0 / 3.0};
      const double l[3] = {1.0, -1.0, 0.0};
#pragma unroll
      for (int i = 0; i < O; ++i) {
        s.hc[i] = h[i % 3];
        s.lc[i] = l[i % 3];
      }
    }
    s.dt_max = a.dt_max;
    s.dt_min = a.dt_min < a.dt_max ? a.dt_min : a.dt_max;
    s.time = a.t0 ? a.t0[idx] : a.t0_s;
    s.end = a.t_end ? a.t_end[idx] : a.t_end_s;
    s.tol = a.tol;
    s.dt = Op::mul(Op::add(s.dt_max, s.dt_min), 0.5);
    s.order = static_cast<double>(O);
    s.hfront = 0;
    s.hlen = 0;
    s.ym = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) s.state[d] = a.y0[d * n + idx];
    double last_t = s.time, last_y[D];
#pragma unroll
    for (int d = 0; d < D; ++d) last_y[d] = s.state[d];
    int32_t acc = 0, rej = 0, status = kStOk;
    int64_t calls = 0;
    if (s.time >= s.end) status = kStTimeEndOob;
    while (status == kStOk) {
      if (calls >= a.max_steps) {
        status = kStMaxAttempts;
        break;
      }
      ++calls;
      int32_t fail = kStOk;
      double it_t, it_y[D];
      const int r = ref_step<Rhs>(s, p, a.max_iter, dyn, it_t, it_y, fail);
      if (r == kRefDone) break;
      if (r == kRefFail) {
        status = fail;
        break;
      }
      if (r == kRefRedo) {
        ++rej;
        continue;
      }
      if (a.traj_t != nullptr) {
        const int64_t slot = traj_slot(a.traj_off, a.traj_cap, idx, acc);
        if (slot < 0) {
          status = kStCapacity;  // the trajectory buffer is full: the item is not yielded
          break;
        }
        a.traj_t[slot] = it_t;
#pragma unroll
        for (int d = 0; d < D; ++d) a.traj_y[slot * D + d] = it_y[d];
      }
      ++acc;
      last_t = it_t;
#pragma unroll
      for (int d = 0; d < D; ++d) last_y[d] = it_y[d];
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

}  // namespace bacon
