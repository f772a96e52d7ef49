// Plain GPU baseline: one launch per attempt.
//
// This is the straightforward port of RungeKuttaSolver::step
// (src/ivp/rk.rs:361-423) to one thread per system: the solver state (y, the
// stage matrix K, t, dt, end, counters) lives in HBM between launches, the
// dense S x S tableau (zeros included) is read from constant memory, and the
// host relaunches until no system is still running.  It performs the same
// rounded operations as the persistent kernel in exact mode, so the two give
// bit-identical results; it exists as the baseline the persistent engine is
// measured against.
#include <cstdint>

#include "plain.h"
#include "rhs.cuh"
#include "tableau.cuh"

namespace bacon {

__constant__ double c_plain_m[6][6];
__constant__ double c_plain_c[6];
__constant__ double c_plain_b[6];
__constant__ double c_plain_e[6];

template <class Rhs>
__global__ void __launch_bounds__(256) rk_plain_step_kernel(PlainArgs a) {
  constexpr int D = Rhs::DIM;
  constexpr int P = Rhs::NP > 0 ? Rhs::NP : 1;
  using Ops = ExactOps;
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  if (a.status[i] != kPlainRunning) return;
  const int64_t n = a.n;
  const int S = a.stages;
  double t = a.t[i], dt = a.dt[i];
  const double end = a.end[i];
  int32_t st = kPlainRunning;

  if (t >= end) {
    st = 0;  // Done (rk.rs:362-364)
  } else if (a.attempts[i] >= a.max_attempts) {
    st = 13;
  } else {
    a.attempts[i] += 1;
    double y[D], p[P];
    for (int d = 0; d < D; ++d) y[d] = a.y[d * n + i];
    for (int k = 0; k < Rhs::NP; ++k) p[k] = a.params[k * n + i];
    if (Ops::add(t, dt) >= end) dt = Ops::sub(end, t);
    for (int s = 0; s < S; ++s) {
      double sc[D];
      for (int d = 0; d < D; ++d) sc[d] = y[d];
      for (int j = 0; j < S; ++j)
        for (int d = 0; d < D; ++d)
          sc[d] = Ops::add(sc[d], Ops::mul(a.K[(j * D + d) * n + i], c_plain_m[s][j]));
      const double stime = Ops::add(t, Ops::mul(c_plain_c[s], dt));
      double fv[D];
      Rhs::template eval<Ops>(stime, sc, p, fv);
      for (int d = 0; d < D; ++d) a.K[(s * D + d) * n + i] = Ops::mul(fv[d], dt);
    }
    double ev[D];
    for (int d = 0; d < D; ++d) ev[d] = Ops::mul(a.K[(0 * D + d) * n + i], c_plain_e[0]);
    for (int j = 1; j < S; ++j)
      for (int d = 0; d < D; ++d)
        ev[d] = Ops::add(ev[d], Ops::mul(a.K[(j * D + d) * n + i], c_plain_e[j]));
    double ss;
    if (D == 2) ss = Ops::add(Ops::mul(ev[0], ev[0]), Ops::mul(ev[1], ev[1]));
    else if (D == 3)
      ss = Ops::add(Ops::add(Ops::mul(ev[0], ev[0]), Ops::mul(ev[1], ev[1])),
                    Ops::mul(ev[D - 1], ev[D - 1]));
    else ss = Ops::mul(ev[0], ev[0]);
    const double err = Ops::div(Ops::sqrt(ss), dt);
    const bool ok = err <= a.tol;
    double tn = t, yn[D];
    for (int d = 0; d < D; ++d) yn[d] = y[d];
    if (ok) {
      tn = Ops::add(t, dt);
      for (int j = 0; j < S; ++j)
        for (int d = 0; d < D; ++d)
          yn[d] = Ops::add(yn[d], Ops::mul(a.K[(j * D + d) * n + i], c_plain_b[j]));
    }
    const double delta = qrt(Ops::div(a.tol, err));
    if (delta <= 0.1) dt = Ops::mul(dt, 0.1);
    else if (delta >= 4.0) dt = Ops::mul(dt, 4.0);
    else dt = Ops::mul(dt, delta);
    if (dt > a.dt_max) dt = a.dt_max;
    if (dt < a.dt_min && (ok ? tn : t) < end) {
      st = 8;
    } else if (ok) {
      t = tn;
      for (int d = 0; d < D; ++d) a.y[d * n + i] = yn[d];
      a.accepted[i] += 1;
    } else {
      a.rejected[i] += 1;
    }
    a.t[i] = t;
    a.dt[i] = dt;
  }
  if (st != kPlainRunning) {
    a.status[i] = st;
  } else {
    atomicAdd(a.live, 1u);
  }
}

template <class Lit, int L>
static void fill_tables(PlainTables& tb) {
  using T = Tableau<Lit, L>;
  tb.stages = T::S;
  for (int i = 0; i < 6; ++i) {
    tb.c[i] = i < T::S ? T::c(i) : 0.0;
    tb.b[i] = i < T::S ? T::b(i) : 0.0;
    tb.e[i] = i < T::S ? T::e(i) : 0.0;
    for (int j = 0; j < 6; ++j) tb.m[i][j] = (i < T::S && j < T::S) ? T::M(i, j) : 0.0;
  }
}

bool plain_tables(int method, int layout, PlainTables& tb) {
  if (method == 0) {
    if (layout == 0) fill_tables<Rkf45Literal, kAsCompiled>(tb);
    else if (layout == 1) fill_tables<Rkf45Literal, kAsWritten>(tb);
    else fill_tables<Rkf45Literal, kFehlberg>(tb);
  } else {
    if (layout == 0) fill_tables<Bs23Literal, kAsCompiled>(tb);
    else fill_tables<Bs23Literal, kAsWritten>(tb);
  }
  return true;
}

cudaError_t plain_upload_tables(const PlainTables& tb, cudaStream_t s) {
  cudaError_t e = cudaMemcpyToSymbolAsync(c_plain_m, tb.m, sizeof(tb.m), 0, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_plain_c, tb.c, sizeof(tb.c), 0, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_plain_b, tb.b, sizeof(tb.b), 0, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_plain_e, tb.e, sizeof(tb.e), 0, cudaMemcpyHostToDevice, s);
  return e;
}

const void* plain_kernel(int rhs, int dim) {
  switch (rhs) {
    case kRhsExp: return dim == 1 ? (const void*)&rk_plain_step_kernel<RhsExp<1>> : dim == 2 ? (const void*)&rk_plain_step_kernel<RhsExp<2>> : nullptr;
    case kRhsDecay: return dim == 1 ? (const void*)&rk_plain_step_kernel<RhsDecay<1>> : dim == 2 ? (const void*)&rk_plain_step_kernel<RhsDecay<2>> : nullptr;
    case kRhsQuadratic: return dim == 1 ? (const void*)&rk_plain_step_kernel<RhsQuadratic<1>> : nullptr;
    case kRhsSine: return dim == 1 ? (const void*)&rk_plain_step_kernel<RhsSine<1>> : dim == 2 ? (const void*)&rk_plain_step_kernel<RhsSine<2>> : nullptr;
    case kRhsHarmonic: return dim == 2 ? (const void*)&rk_plain_step_kernel<RhsHarmonic> : nullptr;
    case kRhsVdp: return dim == 2 ? (const void*)&rk_plain_step_kernel<RhsVdp> : nullptr;
    case kRhsLorenz: return dim == 3 ? (const void*)&rk_plain_step_kernel<RhsLorenz> : nullptr;
    case kRhsLotka: return dim == 2 ? (const void*)&rk_plain_step_kernel<RhsLotka> : nullptr;
    case kRhsRobertson: return dim == 3 ? (const void*)&rk_plain_step_kernel<RhsRobertson> : nullptr;
    default: return nullptr;
  }
}

}  // namespace bacon

namespace bacon {

// Solver construction for every system (rk.rs:249-343): y = y0, K = 0,
// dt = (dt_max + dt_min) / 2, and the builder's end <= start rejection.
__global__ void rk_plain_init_kernel(PlainInitArgs a) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int64_t n = a.n;
  for (int d = 0; d < a.dim; ++d) a.st.y[d * n + i] = a.y0[d * n + i];
  for (int k = 0; k < a.stages * a.dim; ++k) a.st.K[k * n + i] = 0.0;
  const double t0 = a.t0 ? a.t0[i] : a.t0_s;
  const double te = a.t_end ? a.t_end[i] : a.t_end_s;
  a.st.t[i] = t0;
  a.st.end[i] = te;
  a.st.dt[i] = a.dt0;
  a.st.attempts[i] = 0;
  a.st.accepted[i] = 0;
  a.st.rejected[i] = 0;
  a.st.status[i] = (t0 >= te) ? 5 : kPlainRunning;
}

const void* plain_init_kernel() { return reinterpret_cast<const void*>(&rk_plain_init_kernel); }

}  // namespace bacon
