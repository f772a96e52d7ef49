// Corrected BDF for batches whose systems differ in size: one warp per system.
//
// A damped spring-mass chain of N_i masses (dim 2 N_i, up to 128) is too big
// for one thread's registers, and its Newton matrix (dim x dim) too big for
// shared memory at useful occupancy.  So one warp owns one system: lane l
// owns rows l, l+32, l+64, l+96 of every vector; the history H[0..6] and the
// interpolated history HH live in the warp's slice of shared memory; the LU
// factors of M = I - h b_q J live in a per-warp workspace in device memory
// (column-major, so a column is one coalesced load).  Every floating-point
// operation is the one-thread corrected BDF's (bdf_corrected_system, and the
// CPU oracle's bdf_corrected) on the same operands in the same order, so the
// results are bit-identical to them:
//   - partial-pivot LU: pivot = first row of maximum |M[r][i]| (a warp
//     arg-max with lowest-index ties), whole-row swaps, l = M[r][i] * (1 /
//     M[i][i]), M[r][k] -= l M[i][k] row by row and pivot by pivot;
//   - substitutions: row r receives its updates in pivot order; the
//     permutation is applied as one gather (it only moves values);
//   - ordered sums (the Newton step norm, the error norm's lanes) run on one
//     lane in the oracle's order.
// The chain Jacobian is constant, so M depends on h b_q alone: the factors of
// the last two values of h b_q are kept (one slot per parity of q, as orders
// q and q-1 alternate within a step), which is bit-identical to refactoring.
#pragma once

#include <type_traits>

#include "bdf_kernel.cuh"

namespace bacon {

constexpr int kRagMaxDim = 128;
constexpr int kRagChunks = kRagMaxDim / 32;  // rows per lane

struct RaggedArgs {
  int64_t n;
  const int64_t* y_off;  // [n+1] system i's state is y0[y_off[i] .. y_off[i+1])
  const int64_t* p_off;  // [n+1] and its parameters params[p_off[i] ..)
  const double* y0;
  const double* params;
  const double* t0;      // [n] or null
  const double* t_end;   // [n] or null
  double t0_s, t_end_s;
  double tol, dt_min, dt_max;
  int64_t max_steps;
  int32_t max_iter;
  int32_t qmax;
  double* y_out;         // [y_off[n]]
  double* t_out;
  int32_t* accepted;
  int32_t* rejected;
  int32_t* status;
  const uint32_t* order;  // work order (largest systems first) or null
  double* lu;             // per warp: 2 slots of ld*ld doubles
  int32_t* perm;          // per warp: 2 slots of ld ints
  int32_t ld;             // largest dim in the batch (<= kRagMaxDim)
  unsigned long long* queue;
  unsigned long long* first_fail;
};

// Doubles of shared memory per warp: H and HH (7 x ld each), one staging
// vector (ld) and the parameters (ld/2 + 1), rounded to an even count.
__host__ __device__ constexpr int rag_smem_doubles(int ld) { return ((15 * ld + ld / 2 + 1) + 1) & ~1; }

// Damped spring-mass chain (unit masses): rows 0..N-1 are x' = v, rows
// N..2N-1 the forces; y and p in shared memory.  Same expressions as RhsChain
// and the oracle's chain right-hand side.
struct RagChain {
  __device__ __forceinline__ static double f(int r, int N, const double* y, const double* p) {
    using O = ExactOps;
    if (r < N) return y[N + r];
    const int i = r - N;
    const double xl = (i == 0) ? 0.0 : y[i - 1];
    const double xr = (i + 1 < N) ? y[i + 1] : 0.0;
    const double kl = p[i];
    const double kr = (i + 1 < N) ? p[i + 1] : 0.0;
    const double force = O::add(O::mul(kl, O::sub(xl, y[i])), O::mul(kr, O::sub(xr, y[i])));
    return O::sub(force, O::mul(p[N], y[N + i]));
  }
  // d f_r / d y_k (the oracle's oracle_rhs_jacobian for the chain).
  __device__ __forceinline__ static double jac(int r, int k, int N, const double* p) {
    using O = ExactOps;
    if (r < N) return (k == N + r) ? 1.0 : 0.0;
    const int i = r - N;
    if (k == i) return -O::add(p[i], (i + 1 < N) ? p[i + 1] : 0.0);
    if (k == i - 1) return p[i];
    if (k == i + 1 && i + 1 < N) return p[i + 1];
    if (k == N + i) return -p[N];
    return 0.0;
  }
};

// Factor slots of one warp: the h*b_q each holds and whether it is usable.
struct RagLuCache {
  double key[2];
  int state[2];  // 0 empty, 1 factored, 2 singular
};

// M = I - hb J, then the partial-pivot LU in place; perm[pos] = the original
// row now at pos.  Returns false on an exactly zero pivot.
__device__ __forceinline__ bool rag_factor(int lane, int D, int N, const double* sp, double hb, double* M,
                                           int32_t* perm) {
  using O = ExactOps;
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      if (r < D) M[k * D + r] = O::sub((r == k) ? 1.0 : 0.0, O::mul(hb, RagChain::jac(r, k, N, sp)));
    }
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) {
    const int r = lane + 32 * j;
    if (r < D) perm[r] = r;
  }
  __syncwarp();
  for (int i = 0; i < D; ++i) {
    double* col = M + i * D;
    const double diag = fabs(col[i]);
    int pr = i;
    if (diag == diag) {
      double bv = diag;
      int br = i;
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        if (r > i && r < D) {
          const double v = fabs(col[r]);
          if (v > bv) {
            bv = v;
            br = r;
          }
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, off);
        const int orr = __shfl_xor_sync(0xffffffffu, br, off);
        if (ov > bv || (ov == bv && orr < br)) {
          bv = ov;
          br = orr;
        }
      }
      pr = br;
    }
    if (pr != i) {
      for (int k = lane; k < D; k += 32) {
        const double a = M[k * D + i];
        M[k * D + i] = M[k * D + pr];
        M[k * D + pr] = a;
      }
      if (lane == 0) {
        const int32_t a = perm[i];
        perm[i] = perm[pr];
        perm[pr] = a;
      }
      __syncwarp();
    }
    const double piv = col[i];
    if (piv == 0.0) return false;
    const double inv = O::div(1.0, piv);
    double l[kRagChunks];
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      l[j] = 0.0;
      if (r > i && r < D) {
        l[j] = O::mul(col[r], inv);
        col[r] = l[j];
      }
    }
    for (int k = i + 1; k < D; ++k) {
      double* ck = M + k * D;
      const double mik = ck[i];
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        if (r > i && r < D) ck[r] = O::sub(ck[r], O::mul(l[j], mik));
      }
    }
    __syncwarp();
  }
  return true;
}

// Newton solve of y - hb f(y) + sum_j a_{q,j} HH[j-1] = 0 from the guess in
// y (own rows), with the factors of M for hb (cached per parity of q).
__device__ __forceinline__ bool rag_newton(int lane, int D, int N, const double* sp, double* sv, const double* HH,
                                           int ld, int q, double h, RagLuCache& cache, double* lu, int32_t* perm,
                                           int max_newton, double tol, double (&y)[kRagChunks]) {
  using O = ExactOps;
  const double hb = O::mul(h, bdf_b(q));
  double c[kRagChunks];
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) c[j] = 0.0;
  for (int jj = 1; jj <= q; ++jj) {
    const double aj = bdf_a(q, jj);
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      if (r < D) c[j] = O::add(c[j], O::mul(aj, HH[(jj - 1) * ld + r]));
    }
  }
  const int slot = q & 1;
  double* M = lu + static_cast<size_t>(slot) * ld * ld;
  int32_t* pm = perm + slot * ld;
  if (cache.state[slot] == 0 || cache.key[slot] != hb) {
    cache.key[slot] = hb;
    cache.state[slot] = rag_factor(lane, D, N, sp, hb, M, pm) ? 1 : 2;
  }
  if (cache.state[slot] != 1) return false;
  int32_t src[kRagChunks];
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) {
    const int r = lane + 32 * j;
    src[j] = (r < D) ? pm[r] : 0;
  }
  const double conv = O::mul(1e-3, tol);
  for (int it = 0; it < max_newton; ++it) {
    __syncwarp();
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      if (r < D) sv[r] = y[j];
    }
    __syncwarp();
    double g[kRagChunks];
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      g[j] = 0.0;
      if (r < D) g[j] = O::add(O::sub(y[j], O::mul(hb, RagChain::f(r, N, sv, sp))), c[j]);
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      if (r < D) sv[r] = g[j];
    }
    __syncwarp();
    double dx[kRagChunks];
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      dx[j] = (r < D) ? -sv[src[j]] : 0.0;
    }
    // forward substitution with the unit lower factor
#pragma unroll
    for (int jb = 0; jb < kRagChunks; ++jb) {
      const int iend = min(32, D - 1 - 32 * jb);
      for (int ii = 0; ii < iend; ++ii) {
        const int i = 32 * jb + ii;
        const double xi = __shfl_sync(0xffffffffu, dx[jb], ii);
        const double* col = M + i * D;
#pragma unroll
        for (int j = jb; j < kRagChunks; ++j) {
          const int r = lane + 32 * j;
          if (r > i && r < D) dx[j] = O::sub(dx[j], O::mul(col[r], xi));
        }
      }
    }
    // back substitution with the upper factor
#pragma unroll
    for (int jb = kRagChunks - 1; jb >= 0; --jb) {
      const int ihi = min(31, D - 1 - 32 * jb);
      for (int ii = ihi; ii >= 0; --ii) {
        const int i = 32 * jb + ii;
        const double* col = M + i * D;
        if (static_cast<int>(lane) == ii) dx[jb] = O::div(dx[jb], col[i]);
        const double xi = __shfl_sync(0xffffffffu, dx[jb], ii);
#pragma unroll
        for (int j = 0; j <= jb; ++j) {
          const int r = lane + 32 * j;
          if (r < i) dx[j] = O::sub(dx[j], O::mul(col[r], xi));
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      if (r < D) {
        y[j] = O::add(y[j], dx[j]);
        sv[r] = dx[j];
      }
    }
    __syncwarp();
    double dn = 0.0;
    if (lane == 0)
      for (int d = 0; d < D; ++d) dn = O::add(dn, O::mul(sv[d], sv[d]));
    dn = __shfl_sync(0xffffffffu, dn, 0);
    if (!(dn == dn)) return false;
    if (O::sqrt(dn) <= conv) return true;
  }
  return false;
}

// Euclidean norm of the vector in sv[0..D) in nalgebra's order for a
// dynamically sized vector (eight partial sums, then the tail), warp-uniform.
__device__ __forceinline__ double rag_norm(int lane, int D, const double* sv) {
  using O = ExactOps;
  double acc = 0.0;
  const int full = D - D % 8;
  if (lane < 8)
    for (int i = 0; i < full; i += 8) acc = O::add(acc, O::mul(sv[i + lane], sv[i + lane]));
  double a[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) a[l] = __shfl_sync(0xffffffffu, acc, l);
  double res = 0.0;
  if (lane == 0) {
    res = O::add(res, O::add(a[0], a[4]));
    res = O::add(res, O::add(a[1], a[5]));
    res = O::add(res, O::add(a[2], a[6]));
    res = O::add(res, O::add(a[3], a[7]));
    for (int k = full; k < D; ++k) res = O::add(res, O::mul(sv[k], sv[k]));
    res = O::sqrt(O::add(0.0, res));
  }
  return __shfl_sync(0xffffffffu, res, 0);
}

// Interpolates the k history rows of this lane onto nodes -s*j (j < k).
__device__ __forceinline__ void rag_interp_rows(int lane, int D, int ld, int k, double s, const double* src,
                                                double* dst) {
  using O = ExactOps;
  double w[7];
  for (int j = 0; j < k; ++j) {
    lagrange_weights(k - 1, O::mul(-s, static_cast<double>(j)), w);
#pragma unroll
    for (int jj = 0; jj < kRagChunks; ++jj) {
      const int r = lane + 32 * jj;
      if (r < D) {
        double acc = 0.0;
        for (int i = 0; i < k; ++i) acc = O::add(acc, O::mul(w[i], src[i * ld + r]));
        dst[j * ld + r] = acc;
      }
    }
  }
}

// One ragged system integrated by the calling warp.
__device__ __forceinline__ void rag_solve_system(const RaggedArgs& a, int64_t item, int lane, double* ws,
                                                 double* lu, int32_t* perm) {
  using O = ExactOps;
  const int ld = a.ld;
  double* H = ws;
  double* HH = ws + 7 * ld;
  double* sv = ws + 14 * ld;
  double* sp = ws + 15 * ld;
  const int64_t idx = a.order ? static_cast<int64_t>(a.order[item]) : item;
  const int64_t yo = a.y_off[idx];
  const int D = static_cast<int>(a.y_off[idx + 1] - yo);
  const int N = D / 2;
  const int64_t po = a.p_off[idx];
  __syncwarp();
  for (int k = lane; k <= N; k += 32) sp[k] = a.params[po + k];
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) {
    const int r = lane + 32 * j;
    if (r < D) H[r] = a.y0[yo + r];
  }
  double ly[kRagChunks];
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) {
    const int r = lane + 32 * j;
    ly[j] = (r < D) ? a.y0[yo + r] : 0.0;
  }
  __syncwarp();
  double dt_min = a.dt_min;
  const double dt_max = a.dt_max;
  if (dt_min > dt_max) dt_min = dt_max;
  const int qmax = a.qmax;
  double t = a.t0 ? a.t0[idx] : a.t0_s;
  const double t_end = a.t_end ? a.t_end[idx] : a.t_end_s;
  double dt = O::mul(O::add(dt_max, dt_min), 0.5);
  int k = 1;
  int32_t acc = 0, rej = 0, status = kStOk;
  double last_t = t;
  RagLuCache cache;
  cache.key[0] = cache.key[1] = 0.0;
  cache.state[0] = cache.state[1] = 0;
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
    const double* HHp = H;
    if (h != dt && k > 1) {
      rag_interp_rows(lane, D, ld, k, O::div(h, dt), H, HH);
      HHp = HH;
    }
    // predictor: extrapolation through the history points
    double w[7];
    lagrange_weights(k - 1, 1.0, w);
    double yh[kRagChunks], yl[kRagChunks];
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) {
      const int r = lane + 32 * j;
      double s = 0.0;
      if (r < D)
        for (int i = 0; i < k; ++i) s = O::add(s, O::mul(w[i], HHp[i * ld + r]));
      yh[j] = s;
    }
    __syncwarp();
    const double t1 = O::add(t, h);
    bool ok = rag_newton(lane, D, N, sp, sv, HHp, ld, q, h, cache, lu, perm, a.max_iter, a.tol, yh);
    double error;
    if (ok && q >= 2) {
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) yl[j] = yh[j];
      ok = rag_newton(lane, D, N, sp, sv, HHp, ld, q - 1, h, cache, lu, perm, a.max_iter, a.tol, yl);
      __syncwarp();
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        if (r < D) sv[r] = O::sub(yh[j], yl[j]);
      }
      __syncwarp();
      error = rag_norm(lane, D, sv);
    } else {
      // order 1: half the gap between backward and forward Euler
      double diff[kRagChunks];
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        diff[j] = 0.0;
        if (r < D) diff[j] = O::mul(0.5, O::sub(yh[j], O::add(H[r], O::mul(h, RagChain::f(r, N, H, sp)))));
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        if (r < D) sv[r] = diff[j];
      }
      __syncwarp();
      error = rag_norm(lane, D, sv);
    }
    if (ok && error <= a.tol) {
      const int kk = (k < 7) ? k + 1 : 7;
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        if (r < D) {
          for (int i = kk - 1; i >= 1; --i) H[i * ld + r] = H[(i - 1) * ld + r];
          H[r] = yh[j];
          ly[j] = yh[j];
        }
      }
      __syncwarp();
      k = kk;
      t = t1;
      ++acc;
      last_t = t;
      if (h != dt) continue;
      if (error < O::mul(0.1, a.tol) && k == qmax + 1 && O::mul(dt, 2.0) <= dt_max) {
        const int nk = (k + 1) / 2;
#pragma unroll
        for (int j = 0; j < kRagChunks; ++j) {
          const int r = lane + 32 * j;
          if (r < D)
            for (int i = 1; i < nk; ++i) H[i * ld + r] = H[2 * i * ld + r];
        }
        __syncwarp();
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
      rag_interp_rows(lane, D, ld, k, 0.5, H, HH);
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        if (r < D)
          for (int i = 0; i < k; ++i) H[i * ld + r] = HH[i * ld + r];
      }
      __syncwarp();
    }
    dt = nd;
  }
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) {
    const int r = lane + 32 * j;
    if (r < D) a.y_out[yo + r] = ly[j];
  }
  if (lane == 0) {
    a.t_out[idx] = last_t;
    a.accepted[idx] = acc;
    a.rejected[idx] = rej;
    a.status[idx] = status;
    if (status != kStOk) atomicMin(a.first_fail, static_cast<unsigned long long>(idx));
  }
  __syncwarp();
}

// Marker for a mixed launch without a uniform (one-thread-per-system) part.
struct NoSmall {};

// One launch for a stiff batch of two parts: ragged systems (a warp each,
// largest first) and a uniform batch of small systems (a thread each).  A
// warp takes ragged systems until none is left, then its threads take small
// systems from the second work counter.
template <class Small>
__global__ void __launch_bounds__(128) bdf_mixed_kernel(const BdfArgs small, int small_dyn, const RaggedArgs rg) {
  extern __shared__ double rag_smem[];
  const int warp = static_cast<int>(threadIdx.x >> 5);
  const int lane = static_cast<int>(threadIdx.x & 31u);
  const int64_t wslot = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + warp;
  if (rg.n > 0) {
    double* ws = rag_smem + static_cast<size_t>(warp) * rag_smem_doubles(rg.ld);
    double* lu = rg.lu + static_cast<size_t>(wslot) * 2 * rg.ld * rg.ld;
    int32_t* perm = rg.perm + static_cast<size_t>(wslot) * 2 * rg.ld;
    for (;;) {
      unsigned long long item = 0;
      if (lane == 0) item = atomicAdd(rg.queue, 1ull);
      item = __shfl_sync(0xffffffffu, item, 0);
      if (item >= static_cast<unsigned long long>(rg.n)) break;
      rag_solve_system(rg, static_cast<int64_t>(item), lane, ws, lu, perm);
    }
  }
  if constexpr (!std::is_same<Small, NoSmall>::value) {
    if (small.n > 0) bdf_corrected_thread_loop<Small>(small, small_dyn != 0);
  }
}

}  // namespace bacon
