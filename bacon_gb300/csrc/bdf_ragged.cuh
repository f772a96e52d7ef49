// Corrected BDF for batches whose systems differ in size: one warp per system.
//
// A damped spring-mass chain of N_i masses (dim 2 N_i, up to 128) is too big
// for one thread's registers, so one warp owns one system: lane l owns rows
// l, l+32, l+64, l+96 of every vector.  Everything the warp touches in its
// inner loops lives in its slice of shared memory: the LU factors of
// M = I - h b_q J in use (column-major, so lane r reads row r of a column
// without bank conflicts), their row permutation, the history H[0..6], the
// interpolated history HH, a staging vector and the parameters.
//
// Factors are costly to recompute (2/3 dim^3 flops) and the chain Jacobian is
// constant, so M depends on h b_q alone.  A solve meets ~100 distinct values
// of h b_q (h moves by factors of 2, q ramps 1..6 after every doubling) and
// revisits them constantly (orders q and q-1 alternate within every step).
// Each warp therefore keeps a 16-entry least-recently-used cache of factor
// sets in device memory, keyed by the bits of h b_q: a hit copies the factors
// into shared memory, a miss factors in shared memory and writes them back.
// Reusing a factorisation of the same matrix is bit-identical to redoing it.
//
// Occupancy follows size.  GB300 issues one FP64 warp instruction every 16
// cycles per SM, so one warp with four independent row updates per pivot
// keeps the FP64 pipe busy at dim 128, while small systems need many warps to
// cover shuffle and shared-memory latency.  A CTA of 8 warps and ~206 KB of
// shared memory runs four phases, one per size class (dim <= 128, 96, 64, 32),
// with 1, 2, 5 and 8 warps working; each class has its own work counter and
// largest-first order, and a CTA moves to the next class when the counter of
// the current one runs out.  The uniform part of a mixed batch (one thread per
// system) runs after the last phase on all 8 warps.
//
// Every floating-point operation is the one-thread corrected BDF's
// (bdf_corrected_system, and the CPU oracle's bdf_corrected) on the same
// operands in the same order, so the results are bit-identical to them:
//   - partial-pivot LU: pivot = first row of maximum |M[r][i]| (a warp
//     arg-max with lowest-index ties), whole-row swaps, l = M[r][i] * (1 /
//     M[i][i]), M[r][k] -= l M[i][k] row by row and pivot by pivot;
//   - substitutions: row r receives its updates in pivot order, the back
//     substitution multiplies by the pivot reciprocals the elimination
//     formed (no division on its critical path); the permutation is applied
//     as one gather (it only moves values);
//   - the Newton step norm and the error norm only feed comparisons with
//     thresholds: a warp tree sum decides them unless it lies within 1e-10
//     of a threshold, where the oracle's ordered sum on one lane decides.
#pragma once

#include <type_traits>

#include "bdf_kernel.cuh"

namespace bacon {

constexpr int kRagMaxDim = 128;
constexpr int kRagChunks = kRagMaxDim / 32;  // rows per lane
constexpr int kRagWarps = 8;                 // warps per CTA
constexpr int kRagClasses = 4;
constexpr int kRagCacheSlots = 16;

// Size classes: the largest dim of the class and the warps of its phase.
__host__ __device__ constexpr int rag_class_dim(int c) { return c == 0 ? 128 : c == 1 ? 96 : c == 2 ? 64 : 32; }
__host__ __device__ constexpr int rag_class_warps(int c) { return c == 0 ? 1 : c == 1 ? 2 : c == 2 ? 5 : 8; }
__host__ __device__ constexpr int rag_class_of(int dim) { return dim > 96 ? 0 : dim > 64 ? 1 : dim > 32 ? 2 : 3; }
// The largest dim warp w of a CTA ever works on (the first class it joins).
__host__ __device__ constexpr int rag_warp_max_dim(int w) { return w == 0 ? 128 : w == 1 ? 96 : w < 5 ? 64 : 32; }

// One warp's shared-memory slice for systems of dim <= ld, in doubles:
// factors ld*ld, pivot reciprocals ld, H 7*ld, HH 7*ld, staging ld, params
// ld/2+2, permutation ld/2 (ld ints), cache table 48 (16 keys, 16 stamps,
// 16 states).
struct RagSmem {
  __host__ __device__ static constexpr int M(int) { return 0; }
  __host__ __device__ static constexpr int rinv(int ld) { return ld * ld; }
  __host__ __device__ static constexpr int H(int ld) { return ld * ld + ld; }
  __host__ __device__ static constexpr int HH(int ld) { return ld * ld + 8 * ld; }
  __host__ __device__ static constexpr int sv(int ld) { return ld * ld + 15 * ld; }
  __host__ __device__ static constexpr int sp(int ld) { return ld * ld + 16 * ld; }
  __host__ __device__ static constexpr int perm(int ld) { return ld * ld + 16 * ld + ld / 2 + 2; }
  __host__ __device__ static constexpr int table(int ld) { return perm(ld) + ld / 2; }
  __host__ __device__ static constexpr int doubles(int ld) { return table(ld) + 48; }
};

// Shared memory of a CTA for the classes present (bit c of mask = class c).
__host__ __device__ constexpr size_t rag_cta_smem_bytes(unsigned mask) {
  size_t b = 0;
  for (int c = 0; c < kRagClasses; ++c)
    if (mask & (1u << c)) {
      const size_t need = static_cast<size_t>(rag_class_warps(c)) * RagSmem::doubles(rag_class_dim(c)) * 8;
      if (need > b) b = need;
    }
  return b;
}

// Device-memory factor cache of warp w: 16 slots of ld*ld factors, ld pivot
// reciprocals and ld permutation ints, ld = rag_warp_max_dim(w); a CTA's
// warps are laid out back to back.
__host__ __device__ constexpr size_t rag_gslot_doubles(int ld) { return static_cast<size_t>(ld) * ld + ld + ld / 2; }
__host__ __device__ constexpr size_t rag_gcache_warp_doubles(int w) {
  return kRagCacheSlots * rag_gslot_doubles(rag_warp_max_dim(w));
}
__host__ __device__ constexpr size_t rag_gcache_cta_doubles() {
  size_t s = 0;
  for (int w = 0; w < kRagWarps; ++w) s += rag_gcache_warp_doubles(w);
  return s;
}
__host__ __device__ constexpr size_t rag_gcache_warp_offset(int w) {
  size_t s = 0;
  for (int i = 0; i < w; ++i) s += rag_gcache_warp_doubles(i);
  return s;
}

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
  const uint32_t* order;       // systems grouped by size class, largest first within a class
  int64_t class_start[kRagClasses];
  int64_t class_n[kRagClasses];
  double* gcache;              // per CTA rag_gcache_cta_doubles()
  unsigned long long* queues;  // [kRagClasses] work counters, zero at launch
  unsigned long long* first_fail;
};

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

// M = I - hb J, then the partial-pivot LU in place (shared memory);
// perm[pos] = the original row now at pos, rinv[i] = 1 / U[i][i] (the
// elimination's own reciprocal, used again by the back substitution).
// Returns false on an exactly zero pivot.
__device__ __forceinline__ bool rag_factor(int lane, int D, int N, const double* sp, double hb, double* M,
                                           double* rinv, int32_t* perm) {
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
    if (lane == 0) rinv[i] = inv;
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

// Warp copy of n doubles (n even; both pointers 16-byte aligned).
__device__ __forceinline__ void rag_copy(int lane, double* dst, const double* src, int n) {
  const double2* s = reinterpret_cast<const double2*>(src);
  double2* d = reinterpret_cast<double2*>(dst);
  const int n2 = n / 2;
  int i = lane;
  for (; i + 96 < n2; i += 128) {
    const double2 a = s[i], b = s[i + 32], c = s[i + 64], e = s[i + 96];
    d[i] = a;
    d[i + 32] = b;
    d[i + 64] = c;
    d[i + 96] = e;
  }
  for (; i < n2; i += 32) d[i] = s[i];
}

// The factor cache of one warp: shared-memory table of 16 (key, stamp,
// state) entries for the device-memory slots, plus the key and state of the
// factors currently in shared memory.
struct RagCache {
  long long cur_key;
  int cur_state;  // 0 none, 1 factored, 2 singular
  int clock;
};

// Makes the factors of M(hb) current in shared memory; returns 1 (factored)
// or 2 (singular).
__device__ __forceinline__ int rag_get_factors(int lane, int D, int N, const double* sp, double hb, double* sM,
                                               double* srinv, int32_t* sperm, double* table, double* gcache,
                                               int gld, RagCache& cache) {
  const long long key = __double_as_longlong(hb);
  if (cache.cur_state != 0 && cache.cur_key == key) return cache.cur_state;
  long long* keys = reinterpret_cast<long long*>(table);
  int* stamps = reinterpret_cast<int*>(table + 16);
  int* states = stamps + 16;
  ++cache.clock;
  int hit = -1;
  for (int s = 0; s < kRagCacheSlots; ++s)
    if (states[s] != 0 && keys[s] == key) hit = s;
  const size_t slot_doubles = rag_gslot_doubles(gld);
  if (hit >= 0) {
    const int st = states[hit];
    if (st == 1) {
      const double* g = gcache + hit * slot_doubles;
      rag_copy(lane, sM, g, D * D);
      rag_copy(lane, srinv, g + static_cast<size_t>(gld) * gld, D);
      const int32_t* gp = reinterpret_cast<const int32_t*>(g + static_cast<size_t>(gld) * gld + gld);
      for (int r = lane; r < D; r += 32) sperm[r] = gp[r];
    }
    __syncwarp();
    if (lane == 0) stamps[hit] = cache.clock;
    __syncwarp();
    cache.cur_key = key;
    cache.cur_state = st;
    return st;
  }
  // miss: the first empty slot, else the least recently used one
  int victim = -1;
  for (int s = 0; s < kRagCacheSlots && victim < 0; ++s)
    if (states[s] == 0) victim = s;
  if (victim < 0) {
    victim = 0;
    for (int s = 1; s < kRagCacheSlots; ++s)
      if (stamps[s] < stamps[victim]) victim = s;
  }
  const int st = rag_factor(lane, D, N, sp, hb, sM, srinv, sperm) ? 1 : 2;
  __syncwarp();
  if (st == 1) {
    double* g = gcache + victim * slot_doubles;
    rag_copy(lane, g, sM, D * D);
    rag_copy(lane, g + static_cast<size_t>(gld) * gld, srinv, D);
    int32_t* gp = reinterpret_cast<int32_t*>(g + static_cast<size_t>(gld) * gld + gld);
    for (int r = lane; r < D; r += 32) gp[r] = sperm[r];
  }
  if (lane == 0) {
    keys[victim] = key;
    stamps[victim] = cache.clock;
    states[victim] = st;
  }
  __syncwarp();
  cache.cur_key = key;
  cache.cur_state = st;
  return st;
}

// Newton solve of y - hb f(y) + sum_j a_{q,j} HH[j-1] = 0 from the guess in
// y (own rows), with the factors of M for hb.
__device__ __forceinline__ bool rag_newton(int lane, int D, int N, const double* sp, double* sv, const double* HH,
                                           int ld, int q, double h, double* sM, double* srinv, int32_t* sperm,
                                           double* table, double* gcache, int gld, RagCache& cache,
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
  if (rag_get_factors(lane, D, N, sp, hb, sM, srinv, sperm, table, gcache, gld, cache) != 1) return false;
  const double* M = sM;
  int32_t src[kRagChunks];
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) {
    const int r = lane + 32 * j;
    src[j] = (r < D) ? sperm[r] : 0;
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
        if (static_cast<int>(lane) == ii) dx[jb] = O::mul(dx[jb], srinv[i]);
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
    // ||dx||^2: the oracle sums it in order on one lane and tests
    // sqrt(dn) <= conv.  A warp tree sum differs from that by ~dim * 2^-53
    // (all terms are non-negative), so it decides alone unless it lies within
    // 1e-10 of conv^2; then the ordered sum decides.  NaN in either exactly
    // when some dx is NaN.
    double part = 0.0;
#pragma unroll
    for (int j = 0; j < kRagChunks; ++j) part = O::add(part, O::mul(dx[j], dx[j]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) part = O::add(part, __shfl_xor_sync(0xffffffffu, part, off));
    if (!(part == part)) return false;
    const double thr = O::mul(conv, conv);
    if (fabs(O::sub(part, thr)) > O::mul(1e-10, thr)) {
      if (part < thr) return true;
      continue;
    }
    double dn = 0.0;
    if (lane == 0)
      for (int d = 0; d < D; ++d) dn = O::add(dn, O::mul(sv[d], sv[d]));
    dn = __shfl_sync(0xffffffffu, dn, 0);
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

// A value that compares with tol and 0.1*tol exactly as rag_norm(sv) does:
// the warp tree-sum norm (within ~dim * 2^-53 of the ordered one) unless it
// lies within 1e-10 of either threshold, else the ordered norm itself.
__device__ __forceinline__ double rag_norm_decide(int lane, int D, const double* sv, double tol) {
  using O = ExactOps;
  double part = 0.0;
#pragma unroll
  for (int j = 0; j < kRagChunks; ++j) {
    const int r = lane + 32 * j;
    if (r < D) part = O::add(part, O::mul(sv[r], sv[r]));
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) part = O::add(part, __shfl_xor_sync(0xffffffffu, part, off));
  const double e = O::sqrt(part);
  if (!(e == e)) return e;
  const double t2 = O::mul(0.1, tol);
  if (fabs(O::sub(e, tol)) > O::mul(1e-10, tol) && fabs(O::sub(e, t2)) > O::mul(1e-10, t2)) return e;
  return rag_norm(lane, D, sv);
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

// One ragged system integrated by the calling warp; ws is its shared-memory
// slice for dims <= ld, gcache its device-memory factor slots of dim <= gld.
__device__ __forceinline__ void rag_solve_system(const RaggedArgs& a, int64_t idx, int lane, double* ws, int ld,
                                                 double* gcache, int gld) {
  using O = ExactOps;
  double* sM = ws + RagSmem::M(ld);
  double* srinv = ws + RagSmem::rinv(ld);
  double* H = ws + RagSmem::H(ld);
  double* HH = ws + RagSmem::HH(ld);
  double* sv = ws + RagSmem::sv(ld);
  double* sp = ws + RagSmem::sp(ld);
  int32_t* sperm = reinterpret_cast<int32_t*>(ws + RagSmem::perm(ld));
  double* table = ws + RagSmem::table(ld);
  const int64_t yo = a.y_off[idx];
  const int D = static_cast<int>(a.y_off[idx + 1] - yo);
  const int N = D / 2;
  const int64_t po = a.p_off[idx];
  __syncwarp();
  for (int k = lane; k <= N; k += 32) sp[k] = a.params[po + k];
  if (lane < 32) reinterpret_cast<int*>(table + 16)[lane] = 0;  // stamps and states of the 16 slots
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
  RagCache cache;
  cache.cur_key = 0;
  cache.cur_state = 0;
  cache.clock = 0;
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
    bool ok = rag_newton(lane, D, N, sp, sv, HHp, ld, q, h, sM, srinv, sperm, table, gcache, gld, cache,
                         a.max_iter, a.tol, yh);
    double error;
    if (ok && q >= 2) {
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) yl[j] = yh[j];
      ok = rag_newton(lane, D, N, sp, sv, HHp, ld, q - 1, h, sM, srinv, sperm, table, gcache, gld, cache,
                      a.max_iter, a.tol, yl);
      __syncwarp();
#pragma unroll
      for (int j = 0; j < kRagChunks; ++j) {
        const int r = lane + 32 * j;
        if (r < D) sv[r] = O::sub(yh[j], yl[j]);
      }
      __syncwarp();
      error = rag_norm_decide(lane, D, sv, a.tol);
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
      error = rag_norm_decide(lane, D, sv, a.tol);
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

// One launch for a stiff batch of two parts: ragged systems (a warp each, in
// four size-class phases) and a uniform batch of small systems (a thread
// each, after the last phase).  Launched with kRagWarps * 32 threads and
// rag_cta_smem_bytes(classes present) of dynamic shared memory.
template <class Small>
__global__ void __launch_bounds__(kRagWarps * 32, 1)
    bdf_mixed_kernel(const BdfArgs small, int small_dyn, const RaggedArgs rg) {
  extern __shared__ __align__(16) double rag_smem[];
  const int warp = static_cast<int>(threadIdx.x >> 5);
  const int lane = static_cast<int>(threadIdx.x & 31u);
  double* gcache = rg.gcache + static_cast<size_t>(blockIdx.x) * rag_gcache_cta_doubles() +
                   rag_gcache_warp_offset(warp);
  for (int c = 0; c < kRagClasses; ++c) {
    if (rg.class_n[c] == 0) continue;
    if (warp < rag_class_warps(c)) {
      const int ld = rag_class_dim(c);
      double* ws = rag_smem + static_cast<size_t>(warp) * RagSmem::doubles(ld);
      for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(rg.queues + c, 1ull);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= static_cast<unsigned long long>(rg.class_n[c])) break;
        const int64_t idx = static_cast<int64_t>(rg.order[rg.class_start[c] + static_cast<int64_t>(item)]);
        rag_solve_system(rg, idx, lane, ws, ld, gcache, rag_warp_max_dim(warp));
      }
    }
    __syncthreads();
  }
  if constexpr (!std::is_same<Small, NoSmall>::value) {
    if (small.n > 0) bdf_corrected_thread_loop<Small>(small, small_dyn != 0);
  }
}

}  // namespace bacon
