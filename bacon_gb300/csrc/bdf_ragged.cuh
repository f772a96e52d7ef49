// Corrected BDF for batches whose systems differ in size: a group of warps
// per system, one row per thread.
//
// A damped spring-mass chain of N_i masses (dim 2 N_i, up to 128) is too big
// for one thread's registers.  A group of G = ceil(dim / 32) warps owns one
// system: thread r of the group owns row r of every vector.  Everything the
// group's inner loops touch lives in its slice of shared memory: the LU
// factors of M = I - h b_q J in use (column-major: a column is one
// conflict-free read across the group), the pivot reciprocals and the row
// permutation, the history H[0..6], the interpolated history HH, a staging
// vector, the parameters and a small exchange area for broadcasts and
// reductions.  The substitutions go by 32-row blocks whose diagonal blocks
// hold their own inverses: the block's warp forms the product of the inverse
// with its complete right-hand side (staged in shared memory; no dependent
// chain over the pivots) and publishes the values in chunks of 8 or 16,
// arriving on a named barrier per chunk without waiting; the warps below wait
// on it and apply each chunk while the block's warp continues, so the next
// block's warp starts its product almost at once.
//
// Factors are costly to recompute (2/3 dim^3 flops) and the chain Jacobian is
// constant, so M depends on h b_q alone.  A solve meets ~100 distinct values
// of h b_q (h moves by factors of 2, q ramps 1..6 after every doubling) and
// revisits them constantly (orders q and q-1 alternate within every step).
// Each group therefore keeps a 16-entry least-recently-used cache of factor
// sets in device memory, keyed by the bits of h b_q: a hit copies the factors
// into shared memory, a miss factors in shared memory and writes them back.
// Reusing a factorisation of the same matrix is bit-identical to redoing it.
//
// A CTA of 8 warps (one per SM: its shared memory fills the SM) runs four
// phases, one per size class: dim <= 128 (one group of 4 warps), <= 96 (two
// groups of 3), <= 64 (four of 2), <= 32 (eight of 1).  Each class has its own
// work counter and largest-first order; a CTA moves to the next class when
// the counter of the current one runs out.  The uniform part of a mixed batch
// (one thread per system) runs after the last phase on all 8 warps.
//
// Every floating-point operation is the one-thread corrected BDF's
// (bdf_corrected_system, and the CPU oracle's bdf_corrected) on the same
// operands in the same order, so the results are bit-identical to them:
//   - partial-pivot LU: pivot = first row of maximum |M[r][i]| (a group
//     arg-max with lowest-index ties), whole-row swaps, l = M[r][i] * (1 /
//     M[i][i]), M[r][k] = fma(-l, M[i][k], M[r][k]) pivot by pivot;
//   - the rows of U are then scaled by the pivot reciprocals the elimination
//     formed (a unit upper factor); the back substitution scales its
//     right-hand side by them once;
//   - each 32x32 diagonal block of L and of the scaled U is replaced by its
//     inverse (column c = the solve of e_c, every update taken for every
//     column in the oracle's order);
//   - substitutions: row r receives the fused updates from the other blocks
//     in pivot order, then the product with its block's inverse accumulates
//     onto it in ascending (L) or descending (U) column order; the
//     permutation is applied as one gather (it only moves values);
//   - the Newton step norm and the error norm only feed comparisons with
//     thresholds: a group tree sum decides them unless it lies within 1e-10
//     of a threshold, where the oracle's ordered sum on one thread decides.
#pragma once

#include <type_traits>

#include "bdf_kernel.cuh"

namespace bacon {

#ifndef BACON_BAR_ARRIVE
#define BACON_BAR_ARRIVE(id, cnt) \
  asm volatile("bar.arrive %0, %1;" ::"r"(static_cast<unsigned>(id)), "r"(static_cast<unsigned>(cnt)) : "memory")
#endif

// Bulk copies into shared memory through the async proxy, tracked on an
// mbarrier.  (A host build of this header for testing supplies its own
// versions by defining BACON_RAG_HOST_SHIMS.)
#ifndef BACON_RAG_HOST_SHIMS
__device__ __forceinline__ uint32_t rag_smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void rag_mbar_init(uint32_t mbar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void rag_mbar_inval(uint32_t mbar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(mbar) : "memory");
}
// Every thread, before the barrier that precedes a bulk copy: orders its
// earlier generic accesses (the factors in shared memory, the cache slots in
// global memory) before the async proxy's.
__device__ __forceinline__ void rag_proxy_fence() { asm volatile("fence.proxy.async;" ::: "memory"); }
// One thread: announce the bytes, start the copies.  Sizes are multiples of
// 16 bytes, addresses 16-byte aligned.
__device__ __forceinline__ void rag_bulk_issue2(uint32_t mbar, void* d0, const void* s0, uint32_t b0, void* d1,
                                                const void* s1, uint32_t b1) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(b0 + b1) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   rag_smem_addr(d0)),
               "l"(s0), "r"(b0), "r"(mbar)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   rag_smem_addr(d1)),
               "l"(s1), "r"(b1), "r"(mbar)
               : "memory");
}
// Waits for the mbarrier phase, for about one second of SM clock at most;
// on expiry raises *err and returns false.
__device__ __forceinline__ bool rag_mbar_wait(uint32_t mbar, uint32_t phase, unsigned int* err) {
  const long long start = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
    if (clock64() - start > 2000000000ll) break;
  }
  atomicExch(err, 1u);
  return false;
}
#endif

constexpr int kRagMaxDim = 128;
constexpr int kRagWarps = 8;  // warps per CTA
constexpr int kRagClasses = 4;
constexpr int kRagCacheSlots = 16;

// Size classes: the largest dim, the warps of one group (one row per
// thread) and the groups a CTA runs at a time.
__host__ __device__ constexpr int rag_class_dim(int c) { return c == 0 ? 128 : c == 1 ? 96 : c == 2 ? 64 : 32; }
__host__ __device__ constexpr int rag_class_gwarps(int c) { return c == 0 ? 4 : c == 1 ? 3 : c == 2 ? 2 : 1; }
__host__ __device__ constexpr int rag_class_groups(int c) { return c == 0 ? 1 : c == 1 ? 2 : c == 2 ? 4 : 8; }
__host__ __device__ constexpr int rag_class_of(int dim) { return dim > 96 ? 0 : dim > 64 ? 1 : dim > 32 ? 2 : 3; }
// Chunks per 32-row block in the substitutions' hand-off.  Named barrier ids:
// 0 is __syncthreads, 1..groups the groups' own, then each group's chunk
// barriers (at most 1 + 4 + 4*2 = 12 < 16).
__host__ __device__ constexpr int rag_class_chunks(int c) { return c <= 1 ? 4 : c == 2 ? 2 : 0; }

// One group's shared-memory slice for systems of dim <= ld, in doubles:
// factors ld*ld, pivot reciprocals ld, H 7*ld, HH 7*ld, staging ld, params
// ld/2+2, permutation ld/2 (ld ints), cache table 48 (16 keys, 16 stamps,
// 16 states), exchange area (2 broadcast slots, 2 x 4 reduction values,
// 2 x 4 reduction indices, the bulk-copy mbarrier at 14, the work item at 15,
// 2 x 32 block values of the substitutions from 16, the producing block's
// right-hand side from 80; 112 in all).
struct RagSmem {
  __host__ __device__ static constexpr int M(int) { return 0; }
  __host__ __device__ static constexpr int rinv(int ld) { return ld * ld; }
  __host__ __device__ static constexpr int H(int ld) { return ld * ld + ld; }
  __host__ __device__ static constexpr int HH(int ld) { return ld * ld + 8 * ld; }
  __host__ __device__ static constexpr int sv(int ld) { return ld * ld + 15 * ld; }
  __host__ __device__ static constexpr int sp(int ld) { return ld * ld + 16 * ld; }
  __host__ __device__ static constexpr int perm(int ld) { return ld * ld + 16 * ld + ld / 2 + 2; }
  __host__ __device__ static constexpr int table(int ld) { return perm(ld) + ld / 2; }
  __host__ __device__ static constexpr int xch(int ld) { return table(ld) + 48; }
  __host__ __device__ static constexpr int doubles(int ld) { return xch(ld) + 112; }
};

// Shared memory of a CTA for the classes present (bit c of mask = class c).
__host__ __device__ constexpr size_t rag_cta_smem_bytes(unsigned mask) {
  size_t b = 0;
  for (int c = 0; c < kRagClasses; ++c)
    if (mask & (1u << c)) {
      const size_t need = static_cast<size_t>(rag_class_groups(c)) * RagSmem::doubles(rag_class_dim(c)) * 8;
      if (need > b) b = need;
    }
  return b;
}

// Device-memory factor cache of one group: 16 slots of ld*ld factors, ld
// pivot reciprocals and ld permutation ints.  A CTA's phases run one after
// another, so they share one region sized for the largest phase.
__host__ __device__ constexpr size_t rag_gslot_doubles(int ld) { return static_cast<size_t>(ld) * ld + ld + ld / 2; }
__host__ __device__ constexpr size_t rag_gcache_group_doubles(int c) {
  return kRagCacheSlots * rag_gslot_doubles(rag_class_dim(c));
}
__host__ __device__ constexpr size_t rag_gcache_cta_doubles() {
  size_t s = 0;
  for (int c = 0; c < kRagClasses; ++c) {
    const size_t need = rag_class_groups(c) * rag_gcache_group_doubles(c);
    if (need > s) s = need;
  }
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
  unsigned int* error_flag;    // raised when a bounded wait on a bulk copy gives up
  // packed dense output, or null: system i's items (t, y) are the slots
  // [traj_off[i], traj_off[i+1]) of traj_t, its values from traj_voff[i] of
  // traj_y (item k at traj_voff[i] + k * dim_i)
  double* traj_t;
  double* traj_y;
  const int64_t* traj_off;
  const int64_t* traj_voff;
};

// Damped spring-mass chain (unit masses): rows 0..N-1 are x' = v, rows
// N..2N-1 the forces; y and p in shared memory.  Same expressions as RhsChain
// and the oracle's chain right-hand side.
struct RagChain {
  static constexpr bool kAffine = true;  // f = J y, J constant
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

// The threads that own one system: thread t owns row t.  Synchronisation is
// __syncwarp for a one-warp group, else the group's own named barrier.
struct RagGroup {
  int t;         // thread (= row) index in the group
  int nthr;      // 32 * warps
  int bar;       // named barrier id
  int cbar;      // first of the substitutions' chunk barrier ids
  int nchunk;    // chunks per 32-row block (0 for a one-warp group)
  double* xch;   // exchange area (RagSmem::xch)
  int par;       // parity of the next reduction's buffer
  uint32_t mbar;   // the group's mbarrier for bulk copies (shared address)
  uint32_t mphase; // its next phase parity
  unsigned int* err;  // raised when a bounded wait gives up

  // Producer/consumer hand-off on a named barrier: the producing warp
  // arrives (and moves on), the consuming warps wait.  cnt counts both.
  __device__ __forceinline__ static void arrive(int id, unsigned cnt) { BACON_BAR_ARRIVE(id, cnt); }
  __device__ __forceinline__ static void wait(int id, unsigned cnt) {
    __barrier_sync_count(static_cast<unsigned>(id), cnt);
  }

  __device__ __forceinline__ void sync() const {
    if (nthr == 32) __syncwarp();
    else __barrier_sync_count(static_cast<unsigned>(bar), static_cast<unsigned>(nthr));
  }
  // value of thread src, to every thread; slot alternates with the caller's
  // step parity so that one barrier per broadcast suffices
  __device__ __forceinline__ double bcast(double v, int src, int slot) const {
    if (nthr == 32) return __shfl_sync(0xffffffffu, v, src);
    if (t == src) xch[slot & 1] = v;
    sync();
    return xch[slot & 1];
  }
  // sum over the group in a fixed order (warp trees, then warps in order)
  __device__ __forceinline__ double sum(double v) {
    using O = ExactOps;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = O::add(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (nthr == 32) return v;
    double* red = xch + 2 + 4 * par;
    if ((t & 31) == 0) red[t >> 5] = v;
    par ^= 1;
    sync();
    double s = red[0];
    for (int w = 1; w < nthr / 32; ++w) s = O::add(s, red[w]);
    return s;
  }
  // arg-max of (magnitude, index) with the lowest index winning ties, for
  // magnitudes that are non-negative and not NaN, given as their bit
  // patterns: integer order is then numeric order, and the compares stay off
  // the FP64 pipe
  __device__ __forceinline__ int argmax_bits(unsigned long long v, int idx) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long ov = __shfl_xor_sync(0xffffffffu, v, off);
      const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
      if (ov > v || (ov == v && oi < idx)) {
        v = ov;
        idx = oi;
      }
    }
    if (nthr == 32) return idx;
    unsigned long long* red = reinterpret_cast<unsigned long long*>(xch + 2 + 4 * par);
    int* redi = reinterpret_cast<int*>(xch + 10) + 4 * par;
    if ((t & 31) == 0) {
      red[t >> 5] = v;
      redi[t >> 5] = idx;
    }
    par ^= 1;
    sync();
    unsigned long long bv = red[0];
    int bi = redi[0];
    for (int w = 1; w < nthr / 32; ++w)
      if (red[w] > bv || (red[w] == bv && redi[w] < bi)) {
        bv = red[w];
        bi = redi[w];
      }
    return bi;
  }
};

// M = I - hb J, then the partial-pivot LU in place (shared memory);
// perm[pos] = the original row now at pos, rinv[i] = 1 / U[i][i] (the
// elimination's own reciprocal, used again by the back substitution).
// Returns false on an exactly zero pivot.
__device__ __forceinline__ bool rag_factor(RagGroup& g, int D, int N, const double* sp, double hb, double* M,
                                           double* rinv, int32_t* perm) {
  using O = ExactOps;
  const int r = g.t;
  if (r < D) {
    for (int k = 0; k < D; ++k) M[k * D + r] = O::sub((r == k) ? 1.0 : 0.0, O::mul(hb, RagChain::jac(r, k, N, sp)));
    perm[r] = r;
  }
  g.sync();
  for (int i = 0; i < D; ++i) {
    double* col = M + i * D;
    // pivot: the first row of maximum |M[r][i]| from the diagonal down (a NaN
    // below the diagonal never wins, a NaN diagonal stays), on the magnitudes'
    // bit patterns
    constexpr unsigned long long kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
    const unsigned long long diag = static_cast<unsigned long long>(__double_as_longlong(col[i])) & kAbs;
    int pr = i;
    if (diag <= kInf) {
      unsigned long long v = diag;
      int idx = i;
      if (r > i && r < D) {
        const unsigned long long a = static_cast<unsigned long long>(__double_as_longlong(col[r])) & kAbs;
        if (a > diag && a <= kInf) {
          v = a;
          idx = r;
        }
      }
      pr = g.argmax_bits(v, idx);
    }
    if (pr != i) {
      for (int k = r; k < D; k += g.nthr) {
        const double a = M[k * D + i];
        M[k * D + i] = M[k * D + pr];
        M[k * D + pr] = a;
      }
      if (r == 0) {
        const int32_t a = perm[i];
        perm[i] = perm[pr];
        perm[pr] = a;
      }
      g.sync();
    }
    const double piv = col[i];
    if ((static_cast<unsigned long long>(__double_as_longlong(piv)) & kAbs) == 0ull) return false;  // piv == 0
    const double inv = O::div(1.0, piv);
    if (r == 0) rinv[i] = inv;
    if (r > i && r < D) col[r] = O::mul(col[r], inv);
    const int m = D - 1 - i;  // rows (and columns) below / right of the pivot
    if (m > 0) {
      g.sync();  // the multipliers
      // Trailing update, balanced over the whole group: columns dealt
      // round-robin to the warps, the m rows to the lanes (up to four each,
      // independent FMAs).  Every element receives the same FMA in the same
      // pivot order as with one row per thread.  An update with an exactly
      // zero multiplier or pivot-row entry is skipped (the oracle's rule):
      // a zero U[i][k] skips the warp's column, a 32-row chunk without a
      // nonzero multiplier is skipped by the whole warp, so the sparse
      // factors of the chains cost a fraction of the dense update.
      const int w = r >> 5, lane = r & 31, nw = g.nthr >> 5;
      const double* lc = col + i + 1;
      const double l0 = lane < m ? lc[lane] : 0.0;
      const double l1 = lane + 32 < m ? lc[lane + 32] : 0.0;
      const double l2 = lane + 64 < m ? lc[lane + 64] : 0.0;
      const double l3 = lane + 96 < m ? lc[lane + 96] : 0.0;
      const bool n0 = !bits_zero(l0), n1 = !bits_zero(l1), n2 = !bits_zero(l2), n3 = !bits_zero(l3);
      const bool g0 = __any_sync(0xffffffffu, n0), g1 = __any_sync(0xffffffffu, n1);
      const bool g2 = __any_sync(0xffffffffu, n2), g3 = __any_sync(0xffffffffu, n3);
      if (g0 || g1 || g2 || g3) {
        for (int k = i + 1 + w; k < D; k += nw) {
          double* ck = M + k * D + i + 1;
          const double u = ck[-1];  // U[i][k], the same for the warp
          if (bits_zero(u)) continue;
          if (g0 && n0) ck[lane] = __fma_rn(-l0, u, ck[lane]);
          if (g1 && n1) ck[lane + 32] = __fma_rn(-l1, u, ck[lane + 32]);
          if (g2 && n2) ck[lane + 64] = __fma_rn(-l2, u, ck[lane + 64]);
          if (g3 && n3) ck[lane + 96] = __fma_rn(-l3, u, ck[lane + 96]);
        }
      }
    }
    g.sync();
  }
  // the rows of U scaled by their pivot reciprocal (a unit upper factor for
  // the back substitution)
  if (r < D) {
    const double s = rinv[r];
    for (int k = r + 1; k < D; ++k) M[k * D + r] = O::mul(M[k * D + r], s);
  }
  // The diagonal 32-row blocks of L and of the scaled U replaced by their
  // inverses (strict parts in place): block b by warp b (its own rows), lane
  // c computing column c as the solve of e_c, every update taken for every
  // column in the oracle's order.  (Skipping the zero entries, a uniform test
  // per update, measured slower: the unrolled FMAs cost less than the
  // branches.)  The caller syncs before the factors are read.
  const int nw = g.nthr >> 5, lane = r & 31;
  for (int b = r >> 5; b * 32 < D; b += nw) {
    __syncwarp();
    const int s0 = 32 * b;
    const int nb = min(32, D - s0);
    double* blk = M + s0 * D + s0;  // element (j, k) of the block at blk[k * D + j]
    double x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) x[j] = (j == lane) ? 1.0 : 0.0;
#pragma unroll
    for (int k = 0; k < 31; ++k)
      if (k + 1 < nb) {
#pragma unroll
        for (int j = k + 1; j < 32; ++j)
          if (j < nb) x[j] = __fma_rn(-blk[k * D + j], x[k], x[j]);
      }
    __syncwarp();  // every lane has read the lower block
    if (lane < nb) {
#pragma unroll
      for (int j = 1; j < 32; ++j)
        if (j > lane && j < nb) blk[lane * D + j] = x[j];
    }
#pragma unroll
    for (int j = 0; j < 32; ++j) x[j] = (j == lane) ? 1.0 : 0.0;
#pragma unroll
    for (int k = 31; k > 0; --k)
      if (k < nb) {
#pragma unroll
        for (int j = 0; j < k; ++j) x[j] = __fma_rn(-blk[k * D + j], x[k], x[j]);
      }
    __syncwarp();  // every lane has read the upper block
    if (lane < nb) {
#pragma unroll
      for (int j = 0; j < 31; ++j)
        if (j < lane) blk[lane * D + j] = x[j];
    }
  }
  return true;
}

// Group copy of n doubles (n even; both pointers 16-byte aligned).
__device__ __forceinline__ void rag_copy(const RagGroup& g, double* dst, const double* src, int n) {
  const double2* s = reinterpret_cast<const double2*>(src);
  double2* d = reinterpret_cast<double2*>(dst);
  const int n2 = n / 2, st = g.nthr;
  int i = g.t;
  for (; i + 3 * st < n2; i += 4 * st) {
    const double2 a = s[i], b = s[i + st], c = s[i + 2 * st], e = s[i + 3 * st];
    d[i] = a;
    d[i + st] = b;
    d[i + 2 * st] = c;
    d[i + 3 * st] = e;
  }
  for (; i < n2; i += st) d[i] = s[i];
}

// The factors currently in shared memory (their key and state: 0 none,
// 1 factored, 2 singular) and the cache clock.  The device-memory slots are
// described by a shared-memory table of 16 (key, stamp, state) entries.
struct RagCache {
  long long cur_key;
  int cur_state;
  int clock;
};

// Makes the factors of M(hb) current in shared memory; returns 1 (factored)
// or 2 (singular).
__device__ __forceinline__ int rag_get_factors(RagGroup& g, int D, int N, const double* sp, double hb, double* sM,
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
      // factors and reciprocals by one bulk copy each (D is even, so both
      // sizes are multiples of 16 bytes), the permutation by plain loads
      const double* gs = gcache + hit * slot_doubles;
      rag_proxy_fence();
      g.sync();  // every earlier access of the factors and the slots is done
      if (g.t == 0)
        rag_bulk_issue2(g.mbar, sM, gs, static_cast<uint32_t>(D * D * 8), srinv, gs + static_cast<size_t>(gld) * gld,
                        static_cast<uint32_t>(D * 8));
      const int32_t* gp = reinterpret_cast<const int32_t*>(gs + static_cast<size_t>(gld) * gld + gld);
      for (int r = g.t; r < D; r += g.nthr) sperm[r] = gp[r];
      rag_mbar_wait(g.mbar, g.mphase, g.err);
      g.mphase ^= 1u;
    }
    g.sync();
    if (g.t == 0) stamps[hit] = cache.clock;
    g.sync();
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
  const int st = rag_factor(g, D, N, sp, hb, sM, srinv, sperm) ? 1 : 2;
  g.sync();
  if (st == 1) {
    double* gs = gcache + victim * slot_doubles;
    rag_copy(g, gs, sM, D * D);
    rag_copy(g, gs + static_cast<size_t>(gld) * gld, srinv, D);
    int32_t* gp = reinterpret_cast<int32_t*>(gs + static_cast<size_t>(gld) * gld + gld);
    for (int r = g.t; r < D; r += g.nthr) gp[r] = sperm[r];
  }
  if (g.t == 0) {
    keys[victim] = key;
    stamps[victim] = cache.clock;
    states[victim] = st;
  }
  g.sync();
  cache.cur_key = key;
  cache.cur_state = st;
  return st;
}

// Newton solve of y - hb f(y) + sum_j a_{q,j} HH[j-1] = 0 from the guess in
// y (this thread's row), with the factors of M for hb.
__device__ __forceinline__ bool rag_newton(RagGroup& g, int D, int N, const double* sp, double* sv, const double* HH,
                                           int ld, int q, double h, double* sM, double* srinv, int32_t* sperm,
                                           double* table, double* gcache, int gld, RagCache& cache,
                                           int max_newton, double tol, double& y) {
  using O = ExactOps;
  const int r = g.t;
  const bool own = r < D;
  const double hb = O::mul(h, bdf_b(q));
  double c = 0.0;
  if (own)
    for (int jj = 1; jj <= q; ++jj) c = O::add(c, O::mul(bdf_a(q, jj), HH[(jj - 1) * ld + r]));
  if (rag_get_factors(g, D, N, sp, hb, sM, srinv, sperm, table, gcache, gld, cache) != 1) return false;
  const double* M = sM;
  const int src = own ? sperm[r] : 0;
  const double conv = O::mul(1e-3, tol);
  for (int it = 0; it < max_newton; ++it) {
    g.sync();
    if (own) sv[r] = y;
    g.sync();
    const double gr = own ? O::add(O::sub(y, O::mul(hb, RagChain::f(r, N, sv, sp))), c) : 0.0;
    g.sync();
    if (own) sv[r] = gr;
    g.sync();
    double dx = own ? -sv[src] : 0.0;
    // Substitutions by 32-row blocks (block b = warp b of the group).  The
    // block's warp runs its triangle with shuffles and publishes the values
    // chunk by chunk (it arrives on the chunk's barrier and moves on); the
    // warps that need them wait on that barrier and apply the chunk while the
    // block's warp continues.  Every row receives its updates in the order of
    // the unblocked loops.  A chunk barrier is reused by the next block only
    // after every participant of its previous phase has arrived: the next
    // block's warps all waited on the earlier chunks.
    const int wg = r >> 5, lane = r & 31;
    const int nblk = (D + 31) >> 5;
    double* xs = g.xch + 16;  // [2][32], alternating blocks
    double* rin = g.xch + 80;  // the producing block's right-hand side
    const int cs = g.nchunk > 0 ? 32 / g.nchunk : 32;
    // forward, unit lower factor
    for (int b = 0; b < nblk; ++b) {
      const int base = 32 * b;
      const int nb = min(32, D - base);
      const unsigned cnt = 32u * static_cast<unsigned>(nblk - b);
      double* xb = xs + (b & 1) * 32;
      if (wg == b) {
        // x = Linv r: lane j adds Linv[j][k] r_k for k < j, ascending.  The
        // right-hand side is complete, so it is staged once in shared memory
        // and read back as broadcasts (a shuffle per term would cost ~50
        // cycles more per FMA)
        rin[lane] = dx;
        __syncwarp();
        for (int lo = 0; lo < nb; lo += cs) {
          const int hi = min(lo + cs, nb);
          for (int k0 = lo; k0 < hi; k0 += 8) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int k = k0 + q;
              if (k < hi) {
                const double m = own ? M[(base + k) * D + r] : 0.0;
                const double rk = rin[k];
                if (lane > k && own) dx = __fma_rn(m, rk, dx);
              }
            }
          }
          if (b + 1 < nblk) {
            if (lane >= lo && lane < hi) xb[lane] = dx;
            g.arrive(g.cbar + lo / cs, cnt);
          }
        }
      } else if (wg > b) {
        for (int lo = 0; lo < nb; lo += cs) {
          const int hi = min(lo + cs, nb);
          g.wait(g.cbar + lo / cs, cnt);
          if (own)
            for (int k0 = lo; k0 < hi; k0 += 8) {
#pragma unroll
              for (int q = 0; q < 8; ++q) {
                const int k = k0 + q;
                if (k < hi) dx = __fma_rn(-M[(base + k) * D + r], xb[k], dx);
              }
            }
        }
      }
    }
    // back, on the row-scaled unit upper factor.  The group sync closes every
    // forward chunk phase first (warp 0 only arrived on block 0's chunk
    // barriers, and its waits below use the same ids) and every read of the
    // staged right-hand side.  It costs no time on the critical path (the
    // last block's warp finishes the forward last and starts the back first).
    g.sync();
    if (own) dx = O::mul(dx, srinv[r]);
    for (int b = nblk - 1; b >= 0; --b) {
      const int base = 32 * b;
      const int nb = min(32, D - base);
      const unsigned cnt = 32u * static_cast<unsigned>(b + 1);
      double* xb = xs + (b & 1) * 32;
      if (wg == b) {
        // x = Uinv r: lane j adds Uinv[j][k] r_k for k > j, descending
        rin[lane] = dx;
        __syncwarp();
        for (int hi = nb; hi > 0; hi -= cs) {
          const int lo = max(hi - cs, 0);
          for (int k1 = hi - 1; k1 >= lo; k1 -= 8) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int k = k1 - q;
              if (k >= lo) {
                const double m = own ? M[(base + k) * D + r] : 0.0;
                const double rk = rin[k];
                if (lane < k) dx = __fma_rn(m, rk, dx);
              }
            }
          }
          if (b > 0) {
            if (lane >= lo && lane < hi) xb[lane] = dx;
            g.arrive(g.cbar + (nb - hi) / cs, cnt);
          }
        }
      } else if (wg < b) {
        for (int hi = nb; hi > 0; hi -= cs) {
          const int lo = max(hi - cs, 0);
          g.wait(g.cbar + (nb - hi) / cs, cnt);
          for (int k1 = hi - 1; k1 >= lo; k1 -= 8) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int k = k1 - q;
              if (k >= lo) dx = __fma_rn(-M[(base + k) * D + r], xb[k], dx);
            }
          }
        }
      }
    }
    if (own) {
      y = O::add(y, dx);
      sv[r] = dx;
    }
    // ||dx||^2: the oracle sums it in order on one thread and tests
    // sqrt(dn) <= conv.  The group tree sum differs from that by ~dim * 2^-53
    // (all terms are non-negative), so it decides alone unless it lies within
    // 1e-10 of conv^2; then the ordered sum decides.  NaN in either exactly
    // when some dx is NaN.
    const double part = g.sum(own ? O::mul(dx, dx) : 0.0);
    if (!(part == part)) return false;
    // The chain is affine in y and M holds its exact Jacobian, so the first
    // update solves the linear system: the solve ends here (the oracle's
    // rule for affine right-hand sides).
    if (RagChain::kAffine) return true;
    const double thr = O::mul(conv, conv);
    if (fabs(O::sub(part, thr)) > O::mul(1e-10, thr)) {
      if (part < thr) return true;
      continue;
    }
    g.sync();  // every row's dx is in sv
    double dn = 0.0;
    if (r == 0)
      for (int d = 0; d < D; ++d) dn = O::add(dn, O::mul(sv[d], sv[d]));
    dn = g.bcast(dn, 0, 0);
    g.sync();
    if (O::sqrt(dn) <= conv) return true;
  }
  return false;
}

// Euclidean norm of sv[0..D) in nalgebra's order for a dynamically sized
// vector (eight partial sums, then the tail); group-uniform.
__device__ __forceinline__ double rag_norm(RagGroup& g, int D, const double* sv) {
  using O = ExactOps;
  double acc = 0.0;
  const int full = D - D % 8;
  if (g.t < 8)
    for (int i = 0; i < full; i += 8) acc = O::add(acc, O::mul(sv[i + g.t], sv[i + g.t]));
  double a[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) a[l] = __shfl_sync(0xffffffffu, acc, l);
  double res = 0.0;
  if (g.t == 0) {
    res = O::add(res, O::add(a[0], a[4]));
    res = O::add(res, O::add(a[1], a[5]));
    res = O::add(res, O::add(a[2], a[6]));
    res = O::add(res, O::add(a[3], a[7]));
    for (int k = full; k < D; ++k) res = O::add(res, O::mul(sv[k], sv[k]));
    res = O::sqrt(O::add(0.0, res));
  }
  res = g.bcast(res, 0, 1);
  g.sync();
  return res;
}

// A value that compares with tol and 0.1*tol exactly as rag_norm(sv) does:
// the group tree-sum norm (within ~dim * 2^-53 of the ordered one) unless it
// lies within 1e-10 of either threshold, else the ordered norm itself.
// sv must be written and synchronised by the caller.
__device__ __forceinline__ double rag_norm_decide(RagGroup& g, int D, const double* sv, double tol) {
  using O = ExactOps;
  const double v = g.t < D ? sv[g.t] : 0.0;
  const double e = O::sqrt(g.sum(O::mul(v, v)));
  if (!(e == e)) return e;
  const double t2 = O::mul(0.1, tol);
  if (fabs(O::sub(e, tol)) > O::mul(1e-10, tol) && fabs(O::sub(e, t2)) > O::mul(1e-10, t2)) return e;
  return rag_norm(g, D, sv);
}

// Lagrange weights the ragged steps use at fixed points, computed once per
// CTA by lagrange_weights itself (so the same values): the predictor's, at
// s = 1 over k = 1..7 history points, and the halving's, at the nodes
// s = -0.5 j (j < k).  Each is a division chain of ~k dependent FP64 divisions
// that every step (or rejection) would otherwise repeat.
struct RagWeights {
  double pred[7][7];     // [k-1][i]
  double half[7][7][7];  // [k-1][j][i]
};

__device__ __forceinline__ void rag_weights_init(RagWeights& wt) {
  using O = ExactOps;
  for (int u = static_cast<int>(threadIdx.x); u < 7 + 49; u += static_cast<int>(blockDim.x)) {
    double w[7];
    if (u < 7) {
      lagrange_weights(u, 1.0, w);
      for (int i = 0; i <= u; ++i) wt.pred[u][i] = w[i];
    } else {
      const int q = (u - 7) / 7, j = (u - 7) % 7;
      if (j > q) continue;
      lagrange_weights(q, O::mul(-0.5, static_cast<double>(j)), w);
      for (int i = 0; i <= q; ++i) wt.half[q][j][i] = w[i];
    }
  }
}

// Interpolates this thread's k history values onto nodes -s*j (j < k), with
// the weights of the table wt ([j][i]) when given.
__device__ __forceinline__ void rag_interp_row(int r, int ld, int k, double s, const double* src, double* dst,
                                               const double (*wt)[7]) {
  using O = ExactOps;
  double w[7];
  for (int j = 0; j < k; ++j) {
    const double* wj = w;
    if (wt != nullptr) wj = wt[j];
    else lagrange_weights(k - 1, O::mul(-s, static_cast<double>(j)), w);
    double acc = 0.0;
    for (int i = 0; i < k; ++i) acc = O::add(acc, O::mul(wj[i], src[i * ld + r]));
    dst[j * ld + r] = acc;
  }
}

// One ragged system integrated by the calling group; ws is its shared-memory
// slice for dims <= ld, gcache its device-memory factor slots.
__device__ __forceinline__ void rag_solve_system(const RaggedArgs& a, int64_t idx, RagGroup& g, double* ws, int ld,
                                                 double* gcache, const RagWeights& wt) {
  using O = ExactOps;
  double* sM = ws + RagSmem::M(ld);
  double* srinv = ws + RagSmem::rinv(ld);
  double* H = ws + RagSmem::H(ld);
  double* HH = ws + RagSmem::HH(ld);
  double* sv = ws + RagSmem::sv(ld);
  double* sp = ws + RagSmem::sp(ld);
  int32_t* sperm = reinterpret_cast<int32_t*>(ws + RagSmem::perm(ld));
  double* table = ws + RagSmem::table(ld);
  const int r = g.t;
  const int64_t yo = a.y_off[idx];
  const int D = static_cast<int>(a.y_off[idx + 1] - yo);
  const int N = D / 2;
  const bool own = r < D;
  const int64_t po = a.p_off[idx];
  g.sync();
  for (int k = r; k <= N; k += g.nthr) sp[k] = a.params[po + k];
  if (r < 32) reinterpret_cast<int*>(table + 16)[r] = 0;  // stamps and states of the 16 slots
  double ly = 0.0;
  if (own) {
    ly = a.y0[yo + r];
    H[r] = ly;
  }
  g.sync();
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
      if (own) rag_interp_row(r, ld, k, O::div(h, dt), H, HH, nullptr);
      HHp = HH;
    }
    // predictor: extrapolation through the history points
    const double* w = wt.pred[k - 1];
    double yh = 0.0, yl = 0.0;
    if (own)
      for (int i = 0; i < k; ++i) yh = O::add(yh, O::mul(w[i], HHp[i * ld + r]));
    const double t1 = O::add(t, h);
    bool ok = rag_newton(g, D, N, sp, sv, HHp, ld, q, h, sM, srinv, sperm, table, gcache, ld, cache, a.max_iter,
                         a.tol, yh);
    double error;
    if (ok && q >= 2) {
      yl = yh;
      ok = rag_newton(g, D, N, sp, sv, HHp, ld, q - 1, h, sM, srinv, sperm, table, gcache, ld, cache, a.max_iter,
                      a.tol, yl);
      g.sync();
      if (own) sv[r] = O::sub(yh, yl);
      g.sync();
      error = rag_norm_decide(g, D, sv, a.tol);
    } else {
      // order 1: half the gap between backward and forward Euler
      const double diff =
          own ? O::mul(0.5, O::sub(yh, O::add(H[r], O::mul(h, RagChain::f(r, N, H, sp))))) : 0.0;
      g.sync();
      if (own) sv[r] = diff;
      g.sync();
      error = rag_norm_decide(g, D, sv, a.tol);
    }
    if (ok && error <= a.tol && a.traj_t != nullptr && a.traj_off[idx] + acc >= a.traj_off[idx + 1]) {
      status = kStCapacity;  // the dense output is full: the item is not yielded
      break;
    }
    if (ok && error <= a.tol) {
      if (a.traj_t != nullptr) {
        if (r == 0) a.traj_t[a.traj_off[idx] + acc] = t1;
        if (own) a.traj_y[a.traj_voff[idx] + static_cast<int64_t>(acc) * D + r] = yh;
      }
      const int kk = (k < 7) ? k + 1 : 7;
      g.sync();  // every row has finished reading H
      if (own) {
        for (int i = kk - 1; i >= 1; --i) H[i * ld + r] = H[(i - 1) * ld + r];
        H[r] = yh;
        ly = yh;
      }
      g.sync();
      k = kk;
      t = t1;
      ++acc;
      last_t = t;
      if (h != dt) continue;
      if (error < O::mul(0.1, a.tol) && k == qmax + 1 && O::mul(dt, 2.0) <= dt_max) {
        const int nk = (k + 1) / 2;
        if (own)
          for (int i = 1; i < nk; ++i) H[i * ld + r] = H[2 * i * ld + r];
        g.sync();
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
      g.sync();  // every row has finished reading H
      if (own) {
        rag_interp_row(r, ld, k, 0.5, H, HH, wt.half[k - 1]);
        for (int i = 0; i < k; ++i) H[i * ld + r] = HH[i * ld + r];
      }
      g.sync();
    }
    dt = nd;
  }
  if (own) a.y_out[yo + r] = ly;
  if (r == 0) {
    a.t_out[idx] = last_t;
    a.accepted[idx] = acc;
    a.rejected[idx] = rej;
    a.status[idx] = status;
    if (status != kStOk) atomicMin(a.first_fail, static_cast<unsigned long long>(idx));
  }
  g.sync();
}

// Marker for a mixed launch without a uniform (one-thread-per-system) part.
struct NoSmall {};

// One launch for a stiff batch of two parts: ragged systems (a group of
// warps each, in four size-class phases) and a uniform batch of small systems
// (a thread each, after the last phase).  Launched with kRagWarps * 32 threads
// and rag_cta_smem_bytes(classes present) of dynamic shared memory.
template <class Small>
__global__ void __launch_bounds__(kRagWarps * 32, 1)
    bdf_mixed_kernel(const BdfArgs small, int small_dyn, const RaggedArgs rg) {
  extern __shared__ __align__(16) double rag_smem[];
  __shared__ RagWeights rag_w;
  rag_weights_init(rag_w);
  __syncthreads();
  const int warp = static_cast<int>(threadIdx.x >> 5);
  double* gcache_cta = rg.gcache + static_cast<size_t>(blockIdx.x) * rag_gcache_cta_doubles();
  for (int c = 0; c < kRagClasses; ++c) {
    if (rg.class_n[c] == 0) continue;
    const int gw = rag_class_gwarps(c);
    const int grp = warp / gw;
    if (grp < rag_class_groups(c)) {
      const int ld = rag_class_dim(c);
      double* ws = rag_smem + static_cast<size_t>(grp) * RagSmem::doubles(ld);
      RagGroup g;
      g.t = static_cast<int>(threadIdx.x) - grp * gw * 32;
      g.nthr = gw * 32;
      g.bar = 1 + grp;
      g.nchunk = rag_class_chunks(c);
      g.cbar = 1 + rag_class_groups(c) + grp * g.nchunk;
      g.xch = ws + RagSmem::xch(ld);
      g.par = 0;
      g.mbar = rag_smem_addr(g.xch + 14);
      g.mphase = 0u;
      g.err = rg.error_flag;
      if (g.t == 0) rag_mbar_init(g.mbar);
      g.sync();
      double* gcache = gcache_cta + static_cast<size_t>(grp) * rag_gcache_group_doubles(c);
      unsigned long long* slot = reinterpret_cast<unsigned long long*>(g.xch + 15);
      for (;;) {
        if (g.t == 0) *slot = atomicAdd(rg.queues + c, 1ull);
        g.sync();
        const unsigned long long item = *slot;
        g.sync();
        if (item >= static_cast<unsigned long long>(rg.class_n[c])) break;
        const int64_t idx = static_cast<int64_t>(rg.order[rg.class_start[c] + static_cast<int64_t>(item)]);
        rag_solve_system(rg, idx, g, ws, ld, gcache, rag_w);
      }
      g.sync();
      if (g.t == 0) rag_mbar_inval(g.mbar);  // before the next phase reuses this memory
    }
    __syncthreads();
  }
  if constexpr (!std::is_same<Small, NoSmall>::value) {
    if (small.n > 0) bdf_corrected_thread_loop<Small>(small, small_dyn != 0);
  }
}

}  // namespace bacon
