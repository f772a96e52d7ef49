// Tensor-core stage GEMM for the linear (shared-A) engine: split-precision
// emulation of the FP64 product A * Y on tcgen05 (bf16 operands, FP32
// accumulators in tensor memory).
//
// Splitting (the Ozaki scheme): every row of A and every system's stage
// vector (a column of Y) is scaled by a power of two so that its largest
// entry is below 1, then cut into NS = 5 slices of B = 8 bits each:
//     x = 2^e * sum_s q_s 2^(-8(s+1)),  q_s integer, |q_s| <= 255.
// Integers of at most 8 significant bits are exact in bf16, and a K = 256 dot
// product of two slices is an integer of magnitude at most 256 * 255^2 =
// 16,646,400 < 2^24, so the tensor cores compute every slice product exactly
// in FP32.  Pairs (s, t) with s + t = d share the scale 2^(-8(d+2)).  The
// pairs of diagonals 0..2 (1 + 2 + 3) get one TMEM accumulator each, so their
// sums are exact.  Diagonal 3's four pairs share one accumulator and diagonal
// 4's five another: those sums can round in FP32 (at most ~2^26), but they
// weigh at most 2^-24 of diagonal 0, so their rounding stays near 2^-40 of
// the product.  Eight accumulators x 64 columns fill the 512 TMEM columns.
// The epilogue combines them as 64-bit integers, applies 2^(e_row + e_sys)
// and writes the product: the engine forms v_k = A v_{k-1}.  Pairs with
// s + t >= NS are dropped.
// The relative error of the product is ~2^-39 (40-bit operands), with 15
// slice products per K step; six 6-bit slices (exact sums in six
// accumulators, 21 products) reached ~2^-35.
//
// CTA tile: 128 rows of A x 64 systems, K = D in chunks of 32 staged in
// shared memory in the canonical no-swizzle K-major layout (8 x 16-byte core
// matrices).  One producer thread issues the copies and the MMAs (M128 N64
// K16) and commits them to mbarriers; eight epilogue warps drain the
// accumulators, so a tile's epilogue overlaps the next tile's MMAs.  Every
// wait on an mbarrier is bounded.
#pragma once

#include <cstdint>

#include "linear.cuh"

namespace bacon {

constexpr int kTcSlices = 5;      // slices per operand (40 bits)
constexpr int kTcBits = 8;        // bits per slice
constexpr int kTcFracBits = kTcSlices * kTcBits;
constexpr int kTcAccs = 8;        // TMEM accumulators
constexpr int kTcExactDiags = 3;  // diagonals 0..2 accumulate exactly, a pair per accumulator
constexpr int kTcM = 128;         // rows per CTA
constexpr int kTcN = 64;          // systems per CTA
constexpr int kTcKc = 32;         // K per shared-memory chunk (two buffers)
constexpr int kTcTmemCols = 512;  // kTcAccs accumulators x 64 columns, rounded to a power of two

// Accumulator of the slice pair (s, t): one per pair on diagonals 0..2
// (accumulators 0 | 1, 2 | 3, 4, 5), one per diagonal for 3 and 4 (6, 7);
// the diagonal an accumulator holds; and the first s (in the MMA loop's
// order) that writes it.
__host__ __device__ constexpr int tc_acc(int s, int t) {
  return s + t == 0 ? 0 : s + t == 1 ? 1 + s : s + t == 2 ? 3 + s : s + t == 3 ? 6 : 7;
}
__host__ __device__ constexpr int tc_acc_diag(int acc) {
  return acc == 0 ? 0 : acc <= 2 ? 1 : acc <= 5 ? 2 : acc == 6 ? 3 : 4;
}
__host__ __device__ constexpr int tc_acc_first_s(int acc) {
  return acc == 2 ? 1 : acc == 4 ? 1 : acc == 5 ? 2 : 0;
}
__host__ __device__ constexpr bool tc_split_exact(int k) {
  // the accumulators of diagonals 0..2 take one pair each, at most
  // k * 255^2, an exact FP32 integer; every accumulator index is in range
  // and its first pair is the one tc_acc_first_s names
  for (int acc = 0; acc < kTcAccs; ++acc) {
    int pairs = 0, first = -1;
    for (int s = 0; s < kTcSlices; ++s)
      for (int t = 0; s + t < kTcSlices; ++t)
        if (tc_acc(s, t) == acc) {
          if (tc_acc_diag(acc) != s + t) return false;
          if (first < 0) first = s;
          ++pairs;
        }
    if (pairs == 0 || first != tc_acc_first_s(acc)) return false;
    if (tc_acc_diag(acc) < kTcExactDiags && (pairs != 1 || static_cast<long long>(k) * 255 * 255 >= (1ll << 24)))
      return false;
  }
  return true;
}
static_assert(tc_split_exact(256), "slice products must accumulate exactly in FP32 for K = 256");
static_assert(kTcAccs * kTcN <= kTcTmemCols, "the accumulators fit the TMEM allocation");

struct TcArgs {
  LinArgs st;
  const __nv_bfloat16* sa;  // slices of A, chunk images (tc_tile_index, 128-row tiles)
  const int32_t* ea;        // [D]          row exponents of A
  const __nv_bfloat16* sy;  // slices of the stage inputs, chunk images (64-system tiles, padded)
  const int32_t* ey;        // [n]          system exponents
  int stage;                // the product written: K[stage] = A * (the sliced vector)
  unsigned int* error_flag; // set when a bounded wait gives up
  long long wait_limit;     // SM clock cycles an mbarrier wait may take (about one second)
  int withhold_tmem_full;   // fault injection for tests: the producer never signals the epilogue
};

// --- PTX wrappers -----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor, no swizzle, K-major: lbo = byte distance
// between core matrices along K, sbo = along M/N.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= static_cast<uint64_t>(1) << 46;  // descriptor version for tcgen05
  return d;                             // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor for kind::f16: F32 accumulators, bf16 A and B, both
// K-major, M = 128, N = 64.
__host__ __device__ constexpr uint32_t tc_idesc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(kTcN >> 3) << 17) |
         (static_cast<uint32_t>(kTcM >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

// Waits for the mbarrier phase for at most `limit` SM clock cycles; on
// expiry it raises the error flag and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t phase, unsigned int* error_flag,
                                                  long long limit) {
  const long long start = clock64();
  for (;;) {
    if (clock64() - start > limit) break;
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  atomicExch(error_flag, 1u);
  return false;
}

// 16 consecutive 32-bit TMEM columns of this warp's 32 lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// --- the stage GEMM ------------------------------------------------------------
// Persistent: one CTA per SM walks the (64-system, 128-row) tiles.  K = D is
// staged in chunks of 32 into two buffers, each holding the A slices
// [NS][128 x 32] (8 KiB each) and B slices [NS][64 x 32] (4 KiB each):
// 2 x 72 KiB.  The slices are stored in global memory as images of these
// chunks, so a chunk arrives by two bulk copies (cp.async.bulk, completion
// counted in bytes on the buffer's full barrier) issued by one thread; with
// 16-byte cp.async from every thread, issuing the copies took 4.4k cycles per
// chunk, more than the MMAs.  The chunk after the current one loads while the
// tensor cores work on the current one; the buffer it overwrites is released
// by the mbarrier its last MMAs committed to.  Every wait is bounded.
constexpr int kTcBufBytes = kTcSlices * (kTcM + kTcN) * kTcKc * 2;

// The slices live in global memory as images of the shared-memory chunks:
// chunk c of a tile (128 rows of A, or 64 systems) is kTcSlices blocks of
// (rows x 32) bf16 in the canonical no-swizzle K-major order (8 x 16-byte
// core matrices, K-adjacent core matrices 128 bytes apart, 8-row groups
// kTcKc * 16 bytes apart), back to back.  A chunk is then two contiguous
// copies (A and B parts), issued by one thread.
template <int D>
__device__ __forceinline__ int64_t tc_tile_index(int rows, int64_t r, int s, int k) {
  constexpr int kChunks = D / kTcKc;
  const int64_t tile = r / rows;
  const int m = static_cast<int>(r - tile * rows);
  const int c = k / kTcKc, kk = k % kTcKc;
  const int64_t block = (tile * kChunks + c) * kTcSlices + s;
  return block * (rows * kTcKc) + (m / 8) * (kTcKc * 8) + (kk / 8) * 64 + (m % 8) * 8 + (kk % 8);
}

// One thread: announce a chunk's bytes on the buffer's mbarrier and start
// its two bulk copies (sizes multiples of 16 bytes, addresses 16-byte
// aligned).  Only the leading kSl slices of each operand are copied (they
// come first in a chunk image); the B part starts after room for all of A's.
template <int kSl>
__device__ __forceinline__ void tc_issue_chunk(uint32_t full_bar, unsigned char* dst, const __nv_bfloat16* srcA,
                                               const __nv_bfloat16* srcB) {
  constexpr uint32_t kABytes = kSl * kTcM * kTcKc * 2;
  constexpr uint32_t kBBytes = kSl * kTcN * kTcKc * 2;
  constexpr uint32_t kBOff = kTcSlices * kTcM * kTcKc * 2;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full_bar), "r"(kABytes + kBBytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(srcA), "r"(kABytes), "r"(full_bar)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst + kBOff)),
               "l"(srcB), "r"(kBBytes), "r"(full_bar)
               : "memory");
}

// Warp roles.  Warps 0..7 run the epilogue: warp w reads TMEM lanes
// 32(w%4)..32(w%4)+31 (the rows of its quadrant) for half of the tile's 64
// columns.  Warp 8 is the producer: its lane 0 issues the copies and the MMAs.
// The accumulators are handed over through two mbarriers: tmem_full (the
// tile's last MMAs are done, by tcgen05.commit) and tmem_empty (the epilogue
// warps have read every diagonal into registers).  The FP64 conversion,
// scaling and stores of tile j then run while the MMAs of tile j+1 fill TMEM.
constexpr int kTcEpiWarps = 8;
constexpr int kTcThreads = 32 * (kTcEpiWarps + 1);

__device__ __forceinline__ void tc_epi_sync() {  // named barrier 1: the epilogue warps only
  asm volatile("bar.sync 1, %0;" ::"n"(32 * kTcEpiWarps) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// kDiags: the leading diagonals s + t < kDiags of the slice products that
// are formed (kTcSlices: all 15 pairs, ~2^-39; 2: the pairs (0,0), (0,1),
// (1,0), ~2^-15, for a product that feeds only the error estimate).
template <int D, int kDiags = kTcSlices>
__global__ void __launch_bounds__(kTcThreads, 1) lin_tc_stage_kernel(const TcArgs a) {
  static_assert(kDiags >= 1 && kDiags <= kTcSlices, "diagonals of the slice products");
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  constexpr int kABytes = kTcM * kTcKc * 2;  // 8192
  constexpr int kBBytes = kTcN * kTcKc * 2;  // 4096
  constexpr int kChunks = D / kTcKc;
  constexpr int kKg = kTcKc / 8;
  static_assert(kChunks >= 2 && kChunks % 2 == 0, "every tile starts in buffer 0 of the two-buffer pipeline");
  __shared__ __align__(8) uint64_t mbar[2];      // the MMAs of the buffer's chunk are done
  __shared__ __align__(8) uint64_t full_bar[2];  // the buffer's chunk has arrived
  __shared__ __align__(8) uint64_t tmem_full;    // the tile's accumulators are complete
  __shared__ __align__(8) uint64_t tmem_empty;   // the epilogue has read them
  __shared__ uint32_t tmem_base_sh;
  __shared__ int any_w[2];
  __shared__ int ok_sh;
  __shared__ int tile_live[kTcN];          // the tile's systems: running (and < n)
  __shared__ int tile_ey[kTcN];            // their exponents

  const int tid = threadIdx.x;
  const int warp = tid / 32;
  const int lane = tid % 32;
  const int64_t n = a.st.n;
  const int64_t ntx = (n + kTcN - 1) / kTcN;
  // The row tiles of one system tile are consecutive tiles, so the CTAs that
  // take them run at about the same time and the second read of the system
  // tile's slices hits L2 (at 65,536 systems the slices of all tiles, 168 MB,
  // exceed it).
  constexpr int kRowTiles = D / kTcM;
  const int64_t ntiles = ntx * kRowTiles;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_sh)),
                 "r"(kTcTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full_bar[b])) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&tmem_full)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&tmem_empty)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_sh;

  if (warp == kTcEpiWarps) {
    // ---- producer ----------------------------------------------------------
    // Both roles walk the same tiles and skip the same ones (a tile whose 64
    // systems have all stopped); status is not written during the launch.
    // Lane 0 runs the pipeline: chunk c+1 copies into the other buffer once
    // the MMAs of its last reader are done, chunk c's MMAs are issued when
    // its copies have arrived, and a tile's first MMAs wait until the
    // epilogue has read the previous tile's accumulators.  Every wait is
    // bounded; after a timeout no wait is attempted again until the drain.
    uint32_t phase[2] = {0u, 0u}, fphase[2] = {0u, 0u}, ephase = 0u;
    bool pending[2] = {false, false};   // MMAs committed to mbar[b], not yet waited for
    bool inflight[2] = {false, false};  // copies issued, their arrival not yet waited for
    bool ok = true, first = true;
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int r0 = static_cast<int>(tile % kRowTiles) * kTcM;
      const int64_t s0 = (tile / kRowTiles) * kTcN;
      const int64_t sa0 = s0 + lane, sa1 = s0 + 32 + lane;
      const bool live = (sa0 < n && a.st.status[sa0] == kLinRunning) || (sa1 < n && a.st.status[sa1] == kLinRunning);
      if (!__any_sync(0xffffffffu, live)) continue;
      if (lane == 0) {
        const __nv_bfloat16* srcA = a.sa + static_cast<int64_t>(r0 / kTcM) * kChunks * kTcSlices * (kTcM * kTcKc);
        const __nv_bfloat16* srcB = a.sy + static_cast<int64_t>(s0 / kTcN) * kChunks * kTcSlices * (kTcN * kTcKc);
        constexpr int64_t kAChunk = kTcSlices * kTcM * kTcKc, kBChunk = kTcSlices * kTcN * kTcKc;  // elements
        auto load = [&](int b, int c) {
          if (pending[b]) {
            if (ok && !mbar_wait_bounded(smem_addr(&mbar[b]), phase[b], a.error_flag, a.wait_limit)) ok = false;
            phase[b] ^= 1u;
            pending[b] = false;
          }
          if (ok) {
            tc_issue_chunk<kDiags>(smem_addr(&full_bar[b]), tc_smem + b * kTcBufBytes, srcA + c * kAChunk,
                                   srcB + c * kBChunk);
            inflight[b] = true;
          }
        };
        load(0, 0);
        // unrolled, so the buffer index and the per-buffer phases are
        // compile-time (registers, not a stack frame)
#pragma unroll
        for (int c = 0; c < kChunks; ++c) {
          const int buf = c & 1;
          if (c + 1 < kChunks) load(buf ^ 1, c + 1);
          if (ok) {
            if (mbar_wait_bounded(smem_addr(&full_bar[buf]), fphase[buf], a.error_flag, a.wait_limit)) inflight[buf] = false;
            else ok = false;
            fphase[buf] ^= 1u;
          }
          if (ok && c == 0 && !first) {
            if (!mbar_wait_bounded(smem_addr(&tmem_empty), ephase, a.error_flag, a.wait_limit)) ok = false;
            ephase ^= 1u;
          }
          if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            constexpr uint32_t idesc = tc_idesc();
            unsigned char* sA = tc_smem + buf * kTcBufBytes;
            unsigned char* sB = sA + kTcSlices * kABytes;
            // One descriptor per operand buffer; each MMA's operand is a
            // compile-time byte offset from it, added to the 14-bit
            // start-address field (addresses stay below 228 KiB, so the
            // field never carries).
            const uint64_t a0 = umma_desc(smem_addr(sA), 128, kKg * 128);
            const uint64_t b0 = umma_desc(smem_addr(sB), 128, kKg * 128);
#pragma unroll
            for (int ks = 0; ks < kTcKc / 16; ++ks) {
#pragma unroll
              for (int s = 0; s < kDiags; ++s) {
#pragma unroll
                for (int t = 0; s + t < kDiags; ++t) {
                  const int ac = tc_acc(s, t);
                  const uint64_t ad = a0 + static_cast<uint64_t>((s * kABytes + ks * 256) >> 4);
                  const uint64_t bd = b0 + static_cast<uint64_t>((t * kBBytes + ks * 256) >> 4);
                  // The first product into an accumulator (its first pair
                  // of the first K step) overwrites it.
                  const uint32_t acc = (c == 0 && ks == 0 && s == tc_acc_first_s(ac)) ? 0u : 1u;
                  tc_mma(tmem + static_cast<uint32_t>(ac * kTcN), ad, bd, idesc, acc);
                }
              }
            }
            tc_commit(smem_addr(&mbar[buf]));
            pending[buf] = true;
            if (c + 1 == kChunks && !a.withhold_tmem_full) tc_commit(smem_addr(&tmem_full));
          }
        }
      }
      first = false;
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    }
    if (lane == 0) {
      // drain (bounded): the MMAs and the copies still in flight into this
      // CTA's shared memory and tensor memory
#pragma unroll
      for (int b = 0; b < 2; ++b)
        if (pending[b]) mbar_wait_bounded(smem_addr(&mbar[b]), phase[b], a.error_flag, a.wait_limit);
#pragma unroll
      for (int b = 0; b < 2; ++b)
        if (inflight[b]) mbar_wait_bounded(smem_addr(&full_bar[b]), fphase[b], a.error_flag, a.wait_limit);
    }
  } else {
    // ---- epilogue ----------------------------------------------------------
    // Warps 0..3 own TMEM lanes (rows) 32w..32w+31 for columns 0..31, warps
    // 4..7 the same rows for columns 32..63.  Every decision that ends or
    // skips an iteration is read from shared memory after a barrier of all
    // 256 epilogue threads, so they all take the same path.
    const int rw = warp % 4;
    const int cbase = (warp / 4) * 32;
    uint32_t tphase = 0u;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      const int r0 = static_cast<int>(tile % kRowTiles) * kTcM;
      const int64_t s0 = (tile / kRowTiles) * kTcN;
      tc_epi_sync();  // the previous tile's readers of tile_* are done
      if (tid < kTcN) {
        // the epilogue's per-system data, read once per tile
        const int64_t sys = s0 + tid;
        const bool live = sys < n && a.st.status[sys] == kLinRunning;
        tile_live[tid] = live ? 1 : 0;
        tile_ey[tid] = live ? a.ey[sys] : 0;
        const bool any = __any_sync(0xffffffffu, live);
        if (lane == 0) any_w[warp] = any ? 1 : 0;
      }
      tc_epi_sync();
      if (!(any_w[0] | any_w[1])) continue;  // the producer skips it too
      if (tid == 0) ok_sh = mbar_wait_bounded(smem_addr(&tmem_full), tphase, a.error_flag, a.wait_limit) ? 1 : 0;
      tc_epi_sync();
      tphase ^= 1u;
      if (!ok_sh) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // An accumulator of diagonal d holds an integer (exact below 2^24 for
      // d <= 2, at most ~2^26.4 for d = 3, 4) scaled by 2^(-8(d+2)): the sum
      // over the accumulators, each shifted by 8(4 - d), is a 64-bit integer
      // (below 2^57) times 2^-48.
      long long acc[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) acc[j] = 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int ac = 0; ac < kTcAccs; ++ac) {
          if (tc_acc_diag(ac) >= kDiags) continue;  // not formed (compile time)
          float v[16];
          tmem_ld16(tmem + (static_cast<uint32_t>(rw * 32) << 16) + static_cast<uint32_t>(ac * kTcN + cbase + 16 * h),
                    v);
#pragma unroll
          for (int j = 0; j < 16; ++j)
            acc[16 * h + j] += static_cast<long long>(__float2int_rz(v[j]))
                               << (kTcBits * (kTcSlices - 1 - tc_acc_diag(ac)));
        }
      }
      // hand the accumulators back to the producer
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      tc_epi_sync();
      if (tid == 0) mbar_arrive(smem_addr(&tmem_empty));
      const int row = r0 + rw * 32 + lane;
      const int erow = a.ea[row];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int col = cbase + j;
        if (!tile_live[col]) continue;
        const int64_t sys = s0 + col;
        const int pe = erow + tile_ey[col] - kTcBits * (kTcSlices + 1);
        const double x = __ll2double_rn(acc[j]);
        // x 2^pe: a product by a normal power of two, exact unless the result
        // is subnormal; outside that exponent range ldexp rounds once
        const double k = (pe >= -1022 && pe <= 1023)
                             ? x * __longlong_as_double(static_cast<long long>(pe + 1023) << 52)
                             : ldexp(x, pe);
        a.st.K[(static_cast<int64_t>(a.stage) * n + sys) * D + row] = k;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
  }
}

// Integer slicing.  With e the exponent of the largest |x| of a row (or a
// system), |x| / 2^e < 1 and its first 40 fraction bits, F = floor(|x| *
// 2^(40-e)), are the mantissa shifted right; slice s is bits 39-8s..32-8s of
// F with the sign of x.  This equals truncating 256 r, r -= trunc, five times
// in FP64 (every step of that is exact), without the FP64 instructions GB300
// runs at 1/64 of its integer rate.  Returns e for the largest magnitude bits.
__device__ __forceinline__ int tc_exponent_of(unsigned long long max_abs_bits) {
  // max_abs_bits = bits of the largest |x|; e with |x| < 2^e, 0 for zero
  if (max_abs_bits == 0ull) return 0;
  const int ex = static_cast<int>(max_abs_bits >> 52);
  if (ex == 0) return -1010 - __clzll(static_cast<long long>(max_abs_bits));  // subnormal: top bit p, 2^(p-1074)
  return ex - 1022;  // |x| in [2^(ex-1023), 2^(ex-1022))
}

__device__ __forceinline__ void tc_slices(double x, int e, __nv_bfloat16 (&q)[kTcSlices]) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const int ex = static_cast<int>((b >> 52) & 0x7ff);
  const unsigned long long m = (b & 0xfffffffffffffull) | (ex ? (1ull << 52) : 0ull);
  // |x| = m * 2^(ex' - 1075) with ex' = max(ex, 1); F = m * 2^(ex' - 1075 + 40 - e)
  const int sh = 1075 - kTcFracBits + e - (ex ? ex : 1);  // right shift, >= 13 since |x| < 2^e
  const unsigned long long F = sh >= 64 ? 0ull : (m >> sh);
  const bool neg = (b >> 63) != 0ull;
#pragma unroll
  for (int s = 0; s < kTcSlices; ++s) {
    const int v = static_cast<int>((F >> (kTcFracBits - kTcBits * (s + 1))) & ((1ull << kTcBits) - 1ull));
    q[s] = __float2bfloat16_rz(static_cast<float>(neg ? -v : v));
  }
}

__device__ __forceinline__ unsigned long long tc_abs_bits(double x) {
  return static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffull;
}

// Slices of a vector per system (the GEMM's B operand), one warp per system.
// Lane l owns the PER = D/32 consecutive elements from PER*l: it loads them
// as 16-byte vectors and writes each slice's PER bf16 values with one store
// (16 bytes for D = 256, 8 for D = 128), since in a chunk image the K index
// is contiguous in runs of 8.
template <int PER>
struct TcSliceVec;
template <>
struct TcSliceVec<8> {
  using T = uint4;
};
template <>
struct TcSliceVec<4> {
  using T = uint2;
};

template <int PER>
__device__ __forceinline__ void tc_load_run(const double* p, double (&v)[PER]) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < PER / 2; ++i) {
    const double2 x = q[i];
    v[2 * i] = x.x;
    v[2 * i + 1] = x.y;
  }
}

// The slices of a system's PER values from PER*lane (one warp per system,
// every lane of the warp calling it) and its exponent.
template <int D>
__device__ __forceinline__ int tc_slice_values(const double (&v)[D / 32], __nv_bfloat16 (&qs)[D / 32][kTcSlices]) {
  constexpr int PER = D / 32;
  unsigned long long mx = 0ull;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const unsigned long long ab = tc_abs_bits(v[i]);
    mx = ab > mx ? ab : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = other > mx ? other : mx;
  }
  const int e = tc_exponent_of(mx);
#pragma unroll
  for (int i = 0; i < PER; ++i) tc_slices(v[i], e, qs[i]);
  return e;
}

// Slices of the vectors x (per system contiguous, [n][D]) of the running
// systems: y, or the product v_k = A^k y for the next one.  A block of eight
// warps takes eight consecutive systems, one each.  In a chunk image those
// eight systems' entries of one (chunk, slice) block are one contiguous run
// of 8 x 32 values (512 B), so the warps assemble the runs in shared memory
// and the block writes them with whole 16-byte stores across lines, instead
// of every lane scattering 16 bytes into eight different 128-byte lines.
// Systems that are not running (or past n) get zero slices: the GEMM's
// epilogue skips their columns.
template <int D>
__global__ void __launch_bounds__(256) lin_tc_slice_vec_kernel(const TcArgs a, const double* x, __nv_bfloat16* sy,
                                                               int32_t* ey) {
  constexpr int PER = D / 32;
  constexpr int kChunks = D / kTcKc;
  constexpr int kRun = kTcKc * 8;  // values of one (chunk, slice) run of 8 systems
  static_assert(PER == 4 || PER == 8, "vector stores of 8 or 16 bytes");
  static_assert(kTcN % 8 == 0, "8-system groups within a tile");
  using Vec = typename TcSliceVec<PER>::T;
  __shared__ __align__(16) __nv_bfloat16 staged[kChunks * kTcSlices * kRun];
  const unsigned lane = threadIdx.x & 31u;
  const int w = static_cast<int>(threadIdx.x >> 5);
  const int64_t first = static_cast<int64_t>(blockIdx.x) * 8;
  const int64_t sys = first + w;
  const bool run = sys < a.st.n && a.st.status[sys] == kLinRunning;  // the same for the whole warp
  __nv_bfloat16 qs[PER][kTcSlices];
  if (run) {
    double v[PER];
    tc_load_run<PER>(x + sys * D + PER * lane, v);
    const int e = tc_slice_values<D>(v, qs);
    if (lane == 0) ey[sys] = e;
  } else {
#pragma unroll
    for (int i = 0; i < PER; ++i)
#pragma unroll
      for (int q = 0; q < kTcSlices; ++q) qs[i][q] = __float2bfloat16_rz(0.0f);
  }
  // this lane's PER values are contiguous in the run: chunk c, at
  // (kk / 8) * 64 + w * 8 + kk % 8 for its first K index kk in the chunk
  const int k0 = PER * static_cast<int>(lane);
  const int c = k0 / kTcKc, kk = k0 % kTcKc;
  const int intra = (kk / 8) * 64 + w * 8 + (kk % 8);
#pragma unroll
  for (int q = 0; q < kTcSlices; ++q) {
    union {
      Vec vec;
      __nv_bfloat16 h[PER];
    } u;
#pragma unroll
    for (int i = 0; i < PER; ++i) u.h[i] = qs[i][q];
    *reinterpret_cast<Vec*>(staged + (c * kTcSlices + q) * kRun + intra) = u.vec;
  }
  __syncthreads();
  const int64_t tile = first / kTcN;
  const int group = static_cast<int>((first % kTcN) / 8);
  constexpr int kVecs = kRun / 8;  // 16-byte stores per run
  for (int i = static_cast<int>(threadIdx.x); i < kChunks * kTcSlices * kVecs; i += 256) {
    const int region = i / kVecs, part = i % kVecs;  // region = chunk * kTcSlices + slice
    const int64_t block = tile * (kChunks * kTcSlices) + region;
    uint4* dst = reinterpret_cast<uint4*>(sy + block * (kTcN * kTcKc) + group * kRun) + part;
    *dst = reinterpret_cast<const uint4*>(staged + region * kRun)[part];
  }
}

// Slices of A, one warp per row (computed once per solve).
template <int D>
__global__ void __launch_bounds__(256) lin_tc_slice_a_kernel(const double* A, __nv_bfloat16* sa, int32_t* ea) {
  constexpr int PER = D / 32;
  const unsigned lane = threadIdx.x & 31u;
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  if (row >= D) return;
  double v[PER];
  unsigned long long mx = 0ull;
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    v[q] = A[static_cast<int64_t>(row) * D + lane + 32 * q];
    const unsigned long long ab = tc_abs_bits(v[q]);
    mx = ab > mx ? ab : mx;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = other > mx ? other : mx;
  }
  const int e = tc_exponent_of(mx);
  if (lane == 0) ea[row] = e;
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    __nv_bfloat16 qs[kTcSlices];
    tc_slices(v[q], e, qs);
#pragma unroll
    for (int s = 0; s < kTcSlices; ++s) sa[tc_tile_index<D>(kTcM, row, s, lane + 32 * q)] = qs[s];
  }
}

}  // namespace bacon
