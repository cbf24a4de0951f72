// K4: split-precision matrix triple product on the 5th-generation tensor
// cores (tcgen05 + TMEM + TMA), sm_103a.
//
// lentil's dft2 (lentil/fourier.py:95-101) computes F = E1 . f . E2 in
// complex128.  Here each complex GEMM runs as ONE real GEMM over a block
// embedding of the complex operands (layouts in dft_matrices.cu), and every
// real operand is split into two 16-bit floats x = hi + lo.  The product is
//     A_hi.B_hi + (A_hi.B_lo + A_lo.B_hi)            (lo.lo is below 2^-16)
//
//   stage 1:  G = E1 . f     A = E1 block, B = f^T (split, transposed)
//             epilogue: scale, split, write G as stage 2's A operand
//   stage 2:  F = G . E2     A = G, B = E2 block
//             epilogue: weight * |F|^2 reduced (red.v4.f32) into the image
//             window, or a complex128 write of F (single dft2)
//
// Accumulation.  The tensor core's FP32 accumulate rounds toward zero on
// every MMA, a bias that grows with the length of the accumulation chain
// (measured: 1.8e-5 relative at K = 2048 with one chain per tile).  So the
// chains are short: with fp16 operands every 64-wide K block is its own chain
// (12 MMAs: 4 k-steps x 3 split products, the small cross terms hi.lo + lo.hi
// first and the dominant hi.hi last, so that only the last 4 MMAs round at
// full magnitude); with bf16 operands two consecutive K blocks share one
// chain, which halves the drains and lets the MMA run twice as far ahead
// while the epilogue writes an item's output (+4.7 % on the broadband
// workload; its error vs the complex128 plan goes from 3.5e-7 to 6.8e-7).
// The chains alternate between two TMEM accumulators, and the epilogue warps
// fold each into round-to-nearest FP32 registers while the MMA fills the
// other one.
//
// CTA pairs (cta_group::2).  Two CTAs of a cluster run on a TPC's two SMs
// and compute one 256 x 256 output tile together: CTA r holds rows
// 128r..128r+127 of the A tile and rows 128r..128r+127 of the B tile in its
// own shared memory, and one tcgen05.mma (M=256, N=256, K=16) issued by the
// even CTA reads both halves.  Each SM thus fetches 64 KB per 64-wide K block
// instead of the 96 KB a lone M=128 x N=256 CTA needs for the same MMA work,
// and three stages fit in shared memory.
//
// Warp roles (320 threads per CTA, one CTA per SM, persistent over items):
//   warp 0       TMA producer (one lane), in both CTAs
//   warp 1       TMEM allocator in both CTAs; MMA issuer (one lane) in the
//                even CTA only
//   warps 2..9   epilogue: warp w owns TMEM lanes 32*(w%4).. and the
//                column half (w-2)/4 of the 256-column tile, in both CTAs
// TMEM accumulators X0 = cols 0..255, X1 = cols 256..511 in each CTA (its
// 128 rows); a 3-stage 64 KB smem ring per CTA (A_hi, A_lo, B_hi, B_lo halves).
// Barriers: a stage's "full" barrier lives in the even CTA and counts both
// CTAs' bytes; "empty" and "accumulator ready" are signalled to both CTAs by
// multicast commits; "accumulator drained" lives in the even CTA and counts
// the epilogue warps of both.
// Every mbarrier wait is bounded in time; on expiry the kernel records
// LGB_ETIMEOUT in a device flag, drains what it issued and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <map>
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {
namespace tc {

constexpr int BM = 128;                                    // A rows per CTA (256 per pair)
constexpr int BK = 64;
constexpr int KSTEPS = BK / 16;                            // MMA k-steps per K block
constexpr uint32_t A_BYTES = BM * BK * 2;                  // 16 KB per plane
constexpr uint32_t BAR_BYTES = 128;
constexpr int EPI_WARPS = 8;
constexpr int NUM_THREADS = 64 + 32 * EPI_WARPS;
constexpr uint32_t STG_BYTES = 4096;                       // output staging per epilogue warp
constexpr unsigned long long WAIT_NS = 2000000000ull;      // default 2 s bound on any wait
// K blocks per accumulator drain (the kernel's KB template argument): 2 for
// bf16 operands when every PSF of the launch carries many wavelengths (the
// fast form: half the drains, and twice the MMA run-ahead across an item's
// output pass; the longer chains' round-toward-zero bias is left in, while
// the band averages the representation error down), 1 otherwise and always
// for fp16 (the shortest round-toward-zero chains).  A compile-time value:
// the single MMA-issuing thread is on the critical path, and runtime chain
// bookkeeping in its loop measurably slowed the pipe.
constexpr int CHAIN2_MIN_WAVELENGTHS = 16;     // wavelengths per PSF for 2-block bf16 chains

// Pair-tile width: 256 output columns (the fast shape for large transforms:
// each A tile feeds twice the MMA work) or 128 (twice the tiles, for launches
// too small to fill every CTA pair).  The autotuner at the end of this file
// picks one per launch shape.  Both use the same 192 KB operand ring.
template <int BN_>
struct TileCfg {
  static constexpr int BN = BN_;                           // output columns per pair tile
  static constexpr int BNC = BN / 2;                       // B rows held per CTA
  static constexpr int STAGES = BN == 256 ? 3 : 4;
  static constexpr uint32_t B_BYTES = BNC * BK * 2;        // 16 / 8 KB per plane
  static constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // 64 / 48 KB per CTA
  static constexpr uint32_t ACC_COLS = BN;                 // one accumulator: 128 lanes x BN fp32
  static constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;      // double-buffered
  static constexpr int RUN = BN / 2;                       // accumulator columns per epilogue warp
  static constexpr uint32_t SMEM_BYTES =
      STAGES * STAGE_BYTES + EPI_WARPS * STG_BYTES + BAR_BYTES + 1024;
};
static_assert(TileCfg<256>::SMEM_BYTES <= 232448 && TileCfg<128>::SMEM_BYTES <= 232448,
              "shared memory per CTA");

struct Params {
  int stage;                 // 1 or 2
  int kblocks;               // K / 64
  int m_tiles, n_tiles;      // pair tiles: 256 A rows x 256 output columns
  int n_items;               // Q * m_tiles * n_tiles
  int L;
  uint32_t idesc;
  int M, N;                  // stage 1: rows of G / stage 2: window shape
  int kp_out;                // stage 1: row half-width of G (kp2)
  int n_last;                // MMA N of the last column tile (<= 256, multiple of 32)
  float sG;                  // stage-2 operand scale (power of two)
  uint16_t* g_hi;
  uint16_t* g_lo;
  const float* maxabs;       // [batch], or null (operands not scaled)
  int epilogue;              // stage 2: 0 intensity, 1 complex
  const double* weights;     // [batch][L] or null
  const double* unit2;       // [L]
  float* wbuf;               // stage 2 intensity: [batch][M][ldw] FP32 window
  int ldw;
  double* out;               // stage 2 complex: [Q][M][N] complex128
  double cscale;
  int* err;
  const int* lam_idx;        // [L] wavelength -> DFT-matrix slot, or null (identity)
  const uint8_t* kflags;     // stage 1: field nonzero flags [batch][kf_units][kf_pitch], or null
  int kf_units;              // kp1 / 32 (== kblocks)
  int kf_pitch;
  unsigned long long wait_ns;  // bound on every mbarrier wait
  // test of the bounded waits: the producers arrive on the full barrier of
  // K block stall_kb of item stall_item without issuing its loads, so that
  // barrier never completes (-1: no such item)
  int stall_item, stall_kb;
};

// MMA N of column tile tn: BN, except a narrower last tile when the
// operand's columns end inside it (no MMA work on padding columns).  The
// pair splits a tile's B rows evenly: CTA r holds rows r*N/2 .. of it.
template <int BN>
__device__ __forceinline__ int tile_n(const Params& p, int tn) {
  return tn == p.n_tiles - 1 ? p.n_last : BN;
}

__device__ __forceinline__ int matrix_slot(const Params& p, int lam) {
  return p.lam_idx ? p.lam_idx[lam] : lam;
}

// ------------------------------------------------------------------ PTX ---
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: true when the phase completed, false on time-out (recorded
// as LGB_ETIMEOUT) or when another role already flagged an error.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err,
                                          unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  for (uint32_t n = 1;; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 63) == 0) {
      if (*(volatile int*)err != 0) return false;
      if (gtimer() - t0 > limit_ns) {
        atomicCAS(err, 0, LGB_ETIMEOUT);
        return false;
      }
    }
  }
}
// Wait for work this CTA already issued (TMA loads in flight, MMAs) before
// leaving: bounded in time only, whatever the error flag says, so that a
// launch that gave up still retires its copies and MMAs before its shared
// memory and TMEM are released.  Copies and MMAs that were issued complete
// on their own; only a barrier whose loads were never issued (the stall
// test) runs out, after limit_ns.
__device__ __forceinline__ void mbar_wait_issued(uint32_t bar, uint32_t parity,
                                                 unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return;
  const uint64_t t0 = gtimer();
  for (uint32_t n = 1;; ++n) {
    if (mbar_try_wait(bar, parity)) return;
    if ((n & 63) == 0 && gtimer() - t0 > limit_ns) return;
  }
}
// Shared-memory address of the same variable in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t map_to_cta(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// arrive (+ expected bytes) on a barrier given by its cluster address.
// Default (CTA-scope release) semantics: what these arrivals publish needs no
// cluster-wide fence -- the producer has written nothing the consumer reads,
// and an epilogue's TMEM reads are complete at tcgen05.wait::ld, ordered
// against the next MMA by the tcgen05 fences around the barrier.  (A
// cluster-scope release here stalled every epilogue warp on a memory barrier
// once per K block: measured 11 % of the whole step.)
__device__ __forceinline__ void mbar_expect_tx_cluster(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cluster.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(bar) : "memory");
}
// TMA tile load into this CTA's shared memory, completion counted on a
// barrier of either CTA of the pair (cluster address).
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}
// Bulk tensor store / FP32 reduce-add of a swizzled shared-memory tile
// (async proxy; completion tracked by bulk groups of the issuing thread).
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, uint32_t src, int x, int y, int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(src), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap* map, uint32_t src, int x, int y,
                                                  int z) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(src), "r"(x), "r"(y), "r"(z)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory sources of this thread's bulk groups may be overwritten
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// this thread's bulk groups have completed their global writes
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// K-major operand tile with the 128-byte swizzle TMA writes: rows of 64
// 16-bit elements (128 B), 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                             // leading byte offset (unused, SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                   // stride byte offset: 8-row group pitch
  d |= (uint64_t)1 << 46;                             // descriptor version
  d |= (uint64_t)2 << 61;                             // 128-byte swizzle
  return d;
}
// D[256 x 256] (+)= A[256 x 16] . B[256 x 16]^T over the CTA pair: each CTA
// supplies 128 rows of A and 128 rows of B at the same shared-memory offset.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
// arrive once on the barrier at this offset in both CTAs when the MMAs
// issued so far have completed
__device__ __forceinline__ void mma_commit_pair(uint32_t bar) {
  const uint16_t both = 3;
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(bar), "h"(both)
      : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b),
               "f"(c), "f"(d)
               : "memory");
}

// ------------------------------------------------------------ schedule ---
// Work item i -> problem q (PSF-major, then wavelength) and output tile.
struct Item {
  int q, lam, psf, tm, tn;
};

__device__ __forceinline__ Item decode(const Params& p, int i) {
  Item it;
  const int tiles = p.m_tiles * p.n_tiles;
  it.q = i / tiles;
  const int t = i - it.q * tiles;
  it.tm = t % p.m_tiles;
  it.tn = t / p.m_tiles;
  it.psf = it.q / p.L;
  it.lam = it.q - it.psf * p.L;
  return it;
}

// ------------------------------------------------------ K-block skipping ---
// Stage 1 with field flags: a K block whose field rows are zero across the
// item's whole column tile adds nothing and is skipped, by the producer, the
// MMA issuer and the epilogues alike (each derives the same set from the
// same flags).  K block kb covers the 32-row K units 2kb and 2kb + 1; K unit
// u is field unit u mod kf_units (the real rows, then the imaginary rows).
// Up to 128 K blocks are tracked; beyond that the host passes no flags.
struct Live {
  uint64_t lo, hi;           // bit kb: K block kb is issued
  int n;                     // K blocks issued
  bool all;
};

// Warp-collective (all 32 lanes, same item): lane l loads the flags of
// field units l, l+32, l+64, l+96 of the item's column tile at once, the
// ballots give the unit bitmask, and lane l then decides K blocks l, l+32,
// ... from it; every lane returns the same set.  One round of loads per
// item, where a single thread walking the units took up to 128.
template <int BN>
__device__ __forceinline__ Live live_kblocks(const Params& p, const Item& w) {
  Live lv{~0ull, ~0ull, p.kblocks, true};
  if (!p.kflags) return lv;
  const int lane = threadIdx.x & 31;
  const int U = p.kf_units;
  const uint8_t* f = p.kflags + (size_t)w.psf * U * p.kf_pitch + w.tn * (BN / 32);
  uint32_t unit[4];                          // bit l of unit[g]: field unit 32g + l is nonzero
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const int u = 32 * g + lane;
    bool nz = false;
    if (u < U) {
      const uint8_t* fu = f + (size_t)u * p.kf_pitch;
      nz = BN == 256 ? __ldg(reinterpret_cast<const unsigned long long*>(fu)) != 0ull
                     : __ldg(reinterpret_cast<const unsigned int*>(fu)) != 0u;
    }
    unit[g] = __ballot_sync(0xffffffffu, nz);
  }
  auto unit_nz = [&](int u) -> uint32_t {      // u < 2U: the imaginary rows wrap onto unit u - U
    if (u >= U) u -= U;
    const uint32_t word = u < 32 ? unit[0] : u < 64 ? unit[1] : u < 96 ? unit[2] : unit[3];
    return (word >> (u & 31)) & 1u;              // (selects, not an indexed load: registers)
  };
  uint32_t live[4];
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const int kb = 32 * g + lane;
    const bool on = kb < p.kblocks && (unit_nz(2 * kb) | unit_nz(2 * kb + 1));
    live[g] = __ballot_sync(0xffffffffu, on);
  }
  lv.lo = live[0] | ((uint64_t)live[1] << 32);
  lv.hi = live[2] | ((uint64_t)live[3] << 32);
  lv.n = __popcll(lv.lo) + __popcll(lv.hi);
  lv.all = false;
  return lv;
}

__device__ __forceinline__ bool is_live(const Live& lv, int kb) {
  return lv.all || (((kb < 64 ? lv.lo >> kb : lv.hi >> (kb - 64)) & 1ull) != 0);
}

// ------------------------------------------------------------- epilogue ---
// Drain this warp's RUN accumulator columns into the running sums (round to
// nearest).  Columns: ch*RUN.. of the tile, except for 128-wide stage-2
// tiles, whose real parts (the even CTA's B rows) fill columns 0..63 and
// imaginary parts 64..127: there warp half ch takes real columns ch*32..
// and the matching imaginary columns 64 + ch*32.., so that each thread holds
// whole complex values.  One 32-column load in flight keeps the epilogue
// within the 168 registers a thread gets when three warps share an SM
// sub-partition.
template <int RUN>
__device__ __forceinline__ void drain_add(uint32_t trow, int stage, int ch, float (&run)[RUN]) {
#pragma unroll
  for (int h = 0; h < RUN / 32; ++h) {
    const int col = (RUN == 64 && stage == 2) ? h * 64 + ch * 32 : ch * RUN + h * 32;
    uint32_t a[32];
    tmem_ld32(trow + col, a);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < 32; ++j) run[h * 32 + j] += __uint_as_float(a[j]);
  }
}

// Output stores go through a 4 KB shared-memory slice per epilogue warp
// (1024-byte aligned): the warp writes its 32 rows (one per lane) of 16-byte
// chunks into the slice in the swizzled layout of a TMA box (16-byte chunk
// index XOR-ed with the row bits, which also keeps both the writes and the
// TMA read free of bank conflicts), and one lane hands the box to a bulk
// tensor store (stage 1) or FP32 bulk reduce-add (stage 2).  The copies run
// asynchronously; the warp returns to draining the next item and waits for
// the TMA to have read the slice only before it rewrites it.  TMA clips the
// rows past M and the columns past the tensor's extent.
// Stage 1: G rows (split into hi/lo planes) = the stage-2 A operand, as two
// 32 x 32 boxes (64-byte rows, 64-byte swizzle) per pass.  A warp's 32 rows
// are 32 consecutive complex rows u with one plane half h.
template <bool BF16, int BN, int RUN>
__device__ __forceinline__ void write_stage1(const Params& p, const Item& w, int row, int ch,
                                             const float (&run)[RUN], uint8_t* stg,
                                             const CUtensorMap* map_hi, const CUtensorMap* map_lo) {
  const int lane = row & 31;
  const int h = row >> 6;
  const int u0 = w.tm * 64 + (row & 63) - lane;            // first row of this warp
  const int c0 = w.tn * BN + ch * RUN;
  const uint32_t s_hi = smem_u32(stg), s_lo = s_hi + 2048;
#pragma unroll
  for (int cc = 0; cc < RUN / 32; ++cc) {
    if (c0 + cc * 32 >= p.kp_out) break;                   // uniform over the warp
    if (lane == 0) bulk_wait_read();                       // previous box read out of the slice
    __syncwarp();
#pragma unroll
    for (int v8 = 0; v8 < 4; ++v8) {
      uint32_t ph[4], pl[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = cc * 32 + v8 * 8 + 2 * j;
        Split16x2<BF16>::split(run[k] * p.sG, run[k + 1] * p.sG, ph[j], pl[j]);
      }
      const uint32_t slot = lane * 64 + ((v8 ^ ((lane >> 1) & 3)) << 4);
      *reinterpret_cast<uint4*>(stg + slot) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
      *reinterpret_cast<uint4*>(stg + 2048 + slot) = make_uint4(pl[0], pl[1], pl[2], pl[3]);
    }
    fence_async_smem();
    __syncwarp();
    if (lane == 0) {
      const int x = h * p.kp_out + c0 + cc * 32;
      tma_store_3d(map_hi, s_hi, x, u0, w.q);
      tma_store_3d(map_lo, s_lo, x, u0, w.q);
      bulk_commit();
    }
  }
}

// Stage 2: a warp holds HALF = RUN/2 complex output columns
// v = tn*(BN/2) + ch*HALF + j, real parts in run[0, HALF), imaginary in
// run[HALF, RUN).  Intensity: 32 x 32 FP32 boxes (128-byte rows, 128-byte
// swizzle) reduce-added into the window.
template <int BN, int RUN>
__device__ __forceinline__ void write_stage2(const Params& p, const Item& w, int row, int ch,
                                             const float (&run)[RUN], uint8_t* stg,
                                             const CUtensorMap* map_w) {
  constexpr int HALF = RUN / 2;
  const int lane = row & 31;
  const int u = w.tm * BM + row, u0 = u - lane;
  const float sf = p.maxabs ? pow2_scale_for(p.maxabs[w.psf]) : 1.f;   // none: unscaled (bf16)
  const int v0 = w.tn * (BN / 2) + ch * HALF;
  if (p.epilogue == 0) {
    const float inv = 1.f / (sf * p.sG);
    const double wt = p.weights ? p.weights[(size_t)w.psf * p.L + w.lam] : 1.0;
    const float coef = (float)(wt * p.unit2[matrix_slot(p, w.lam)]) * inv * inv;
    const uint32_t s0 = smem_u32(stg);
#pragma unroll
    for (int cc = 0; cc < HALF / 32; ++cc) {
      if (v0 + cc * 32 >= p.N) break;                      // uniform over the warp
      if (lane == 0) bulk_wait_read();
      __syncwarp();
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        float r4[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int j = cc * 32 + c * 4 + e;
          r4[e] = coef * fmaf(run[j], run[j], run[HALF + j] * run[HALF + j]);
        }
        *reinterpret_cast<float4*>(stg + lane * 128 + ((c ^ (lane & 7)) << 4)) =
            make_float4(r4[0], r4[1], r4[2], r4[3]);
      }
      fence_async_smem();
      __syncwarp();
      if (lane == 0) {
        tma_reduce_add_3d(map_w, s0, v0 + cc * 32, u0, w.psf);
        bulk_commit();
      }
    }
  } else {
    if (u >= p.M) return;
    const double scl = p.cscale / ((double)sf * (double)p.sG);
    double2* outc = reinterpret_cast<double2*>(p.out) + ((size_t)w.q * p.M + u) * p.N;
#pragma unroll
    for (int j = 0; j < HALF; ++j)
      if (v0 + j < p.N) outc[v0 + j] = make_double2(scl * run[j], scl * run[HALF + j]);
  }
}

// -------------------------------------------------------------- kernel ---
template <bool BF16, int BN, int KB>
__global__ void __launch_bounds__(NUM_THREADS, 1)
split_mft_kernel(const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
                 const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo,
                 const __grid_constant__ CUtensorMap tmC0, const __grid_constant__ CUtensorMap tmC1,
                 const Params p) {
  using C = TileCfg<BN>;
  constexpr int STAGES = C::STAGES;
  constexpr uint32_t STAGE_BYTES = C::STAGE_BYTES, B_BYTES = C::B_BYTES, ACC_COLS = C::ACC_COLS;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* const gbase = smem_raw + (base - raw);
  const uint32_t bars = base + STAGES * STAGE_BYTES + EPI_WARPS * STG_BYTES;
  auto full_bar = [&](int s) { return bars + 8u * s; };           // even CTA: both CTAs' bytes
  auto empty_bar = [&](int s) { return bars + 32u + 8u * s; };    // both CTAs
  auto acc_full = [&](int b) { return bars + 64u + 8u * b; };     // accumulator b ready, both CTAs
  auto acc_empty = [&](int b) { return bars + 80u + 8u * b; };    // accumulator b drained, even CTA
  const uint32_t drain_bar = bars + 96u;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + (bars - base) + 112);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();
  const bool leader = rank == 0;
  const int pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full_bar(s), 2);
      mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), 2 * EPI_WARPS);
    }
    mbar_init(drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(C::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync();                        // both CTAs' barriers and TMEM are ready
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------ TMA producer
    // the whole warp walks the items (the live K-block set is a warp
    // collective); lane 0 issues the copies
    if (lane == 0) {
      prefetch_map(&tmA_hi); prefetch_map(&tmA_lo);
      prefetch_map(&tmB_hi); prefetch_map(&tmB_lo);
    }
    uint32_t it = 0;
    bool ok = true;
    for (int i = pair; ok && i < p.n_items; i += npairs) {
      const Item w = decode(p, i);
      const Live lv = live_kblocks<BN>(p, w);
      if (lane == 0) {
        // stage 1: A = E1 block of lam, B = f^T of q; stage 2: A = G of q, B = E2 block of lam
        const int az = p.stage == 1 ? matrix_slot(p, w.lam) : w.q;
        const int bz = p.stage == 1 ? w.q : matrix_slot(p, w.lam);
        const int ay = (2 * w.tm + (int)rank) * BM;
        const int by = w.tn * BN + (int)rank * (tile_n<BN>(p, w.tn) >> 1);
        for (int kb = 0; kb < p.kblocks; ++kb) {
          if (!is_live(lv, kb)) continue;
          const int s = it % STAGES;
          if (!mbar_wait(empty_bar(s), ((it / STAGES) & 1) ^ 1, p.err, p.wait_ns)) { ok = false; break; }
          const uint32_t fb = map_to_cta(full_bar(s), 0);
          mbar_expect_tx_cluster(fb, STAGE_BYTES);
          if (i == p.stall_item && kb == p.stall_kb) { ++it; continue; }   // loads withheld
          const uint32_t sa = base + s * STAGE_BYTES;
          tma_load_3d(sa, &tmA_hi, fb, kb * BK, ay, az);
          tma_load_3d(sa + A_BYTES, &tmA_lo, fb, kb * BK, ay, az);
          tma_load_3d(sa + 2 * A_BYTES, &tmB_hi, fb, kb * BK, by, bz);
          tma_load_3d(sa + 2 * A_BYTES + B_BYTES, &tmB_lo, fb, kb * BK, by, bz);
          ++it;
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0) != 0;
    }
    // every copy of both CTAs has landed before the pair exits (the even
    // CTA's full barriers count the odd CTA's bytes too)
    if (lane == 0 && leader)
      for (uint32_t k = (it > STAGES ? it - STAGES : 0); k < it; ++k)
        mbar_wait_issued(full_bar(k % STAGES), (k / STAGES) & 1, p.wait_ns);
  } else if (warp == 1) {
    // ------------------------------------------------------- MMA issuer
    // (even CTA) the whole warp walks the items (the live K-block set is a
    // warp collective); lane 0 issues the MMAs and the commits
    if (leader) {
      uint32_t it = 0;                       // K blocks issued (stage ring)
      uint32_t gi = 0;                       // accumulator groups issued (accumulator uses)
      bool ok = true;
      for (int i = pair; ok && i < p.n_items; i += npairs) {
        const Item w = decode(p, i);
        const Live lv = live_kblocks<BN>(p, w);
        if (lane == 0) {
          const uint32_t idesc = (p.idesc & ~(0x3Fu << 17)) |
                                 ((uint32_t)(tile_n<BN>(p, w.tn) >> 3) << 17);
          int j = 0;                         // live K blocks of this item issued
          for (int kb = 0; kb < p.kblocks; ++kb) {
            if (!is_live(lv, kb)) continue;
            const int s = it % STAGES, xb = gi & 1;
            const bool first = j % KB == 0;
            const bool last = j % KB == KB - 1 || j == lv.n - 1;
            if (!mbar_wait(full_bar(s), (it / STAGES) & 1, p.err, p.wait_ns)) { ok = false; break; }
            // accumulator xb was drained by both CTAs (its previous group, gi - 2)
            if (first && !mbar_wait(acc_empty(xb), ((gi >> 1) & 1) ^ 1, p.err, p.wait_ns)) { ok = false; break; }
            tc_fence_after();
            const uint32_t sa = base + s * STAGE_BYTES, X = tmem + xb * ACC_COLS;
#pragma unroll
            for (int k = 0; k < KSTEPS; ++k) {   // hi.lo + lo.hi: small terms first
              mma_f16(X, smem_desc(sa + k * 32), smem_desc(sa + 2 * A_BYTES + B_BYTES + k * 32),
                      idesc, (first && k == 0) ? 0u : 1u);
              mma_f16(X, smem_desc(sa + A_BYTES + k * 32), smem_desc(sa + 2 * A_BYTES + k * 32),
                      idesc, 1u);
            }
#pragma unroll
            for (int k = 0; k < KSTEPS; ++k)     // hi.hi last
              mma_f16(X, smem_desc(sa + k * 32), smem_desc(sa + 2 * A_BYTES + k * 32), idesc, 1u);
            mma_commit_pair(empty_bar(s));       // both CTAs' stage s free once these retire
            if (last) {
              mma_commit_pair(acc_full(xb));     // accumulator xb ready for the epilogues
              ++gi;
            }
            ++j;
            ++it;
          }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0) != 0;
      }
      // all issued MMAs have retired before TMEM is released
      if (lane == 0) {
        mma_commit_pair(drain_bar);
        mbar_wait_issued(drain_bar, 0, p.wait_ns);
      }
      __syncwarp();
    }
  } else {
    // --------------------------------------------------------- epilogue
    const int q4 = warp & 3;                 // TMEM lane quadrant of this warp
    const int ch = (warp - 2) >> 2;          // column half of the tile
    const int row = q4 * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(q4 * 32) << 16);
    const uint32_t empty_lead[2] = {map_to_cta(acc_empty(0), 0), map_to_cta(acc_empty(1), 0)};
    uint8_t* const stg = gbase + STAGES * STAGE_BYTES + (warp - 2) * STG_BYTES;
    uint32_t gi = 0;                         // accumulator groups drained
    bool ok = true;
    for (int i = pair; ok && i < p.n_items; i += npairs) {
      Item w = decode(p, i);
      // accumulator groups of the item (none when its field tile is zero:
      // the output tile is then written as zeros)
      const int groups = (live_kblocks<BN>(p, w).n + KB - 1) / KB;
      w.tm = 2 * w.tm + (int)rank;           // this CTA's 128-row tile
      float run[C::RUN];
#pragma unroll
      for (int j = 0; j < C::RUN; ++j) run[j] = 0.f;
      for (int g = 0; g < groups; ++g, ++gi) {
        const int xb = gi & 1;
        ok = __all_sync(0xffffffffu, mbar_wait(acc_full(xb), (gi >> 1) & 1, p.err, p.wait_ns));
        if (!ok) break;
        tc_fence_after();
        drain_add<C::RUN>(trow + xb * ACC_COLS, p.stage, ch, run);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_cluster(empty_lead[xb]);
      }
      if (!ok) break;
      if (p.stage == 1) write_stage1<BF16, BN, C::RUN>(p, w, row, ch, run, stg, &tmC0, &tmC1);
      else write_stage2<BN, C::RUN>(p, w, row, ch, run, stg, &tmC0);
    }
    // the bulk stores / reduce-adds this warp issued have landed
    if (lane == 0) bulk_wait_all();
  }

  tc_fence_before();
  __syncthreads();
  cluster_sync();                        // no CTA leaves while its pair may still use it
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS));
  }
}

// ------------------------------------------------------------------ host ---
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

// 3-D row-major map: dims {K, rows, batch} of elem_bytes-wide elements, box
// {box_k, box_rows, 1}.
static int make_map_any(CUtensorMap* map, const void* ptr, CUtensorMapDataType dtype, int elem_bytes,
                        int K, int rows, int batch, int box_k, int box_rows, CUtensorMapSwizzle swz) {
  auto enc = encode_fn();
  LGB_REQUIRE(enc, LGB_ECUDA, "cuTensorMapEncodeTiled is unavailable");
  LGB_REQUIRE(((uintptr_t)ptr & 15) == 0, LGB_EINVAL, "tensor map base must be 16-byte aligned");
  LGB_REQUIRE(((size_t)K * elem_bytes) % 16 == 0, LGB_EINVAL, "tensor map row pitch must be a multiple of 16 bytes");
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)K * elem_bytes, (cuuint64_t)K * elem_bytes * rows};
  cuuint32_t box[3] = {(cuuint32_t)box_k, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult res = enc(map, dtype, 3, const_cast<void*>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (res != CUDA_SUCCESS)
    return set_error(LGB_ECUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)res));
  return LGB_OK;
}

static CUtensorMapDataType half_type(bool bf16) {
  return bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
}

// K-major 16-bit MMA operand: box {64, box_rows}, 128-byte swizzle.
static int make_map(CUtensorMap* map, const void* ptr, bool bf16, int K, int rows, int batch,
                    int box_rows) {
  LGB_REQUIRE(K % BK == 0, LGB_EINVAL, "tensor map K must be a multiple of 64");
  return make_map_any(map, ptr, half_type(bf16), 2, K, rows, batch, BK, box_rows,
                      CU_TENSOR_MAP_SWIZZLE_128B);
}

}  // namespace tc

int make_field_T_store_map(CUtensorMap* map, const uint16_t* ptr, bool bf16, int kp, int n, int Q) {
  auto enc = tc::encode_fn();
  LGB_REQUIRE(enc, LGB_ECUDA, "cuTensorMapEncodeTiled is unavailable");
  LGB_REQUIRE(((uintptr_t)ptr & 15) == 0, LGB_EINVAL, "tensor map base must be 16-byte aligned");
  LGB_REQUIRE(kp % 32 == 0 && n > 0 && Q > 0, LGB_EINVAL, "split field map: bad shape");
  cuuint64_t dims[4] = {(cuuint64_t)kp, 2, (cuuint64_t)n, (cuuint64_t)Q};
  cuuint64_t strides[3] = {(cuuint64_t)kp * 2, (cuuint64_t)kp * 4, (cuuint64_t)kp * 4 * n};
  cuuint32_t box[4] = {64, 1, 32, 1};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult res = enc(map, tc::half_type(bf16), 4, const_cast<uint16_t*>(ptr), dims, strides, box,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (res != CUDA_SUCCESS)
    return set_error(LGB_ECUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)res));
  return LGB_OK;
}

namespace tc {

constexpr uint32_t make_idesc(bool bf16, int bn) {
  return (1u << 4)                          // D format: FP32
         | ((bf16 ? 1u : 0u) << 7)          // A format: BF16 (1) / FP16 (0)
         | ((bf16 ? 1u : 0u) << 10)         // B format
         | ((uint32_t)(bn >> 3) << 17)      // N = tile width (narrower last tile per item)
         | ((uint32_t)((2 * BM) >> 4) << 24);  // M = 256 (the CTA pair)
}

static cudaLaunchConfig_t pair_config(uint32_t smem, cudaStream_t s, cudaLaunchAttribute* attr) {
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2);
  cfg.blockDim = dim3(NUM_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

template <bool BF16, int BN, int KB>
static cudaError_t set_smem_attr() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    err = cudaFuncSetAttribute(split_mft_kernel<BF16, BN, KB>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)TileCfg<BN>::SMEM_BYTES);
  });
  return err;
}

// Largest number of CTA pairs of this kernel resident at once (per device).
template <bool BF16, int BN, int KB>
static int max_pairs() {
  static std::mutex mu;
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (set_smem_attr<BF16, BN, KB>() != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(mu);
  if (cached[dev] == 0) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = pair_config(TileCfg<BN>::SMEM_BYTES, 0, attr);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, split_mft_kernel<BF16, BN, KB>, &cfg) != cudaSuccess) n = 0;
    cached[dev] = n;
  }
  return cached[dev];
}

template <bool BF16, int BN, int KB>
static int launch_one(const Params& p, const CUtensorMap& a_hi, const CUtensorMap& a_lo,
                      const CUtensorMap& b_hi, const CUtensorMap& b_lo, const CUtensorMap& c0,
                      const CUtensorMap& c1, cudaStream_t s) {
  LGB_CUDA((set_smem_attr<BF16, BN, KB>()));
  if (p.n_items <= 0) return LGB_OK;
  const int pairs = max_pairs<BF16, BN, KB>();
  LGB_REQUIRE(pairs > 0, LGB_ECUDA, "split mft: no CTA pair of the tensor-core kernel fits on this GPU");
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = pair_config(TileCfg<BN>::SMEM_BYTES, s, attr);
  cfg.gridDim = dim3(2 * std::min(p.n_items, pairs));
  LGB_CUDA(cudaLaunchKernelEx(&cfg, split_mft_kernel<BF16, BN, KB>, a_hi, a_lo, b_hi, b_lo, c0, c1, p));
  return LGB_OK;
}

template <int BN>
static int launch_stage(const Params& p, bool bf16, bool chain2, const CUtensorMap* m,
                        cudaStream_t s) {
  if (!bf16) return launch_one<false, BN, 1>(p, m[0], m[1], m[2], m[3], m[4], m[5], s);
  return chain2 ? launch_one<true, BN, 2>(p, m[0], m[1], m[2], m[3], m[4], m[5], s)
                : launch_one<true, BN, 1>(p, m[0], m[1], m[2], m[3], m[4], m[5], s);
}

// Work items and K blocks of each stage at tile width bn.
struct StageShape {
  long long items;
  int kblocks;
};
static void stage_shapes(const SplitMftProblem& q, int bn, StageShape (&st)[2]) {
  const long long Q = (long long)q.batch * q.L;
  st[0].items = Q * cdiv(cdiv(q.M, 64), 2) * cdiv(q.kp2, bn);
  st[0].kblocks = 2 * q.kp1 / BK;
  st[1].items = Q * cdiv(q.M, 2 * BM) * cdiv(q.N, bn / 2);
  st[1].kblocks = 2 * q.kp2 / BK;
}

// One-shot test of the bounded waits (lgb_test_stall_tma): the next stage-1
// launch withholds the loads of one K block and bounds its waits by
// g_stall_wait nanoseconds.
static std::atomic<int> g_stall_item{-1};
static std::atomic<int> g_stall_kb{0};
static std::atomic<unsigned long long> g_stall_wait{WAIT_NS};

// Both stages with pair tiles BN wide; ev (optional [4]) brackets the two
// launches.  Every tensor map is encoded before the first launch, so the
// host leaves no gap between the stages on the stream.
template <int BN>
static int run_split_mft(const SplitMftProblem& q, cudaEvent_t* ev, cudaStream_t s) {
  using C = TileCfg<BN>;
  const int Q = q.batch * q.L;
  const int mrows1 = cdiv(q.M, 64) * 128;      // E1 block rows
  const int nrows2 = cdiv(q.N, 128) * 256;     // E2 block rows
  const int Lm = q.lam_idx ? q.L_bank : q.L;   // DFT-matrix slots held
  CUtensorMap m1[6], m2[6];                    // a_hi, a_lo, b_hi, b_lo, c0, c1 per stage
  StageShape sh[2];
  stage_shapes(q, BN, sh);
  int st;
  // stage 1: G = E1 . f
  if ((st = make_map(&m1[0], q.e1_hi, q.bf16, 2 * q.kp1, mrows1, Lm, BM))) return st;
  if ((st = make_map(&m1[1], q.e1_lo, q.bf16, 2 * q.kp1, mrows1, Lm, BM))) return st;
  if ((st = make_map(&m1[2], q.f_hi, q.bf16, 2 * q.kp1, q.n, Q, C::BNC))) return st;
  if ((st = make_map(&m1[3], q.f_lo, q.bf16, 2 * q.kp1, q.n, Q, C::BNC))) return st;
  if ((st = make_map_any(&m1[4], q.g_hi, half_type(q.bf16), 2, 2 * q.kp2, q.M, Q, 32, 32,
                         CU_TENSOR_MAP_SWIZZLE_64B)))
    return st;
  if ((st = make_map_any(&m1[5], q.g_lo, half_type(q.bf16), 2, 2 * q.kp2, q.M, Q, 32, 32,
                         CU_TENSOR_MAP_SWIZZLE_64B)))
    return st;
  // stage 2: F = G . E2 (+ epilogue)
  if ((st = make_map(&m2[0], q.g_hi, q.bf16, 2 * q.kp2, q.M, Q, BM))) return st;
  if ((st = make_map(&m2[1], q.g_lo, q.bf16, 2 * q.kp2, q.M, Q, BM))) return st;
  if ((st = make_map(&m2[2], q.e2_hi, q.bf16, 2 * q.kp2, nrows2, Lm, C::BNC))) return st;
  if ((st = make_map(&m2[3], q.e2_lo, q.bf16, 2 * q.kp2, nrows2, Lm, C::BNC))) return st;
  m2[4] = m1[4];
  m2[5] = m1[5];
  if (q.epilogue == 0) {
    LGB_REQUIRE(q.ldw % 4 == 0, LGB_EINVAL, "split mft: intensity window pitch must be a multiple of 4");
    if ((st = make_map_any(&m2[4], q.wbuf, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, q.ldw, q.M, q.batch,
                           32, 32, CU_TENSOR_MAP_SWIZZLE_128B)))
      return st;
  }

  // two-block accumulator chains for bf16 PSFs of many wavelengths only
  const bool chain2 = q.bf16 && q.L >= CHAIN2_MIN_WAVELENGTHS;
  Params p{};
  p.stage = 1;
  p.wait_ns = WAIT_NS;
  p.stall_item = g_stall_item.exchange(-1);
  if (p.stall_item >= 0) {
    p.stall_kb = g_stall_kb.load();
    p.wait_ns = g_stall_wait.load();
  }
  p.kblocks = sh[0].kblocks;
  p.m_tiles = cdiv(cdiv(q.M, 64), 2);          // pairs of 64-row (128 block-row) E1 tiles
  p.n_tiles = cdiv(q.kp2, BN);
  p.n_items = (int)sh[0].items;
  p.L = q.L;
  p.idesc = make_idesc(q.bf16, BN);
  p.M = q.M; p.N = q.N;
  p.kp_out = q.kp2;
  p.n_last = q.kp2 - (p.n_tiles - 1) * BN;              // kp2 % 32 == 0, so n_last % 32 == 0
  p.sG = split_g_scale(q.m);
  p.g_hi = q.g_hi; p.g_lo = q.g_lo;
  p.maxabs = q.maxabs;
  p.err = q.err;
  p.lam_idx = q.lam_idx;
  if (q.kflags && q.kp1 / 32 <= 128) {         // Live tracks up to 128 K blocks
    LGB_REQUIRE(q.kf_pitch % 8 == 0 && q.kf_pitch >= kflag_pitch(q.kp2), LGB_EINVAL,
                "split mft: field flag rows too short for the column tiles");
    p.kflags = q.kflags;
    p.kf_units = q.kp1 / 32;
    p.kf_pitch = q.kf_pitch;
  }
  if (ev) LGB_CUDA(cudaEventRecord(ev[0], s));
  if ((st = launch_stage<BN>(p, q.bf16, chain2, m1, s))) return st;
  if (ev) LGB_CUDA(cudaEventRecord(ev[1], s));

  p.stage = 2;
  p.stall_item = -1;
  p.wait_ns = WAIT_NS;
  p.kflags = nullptr;                           // G is dense
  p.kblocks = sh[1].kblocks;
  p.m_tiles = cdiv(q.M, 2 * BM);
  p.n_tiles = cdiv(q.N, BN / 2);                        // BN/2 complex columns per tile
  p.n_last = BN;                                        // E2 blocks are padded to whole tiles
  p.n_items = (int)sh[1].items;
  p.epilogue = q.epilogue;
  p.weights = q.weights;
  p.unit2 = q.unit2;
  p.wbuf = q.wbuf;
  p.ldw = q.ldw;
  p.out = q.out;
  p.cscale = q.complex_scale;
  if (ev) LGB_CUDA(cudaEventRecord(ev[2], s));
  if ((st = launch_stage<BN>(p, q.bf16, chain2, m2, s))) return st;
  if (ev) LGB_CUDA(cudaEventRecord(ev[3], s));
  return LGB_OK;
}

// ------------------------------------------------------------- autotuner ---
// The tile width is chosen per launch class and cached for the process.  A
// class is the precision, field m x n, window M x N, epilogue, and the
// occupancy the problem count gives: the waves of 128-wide tiles of each
// stage over the resident CTA pairs, capped at 8 (launches of eight or more
// waves behave alike).
//
// The occupancy model below prices both widths.  Where it separates them by
// TUNE_DECISIVE or more (many waves: the 256-wide tile; a launch far below
// one wave: the 128-wide one) its choice is final.  In between, measure mode
// (the default) tunes the class online, on the caller's own launches: the
// next TUNE_TRIALS launches alternate the two widths, the model's first, each
// bracketed by CUDA events on its stream; a later launch of the class finds
// them all finished (cudaEventQuery, no host wait), compares the fastest run
// of each width, caches the winner and runs with it -- until then it runs the
// model's width.  No launch is repeated and nothing synchronises.  Both
// widths' kernels are loaded and configured before a trial is timed, so a
// first launch's host-side set-up is not charged to its width.  A launch
// under stream capture uses the cached or the model's width and records
// nothing.  Model mode takes the model's choice at once; a forced width
// overrides everything.
constexpr int TUNE_TRIALS = 4;
constexpr double TUNE_DECISIVE = 1.4;

struct Trial {
  int width = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool recorded = false;
};
struct TuneEntry {
  int best = 0;              // decided width, 0 while trials run
  int trials = 0;            // trials handed out (0..TUNE_TRIALS)
  Trial t[TUNE_TRIALS];
};
using TuneKey = std::array<int, 8>;
struct Tuner {
  std::mutex mu;
  std::map<TuneKey, TuneEntry> table;
  int mode = LGB_TUNE_MEASURE;
  int forced = 0;
};
static Tuner& tuner() {
  static Tuner* t = new Tuner();     // never destroyed: its events may outlive the CUDA context
  return *t;
}
static thread_local int t_last_tile = 0;

static void drop_trials(TuneEntry& e) {
  for (Trial& t : e.t) {
    if (t.e0) cudaEventDestroy(t.e0);
    if (t.e1) cudaEventDestroy(t.e1);
    t = Trial();
  }
}

static TuneKey tune_key(const SplitMftProblem& q) {
  const int pairs = std::max(1, sm_count() / 2);
  StageShape sh[2];
  stage_shapes(q, 128, sh);
  auto waves = [&](long long items) { return (int)std::min<long long>(8, (items + pairs - 1) / pairs); };
  return {q.bf16 ? 1 : 0, q.m, q.n, q.M, q.N, q.epilogue, waves(sh[0].items), waves(sh[1].items)};
}

// Cost of each width: waves of work items over the resident CTA pairs times
// K blocks, a 128-wide item costing 0.78 of a 256-wide one (measured on the
// broadband workload: twice the items took 1.56x the time at full
// occupancy).  Either width holds one CTA per SM, so the pairs are taken as
// half the SMs: no occupancy query, which keeps the model usable inside a
// stream capture.  Returns the cheaper width; *ratio = dearer / cheaper.
static int model_tile(const SplitMftProblem& q, double* ratio = nullptr) {
  double cost[2];
  const int bns[2] = {256, 128};
  const int pairs = std::max(1, sm_count() / 2);
  for (int c = 0; c < 2; ++c) {
    StageShape sh[2];
    stage_shapes(q, bns[c], sh);
    cost[c] = 0.0;
    for (const StageShape& x : sh) cost[c] += (double)((x.items + pairs - 1) / pairs) * x.kblocks;
    cost[c] *= bns[c] == 256 ? 1.0 : 0.78;
  }
  if (ratio) *ratio = std::max(cost[0], cost[1]) / std::max(1e-30, std::min(cost[0], cost[1]));
  return cost[1] < cost[0] ? 128 : 256;
}

static int run_tile(const SplitMftProblem& q, int bn, cudaEvent_t* ev, cudaStream_t s) {
  return bn == 128 ? run_split_mft<128>(q, ev, s) : run_split_mft<256>(q, ev, s);
}

// Loads and configures both widths' kernels (lazy module load, shared-memory
// attribute, occupancy) so that no trial is timed across that set-up.
static void prepare_widths(bool bf16) {
  if (bf16) {
    max_pairs<true, 256, 1>(); max_pairs<true, 128, 1>();
    max_pairs<true, 256, 2>(); max_pairs<true, 128, 2>();
  } else {
    max_pairs<false, 256, 1>(); max_pairs<false, 128, 1>();
  }
}

// Width for this launch; ev[0..1] are set when the launch is to be timed
// (events owned by the tuner's table).
static int choose_tile(const SplitMftProblem& q, cudaStream_t s, int* bn, cudaEvent_t* ev,
                       TuneKey* key) {
  Tuner& T = tuner();
  ev[0] = ev[1] = nullptr;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  LGB_CUDA(cudaStreamIsCapturing(s, &cap));
  *key = tune_key(q);
  double ratio = 1.0;
  const int model = model_tile(q, &ratio);
  std::lock_guard<std::mutex> lock(T.mu);
  if (T.forced) { *bn = T.forced; return LGB_OK; }
  auto it = T.table.find(*key);
  if (it != T.table.end() && it->second.best) { *bn = it->second.best; return LGB_OK; }
  *bn = model;
  if (cap != cudaStreamCaptureStatusNone) return LGB_OK;
  if (T.mode == LGB_TUNE_MODEL || ratio >= TUNE_DECISIVE) {
    T.table[*key].best = model;
    return LGB_OK;
  }
  TuneEntry& e = T.table[*key];
  if (e.trials < TUNE_TRIALS) {                // hand out the next trial
    Trial& t = e.t[e.trials];
    if (cudaEventCreate(&t.e0) != cudaSuccess || cudaEventCreate(&t.e1) != cudaSuccess) {
      drop_trials(e);
      e.best = model;                          // cannot time: keep the model's width
      return LGB_OK;
    }
    t.width = (e.trials & 1) == 0 ? model : (model == 256 ? 128 : 256);
    ++e.trials;
    *bn = t.width;
    ev[0] = t.e0;
    ev[1] = t.e1;
    return LGB_OK;
  }
  float fastest[2] = {1e30f, 1e30f};           // [0]: the model's width, [1]: the other
  for (int k = 0; k < TUNE_TRIALS; ++k) {
    const Trial& t = e.t[k];
    if (!t.recorded) return LGB_OK;            // a trial launch is still being issued
    const cudaError_t qe = cudaEventQuery(t.e1);
    if (qe == cudaErrorNotReady) return LGB_OK;
    float ms = 0.f;
    if (qe != cudaSuccess || cudaEventElapsedTime(&ms, t.e0, t.e1) != cudaSuccess) {
      (void)cudaGetLastError();
      drop_trials(e);
      e.best = model;
      return LGB_OK;
    }
    float& f = fastest[t.width == model ? 0 : 1];
    f = std::min(f, ms);
  }
  e.best = fastest[1] < fastest[0] ? (model == 256 ? 128 : 256) : model;
  drop_trials(e);
  *bn = e.best;
  return LGB_OK;
}

}  // namespace tc

float split_g_scale(int m) {
  // |G * s_f| <= sqrt(2) m, so 2^13 / 2^ceil(log2 m) keeps |G * s_f * s_G| < 2^14
  int e = 0;
  std::frexp((float)m, &e);
  return std::ldexp(1.f, 13 - e);
}

int launch_split_mft(const SplitMftProblem& q, cudaStream_t s) {
  using namespace tc;
  LGB_REQUIRE(q.kp1 % 32 == 0 && q.kp2 % 32 == 0, LGB_EINVAL, "split mft: K padding");
  int bn = q.tile;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  TuneKey key{};
  if (bn != 0) {                               // a forced width overrides the caller's too
    Tuner& T = tuner();
    std::lock_guard<std::mutex> lock(T.mu);
    if (T.forced) bn = T.forced;
  } else {
    const int st = choose_tile(q, s, &bn, ev, &key);
    if (st) return st;
  }
  LGB_REQUIRE(bn == 256 || bn == 128, LGB_EINVAL, "split mft: tile width must be 256 or 128");
  t_last_tile = bn;
  // a timed trial brackets the launch with the entry's events (a concurrent
  // lgb_tuner_clear may have destroyed them: the launch then runs untimed)
  if (ev[0]) prepare_widths(q.bf16);
  bool timed = ev[0] && cudaEventRecord(ev[0], s) == cudaSuccess;
  if (ev[0] && !timed) (void)cudaGetLastError();   // not the launch's error: clear it
  const int st = run_tile(q, bn, q.events, s);
  if (st) return st;
  if (timed && cudaEventRecord(ev[1], s) != cudaSuccess) {
    (void)cudaGetLastError();
    timed = false;
  }
  if (timed) {
    Tuner& T = tuner();
    std::lock_guard<std::mutex> lock(T.mu);
    auto it = T.table.find(key);
    if (it != T.table.end())
      for (Trial& t : it->second.t)
        if (t.e1 == ev[1]) t.recorded = true;
  }
  return LGB_OK;
}

}  // namespace lgb

// ------------------------------------------------------------- tuner ABI ---
using namespace lgb;

extern "C" int lgb_test_stall_tma(int item, int kblock, double wait_ms) {
  LGB_REQUIRE(item >= 0 && kblock >= 0, LGB_EINVAL, "test_stall_tma: item and kblock must be >= 0");
  LGB_REQUIRE(wait_ms > 0.0 && wait_ms <= 2000.0, LGB_EINVAL,
              "test_stall_tma: wait_ms must lie in (0, 2000]");
  tc::g_stall_kb.store(kblock);
  tc::g_stall_wait.store((unsigned long long)(wait_ms * 1e6));
  tc::g_stall_item.store(item);
  return LGB_OK;
}

extern "C" int lgb_tuner_set_mode(int mode) {
  LGB_REQUIRE(mode == LGB_TUNE_MODEL || mode == LGB_TUNE_MEASURE, LGB_EINVAL,
              "tuner_set_mode: mode must be LGB_TUNE_MODEL or LGB_TUNE_MEASURE");
  tc::Tuner& T = tc::tuner();
  std::lock_guard<std::mutex> lock(T.mu);
  T.mode = mode;
  return LGB_OK;
}

extern "C" int lgb_tuner_force_tile(int tile) {
  LGB_REQUIRE(tile == 0 || tile == 128 || tile == 256, LGB_EINVAL,
              "tuner_force_tile: tile must be 0 (tuned), 128 or 256");
  tc::Tuner& T = tc::tuner();
  std::lock_guard<std::mutex> lock(T.mu);
  T.forced = tile;
  return LGB_OK;
}

extern "C" void lgb_tuner_clear(void) {
  tc::Tuner& T = tc::tuner();
  std::lock_guard<std::mutex> lock(T.mu);
  for (auto& kv : T.table) tc::drop_trials(kv.second);
  T.table.clear();
}

extern "C" int lgb_tuner_entries(void) {
  tc::Tuner& T = tc::tuner();
  std::lock_guard<std::mutex> lock(T.mu);
  int n = 0;
  for (const auto& kv : T.table) n += kv.second.best != 0;
  return n;
}

extern "C" int lgb_tuner_lookup(int m, int n, int M, int N, int count, int precision, int epilogue) {
  if (m <= 0 || n <= 0 || M <= 0 || N <= 0 || count <= 0) return 0;
  SplitMftProblem q{};
  q.bf16 = precision == LGB_SPLIT_BF16;
  q.m = m; q.n = n; q.M = M; q.N = N;
  q.kp1 = round_up(m, 32); q.kp2 = round_up(n, 32);
  q.L = count; q.batch = 1;
  q.epilogue = epilogue;
  const tc::TuneKey key = tc::tune_key(q);
  tc::Tuner& T = tc::tuner();
  std::lock_guard<std::mutex> lock(T.mu);
  const auto it = T.table.find(key);
  return it == T.table.end() ? 0 : it->second.best;
}

extern "C" int lgb_tuner_last_tile(void) { return tc::t_last_tile; }

extern "C" int lgb_tuner_export(int* rows, int max_rows) {
  tc::Tuner& T = tc::tuner();
  std::lock_guard<std::mutex> lock(T.mu);
  int n = 0;
  for (const auto& kv : T.table) {
    if (!kv.second.best) continue;
    if (rows && n < max_rows) {
      for (int j = 0; j < 8; ++j) rows[9 * n + j] = kv.first[j];
      rows[9 * n + 8] = kv.second.best;
    }
    ++n;
  }
  return n;
}

extern "C" int lgb_tuner_import(const int* rows, int n) {
  LGB_REQUIRE(n >= 0 && (rows || n == 0), LGB_EINVAL, "tuner_import: bad rows");
  for (int i = 0; i < n; ++i)
    LGB_REQUIRE(rows[9 * i + 8] == 128 || rows[9 * i + 8] == 256, LGB_EINVAL,
                "tuner_import: a width is not 128 or 256");
  tc::Tuner& T = tc::tuner();
  std::lock_guard<std::mutex> lock(T.mu);
  for (int i = 0; i < n; ++i) {
    tc::TuneKey key;
    for (int j = 0; j < 8; ++j) key[j] = rows[9 * i + j];
    tc::TuneEntry& e = T.table[key];
    tc::drop_trials(e);
    e.trials = 0;
    e.best = rows[9 * i + 8];
  }
  return LGB_OK;
}
