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
// (measured: 1.8e-5 relative at K = 2048).  So the dominant hi.hi products
// are accumulated in short chains: TMEM region X is restarted every KSUB
// (= 4, one 64-wide K block) k-steps and the epilogue warps fold each chunk into round-to-nearest FP32
// registers, while the MMA issues the small cross terms into region Y (one
// long chain; its truncation is 2^-8 smaller).  The epilogue drain of X
// hides behind the Y instructions.
//
// Warp roles (320 threads, one CTA per SM, persistent over work items):
//   warp 0       TMA producer (one lane)
//   warp 1       TMEM allocator + MMA issuer (one lane)
//   warps 2..9   epilogue: warp w owns TMEM lanes 32*(w%4).. and the
//                column half (w-2)/4 of the 256-column tile
// Tiles: M=128 x N=256 per MMA instruction, K=16; TMEM X = cols 0..255,
// Y = cols 256..511; a 2-stage 96 KB smem ring (A_hi, A_lo, B_hi, B_lo).
// Every mbarrier wait is bounded in time; on expiry the kernel records
// LGB_ETIMEOUT in a device flag, drains what it issued and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {
namespace tc {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 2;
constexpr int KSTEPS = BK / 16;                            // MMA k-steps per K block
#ifndef LGB_KSUB
#define LGB_KSUB 4
#endif
constexpr int KSUB = LGB_KSUB;                             // k-steps per hi.hi chain
constexpr int CHUNKS = KSTEPS / KSUB;                      // X chunks per K block
constexpr uint32_t A_BYTES = BM * BK * 2;                  // 16 KB per plane
constexpr uint32_t B_BYTES = BN * BK * 2;                  // 32 KB per plane
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // 96 KB
constexpr uint32_t BAR_BYTES = 128;
constexpr uint32_t SMEM_BYTES = STAGES * STAGE_BYTES + BAR_BYTES + 1024;
constexpr int EPI_WARPS = 8;
constexpr int NUM_THREADS = 64 + 32 * EPI_WARPS;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t X_COL = 0, Y_COL = 256;
constexpr unsigned long long WAIT_NS = 2000000000ull;      // 2 s bound on any wait

struct Params {
  int stage;                 // 1 or 2
  int kblocks;               // K / 64
  int m_tiles, n_tiles;
  int n_items;               // Q * m_tiles * n_tiles
  int L;
  uint32_t idesc;
  int M, N;                  // stage 1: rows of G / stage 2: window shape
  int kp_out;                // stage 1: row half-width of G (kp2)
  float sG;                  // stage-2 operand scale (power of two)
  uint16_t* g_hi;
  uint16_t* g_lo;
  const float* maxabs;       // [batch]
  int epilogue;              // stage 2: 0 intensity, 1 complex
  const double* weights;     // [batch][L] or null
  const double* unit2;       // [L]
  float* wbuf;               // stage 2 intensity: [batch][M][ldw] FP32 window
  int ldw;
  double* out;               // stage 2 complex: [M][N] complex128
  double cscale;
  int* err;
  const int* lam_idx;        // [L] wavelength -> DFT-matrix slot, or null (identity)
};

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
// Bounded wait: true when the phase completed, false on time-out or when
// another role already flagged an error.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  for (uint32_t n = 1;; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 63) == 0) {
      if (*(volatile int*)err != 0) return false;
      if (gtimer() - t0 > WAIT_NS) {
        atomicCAS(err, 0, LGB_ETIMEOUT);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
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
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
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

// ------------------------------------------------------------- epilogue ---
// Drain 128 columns of a TMEM region into the running sums (round to nearest).
// One 32-column load in flight keeps the epilogue within the 168 registers
// a thread gets when three warps share an SM sub-partition.
__device__ __forceinline__ void drain_add(uint32_t taddr, float (&run)[128]) {
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    uint32_t a[32];
    tmem_ld32(taddr + h * 32, a);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < 32; ++j) run[h * 32 + j] += __uint_as_float(a[j]);
  }
}

template <bool BF16>
__device__ __forceinline__ void write_stage1(const Params& p, const Item& w, int row, int ch,
                                             const float (&run)[128]) {
  const int h = row >> 6, u = w.tm * 64 + (row & 63);
  if (u >= p.M) return;
  const size_t K2 = 2 * (size_t)p.kp_out;
  const int c0 = w.tn * BN + ch * 128;
  const size_t off = ((size_t)w.q * p.M + u) * K2 + (size_t)h * p.kp_out + c0;
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    if (c0 + cc * 32 >= p.kp_out) break;
#pragma unroll
    for (int v8 = 0; v8 < 4; ++v8) {          // 8 columns -> one 16-byte store per plane
      uint32_t ph[4], pl[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = cc * 32 + v8 * 8 + 2 * j;
        uint16_t h0, l0, h1, l1;
        Split16<BF16>::split(run[k] * p.sG, h0, l0);
        Split16<BF16>::split(run[k + 1] * p.sG, h1, l1);
        ph[j] = (uint32_t)h0 | ((uint32_t)h1 << 16);
        pl[j] = (uint32_t)l0 | ((uint32_t)l1 << 16);
      }
      *reinterpret_cast<uint4*>(p.g_hi + off + cc * 32 + v8 * 8) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
      *reinterpret_cast<uint4*>(p.g_lo + off + cc * 32 + v8 * 8) = make_uint4(pl[0], pl[1], pl[2], pl[3]);
    }
  }
}

// Stage 2 column layout of a 256-column tile: half ch holds output columns
// v = tn*128 + ch*64 + j, real parts in [0, 64), imaginary in [64, 128).
__device__ __forceinline__ void write_stage2(const Params& p, const Item& w, int row, int ch,
                                             const float (&run)[128]) {
  const int u = w.tm * BM + row;
  if (u >= p.M) return;
  const float sf = pow2_scale_for(p.maxabs[w.psf]);
  const int v0 = w.tn * 128 + ch * 64;
  if (p.epilogue == 0) {
    const float inv = 1.f / (sf * p.sG);
    const double wt = p.weights ? p.weights[(size_t)w.psf * p.L + w.lam] : 1.0;
    const float coef = (float)(wt * p.unit2[matrix_slot(p, w.lam)]) * inv * inv;
    float* dst = p.wbuf + ((size_t)w.psf * p.M + u) * p.ldw + v0;
#pragma unroll
    for (int j = 0; j < 64; j += 4) {
      if (v0 + j >= p.N) break;
      float r[4];
#pragma unroll
      for (int e = 0; e < 4; ++e)
        r[e] = coef * fmaf(run[j + e], run[j + e], run[64 + j + e] * run[64 + j + e]);
      red_add_v4(dst + j, r[0], r[1], r[2], r[3]);
    }
  } else {
    const double scl = p.cscale / ((double)sf * (double)p.sG);
    double2* outc = reinterpret_cast<double2*>(p.out) + (size_t)u * p.N;
#pragma unroll
    for (int j = 0; j < 64; ++j)
      if (v0 + j < p.N) outc[v0 + j] = make_double2(scl * run[j], scl * run[64 + j]);
  }
}

// -------------------------------------------------------------- kernel ---
template <bool BF16>
__global__ void __launch_bounds__(NUM_THREADS, 1)
split_mft_kernel(const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
                 const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo,
                 const Params p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* const gbase = smem_raw + (base - raw);
  const uint32_t bars = base + STAGES * STAGE_BYTES;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 16u + 8u * s; };
  const uint32_t xf_bar = bars + 32u;    // X chunk ready       (MMA -> epilogue)
  const uint32_t xe_bar = bars + 40u;    // X chunk drained     (epilogue -> MMA)
  const uint32_t yf_bar = bars + 48u;    // Y ready (item end)  (MMA -> epilogue)
  const uint32_t ye_bar = bars + 56u;    // Y drained           (epilogue -> MMA)
  const uint32_t drain_bar = bars + 64u;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + STAGES * STAGE_BYTES + 72);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    mbar_init(xf_bar, 1);
    mbar_init(xe_bar, EPI_WARPS);
    mbar_init(yf_bar, 1);
    mbar_init(ye_bar, EPI_WARPS);
    mbar_init(drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------ TMA producer
    if (lane == 0) {
      prefetch_map(&tmA_hi); prefetch_map(&tmA_lo);
      prefetch_map(&tmB_hi); prefetch_map(&tmB_lo);
      uint32_t it = 0;
      bool ok = true;
      for (int i = blockIdx.x; ok && i < p.n_items; i += gridDim.x) {
        const Item w = decode(p, i);
        // stage 1: A = E1 block of lam, B = f^T of q; stage 2: A = G of q, B = E2 block of lam
        const int az = p.stage == 1 ? matrix_slot(p, w.lam) : w.q;
        const int bz = p.stage == 1 ? w.q : matrix_slot(p, w.lam);
        for (int kb = 0; kb < p.kblocks; ++kb, ++it) {
          const int s = it % STAGES;
          if (!mbar_wait(empty_bar(s), ((it / STAGES) & 1) ^ 1, p.err)) { ok = false; break; }
          mbar_expect_tx(full_bar(s), STAGE_BYTES);
          const uint32_t sa = base + s * STAGE_BYTES;
          tma_load_3d(sa, &tmA_hi, full_bar(s), kb * BK, w.tm * BM, az);
          tma_load_3d(sa + A_BYTES, &tmA_lo, full_bar(s), kb * BK, w.tm * BM, az);
          tma_load_3d(sa + 2 * A_BYTES, &tmB_hi, full_bar(s), kb * BK, w.tn * BN, bz);
          tma_load_3d(sa + 2 * A_BYTES + B_BYTES, &tmB_lo, full_bar(s), kb * BK, w.tn * BN, bz);
        }
      }
      // every copy this thread issued has landed before the CTA exits
      for (uint32_t k = (it > STAGES ? it - STAGES : 0); k < it; ++k)
        mbar_wait(full_bar(k % STAGES), (k / STAGES) & 1, p.err);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------- MMA issuer
    if (lane == 0) {
      uint32_t it = 0, xc = 0, yi = 0;
      bool ok = true;
      const uint32_t X = tmem + X_COL, Y = tmem + Y_COL;
      for (int i = blockIdx.x; ok && i < p.n_items; i += gridDim.x, ++yi) {
        for (int kb = 0; kb < p.kblocks && ok; ++kb, ++it) {
          const int s = it % STAGES;
          if (!mbar_wait(full_bar(s), (it / STAGES) & 1, p.err)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sa = base + s * STAGE_BYTES;
#pragma unroll
          for (int c = 0; c < CHUNKS; ++c, ++xc) {
            // X <- hi.hi over KSUB k-steps, once the previous chunk is drained
            if (!mbar_wait(xe_bar, (xc & 1) ^ 1, p.err)) { ok = false; break; }
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < KSUB; ++kk) {
              const int k = c * KSUB + kk;
              mma_f16(X, smem_desc(sa + k * 32), smem_desc(sa + 2 * A_BYTES + k * 32), p.idesc,
                      kk ? 1u : 0u);
            }
            mma_commit(xf_bar);
            // Y <- hi.lo + lo.hi (one chain per item, restarted after Y is drained)
            const bool y_first = (kb == 0 && c == 0);
            if (y_first) {
              if (!mbar_wait(ye_bar, (yi & 1) ^ 1, p.err)) { ok = false; break; }
              tc_fence_after();
            }
#pragma unroll
            for (int kk = 0; kk < KSUB; ++kk) {
              const int k = c * KSUB + kk;
              mma_f16(Y, smem_desc(sa + k * 32), smem_desc(sa + 2 * A_BYTES + B_BYTES + k * 32),
                      p.idesc, (y_first && kk == 0) ? 0u : 1u);
              mma_f16(Y, smem_desc(sa + A_BYTES + k * 32), smem_desc(sa + 2 * A_BYTES + k * 32),
                      p.idesc, 1u);
            }
          }
          mma_commit(empty_bar(s));     // smem stage free once these MMAs retire
        }
        if (!ok) break;
        mma_commit(yf_bar);
      }
      // all issued MMAs have retired before TMEM is released
      mma_commit(drain_bar);
      mbar_wait(drain_bar, 0, p.err);
    }
  } else {
    // --------------------------------------------------------- epilogue
    const int q4 = warp & 3;                 // TMEM lane quadrant of this warp
    const int ch = (warp - 2) >> 2;          // column half of the tile
    const int row = q4 * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(q4 * 32) << 16) + ch * 128;
    uint32_t xc = 0, yi = 0;
    bool ok = true;
    for (int i = blockIdx.x; ok && i < p.n_items; i += gridDim.x, ++yi) {
      const Item w = decode(p, i);
      float run[128];
#pragma unroll
      for (int j = 0; j < 128; ++j) run[j] = 0.f;
      for (int kb = 0; kb < p.kblocks && ok; ++kb) {
        for (int c = 0; c < CHUNKS; ++c, ++xc) {
          ok = __all_sync(0xffffffffu, mbar_wait(xf_bar, xc & 1, p.err));
          if (!ok) break;
          tc_fence_after();
          drain_add(trow + X_COL, run);
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(xe_bar);
        }
      }
      if (!ok) break;
      ok = __all_sync(0xffffffffu, mbar_wait(yf_bar, yi & 1, p.err));
      if (!ok) break;
      tc_fence_after();
      drain_add(trow + Y_COL, run);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(ye_bar);
      if (p.stage == 1) write_stage1<BF16>(p, w, row, ch, run);
      else write_stage2(p, w, row, ch, run);
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
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

// 3-D K-major operand map: dims {K, rows, batch}, box {64, box_rows, 1}.
static int make_map(CUtensorMap* map, const void* ptr, bool bf16, int K, int rows, int batch,
                    int box_rows) {
  auto enc = encode_fn();
  LGB_REQUIRE(enc, LGB_ECUDA, "cuTensorMapEncodeTiled is unavailable");
  LGB_REQUIRE(((uintptr_t)ptr & 15) == 0, LGB_EINVAL, "tensor map base must be 16-byte aligned");
  LGB_REQUIRE(K % BK == 0, LGB_EINVAL, "tensor map K must be a multiple of 64");
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)batch};
  cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)K * 2 * rows};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult res = enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16,
                     3, const_cast<void*>(ptr), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (res != CUDA_SUCCESS)
    return set_error(LGB_ECUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)res));
  return LGB_OK;
}

constexpr uint32_t make_idesc(bool bf16) {
  return (1u << 4)                          // D format: FP32
         | ((bf16 ? 1u : 0u) << 7)          // A format: BF16 (1) / FP16 (0)
         | ((bf16 ? 1u : 0u) << 10)         // B format
         | ((uint32_t)(BN >> 3) << 17)      // N
         | ((uint32_t)(BM >> 4) << 24);     // M
}

template <bool BF16>
static int launch_one(const Params& p, const CUtensorMap& a_hi, const CUtensorMap& a_lo,
                      const CUtensorMap& b_hi, const CUtensorMap& b_lo, cudaStream_t s) {
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(split_mft_kernel<BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)SMEM_BYTES);
  });
  LGB_CUDA(attr_err);
  if (p.n_items <= 0) return LGB_OK;
  const int grid = std::min(p.n_items, sm_count());
  split_mft_kernel<BF16><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(a_hi, a_lo, b_hi, b_lo, p);
  LGB_CUDA(cudaGetLastError());
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
  const int Q = q.batch * q.L;
  const int mrows1 = cdiv(q.M, 64) * 128;      // E1 block rows
  const int nrows2 = cdiv(q.N, 128) * 256;     // E2 block rows
  const uint32_t idesc = make_idesc(q.bf16);
  CUtensorMap a_hi, a_lo, b_hi, b_lo;
  int st;

  // ---- stage 1: G = E1 . f
  const int Lm = q.lam_idx ? q.L_bank : q.L;     // DFT-matrix slots held
  if ((st = make_map(&a_hi, q.e1_hi, q.bf16, 2 * q.kp1, mrows1, Lm, BM))) return st;
  if ((st = make_map(&a_lo, q.e1_lo, q.bf16, 2 * q.kp1, mrows1, Lm, BM))) return st;
  if ((st = make_map(&b_hi, q.f_hi, q.bf16, 2 * q.kp1, q.n, Q, BN))) return st;
  if ((st = make_map(&b_lo, q.f_lo, q.bf16, 2 * q.kp1, q.n, Q, BN))) return st;
  Params p{};
  p.stage = 1;
  p.kblocks = 2 * q.kp1 / BK;
  p.m_tiles = cdiv(q.M, 64);
  p.n_tiles = cdiv(q.kp2, BN);
  p.n_items = Q * p.m_tiles * p.n_tiles;
  p.L = q.L;
  p.idesc = idesc;
  p.M = q.M; p.N = q.N;
  p.kp_out = q.kp2;
  p.sG = split_g_scale(q.m);
  p.g_hi = q.g_hi; p.g_lo = q.g_lo;
  p.maxabs = q.maxabs;
  p.err = q.err;
  p.lam_idx = q.lam_idx;
  if (q.events) LGB_CUDA(cudaEventRecord(q.events[0], s));
  st = q.bf16 ? launch_one<true>(p, a_hi, a_lo, b_hi, b_lo, s)
              : launch_one<false>(p, a_hi, a_lo, b_hi, b_lo, s);
  if (st) return st;
  if (q.events) LGB_CUDA(cudaEventRecord(q.events[1], s));

  // ---- stage 2: F = G . E2 (+ epilogue)
  if ((st = make_map(&a_hi, q.g_hi, q.bf16, 2 * q.kp2, q.M, Q, BM))) return st;
  if ((st = make_map(&a_lo, q.g_lo, q.bf16, 2 * q.kp2, q.M, Q, BM))) return st;
  if ((st = make_map(&b_hi, q.e2_hi, q.bf16, 2 * q.kp2, nrows2, Lm, BN))) return st;
  if ((st = make_map(&b_lo, q.e2_lo, q.bf16, 2 * q.kp2, nrows2, Lm, BN))) return st;
  p.stage = 2;
  p.kblocks = 2 * q.kp2 / BK;
  p.m_tiles = cdiv(q.M, BM);
  p.n_tiles = cdiv(q.N, 128);
  p.n_items = Q * p.m_tiles * p.n_tiles;
  p.epilogue = q.epilogue;
  p.weights = q.weights;
  p.unit2 = q.unit2;
  p.wbuf = q.wbuf;
  p.ldw = q.ldw;
  p.out = q.out;
  p.cscale = q.complex_scale;
  if (q.events) LGB_CUDA(cudaEventRecord(q.events[2], s));
  st = q.bf16 ? launch_one<true>(p, a_hi, a_lo, b_hi, b_lo, s)
              : launch_one<false>(p, a_hi, a_lo, b_hi, b_lo, s);
  if (st) return st;
  if (q.events) LGB_CUDA(cudaEventRecord(q.events[3], s));
  return LGB_OK;
}

}  // namespace lgb
