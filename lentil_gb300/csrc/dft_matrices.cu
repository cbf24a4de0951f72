// K1: DFT-matrix builders (lentil/fourier.py:106-121).
//
// complex128 form: E1 (M x m) and E2 (n x N) exactly as lentil lays them out.
// split form: the real block embeddings consumed by the tcgen05 MFT
// (mft_split.cu), stored as two 16-bit planes (hi, lo):
//   stage-1 A operand ("E1 block", rows in tiles of 128 = 64 real + 64 imag
//   output rows, K = [real part | imaginary part] of the input rows, padded
//   to kp = round_up(m, 32)):
//     row (t*128 + i)      <- output row u = t*64 + i, real part:  [ Re E1[u,:] | -Im E1[u,:] ]
//     row (t*128 + 64 + i) <- output row u, imaginary part:        [ Im E1[u,:] |  Re E1[u,:] ]
//   stage-2 B operand ("E2 block", rows in tiles of 256 covering 128 output
//   columns as two halves of 64 real + 64 imaginary rows, K = [real |
//   imaginary] of the intermediate, padded to kp = round_up(n, 32)):
//     row (t*256 + h*128 + j)      <- v = t*128 + h*64 + j, real:  [ Re E2[:,v] | -Im E2[:,v] ]
//     row (t*256 + h*128 + 64 + j) <- v, imaginary:                [ Im E2[:,v] |  Re E2[:,v] ]
#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

__global__ void dft_matrix_c128_kernel(PhaseAxis ax, int len_in, int len_out, double2* E,
                                       int transpose_out) {
  // E is (len_out x len_in) when transpose_out (E1 layout), else (len_in x len_out) (E2).
  const int i = blockIdx.x * blockDim.x + threadIdx.x;   // fastest index of E
  const int j = blockIdx.y;
  if (transpose_out) {
    // E1[u = j][r = i]
    if (i < len_in && j < len_out) E[(size_t)j * len_in + i] = expm2pi_fixed_f64(phase_fixed(ax, i, j));
  } else {
    // E2[s = j][v = i]
    if (i < len_out && j < len_in) E[(size_t)j * len_out + i] = expm2pi_fixed_f64(phase_fixed(ax, j, i));
  }
}

int launch_dft_matrix_c128(const PhaseAxis& ax, int len_in, int len_out, double2* E,
                           bool e1_layout, cudaStream_t s) {
  if (len_in <= 0 || len_out <= 0) return LGB_OK;
  const int fast = e1_layout ? len_in : len_out;
  const int slow = e1_layout ? len_out : len_in;
  dim3 grid(cdiv(fast, 256), slow);
  dft_matrix_c128_kernel<<<grid, 256, 0, s>>>(ax, len_in, len_out, E, e1_layout ? 1 : 0);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// Both split builders: a thread makes 4 consecutive K entries of one
// output row/column.  The phase is taken once in fixed point and stepped by
// its exact per-index increment; the four values are split in pairs and
// written as 8-byte stores to the four places a block embedding holds them
// ([Re | -Im] and [Im | Re] rows).  The negated imaginary part is the split
// of the imaginary part with the sign bits flipped (round-to-nearest is
// symmetric, so this equals splitting -Im).  (The SFU sine in place of
// sincospif for the bf16 form was tried: it moved a bf16 golden case from
// just under its bound to 2.1e-6, for little speed, the build being near the
// HBM rate already.)
constexpr int SPLIT_PER_THREAD = 4;
constexpr int SPLIT_THREADS = 128;

template <bool BF16>
__device__ __forceinline__ void block_entries_store(const PhaseAxis& ax, int k0, int len_in,
                                                    int j_out, bool live_row, int kp,
                                                    size_t row_re, size_t row_im,
                                                    uint16_t* __restrict__ hi,
                                                    uint16_t* __restrict__ lo) {
  float2 e[SPLIT_PER_THREAD];
  uint64_t ph = phase_fixed(ax, k0, j_out);
  const uint64_t step = phase_step_in(ax, j_out);
#pragma unroll
  for (int t = 0; t < SPLIT_PER_THREAD; ++t) {
    e[t] = (live_row && k0 + t < len_in) ? expm2pi_fixed_f32(ph) : make_float2(0.f, 0.f);
    ph += step;
  }
  uint32_t rh[2], rl[2], ih[2], il[2];
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    Split16x2<BF16>::split(e[2 * t].x, e[2 * t + 1].x, rh[t], rl[t]);
    Split16x2<BF16>::split(e[2 * t].y, e[2 * t + 1].y, ih[t], il[t]);
  }
  constexpr uint32_t SIGN = 0x80008000u;
  const uint2 re_h = make_uint2(rh[0], rh[1]), re_l = make_uint2(rl[0], rl[1]);
  const uint2 im_h = make_uint2(ih[0], ih[1]), im_l = make_uint2(il[0], il[1]);
  const uint2 nim_h = make_uint2(ih[0] ^ SIGN, ih[1] ^ SIGN);
  const uint2 nim_l = make_uint2(il[0] ^ SIGN, il[1] ^ SIGN);
  auto st = [&](uint16_t* base, size_t off, uint2 v) {
    *reinterpret_cast<uint2*>(base + off) = v;
  };
  st(hi, row_re + k0, re_h);       st(lo, row_re + k0, re_l);        // [ Re | . ]
  st(hi, row_re + kp + k0, nim_h); st(lo, row_re + kp + k0, nim_l);  // [ . | -Im ]
  st(hi, row_im + k0, im_h);       st(lo, row_im + k0, im_l);        // [ Im | . ]
  st(hi, row_im + kp + k0, re_h);  st(lo, row_im + kp + k0, re_l);   // [ . | Re ]
}

// Stage-1 A operand, one wavelength per blockIdx.z.
template <bool BF16>
__global__ void __launch_bounds__(SPLIT_THREADS) e1_block_split_kernel(
    const PhaseAxis* __restrict__ axes, int m, int M, int kp, int rows_padded,
    uint16_t* __restrict__ hi, uint16_t* __restrict__ lo) {
  const int r0 = SPLIT_PER_THREAD * (blockIdx.x * blockDim.x + threadIdx.x);   // K index
  const int u = blockIdx.y;                                // output row
  const int z = blockIdx.z;
  if (r0 >= kp) return;
  const int t = u >> 6, i = u & 63;
  const size_t K = 2 * (size_t)kp;
  const size_t base = (size_t)z * rows_padded * K;
  block_entries_store<BF16>(axes[z], r0, m, u, u < M, kp, base + (size_t)(t * 128 + i) * K,
                            base + (size_t)(t * 128 + 64 + i) * K, hi, lo);
}

// Stage-2 B operand, one wavelength per blockIdx.z.
template <bool BF16>
__global__ void __launch_bounds__(SPLIT_THREADS) e2_block_split_kernel(
    const PhaseAxis* __restrict__ axes, int n, int N, int kp, int rows_padded,
    uint16_t* __restrict__ hi, uint16_t* __restrict__ lo) {
  const int c0 = SPLIT_PER_THREAD * (blockIdx.x * blockDim.x + threadIdx.x);   // K index
  const int v = blockIdx.y;                                // output column
  const int z = blockIdx.z;
  if (c0 >= kp) return;
  const int t = v >> 7, h2 = (v >> 6) & 1, j = v & 63;
  const size_t K = 2 * (size_t)kp;
  const size_t base = (size_t)z * rows_padded * K;
  block_entries_store<BF16>(axes[z], c0, n, v, v < N, kp,
                            base + (size_t)(t * 256 + h2 * 128 + j) * K,
                            base + (size_t)(t * 256 + h2 * 128 + 64 + j) * K, hi, lo);
}

int launch_e1_block_split(const PhaseAxis* d_axes, int L, int m, int M, int kp, int rows_padded,
                          bool bf16, uint16_t* hi, uint16_t* lo, cudaStream_t s) {
  LGB_REQUIRE(kp % SPLIT_PER_THREAD == 0, LGB_EINVAL, "e1 block: K padding must be a multiple of 4");
  // rows_padded/2 output rows incl. padding
  dim3 grid(cdiv(kp, SPLIT_PER_THREAD * SPLIT_THREADS), rows_padded / 2, L);
  if (bf16) e1_block_split_kernel<true><<<grid, SPLIT_THREADS, 0, s>>>(d_axes, m, M, kp, rows_padded, hi, lo);
  else e1_block_split_kernel<false><<<grid, SPLIT_THREADS, 0, s>>>(d_axes, m, M, kp, rows_padded, hi, lo);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

int launch_e2_block_split(const PhaseAxis* d_axes, int L, int n, int N, int kp, int rows_padded,
                          bool bf16, uint16_t* hi, uint16_t* lo, cudaStream_t s) {
  LGB_REQUIRE(kp % SPLIT_PER_THREAD == 0, LGB_EINVAL, "e2 block: K padding must be a multiple of 4");
  dim3 grid(cdiv(kp, SPLIT_PER_THREAD * SPLIT_THREADS), rows_padded / 2, L);
  if (bf16) e2_block_split_kernel<true><<<grid, SPLIT_THREADS, 0, s>>>(d_axes, n, N, kp, rows_padded, hi, lo);
  else e2_block_split_kernel<false><<<grid, SPLIT_THREADS, 0, s>>>(d_axes, n, N, kp, rows_padded, hi, lo);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

}  // namespace lgb

extern "C" int lgb_dft2_matrices(int m, int n, int M, int N, double alpha_r, double alpha_c,
                                 double shift_r, double shift_c, double offset_r,
                                 double offset_c, lgb_c128* E1, lgb_c128* E2, lgb_stream stream) {
  LGB_RANGE("lgb_dft2_matrices");
  using namespace lgb;
  LGB_REQUIRE(m > 0 && n > 0 && M > 0 && N > 0, LGB_EINVAL, "dft2_matrices: sizes must be positive");
  LGB_REQUIRE(E1 && E2, LGB_EINVAL, "dft2_matrices: null output");
  PhaseAxis ar, ac;
  int st = make_phase_axis(alpha_r, shift_r, offset_r, m, M, &ar);
  if (st) return st;
  st = make_phase_axis(alpha_c, shift_c, offset_c, n, N, &ac);
  if (st) return st;
  cudaStream_t s = as_stream(stream);
  st = launch_dft_matrix_c128(ar, m, M, reinterpret_cast<double2*>(E1), true, s);
  if (st) return st;
  return launch_dft_matrix_c128(ac, n, N, reinterpret_cast<double2*>(E2), false, s);
}
