// Launchers shared between the translation units of the library.
#pragma once

#include <cuda.h>

#include "common.cuh"

namespace lgb {

// dft_matrices.cu --------------------------------------------------------
int launch_dft_matrix_c128(const PhaseAxis& ax, int len_in, int len_out, double2* E,
                           bool e1_layout, cudaStream_t s);
int launch_e1_block_split(const PhaseAxis* d_axes, int L, int m, int M, int kp, int rows_padded,
                          bool bf16, uint16_t* hi, uint16_t* lo, cudaStream_t s);
int launch_e2_block_split(const PhaseAxis* d_axes, int L, int n, int N, int kp, int rows_padded,
                          bool bf16, uint16_t* hi, uint16_t* lo, cudaStream_t s);

// elementwise.cu ---------------------------------------------------------
// per-PSF scale of the field fed to the 16-bit split: 2^-e with
// max|component| <= 2^e, so every scaled component lies in [-1, 1]
__device__ __forceinline__ float pow2_scale_for(float maxabs) {
  if (!(maxabs > 0.f) || !isfinite(maxabs)) return 1.f;
  int e;
  frexpf(maxabs, &e);
  return ldexpf(1.f, -e);
}

// A double as an unevaluated float pair hi + lo, by integer operations only
// (this part's FP64 pipe runs double<->float conversions at a small
// fraction of the FP32 rate): hi = d with its significand truncated to 24
// bits (the funnel shift moves the exponent and top significand bits into
// float position, the subtraction rebiases the exponent from 1023 to 127),
// lo = the remaining 29 significand bits, converted to float (rounded to 24
// bits) and scaled by 2^(exponent - 52), with d's sign.  hi + lo is d to
// 2^-48 relative for |d| >= 2^-74; below that lo is 0 (hi still exact to
// 2^-23), and |d| < 2^-126 gives 0.  Non-finite or |d| >= 2^128 take the
// plain conversion.
__device__ __forceinline__ float2 split_double(double d) {
  const uint32_t lo32 = (uint32_t)__double2loint(d), hi32 = (uint32_t)__double2hiint(d);
  const uint32_t e = (hi32 >> 20) & 0x7FFu;            // biased exponent
  const uint32_t sign = hi32 & 0x80000000u;
  if (e < 897u) return make_float2(0.f, 0.f);
  if (e > 1150u) return make_float2(__double2float_rn(d), 0.f);
  const uint32_t hb = (__funnelshift_l(lo32, hi32, 3) - (896u << 23)) | sign;
  float lo = 0.f;
  if (e >= 949u) {
    lo = __uint2float_rn(lo32 & 0x1FFFFFFFu) * __uint_as_float((e - 948u) << 23);
    lo = __uint_as_float(__float_as_uint(lo) | sign);
  }
  return make_float2(__uint_as_float(hb), lo);
}

// The float nearest below |d| in magnitude (significand truncated to 24
// bits, relative error below 2^-23), by the same integer operations as
// split_double; |d| < 2^-126 gives 0.
__device__ __forceinline__ float truncate_double(double d) {
  const uint32_t lo32 = (uint32_t)__double2loint(d), hi32 = (uint32_t)__double2hiint(d);
  const uint32_t e = (hi32 >> 20) & 0x7FFu;
  if (e < 897u) return 0.f;
  if (e > 1150u) return __double2float_rn(d);
  return __uint_as_float((__funnelshift_l(lo32, hi32, 3) - (896u << 23)) | (hi32 & 0x80000000u));
}

// float -> double by integer operations (this part's FP64 pipe converts at
// a small fraction of the FP32 rate): exact for normal floats, infinities
// and NaNs; zero and subnormal floats (below 1.2e-38) give a signed zero.
__device__ __forceinline__ double widen_float(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  if (e == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  // exponent rebiased 127 -> 1023 (255, infinity or NaN, -> 2047);
  // significand bits 22..3 in the high word, 2..0 at the top of the low word
  const uint32_t eb = e == 0xFFu ? 0x7FFu : e + 896u;
  const uint32_t hi = (u & 0x80000000u) | (eb << 20) | ((u & 0x7FFFFFu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}

// Input of the split operand builder: either a phasor from amplitude/OPD
// planes (one per PSF, for a list of wavelengths) or a complex field.
struct SplitFieldArgs {
  // phasor mode
  const double* amp;       // [batch][H][W] (mask already applied)
  const double* opd;       // [batch][H][W]
  int H, W, r0, c0;
  const float2* khalf;     // [L] (hi, lo) float pair of 2/lambda
  // complex mode
  const double2* field;    // [batch][m][n] complex128 (L 1)
  // common
  int m, n, kp, L, batch;
  const float* maxabs;     // [batch] max |component| of the field (device), or null: no scale
  uint16_t* hi;            // [batch*L][n][2*kp]
  uint16_t* lo;
  const int* lam_idx;      // optional [L] device: wavelength -> khalf slot
  // optional: nonzero flags of the field's 32 x 32 pieces, [batch][kp/32][kf_pitch]
  // bytes (written in full, padding columns included), for the MFT's K-block skip
  uint8_t* kflags;
  int kf_pitch;            // multiple of 8, >= 8 * ceil(kp2 / 256)
};
int launch_split_field_T(const SplitFieldArgs& a, bool bf16, cudaStream_t s);
// Tensor map of one plane (hi or lo) of the split f^T operand seen as
// [Q][n][2][kp] 16-bit values (x = row within a real/imaginary half of K,
// y = the half, z = field column c, w = problem), box {64, 1, 32, 1} with the
// 128-byte swizzle: the output tiles of the phasor operand kernel, clipped
// at kp and n (mft_split.cu).
int make_field_T_store_map(CUtensorMap* map, const uint16_t* ptr, bool bf16, int kp, int n, int Q);

// max over the slice of |amp| (phasor mode) or max(|re|,|im|) (complex mode)
int launch_maxabs_amp(const double* amp, int batch, int H, int W, int r0, int c0, int m, int n,
                      float* out, cudaStream_t s);
// per field b < batch of `count` entries each: out[b] = max(|re|, |im|)
int launch_maxabs_c128_batch(const double2* f, int count, int batch, float* out, cudaStream_t s);

// out[i,j] (+)= (re, im) scaled; generic complex128 copy/convert kernels
int launch_conj_scale(const double2* in, double2* out, size_t count, double scale, cudaStream_t s);

// mft_fp64.cu ------------------------------------------------------------
// Caller-provided memory for launch_zgemm's split-K partial products.  With
// one given, launch_zgemm never allocates: it splits K only as far as the
// partials fit in `bytes` (not at all when even two splits do not fit).
struct ZgemmScratch {
  void* ptr;
  size_t bytes;
};
// C[b] = alpha * A[b] . B[b] (complex128), row-major with leading dims and
// batch strides (elements).  beta == 0 overwrites C.  Without `scratch`, the
// split-K partials come from the device's stream-ordered pool.
int launch_zgemm(int M, int N, int K, const double2* A, int lda, long long sA,
                 const double2* B, int ldb, long long sB, double2* C, int ldc, long long sC,
                 int batch, double alpha, cudaStream_t s, const ZgemmScratch* scratch = nullptr);
// lgb_dft2_batch's body (plan.cu), with the FP64 GEMMs' split-K partials
// taken from `zs` when it is given (nothing is allocated then)
int dft2_batch(const double2* f, int count, int m, int n, double2* F, int M, int N,
               double alpha_r, double alpha_c, double shift_r, double shift_c, double offset_r,
               double offset_c, int unitary, int precision, void* workspace,
               size_t workspace_bytes, cudaStream_t s, const ZgemmScratch* zs);
// out[b] += sum_l weights[b][l] * unit2[l] * |F[b][l]|^2 into a window (FP64)
int launch_intensity_accum_c128(const double2* F, int M, int N, long long sF, int batch_inner,
                                const double* weights, const double* unit2, double* out,
                                int ld_out, long long s_out, int win_r0, int win_c0, int n_outer,
                                cudaStream_t s);
// batched complex128 phasor: out[b*L + l] = amp[b] * exp(2 pi i opd[b] / lambda_l) on a slice
int launch_phasor_batch_c128(const double* amp, const double* opd, int H, int W, int r0, int c0,
                             int m, int n, const double* two_over_lambda, int L, int batch,
                             double2* out, cudaStream_t s);

// mft_split.cu -----------------------------------------------------------
struct SplitMftProblem {
  // stage 1: G = E1 . f      A: E1 block [L][mrows1][2*kp1]   B: f^T [Q][n][2*kp1]
  // stage 2: F = G . E2      A: G        [Q][M][2*kp2]        B: E2 block [L][nrows2][2*kp2]
  int m, n, M, N;          // field and window shapes
  int kp1, kp2;            // round_up(m, 32), round_up(n, 32)
  int L, batch;            // wavelengths, PSFs; Q = batch * L problems
  bool bf16;
  const uint16_t *e1_hi, *e1_lo, *f_hi, *f_lo, *e2_hi, *e2_lo;
  uint16_t *g_hi, *g_lo;   // stage-1 output / stage-2 A operand
  const float* maxabs;     // [batch], max |component| of the unscaled field, or null: no scale
  // stage-2 epilogue
  int epilogue;            // 0: weighted intensity reduced into wbuf, 1: complex128 out
  const double* weights;   // [batch][L] (intensity) -- may be null (weight 1)
  const double* unit2;     // [L] |alpha_r alpha_c| (or 1)
  float* wbuf;             // intensity: [batch][M][ldw] FP32 window, zeroed by the caller
  int ldw;                 // multiple of 4
  double* out;             // complex: [batch * L][M][N] double2
  double complex_scale;    // complex epilogue: extra scale (unitary factor)
  int* err;                // device error flag
  cudaEvent_t* events;     // optional [4]: recorded around the stage-1 and stage-2 launches
  const int* lam_idx;      // optional [L] device: wavelength -> DFT-matrix slot
  int L_bank;              // DFT-matrix slots held (when lam_idx is set)
  int tile;                // pair-tile width 256 or 128; 0: the autotuner's choice
  // optional stage-1 K-block skip: the field's nonzero flags as written by
  // the split operand kernel ([batch][kp1/32][kf_pitch]); null: dense
  const uint8_t* kflags;
  int kf_pitch;
};
// bytes of a field-flag row (32-column pieces of a kp2-wide operand, padded
// to whole 256-column tiles)
inline int kflag_pitch(int kp2) { return 8 * ((kp2 + 255) / 256); }
int launch_split_mft(const SplitMftProblem& p, cudaStream_t s);
// scale applied to the stage-1 result before its 16-bit split
float split_g_scale(int m);
// out[b][win] += wbuf[b] (add) or out[b][win] = wbuf[b] (FP32 window -> float64 image)
int launch_window_add(const float* wbuf, int M, int N, int ldw, int batch, double* out, int ld_out,
                      long long out_bs, int win_r0, int win_c0, bool add, cudaStream_t s);

}  // namespace lgb
