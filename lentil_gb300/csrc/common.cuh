// Shared helpers for the lentil_gb300 CUDA library (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stddef.h>
#include <string>

#include "../../include/lentil_gb300.h"
#include <nvtx3/nvToolsExt.h>

namespace lgb {

// NVTX range over a C entry point: shows the library's calls on the
// timeline of Nsight tools; inert (one branch) when no tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define LGB_RANGE(name) ::lgb::NvtxRange lgb_nvtx_range_(name)


// ---------------------------------------------------------------------------
// error reporting: every entry point returns an int status and records a
// message retrievable with lgb_last_error() (thread-local, never aborts)
// ---------------------------------------------------------------------------
int set_error(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);

#define LGB_CUDA(call)                                                  \
  do {                                                                  \
    cudaError_t _e = (call);                                            \
    if (_e != cudaSuccess) return ::lgb::check_cuda(_e, #call);         \
  } while (0)

#define LGB_REQUIRE(cond, code, msg)                                    \
  do {                                                                  \
    if (!(cond)) return ::lgb::set_error((code), (msg));                \
  } while (0)

inline cudaStream_t as_stream(lgb_stream s) { return reinterpret_cast<cudaStream_t>(s); }

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
inline int cdiv(int a, int b) { return (a + b - 1) / b; }
inline int round_up(int a, int b) { return cdiv(a, b) * b; }

// Number of SMs of the current device (cached per device).
int sm_count();

// ---------------------------------------------------------------------------
// DFT phase in exact fixed point.
//
// A DFT-matrix entry of lentil's matrix triple product is
//     exp(-2*pi*i * alpha * (R + offset) * (U - shift))
// (lentil/fourier.py:106-110).  The phase argument reaches ~1e2-1e3 cycles,
// so it is reduced modulo one cycle *before* any trigonometry:
//     offset = oi + of,  shift = si + sf   (oi, si integers, |of|,|sf| <= 1/2)
//     X = R + oi,  Y = U - si              (exact integers)
//     alpha*x*y = alpha*X*Y - (alpha*sf)*X + (alpha*of)*Y - alpha*of*sf
// Each product is taken in unsigned 64-bit two's-complement arithmetic with
// the cycle fraction scaled by 2^64, so the reduction modulo 1 is the natural
// integer wrap-around.  alpha mod 1 is carried with 128 fractional bits, which
// makes the dominant alpha*X*Y term exact to 2^-64 cycles for |X*Y| < 2^62.
// ---------------------------------------------------------------------------
struct PhaseAxis {
  uint64_t a_hi, a_lo;   // frac(alpha) * 2^128  (128-bit, high/low words)
  uint64_t b_sf;         // frac(alpha*sf) * 2^64
  uint64_t b_of;         // frac(alpha*of) * 2^64
  uint64_t b_c;          // frac(alpha*of*sf) * 2^64
  int64_t  x0;           // X of input index 0:  -floor(len_in/2) + oi
  int64_t  y0;           // Y of output index 0: -floor(len_out/2) - si
};

// Host: build a PhaseAxis (alpha, shift, offset, input length, output length).
int make_phase_axis(double alpha, double shift, double offset, int len_in, int len_out,
                    PhaseAxis* ax);

// Device: cycle fraction * 2^64 of alpha*(R_i + offset)*(U_j - shift).
__device__ __forceinline__ uint64_t phase_fixed(const PhaseAxis& ax, int i_in, int j_out) {
  const int64_t X = ax.x0 + i_in;
  const int64_t Y = ax.y0 + j_out;
  const int64_t P = X * Y;
  const uint64_t Pu = (uint64_t)P;
  uint64_t hi = __umul64hi(ax.a_lo, Pu);
  if (P < 0) hi -= ax.a_lo;                    // signed high product
  uint64_t ph = ax.a_hi * Pu + hi;             // frac(alpha*P) * 2^64
  ph -= ax.b_sf * (uint64_t)X;
  ph += ax.b_of * (uint64_t)Y;
  ph -= ax.b_c;
  return ph;
}

// Increment of phase_fixed(ax, i, j) from input index i to i + 1 at output
// index j: frac(alpha*Y) - frac(alpha*sf) in the same 2^-64-cycle units.  A
// phase stepped by it agrees with phase_fixed to a few units of 2^-64 cycles
// (the truncated low half of alpha's 128-bit product).
__device__ __forceinline__ uint64_t phase_step_in(const PhaseAxis& ax, int j_out) {
  const int64_t Y = ax.y0 + j_out;
  const uint64_t Yu = (uint64_t)Y;
  uint64_t hi = __umul64hi(ax.a_lo, Yu);
  if (Y < 0) hi -= ax.a_lo;
  return ax.a_hi * Yu + hi - ax.b_sf;
}

// exp(-2*pi*i*phase) in double precision from the fixed-point phase.
__device__ __forceinline__ double2 expm2pi_fixed_f64(uint64_t ph) {
  const double x = (double)(int64_t)ph * 0x1p-63;   // half-cycles in [-1, 1)
  double s, c;
  sincospi(x, &s, &c);
  return make_double2(c, -s);
}

// exp(-2*pi*i*phase) in single precision from the fixed-point phase.
__device__ __forceinline__ float2 expm2pi_fixed_f32(uint64_t ph) {
  const float x = (float)(int32_t)(ph >> 32) * 0x1p-31f;
  float s, c;
  sincospif(x, &s, &c);
  return make_float2(c, -s);
}

// ---------------------------------------------------------------------------
// split of an fp32 value into two 16-bit floats: x ~= hi + lo
// ---------------------------------------------------------------------------
template <bool BF16> struct Split16;
template <> struct Split16<true> {
  static __device__ __forceinline__ void split(float x, uint16_t& hi, uint16_t& lo) {
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    hi = __bfloat16_as_ushort(h);
    lo = __bfloat16_as_ushort(l);
  }
};
template <> struct Split16<false> {
  static __device__ __forceinline__ void split(float x, uint16_t& hi, uint16_t& lo) {
    __half h = __float2half_rn(x);
    __half l = __float2half_rn(x - __half2float(h));
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(l);
  }
};

// Two values at once, packed as two 16-bit lanes (x0 in the low half, x1 in
// the high half) with paired conversions; each lane equals Split16::split.
template <bool BF16> struct Split16x2;
template <> struct Split16x2<true> {
  static __device__ __forceinline__ void split(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  }
};
template <> struct Split16x2<false> {
  static __device__ __forceinline__ void split(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    const __half2 h = __floats2half2_rn(x0, x1);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  }
};

}  // namespace lgb
