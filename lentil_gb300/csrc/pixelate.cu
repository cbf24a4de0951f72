// K6: detector pixel MTF and pixelation (lentil/detector.py:167-251).
//
// lentil applies the pixel MTF as |ifft2(fft2(img) * (s (x) s))| with
// s[k] = sinc(fftfreq(N)[k] * os) (lentil/detector.py:218-222), for square
// N x N images.  Two FP64 evaluations of that product:
//   - N a power of two (<= 8192): the product is separable, C . img . C^T
//     with C = ifft diag(s) fft real and symmetric (s is real and even), so
//     each axis is filtered by this file's shared-memory radix-2 FFTs with two
//     real rows packed into one complex transform (fft, times s, inverse fft:
//     C a + i C b), between tiled transposes (~5 N^2 log2 N flop), in
//     double-float arithmetic (below);
//   - any other N: |C . img . C^T| with C the real symmetric circulant
//     C[i][j] = c[(i - j) mod N], c = ifft(s), as two FP64 GEMMs.
// pixelate then resamples by 1/os with a cubic spline (lentil/util.py:261-349);
// when N is a multiple of os every sample falls on a grid point, so the
// result is d = p[::os, ::os] rescaled by sum(p)/sum(d) and masked where
// d == 0; otherwise the spline evaluation runs as two banded FP64 passes
// (the off-grid section below).
//
// The same FFT machinery also filters white noise for lgb_power_spectrum
// (lentil/wfe.py:8-70), defined at the end of this file.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

__device__ __forceinline__ double sinc_os(int k, int N, double os) {
  const int ff = (k < (N + 1) / 2) ? k : k - N;          // numpy fftfreq ordering
  const double x = (double)ff / N * os;
  return (x == 0.0) ? 1.0 : sinpi(x) / (M_PI * x);
}

// ---------------------------------------------------------------- FFT path
__global__ void real_to_complex_kernel(const double* __restrict__ x, double2* __restrict__ z,
                                       size_t count) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < count;
       p += (size_t)gridDim.x * blockDim.x)
    z[p] = make_double2(x[p], 0.0);
}

// Double-float arithmetic: a value as the unevaluated sum hi + lo of two
// floats (about 48 significant bits).  This part's FP64 units retire about
// two FMAs a clock per SM against 128 FP32 lanes, so the pixel-MTF FFTs run
// in float pairs: ~90 FP32 operations per radix-2 butterfly in place of ~8
// FP64 ones, at a rounding error near 2^-47 per operation (the FFT of
// N <= 8192 points stays near 1e-14 of the signal).  Sums use Knuth's
// error-free two-sum, products the FMA residual, each renormalised with
// Dekker's fast two-sum; the _rn intrinsics keep the compiler from fusing
// the steps whose rounding the transformations rely on.
struct dfl {
  float hi, lo;
};
__device__ __forceinline__ dfl df_renorm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return df_renorm(s, e);
}
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, {-b.hi, -b.lo}); }
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_renorm(p, e);
}
// a complex double-float value (re.hi, re.lo, im.hi, im.lo) as one float4
__device__ __forceinline__ float4 df_pack(dfl re, dfl im) { return make_float4(re.hi, re.lo, im.hi, im.lo); }

// exp(-2 pi i k / N), k < N/2, as double-float pairs
__global__ void twiddle_df_kernel(int N, float4* __restrict__ tw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N / 2) return;
  double s, c;
  sincospi(-2.0 * (double)k / N, &s, &c);
  const float2 cc = split_double(c), ss = split_double(s);
  tw[k] = make_float4(cc.x, cc.y, ss.x, ss.y);
}

// Radix-2 butterflies over a bit-reversed row of complex double-float values
// in shared memory: natural order out (the caller syncs before; this returns
// after a final sync).
__device__ __forceinline__ void fft_stages_df(float4* sm, int N, int logN,
                                              const float4* __restrict__ tw, bool inverse) {
  for (int st = 1; st <= logN; ++st) {
    const int half = 1 << (st - 1);
    const int stride = N >> st;                        // twiddle index step
    for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
      const int pos = b & (half - 1);
      const int i0 = ((b >> (st - 1)) << st) + pos, i1 = i0 + half;
      const float4 w4 = tw[pos * stride];
      const dfl wr{w4.x, w4.y};
      const dfl wi = inverse ? dfl{-w4.z, -w4.w} : dfl{w4.z, w4.w};
      const float4 a4 = sm[i0], v4 = sm[i1];
      const dfl ar{a4.x, a4.y}, ai{a4.z, a4.w}, vr{v4.x, v4.y}, vi{v4.z, v4.w};
      const dfl tr = df_sub(df_mul(wr, vr), df_mul(wi, vi));
      const dfl ti = df_add(df_mul(wr, vi), df_mul(wi, vr));
      sm[i0] = df_pack(df_add(ar, tr), df_add(ai, ti));
      sm[i1] = df_pack(df_sub(ar, tr), df_sub(ai, ti));
    }
    __syncthreads();
  }
}

// In-place FFT of every complex float64 row (length N = 2^logN) in shared
// memory, in double-float arithmetic (the power-spectrum filter); the
// inverse scales by 1/N.
__global__ void __launch_bounds__(512) fft_rows_kernel(double2* __restrict__ data, int N, int logN,
                                                       const float4* __restrict__ tw,
                                                       int inverse) {
  extern __shared__ float4 smf[];
  double2* row = data + (size_t)blockIdx.x * N;
  const int shift = 32 - logN;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double2 v = row[i];
    const float2 re = split_double(v.x), im = split_double(v.y);
    smf[__brev((unsigned)i) >> shift] = make_float4(re.x, re.y, im.x, im.y);
  }
  __syncthreads();
  fft_stages_df(smf, N, logN, tw, inverse != 0);
  const float sc = inverse ? 1.f / (float)N : 1.f;      // a power of two: exact
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const float4 z = smf[i];
    row[i] = make_double2(widen_float(z.x * sc) + widen_float(z.y * sc),
                          widen_float(z.z * sc) + widen_float(z.w * sc));
  }
}

// The pixel MTF along rows: out_row = C . in_row with C = ifft diag(s) fft,
// s = sinc(fftfreq(N) * os) real and even, so C is real.  Two real rows a, b
// ride one complex transform z = a + i b: fft, times s, inverse fft gives
// C a + i C b.  One block per row pair, one N-point buffer (the spectrum is
// bit-reversed in place between the two transforms).  The float64 rows enter
// and leave as double-float pairs by integer conversions (split_double,
// widen_float), so the FP64 pipe only adds each output's two halves.
__global__ void __launch_bounds__(512) pixel_filter_rows_kernel(const double* __restrict__ in,
                                                                double* __restrict__ out, int N,
                                                                int logN,
                                                                const float4* __restrict__ tw,
                                                                const double* __restrict__ sinc) {
  extern __shared__ float4 smf[];
  const size_t r0 = 2 * (size_t)blockIdx.x;
  const double* ra = in + r0 * N;
  const double* rb = ra + N;
  const int shift = 32 - logN;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const float2 a = split_double(ra[i]), b = split_double(rb[i]);
    smf[__brev((unsigned)i) >> shift] = make_float4(a.x, a.y, b.x, b.y);
  }
  __syncthreads();
  fft_stages_df(smf, N, logN, tw, false);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const float2 k2 = split_double(sinc[i]);
    const dfl k{k2.x, k2.y};
    const float4 z = smf[i];
    smf[i] = df_pack(df_mul({z.x, z.y}, k), df_mul({z.z, z.w}, k));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {     // bit-reverse in place
    const int j = (int)(__brev((unsigned)i) >> shift);
    if (i < j) {
      const float4 t = smf[i];
      smf[i] = smf[j];
      smf[j] = t;
    }
  }
  __syncthreads();
  fft_stages_df(smf, N, logN, tw, true);
  const float sc = 1.f / (float)N;                        // a power of two: exact
  double* oa = out + r0 * N;
  double* ob = oa + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const float4 z = smf[i];
    oa[i] = widen_float(z.x * sc) + widen_float(z.y * sc);
    ob[i] = widen_float(z.z * sc) + widen_float(z.w * sc);
  }
}

// out = in^T (N x N float64), 32 x 32 tiles
__global__ void transpose_f64_kernel(const double* __restrict__ in, double* __restrict__ out, int N) {
  __shared__ double t[32][33];
  const int x = blockIdx.x * 32 + threadIdx.x, y0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y)
    if (x < N && y0 + k < N) t[k][threadIdx.x] = in[(size_t)(y0 + k) * N + x];
  __syncthreads();
  const int xo = blockIdx.y * 32 + threadIdx.x, yo0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y)
    if (xo < N && yo0 + k < N) out[(size_t)(yo0 + k) * N + xo] = t[threadIdx.x][k];
}

// out = in^T (N x N complex128), 32 x 32 tiles
__global__ void transpose_c128_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                                      int N) {
  __shared__ double2 t[32][33];
  const int x = blockIdx.x * 32 + threadIdx.x, y0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y)
    if (x < N && y0 + k < N) t[k][threadIdx.x] = in[(size_t)(y0 + k) * N + x];
  __syncthreads();
  const int xo = blockIdx.y * 32 + threadIdx.x, yo0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y)
    if (xo < N && yo0 + k < N) out[(size_t)(yo0 + k) * N + xo] = t[threadIdx.x][k];
}

// s[k] = sinc(fftfreq(N)[k] * os): N values, computed once per call (FP64
// sinpi is slow on this part's FP64 pipe; the N^2 products below only read)
__global__ void sinc_table_kernel(int N, double os, double* __restrict__ s) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < N) s[k] = sinc_os(k, N, os);
}

// ------------------------------------------------------------- GEMM path
// c[k] = (1/N) sum_f s_f cos(2 pi f k / N)
__global__ void pixel_taps_kernel(int N, const double* __restrict__ sinc, double* __restrict__ c) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  double acc = 0.0;
  for (int f = 0; f < N; ++f) {
    const long long ph = ((long long)f * k) % N;         // exact phase index
    acc += sinc[f] * cospi(2.0 * (double)ph / N);
  }
  c[k] = acc / N;
}

__global__ void circulant_kernel(int N, const double* __restrict__ c, double* __restrict__ C) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= N) return;
  C[(size_t)i * N + j] = c[(i - j + N) % N];
}

constexpr int DBM = 64, DBN = 64, DBK = 16;

// C = A . B (real, row-major, N x N), FP64 tiles of 64 x 64, 4 x 4 per thread
__global__ void __launch_bounds__(256) dgemm_kernel(int N, const double* __restrict__ A,
                                                    const double* __restrict__ B,
                                                    double* __restrict__ C) {
  __shared__ double As[DBK][DBM + 1];
  __shared__ double Bs[DBK][DBN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4, tid = threadIdx.x;
  const int m0 = blockIdx.y * DBM, n0 = blockIdx.x * DBN;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  for (int k0 = 0; k0 < N; k0 += DBK) {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int e = tid + 256 * t;
      const int ar = e >> 4, ak = e & 15;
      As[ak][ar] = (m0 + ar < N && k0 + ak < N) ? A[(size_t)(m0 + ar) * N + k0 + ak] : 0.0;
      const int bk = e >> 6, bc = e & 63;
      Bs[bk][bc] = (k0 + bk < N && n0 + bc < N) ? B[(size_t)(k0 + bk) * N + n0 + bc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < DBK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = m0 + ty + 16 * i, c = n0 + tx + 16 * j;
      if (r < N && c < N) C[(size_t)r * N + c] = acc[i][j];
    }
}

// ---------------------------------------------------------- common tail
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// p = |value| written to P; sums[0] += sum p; decimated samples
// d[k][l] = p[k*os][l*os] with sums[1] += sum d.  Reads a real (GEMM path)
// or complex (FFT path) array.
template <bool COMPLEX>
__global__ void pixel_abs_reduce_kernel(int N, int os, const void* __restrict__ src,
                                        double* __restrict__ P, double* __restrict__ d,
                                        double* __restrict__ sums) {
  double s_all = 0.0, s_dec = 0.0;
  const size_t total = (size_t)N * N;
  const int Nd = N / os;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    double v;
    if (COMPLEX) {
      const double2 z = static_cast<const double2*>(src)[p];
      v = hypot(z.x, z.y);
    } else {
      v = fabs(static_cast<const double*>(src)[p]);
    }
    if (P) P[p] = v;
    s_all += v;
    const int i = (int)(p / N), j = (int)(p % N);
    if (d && i % os == 0 && j % os == 0) {
      d[(size_t)(i / os) * Nd + j / os] = v;
      s_dec += v;
    }
  }
  s_all = warp_sum(s_all);
  s_dec = warp_sum(s_dec);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums, s_all);
    if (d) atomicAdd(sums + 1, s_dec);
  }
}

// out = d * sum(p)/sum(d) where d != 0, else 0 (lentil/util.py:341-347)
__global__ void pixelate_scale_kernel(int count, const double* __restrict__ d,
                                      const double* __restrict__ sums, double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  const double v = d[p];
  out[p] = (v != 0.0) ? v * (sums[0] / sums[1]) : 0.0;
}

// ------------------------------------------------- off-grid cubic resampling
// lentil resamples with scipy.ndimage.map_coordinates(order=3,
// mode='nearest') at x_k = (k - S/2) / (1/os) + N/2 on both axes
// (lentil/util.py:323-340).  That evaluation is: pad the image by RS_PAD
// edge copies per side, prefilter each axis of the padded image into cubic
// B-spline coefficients with a half-sample-symmetric boundary, and sum the
// four coefficients around x + RS_PAD weighted by the cubic B-spline
// beta3 (Unser, Aldroubi & Eden, IEEE TSP 41(2), 1993).  The prefilter is
// the symmetric convolution with h[t] = sqrt(3) z^|t|, z = sqrt(3) - 2, so
// each output sample is a fixed linear combination of a window of input
// samples: with h truncated at |t| <= RS_TAPS (|z|^31 < 2e-18 of the
// signal) the window is RS_BW = 2 RS_TAPS + 4 wide, and the whole
// resampling is out = G p G^T with G banded, S x RS_BW plus a start index
// per row.  Both passes are FP64 FMA over L2-resident operands.
constexpr int RS_PAD = 12, RS_TAPS = 30, RS_BW = 2 * RS_TAPS + 4;

__host__ __device__ __forceinline__ double rs_coord(int k, int S, int N, int os) {
  return ((double)k - S / 2.0) / (1.0 / os) + N / 2.0;
}

__device__ __forceinline__ int rs_reflect(int r, int L) {   // half-sample symmetric
  r %= 2 * L;
  if (r < 0) r += 2 * L;
  return r >= L ? 2 * L - 1 - r : r;
}

__device__ __forceinline__ double rs_beta3(double t) {
  t = fabs(t);
  if (t < 1.0) return 2.0 / 3.0 - t * t + t * t * t / 2.0;
  if (t < 2.0) { const double u = 2.0 - t; return u * u * u / 6.0; }
  return 0.0;
}

__device__ __forceinline__ int rs_start(int k, int S, int N, int os) {
  const int i0 = (int)floor(rs_coord(k, S, N, os) + RS_PAD) - 1;
  return min(max(i0 - RS_TAPS - RS_PAD, 0), max(0, N - RS_BW));
}

// Gt[b][k] = weight of input sample q0[k] + b in output sample k
__global__ void resample_operator_kernel(int N, int os, int S, double* __restrict__ Gt,
                                         int* __restrict__ q0) {
  __shared__ double h[RS_TAPS + 1];
  if (threadIdx.x == 0) {
    const double z = sqrt(3.0) - 2.0;
    h[0] = sqrt(3.0);
    for (int a = 1; a <= RS_TAPS; ++a) h[a] = h[a - 1] * z;
  }
  __syncthreads();
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= S * RS_BW) return;
  const int k = idx / RS_BW, b = idx - k * RS_BW;
  const int Np = N + 2 * RS_PAD;
  const double xp = rs_coord(k, S, N, os) + RS_PAD;
  const int i0 = (int)floor(xp) - 1;
  const int start = rs_start(k, S, N, os);
  const int want = start + b;
  double g = 0.0;
  for (int j = i0; j < i0 + 4; ++j) {
    const double w = rs_beta3(xp - j);
    const int jj = rs_reflect(j, Np);
    for (int t = -RS_TAPS; t <= RS_TAPS; ++t) {
      const int q = min(max(rs_reflect(jj - t, Np) - RS_PAD, 0), N - 1);
      if (q == want) g += w * h[t < 0 ? -t : t];
    }
  }
  Gt[(size_t)b * S + k] = g;
  if (b == 0) q0[k] = start;
}

constexpr int RS_ROWS = 8;        // image rows per thread in the row pass

// Tm[r][l] = sum_b Gt[b][l] p[r][q0[l] + b]; block (64, 4), RS_ROWS rows a thread
__global__ void __launch_bounds__(256) resample_rows_kernel(const double* __restrict__ p, int N,
                                                            int S, const double* __restrict__ Gt,
                                                            const int* __restrict__ q0,
                                                            double* __restrict__ Tm) {
  const int l = blockIdx.x * 64 + threadIdx.x;
  const int r0 = (blockIdx.y * 4 + threadIdx.y) * RS_ROWS;
  if (l >= S || r0 >= N) return;
  const int q = q0[l];
  const int nb = min(RS_BW, N - q);
  const int nr = min(RS_ROWS, N - r0);
  const double* src = p + (size_t)r0 * N + q;
  double acc[RS_ROWS];
#pragma unroll
  for (int i = 0; i < RS_ROWS; ++i) acc[i] = 0.0;
  for (int b = 0; b < nb; ++b) {
    const double g = Gt[(size_t)b * S + l];
#pragma unroll
    for (int i = 0; i < RS_ROWS; ++i)
      if (i < nr) acc[i] = fma(g, src[(size_t)i * N + b], acc[i]);
  }
#pragma unroll
  for (int i = 0; i < RS_ROWS; ++i)
    if (i < nr) Tm[(size_t)(r0 + i) * S + l] = acc[i];
}

constexpr int RS_OUT = 4;         // output rows per thread in the column pass

// raw[k][l] = sum_b Gt[b][k] Tm[q0[k] + b][l]; sums[2] += sum raw
__global__ void __launch_bounds__(256) resample_cols_kernel(const double* __restrict__ Tm, int N,
                                                            int S, const double* __restrict__ Gt,
                                                            const int* __restrict__ q0,
                                                            double* __restrict__ raw,
                                                            double* __restrict__ sums) {
  const int l = blockIdx.x * 64 + threadIdx.x;
  const int k0 = (blockIdx.y * 4 + threadIdx.y) * RS_OUT;
  double part = 0.0;
  if (l < S) {
    for (int i = 0; i < RS_OUT && k0 + i < S; ++i) {
      const int k = k0 + i, q = q0[k];
      const int nb = min(RS_BW, N - q);
      const double* src = Tm + (size_t)q * S + l;
      double acc = 0.0;
      for (int b = 0; b < nb; ++b) acc = fma(Gt[(size_t)b * S + k], src[(size_t)b * S], acc);
      raw[(size_t)k * S + l] = acc;
      part += acc;
    }
  }
  part = warp_sum(part);
  if ((threadIdx.x & 31) == 0) atomicAdd(sums + 2, part);
}

// out = (raw * (sum p / sum raw)) * mask, the mask being the order-1
// nearest-mode interpolation of (p != 0) at the same points, zeroed below
// DBL_EPSILON (lentil/util.py:317-320, 333-347)
__global__ void resample_finish_kernel(const double* __restrict__ raw,
                                       const double* __restrict__ p, int N, int S, int os,
                                       const double* __restrict__ sums, double* __restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= S * S) return;
  const int k = idx / S, l = idx - k * S;
  const double y = rs_coord(k, S, N, os), x = rs_coord(l, S, N, os);
  const int iy = (int)floor(y), ix = (int)floor(x);
  const double fy = y - iy, fx = x - ix;
  const int ya = min(max(iy, 0), N - 1), yb = min(max(iy + 1, 0), N - 1);
  const int xa = min(max(ix, 0), N - 1), xb = min(max(ix + 1, 0), N - 1);
  auto m = [&](int r, int c) { return p[(size_t)r * N + c] != 0.0 ? 1.0 : 0.0; };
  double mask = (1.0 - fy) * ((1.0 - fx) * m(ya, xa) + fx * m(ya, xb)) +
                fy * ((1.0 - fx) * m(yb, xa) + fx * m(yb, xb));
  if (mask < 2.220446049250313e-16) mask = 0.0;
  out[idx] = (raw[idx] * (sums[0] / sums[2])) * mask;
}

// S = ceil(N * (1/os)), evaluated as numpy does (lentil/util.py:323-324)
static int resample_size(int N, int os) { return (int)std::ceil((double)N * (1.0 / os)); }

// every resample point an exact grid point k * os
static bool resample_on_grid(int N, int os, int S) {
  if ((long long)S * os != N) return false;
  for (int k = 0; k < S; ++k)
    if (rs_coord(k, S, N, os) != (double)k * os) return false;
  return true;
}

static bool fft_size(int N, int* logN) {
  if (N < 2 || N > 8192 || (N & (N - 1))) return false;
  int l = 0;
  while ((1 << l) < N) ++l;
  *logN = l;
  return true;
}

struct PixelSpace {
  double* sums;          // [0] sum p, [1] sum of the grid samples, [2] sum of the resampled
  double* sinc;          // [N] sinc(fftfreq * os)
  double* d;
  // GEMM path
  double *c, *C, *T, *P;
  // FFT path
  double2 *X, *Y, *tw;
  // off-grid resampling: operator and the two passes
  double *Gt, *Tm, *raw;
  int* q0;
};

static size_t pixel_space(void* ws, int N, int os, PixelSpace* s) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = align_up(off, 256);
    void* p = ws ? static_cast<char*>(ws) + off : nullptr;
    off += bytes;
    return p;
  };
  PixelSpace t{};
  int logN;
  const size_t NN = (size_t)N * N;
  const int Nd = N / std::max(os, 1);
  t.sums = static_cast<double*>(take(4 * sizeof(double)));
  t.sinc = static_cast<double*>(take((size_t)N * sizeof(double)));
  t.d = static_cast<double*>(take((size_t)Nd * Nd * sizeof(double)));
  const bool fft = fft_size(N, &logN);
  if (fft) {
    t.X = static_cast<double2*>(take(NN * sizeof(double2)));
    t.Y = static_cast<double2*>(take(NN * sizeof(double2)));
    t.tw = static_cast<double2*>(take((size_t)(N / 2) * sizeof(double2)));
  } else {
    t.c = static_cast<double*>(take(N * sizeof(double)));
    t.C = static_cast<double*>(take(NN * sizeof(double)));
    t.T = static_cast<double*>(take(NN * sizeof(double)));
    t.P = static_cast<double*>(take(NN * sizeof(double)));
  }
  const int S = resample_size(N, std::max(os, 1));
  if (!resample_on_grid(N, std::max(os, 1), S)) {
    t.Gt = static_cast<double*>(take((size_t)RS_BW * S * sizeof(double)));
    t.q0 = static_cast<int*>(take((size_t)S * sizeof(int)));
    t.Tm = static_cast<double*>(take((size_t)N * S * sizeof(double)));
    t.raw = static_cast<double*>(take((size_t)S * S * sizeof(double)));
  }
  if (s) *s = t;
  return off;
}

// Runs the MTF product; returns (src, complex?) of the pre-abs result.
static int run_pixel(const double* img, int N, int os, void* ws, cudaStream_t s, PixelSpace* w,
                     const void** src, bool* is_complex) {
  pixel_space(ws, N, os, w);
  LGB_CUDA(cudaMemsetAsync(w->sums, 0, 4 * sizeof(double), s));
  sinc_table_kernel<<<cdiv(N, 256), 256, 0, s>>>(N, (double)os, w->sinc);
  int logN;
  if (fft_size(N, &logN)) {
    // separable filter P = C . img . C^T (C real symmetric): filter the rows,
    // transpose, filter the rows again, transpose back; X and Y hold the real
    // N x N intermediates
    double* R = reinterpret_cast<double*>(w->X);
    double* RT = reinterpret_cast<double*>(w->Y);
    float4* const twd = reinterpret_cast<float4*>(w->tw);   // N/2 entries of 16 bytes
    twiddle_df_kernel<<<cdiv(std::max(N / 2, 1), 256), 256, 0, s>>>(N, twd);
    const size_t smem = (size_t)N * sizeof(float4);
    LGB_CUDA(cudaFuncSetAttribute(pixel_filter_rows_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  8192 * (int)sizeof(float4)));
    const int threads = std::min(512, std::max(32, N / 2));
    const dim3 tgrid(cdiv(N, 32), cdiv(N, 32)), tblock(32, 8);
    pixel_filter_rows_kernel<<<N / 2, threads, smem, s>>>(img, R, N, logN, twd, w->sinc);
    transpose_f64_kernel<<<tgrid, tblock, 0, s>>>(R, RT, N);
    pixel_filter_rows_kernel<<<N / 2, threads, smem, s>>>(RT, R, N, logN, twd, w->sinc);
    transpose_f64_kernel<<<tgrid, tblock, 0, s>>>(R, RT, N);
    LGB_CUDA(cudaGetLastError());
    w->P = RT;
    *src = RT;
    *is_complex = false;
    return LGB_OK;
  }
  pixel_taps_kernel<<<cdiv(N, 128), 128, 0, s>>>(N, w->sinc, w->c);
  circulant_kernel<<<dim3(cdiv(N, 128), N), 128, 0, s>>>(N, w->c, w->C);
  dim3 grid(cdiv(N, DBN), cdiv(N, DBM));
  dgemm_kernel<<<grid, 256, 0, s>>>(N, w->C, img, w->T);      // T = C . img
  dgemm_kernel<<<grid, 256, 0, s>>>(N, w->T, w->C, w->P);     // P = T . C^T (C symmetric)
  LGB_CUDA(cudaGetLastError());
  *src = w->P;
  *is_complex = false;
  return LGB_OK;
}

static int abs_reduce(int N, int os, const void* src, bool cplx, double* P, double* d,
                      double* sums, cudaStream_t s) {
  const int blocks = std::max(1, std::min(4 * sm_count(), cdiv(N * N, 256)));
  if (cplx) pixel_abs_reduce_kernel<true><<<blocks, 256, 0, s>>>(N, os, src, P, d, sums);
  else pixel_abs_reduce_kernel<false><<<blocks, 256, 0, s>>>(N, os, src, P, d, sums);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// ------------------------------------------------------ power spectrum
// psd(i, j) of lentil/wfe.py:41-52 on a square N x N grid: offsets from
// (N//2 + 1), cycles per pixel, 1 / (1 + (dr/f0)^exp), 0 at dr == 0
__device__ __forceinline__ double psd_at(int i, int j, int N, double f0, double expo) {
  const double c = floor(N / 2.0) + 1.0;
  const double yy = ((double)i - c) / N, xx = ((double)j - c) / N;
  const double dr = sqrt(xx * xx + yy * yy);
  return dr == 0.0 ? 0.0 : 1.0 / (1.0 + pow(dr / f0, expo));
}

constexpr int PSD_BLOCKS = 128;

// fixed-order two-pass sums: pass 1 writes PSD_BLOCKS partials of (a, b)
__device__ __forceinline__ void psd_block_store2(double a, double b, double* partial) {
  __shared__ double sa[8], sb[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) { sa[threadIdx.x >> 5] = a; sb[threadIdx.x >> 5] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { ta += sa[w]; tb += sb[w]; }
    partial[2 * blockIdx.x] = ta;
    partial[2 * blockIdx.x + 1] = tb;
  }
}

__global__ void __launch_bounds__(256) psd_sum_kernel(int N, double f0, double expo,
                                                      double* __restrict__ partial) {
  const size_t total = (size_t)N * N;
  double a = 0.0;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x)
    a += psd_at((int)(p / N), (int)(p % N), N, f0, expo);
  psd_block_store2(a, 0.0, partial);
}

// opd = Re(z) * N * mask (z complex or real), then (count of nonzero, sum opd^2)
template <bool CPLX>
__global__ void __launch_bounds__(256) psd_mask_kernel(const void* __restrict__ z,
                                                       const double* __restrict__ mask, int N,
                                                       double scale, double* __restrict__ opd,
                                                       double* __restrict__ partial) {
  const size_t total = (size_t)N * N;
  double cnt = 0.0, ss = 0.0;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const double re = CPLX ? static_cast<const double2*>(z)[p].x : static_cast<const double*>(z)[p];
    const double v = re * scale * mask[p];
    opd[p] = v;
    if (v != 0.0) { cnt += 1.0; ss += v * v; }
  }
  psd_block_store2(cnt, ss, partial);
}

__global__ void psd_final_kernel(const double* __restrict__ partial, int nblocks,
                                 double* __restrict__ sums) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nblocks; ++k) { a += partial[2 * k]; b += partial[2 * k + 1]; }
    sums[0] = a;
    sums[1] = b;
  }
}

// Y *= fftshift(sqrt(psd / sum)); psd is symmetric under i <-> j, so the
// transposed spectrum of the FFT path takes the same filter
__global__ void psd_filter_kernel(double2* __restrict__ Y, int N, double f0, double expo,
                                  const double* __restrict__ sums) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= N) return;
  const int h = N / 2;                                  // fftshift: index k <- (k - N//2) mod N
  const int si = (i - h + N) % N, sj = (j - h + N) % N;
  const double H = sqrt(psd_at(si, sj, N, f0, expo) / sums[0]);
  double2 v = Y[(size_t)i * N + j];
  Y[(size_t)i * N + j] = make_double2(v.x * H, v.y * H);
}

__global__ void psd_rescale_kernel(double* __restrict__ opd, size_t count,
                                   const double* __restrict__ sums, double rms) {
  const double k = sqrt(sums[0] / sums[1]) * rms;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < count;
       p += (size_t)gridDim.x * blockDim.x)
    opd[p] *= k;
}

struct PsdSpace {
  double* partial;
  double* sums;          // [0] psd sum, then [0] count / [1] sum of squares
  double2 *X, *Y, *tw;   // FFT path (tw only) / DFT path (E, Ec in tw's place)
  double2 *E, *Ec;
};

static size_t psd_space(void* ws, int N, PsdSpace* s) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    off = align_up(off, 256);
    void* p = ws ? static_cast<char*>(ws) + off : nullptr;
    off += bytes;
    return p;
  };
  PsdSpace t{};
  const size_t NN = (size_t)N * N;
  int logN;
  t.partial = static_cast<double*>(take(2 * PSD_BLOCKS * sizeof(double)));
  t.sums = static_cast<double*>(take(4 * sizeof(double)));
  t.X = static_cast<double2*>(take(NN * sizeof(double2)));
  t.Y = static_cast<double2*>(take(NN * sizeof(double2)));
  if (fft_size(N, &logN)) {
    t.tw = static_cast<double2*>(take((size_t)(N / 2) * sizeof(double2)));
  } else {
    t.E = static_cast<double2*>(take(NN * sizeof(double2)));
    t.Ec = static_cast<double2*>(take(NN * sizeof(double2)));
  }
  if (s) *s = t;
  return off;
}

}  // namespace lgb

using namespace lgb;

extern "C" size_t lgb_pixel_workspace_size(int N, int oversample) {
  if (N <= 0 || oversample <= 0) return 0;
  return pixel_space(nullptr, N, oversample, nullptr);
}

extern "C" int lgb_pixel(const double* img, int rows, int cols, int oversample, double* out,
                         void* workspace, size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_pixel");
  LGB_REQUIRE(img && out && workspace, LGB_EINVAL, "pixel: null pointer");
  LGB_REQUIRE(rows == cols, LGB_EINVAL, "pixel: the pixel MTF is defined for square images");
  LGB_REQUIRE(rows > 0 && oversample > 0, LGB_EINVAL, "pixel: sizes must be positive");
  LGB_REQUIRE(workspace_bytes >= lgb_pixel_workspace_size(rows, oversample), LGB_EWORKSPACE,
              "pixel: workspace too small");
  const int N = rows;
  cudaStream_t s = as_stream(stream);
  PixelSpace w;
  const void* src;
  bool cplx;
  int st = run_pixel(img, N, oversample, workspace, s, &w, &src, &cplx);
  if (st) return st;
  return abs_reduce(N, 1, src, cplx, out, nullptr, w.sums, s);
}

extern "C" int lgb_pixelate(const double* img, int rows, int cols, int oversample, double* out,
                            void* workspace, size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_pixelate");
  LGB_REQUIRE(img && out && workspace, LGB_EINVAL, "pixelate: null pointer");
  LGB_REQUIRE(rows == cols, LGB_EINVAL, "pixelate: the pixel MTF is defined for square images");
  LGB_REQUIRE(rows > 0 && oversample > 0, LGB_EINVAL, "pixelate: sizes must be positive");
  LGB_REQUIRE(workspace_bytes >= lgb_pixel_workspace_size(rows, oversample), LGB_EWORKSPACE,
              "pixelate: workspace too small");
  const int N = rows, os = oversample, S = resample_size(N, os);
  cudaStream_t s = as_stream(stream);
  PixelSpace w;
  const void* src;
  bool cplx;
  int st = run_pixel(img, N, os, workspace, s, &w, &src, &cplx);
  if (st) return st;
  if (resample_on_grid(N, os, S)) {
    if ((st = abs_reduce(N, os, src, cplx, nullptr, w.d, w.sums, s))) return st;
    pixelate_scale_kernel<<<cdiv(S * S, 256), 256, 0, s>>>(S * S, w.d, w.sums, out);
    LGB_CUDA(cudaGetLastError());
    return LGB_OK;
  }
  double* P = w.P;                       // the real MTF product, made |.| in place
  if ((st = abs_reduce(N, 1, src, cplx, P, nullptr, w.sums, s))) return st;
  resample_operator_kernel<<<cdiv(S * RS_BW, 256), 256, 0, s>>>(N, os, S, w.Gt, w.q0);
  resample_rows_kernel<<<dim3(cdiv(S, 64), cdiv(N, 4 * RS_ROWS)), dim3(64, 4), 0, s>>>(
      P, N, S, w.Gt, w.q0, w.Tm);
  resample_cols_kernel<<<dim3(cdiv(S, 64), cdiv(S, 4 * RS_OUT)), dim3(64, 4), 0, s>>>(
      w.Tm, N, S, w.Gt, w.q0, w.raw, w.sums);
  resample_finish_kernel<<<cdiv(S * S, 256), 256, 0, s>>>(w.raw, P, N, S, os, w.sums, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_pixelate_size(int N, int oversample) {
  if (N <= 0 || oversample <= 0) return -1;
  return resample_size(N, oversample);
}

extern "C" size_t lgb_power_spectrum_workspace_size(int N) {
  if (N <= 0) return 0;
  return psd_space(nullptr, N, nullptr);
}

extern "C" int lgb_power_spectrum(const double* noise, const double* mask, int N,
                                  double pixelscale, double rms, double half_power_freq,
                                  double exponent, double* out, void* workspace,
                                  size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_power_spectrum");
  LGB_REQUIRE(noise && mask && out && workspace, LGB_EINVAL, "power_spectrum: null pointer");
  LGB_REQUIRE(N > 0, LGB_EINVAL, "power_spectrum: size must be positive");
  LGB_REQUIRE(workspace_bytes >= lgb_power_spectrum_workspace_size(N), LGB_EWORKSPACE,
              "power_spectrum: workspace smaller than lgb_power_spectrum_workspace_size(N)");
  cudaStream_t s = as_stream(stream);
  PsdSpace w;
  psd_space(workspace, N, &w);
  const size_t NN = (size_t)N * N;
  // half-power point in cycles per pixel (lentil/wfe.py:45): sqrt(m^2 + n^2)
  const double f0 = half_power_freq * pixelscale / sqrt((double)N * N + (double)N * N);
  const int blocks = std::max(1, std::min(4 * sm_count(), (int)((NN + 255) / 256)));
  psd_sum_kernel<<<PSD_BLOCKS, 256, 0, s>>>(N, f0, exponent, w.partial);
  psd_final_kernel<<<1, 32, 0, s>>>(w.partial, PSD_BLOCKS, w.sums);
  real_to_complex_kernel<<<blocks, 256, 0, s>>>(noise, w.X, NN);
  LGB_CUDA(cudaGetLastError());
  int logN;
  const double2* spatial;
  if (fft_size(N, &logN)) {
    const size_t smem = (size_t)N * sizeof(float4);
    LGB_CUDA(cudaFuncSetAttribute(fft_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  8192 * (int)sizeof(float4)));
    const int threads = std::min(512, std::max(32, N / 2));
    const dim3 tgrid(cdiv(N, 32), cdiv(N, 32)), tblock(32, 8);
    float4* const twd = reinterpret_cast<float4*>(w.tw);     // N/2 entries of 16 bytes
    twiddle_df_kernel<<<cdiv(std::max(N / 2, 1), 256), 256, 0, s>>>(N, twd);
    fft_rows_kernel<<<N, threads, smem, s>>>(w.X, N, logN, twd, 0);
    transpose_c128_kernel<<<tgrid, tblock, 0, s>>>(w.X, w.Y, N);
    fft_rows_kernel<<<N, threads, smem, s>>>(w.Y, N, logN, twd, 0);           // Y = fft2(X)^T
    psd_filter_kernel<<<dim3(cdiv(N, 128), N), 128, 0, s>>>(w.Y, N, f0, exponent, w.sums);
    fft_rows_kernel<<<N, threads, smem, s>>>(w.Y, N, logN, twd, 1);
    transpose_c128_kernel<<<tgrid, tblock, 0, s>>>(w.Y, w.X, N);
    fft_rows_kernel<<<N, threads, smem, s>>>(w.X, N, logN, twd, 1);           // X = ifft2(...)
    LGB_CUDA(cudaGetLastError());
    spatial = w.X;
  } else {
    // DFT matrices E[u][r] = exp(-2 pi i u r / N) and their conjugate: the
    // coordinate offset N//2 and shift -(N//2) undo the centring of the
    // library's phase convention
    PhaseAxis ax, axc;
    int st;
    if ((st = make_phase_axis(1.0 / N, -(double)(N / 2), (double)(N / 2), N, N, &ax))) return st;
    if ((st = make_phase_axis(-1.0 / N, -(double)(N / 2), (double)(N / 2), N, N, &axc))) return st;
    if ((st = launch_dft_matrix_c128(ax, N, N, w.E, true, s))) return st;
    if ((st = launch_dft_matrix_c128(axc, N, N, w.Ec, true, s))) return st;
    // fft2(X) = E X E (E symmetric); ifft2(Y) = Ec Y Ec / N^2
    if ((st = launch_zgemm(N, N, N, w.E, N, 0, w.X, N, 0, w.Y, N, 0, 1, 1.0, s))) return st;
    if ((st = launch_zgemm(N, N, N, w.Y, N, 0, w.E, N, 0, w.X, N, 0, 1, 1.0, s))) return st;
    psd_filter_kernel<<<dim3(cdiv(N, 128), N), 128, 0, s>>>(w.X, N, f0, exponent, w.sums);
    LGB_CUDA(cudaGetLastError());
    const double inv = 1.0 / ((double)N * (double)N);
    if ((st = launch_zgemm(N, N, N, w.Ec, N, 0, w.X, N, 0, w.Y, N, 0, 1, 1.0, s))) return st;
    if ((st = launch_zgemm(N, N, N, w.Y, N, 0, w.Ec, N, 0, w.X, N, 0, 1, inv, s))) return st;
    spatial = w.X;
  }
  // opd = Re(.) * sqrt(N * N) * mask, rescaled to rms over its nonzero pixels
  psd_mask_kernel<true><<<PSD_BLOCKS, 256, 0, s>>>(spatial, mask, N, sqrt((double)N * N), out,
                                                   w.partial);
  psd_final_kernel<<<1, 32, 0, s>>>(w.partial, PSD_BLOCKS, w.sums);
  psd_rescale_kernel<<<blocks, 256, 0, s>>>(out, NN, w.sums, rms);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}
