// K6: detector pixel MTF and pixelation (lentil/detector.py:167-251).
//
// lentil applies the pixel MTF as |ifft2(fft2(img) * (s (x) s))| with
// s[k] = sinc(fftfreq(N)[k] * os) (lentil/detector.py:218-222).  For a square
// N x N image that is |C . img . C^T| with C the real symmetric circulant
// C[i][j] = c[(i - j) mod N], c = ifft(s): two real GEMMs on the FP64 pipe,
// the form used here.  pixelate then resamples by 1/os with a cubic spline
// (lentil/util.py:261-349); when N is a multiple of os every sample falls on
// a grid point, so the result is d = p[::os, ::os] rescaled by
// sum(p)/sum(d) and masked where d == 0 -- the only case implemented.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

// c[k] = (1/N) sum_f s_f cos(2 pi f k / N), s_f = sinc(freq_f * os)
__global__ void pixel_taps_kernel(int N, double os, double* __restrict__ c) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  double acc = 0.0;
  for (int f = 0; f < N; ++f) {
    const int ff = (f < (N + 1) / 2) ? f : f - N;        // numpy fftfreq ordering
    const double x = (double)ff / N * os;
    const double s = (x == 0.0) ? 1.0 : sinpi(x) / (M_PI * x);
    const long long ph = ((long long)f * k) % N;         // exact phase index
    acc += s * cospi(2.0 * (double)ph / N);
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

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// p = |P| in place; sums[0] += sum |P|, and the decimated samples
// d[k][l] = |P[k*os][l*os]| with sums[1] += sum d
__global__ void pixel_abs_reduce_kernel(int N, int os, double* __restrict__ P,
                                        double* __restrict__ d, double* __restrict__ sums) {
  double s_all = 0.0, s_dec = 0.0;
  const size_t total = (size_t)N * N;
  const int Nd = N / os;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const double v = fabs(P[p]);
    P[p] = v;
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

struct PixelSpace {
  double *c, *C, *T, *P, *d, *sums;
};

static size_t pixel_space(void* ws, int N, int os, PixelSpace* s) {
  size_t off = 0;
  auto take = [&](size_t n) {
    off = align_up(off, 256);
    double* p = ws ? reinterpret_cast<double*>(static_cast<char*>(ws) + off) : nullptr;
    off += n * sizeof(double);
    return p;
  };
  PixelSpace t;
  t.sums = take(4);
  t.c = take(N);
  t.C = take((size_t)N * N);
  t.T = take((size_t)N * N);
  t.P = take((size_t)N * N);
  t.d = take((size_t)(N / std::max(os, 1)) * (N / std::max(os, 1)));
  if (s) *s = t;
  return off;
}

static int run_pixel(const double* img, int N, int os, void* ws, cudaStream_t s, PixelSpace* w) {
  pixel_space(ws, N, os, w);
  LGB_CUDA(cudaMemsetAsync(w->sums, 0, 4 * sizeof(double), s));
  pixel_taps_kernel<<<cdiv(N, 128), 128, 0, s>>>(N, (double)os, w->c);
  LGB_CUDA(cudaGetLastError());
  circulant_kernel<<<dim3(cdiv(N, 128), N), 128, 0, s>>>(N, w->c, w->C);
  LGB_CUDA(cudaGetLastError());
  dim3 grid(cdiv(N, DBN), cdiv(N, DBM));
  dgemm_kernel<<<grid, 256, 0, s>>>(N, w->C, img, w->T);      // T = C . img
  LGB_CUDA(cudaGetLastError());
  dgemm_kernel<<<grid, 256, 0, s>>>(N, w->T, w->C, w->P);     // P = T . C^T (C symmetric)
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

}  // namespace lgb

using namespace lgb;

extern "C" size_t lgb_pixel_workspace_size(int N, int oversample) {
  if (N <= 0 || oversample <= 0) return 0;
  return pixel_space(nullptr, N, oversample, nullptr);
}

extern "C" int lgb_pixel(const double* img, int rows, int cols, int oversample, double* out,
                         void* workspace, size_t workspace_bytes, lgb_stream stream) {
  LGB_REQUIRE(img && out && workspace, LGB_EINVAL, "pixel: null pointer");
  LGB_REQUIRE(rows == cols, LGB_EINVAL, "pixel: the pixel MTF is defined for square images");
  LGB_REQUIRE(rows > 0 && oversample > 0, LGB_EINVAL, "pixel: sizes must be positive");
  LGB_REQUIRE(workspace_bytes >= lgb_pixel_workspace_size(rows, oversample), LGB_EWORKSPACE,
              "pixel: workspace too small");
  const int N = rows;
  cudaStream_t s = as_stream(stream);
  PixelSpace w;
  int st = run_pixel(img, N, oversample, workspace, s, &w);
  if (st) return st;
  const int blocks = std::max(1, std::min(4 * sm_count(), cdiv(N * N, 256)));
  pixel_abs_reduce_kernel<<<blocks, 256, 0, s>>>(N, 1, w.P, nullptr, w.sums);
  LGB_CUDA(cudaGetLastError());
  LGB_CUDA(cudaMemcpyAsync(out, w.P, sizeof(double) * (size_t)N * N, cudaMemcpyDeviceToDevice, s));
  return LGB_OK;
}

extern "C" int lgb_pixelate(const double* img, int rows, int cols, int oversample, double* out,
                            void* workspace, size_t workspace_bytes, lgb_stream stream) {
  LGB_REQUIRE(img && out && workspace, LGB_EINVAL, "pixelate: null pointer");
  LGB_REQUIRE(rows == cols, LGB_EINVAL, "pixelate: the pixel MTF is defined for square images");
  LGB_REQUIRE(rows > 0 && oversample > 0, LGB_EINVAL, "pixelate: sizes must be positive");
  LGB_REQUIRE(rows % oversample == 0, LGB_EUNSUPPORTED,
              "pixelate: the image size must be a multiple of oversample (the resampling "
              "then falls on grid points)");
  LGB_REQUIRE(workspace_bytes >= lgb_pixel_workspace_size(rows, oversample), LGB_EWORKSPACE,
              "pixelate: workspace too small");
  const int N = rows, os = oversample, Nd = N / os;
  cudaStream_t s = as_stream(stream);
  PixelSpace w;
  int st = run_pixel(img, N, os, workspace, s, &w);
  if (st) return st;
  const int blocks = std::max(1, std::min(4 * sm_count(), cdiv(N * N, 256)));
  pixel_abs_reduce_kernel<<<blocks, 256, 0, s>>>(N, os, w.P, w.d, w.sums);
  LGB_CUDA(cudaGetLastError());
  pixelate_scale_kernel<<<cdiv(Nd * Nd, 256), 256, 0, s>>>(Nd * Nd, w.d, w.sums, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}
