// K3: the plain FP64 (complex128) matrix triple product of lentil's dft2
// (lentil/fourier.py:95-101), as two tiled complex GEMMs on the FP64 pipe.
// This is the parity form (<= 1e-12 peak-normalised against numpy) and the
// baseline the split tensor-core form is measured against.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

constexpr int ZBM = 64, ZBN = 64, ZBK = 16;

// blockIdx.z = b * splits + split: problem b, K range [split * kchunk,
// (split + 1) * kchunk); with splits > 1 each split writes its own partial
// product (C offset by split * sP) for zgemm_reduce_kernel to sum in order.
__global__ void __launch_bounds__(256) zgemm_kernel(int M, int N, int K,
                                                    const double2* __restrict__ A, int lda, long long sA,
                                                    const double2* __restrict__ B, int ldb, long long sB,
                                                    double2* __restrict__ C, int ldc, long long sC,
                                                    double alpha, int splits, int kchunk, long long sP) {
  __shared__ double2 As[ZBK][ZBM];
  __shared__ double2 Bs[ZBK][ZBN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4, tid = threadIdx.x;
  const int m0 = blockIdx.y * ZBM, n0 = blockIdx.x * ZBN;
  const int b = blockIdx.z / splits, split = blockIdx.z - b * splits;
  A += (size_t)b * sA;
  B += (size_t)b * sB;
  C += (size_t)b * sC + (size_t)split * sP;
  const int kbeg = split * kchunk, kend = min(K, kbeg + kchunk);
  double cr[4][4], ci[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) cr[i][j] = ci[i][j] = 0.0;

  for (int k0 = kbeg; k0 < kend; k0 += ZBK) {
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int e = tid + 256 * t;
      const int ar = e >> 4, ak = e & 15;          // A tile: 64 rows x 16 k
      const int gr = m0 + ar, gk = k0 + ak;
      As[ak][ar] = (gr < M && gk < kend) ? A[(size_t)gr * lda + gk] : make_double2(0.0, 0.0);
      const int bk = e >> 6, bc = e & 63;          // B tile: 16 k x 64 cols
      const int hk = k0 + bk, gc = n0 + bc;
      Bs[bk][bc] = (hk < kend && gc < N) ? B[(size_t)hk * ldb + gc] : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < ZBK; ++k) {
      double2 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          cr[i][j] = fma(a[i].x, b[j].x, cr[i][j]);
          cr[i][j] = fma(-a[i].y, b[j].y, cr[i][j]);
          ci[i][j] = fma(a[i].x, b[j].y, ci[i][j]);
          ci[i][j] = fma(a[i].y, b[j].x, ci[i][j]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + ty + 16 * i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx + 16 * j;
      if (c < N) C[(size_t)r * ldc + c] = make_double2(alpha * cr[i][j], alpha * ci[i][j]);
    }
  }
}

// C[b] = alpha * sum_s P[s][b] in split order (deterministic), P[s][b] M x N dense
__global__ void zgemm_reduce_kernel(const double2* __restrict__ P, int splits, long long sP,
                                    int M, int N, double2* __restrict__ C, int ldc, long long sC,
                                    double alpha) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y, b = blockIdx.z;
  if (c >= N) return;
  const double2* p = P + (size_t)b * M * N + (size_t)r * N + c;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < splits; ++k) {
    const double2 v = p[(size_t)k * sP];
    re += v.x;
    im += v.y;
  }
  C[(size_t)b * sC + (size_t)r * ldc + c] = make_double2(alpha * re, alpha * im);
}

// The partials come from the device's default stream-ordered pool; by
// default the pool hands freed memory back at every synchronisation, so the
// next launch would map it again.  This process keeps up to 256 MiB cached
// (a property of the process's pool, gone when the process ends).
static void keep_pool_memory() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { (void)cudaGetLastError(); return; }
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = (uint64_t)256 << 20;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  (void)cudaGetLastError();
  done[dev] = true;
}

// A launch of fewer tiles than SMs would leave the FP64 pipes of most SMs
// idle (a 256 x 256 output is 16 tiles; each SM retires about two FP64 FMAs
// a clock), so such a launch splits K over up to 16 CTAs per tile, each
// writing a partial product to scratch (the caller's, or stream-ordered pool
// memory), and a second kernel sums the partials in split order.
int launch_zgemm(int M, int N, int K, const double2* A, int lda, long long sA, const double2* B,
                 int ldb, long long sB, double2* C, int ldc, long long sC, int batch, double alpha,
                 cudaStream_t s, const ZgemmScratch* scratch) {
  if (M <= 0 || N <= 0 || batch <= 0) return LGB_OK;
  LGB_REQUIRE(batch <= 65535, LGB_EINVAL, "zgemm: batch too large");
  const long long tiles = (long long)cdiv(N, ZBN) * cdiv(M, ZBM) * batch;
  const int sms = sm_count();
  int splits = 1;
  if (tiles < sms && K > 2 * ZBK)
    splits = (int)std::min<long long>({(2LL * sms + tiles - 1) / tiles, (long long)cdiv(K, 2 * ZBK), 16LL,
                                       65535LL / batch});
  const long long sP = (long long)batch * M * N;          // one split's partials
  const size_t part_bytes = (size_t)sP * sizeof(double2);
  if (scratch) {                                          // as many splits as fit
    const size_t fit = scratch->ptr ? scratch->bytes / part_bytes : 0;
    if ((size_t)splits > fit) splits = (int)fit;
  } else if (splits > 1 && (size_t)splits * part_bytes > ((size_t)256 << 20)) {
    splits = 1;
  }
  if (splits <= 1) {
    dim3 grid(cdiv(N, ZBN), cdiv(M, ZBM), batch);
    zgemm_kernel<<<grid, 256, 0, s>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, alpha, 1, K, 0);
    LGB_CUDA(cudaGetLastError());
    return LGB_OK;
  }
  const int kchunk = round_up(cdiv(K, splits), ZBK);
  splits = cdiv(K, kchunk);
  double2* P = nullptr;
  if (scratch) {
    P = static_cast<double2*>(scratch->ptr);
  } else {
    keep_pool_memory();
    LGB_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&P), (size_t)splits * part_bytes, s));
  }
  dim3 grid(cdiv(N, ZBN), cdiv(M, ZBM), batch * splits);
  zgemm_kernel<<<grid, 256, 0, s>>>(M, N, K, A, lda, sA, B, ldb, sB, P, N, (long long)M * N, 1.0,
                                    splits, kchunk, sP);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    dim3 rgrid(cdiv(N, 128), M, batch);
    zgemm_reduce_kernel<<<rgrid, 128, 0, s>>>(P, splits, sP, M, N, C, ldc, sC, alpha);
    e = cudaGetLastError();
  }
  if (!scratch) cudaFreeAsync(P, s);
  LGB_CUDA(e);
  return LGB_OK;
}

// out[b] += sum_l weights[b*L + l] * unit2[l] * |F[b*L + l]|^2 over the window (FP64);
// each output pixel is owned by one thread, so the wavelength sum is
// race-free and in a fixed order.
__global__ void intensity_accum_kernel(const double2* __restrict__ F, int M, int N, long long sF,
                                       int L, const double* __restrict__ weights,
                                       const double* __restrict__ unit2,
                                       double* __restrict__ out, int ld_out, long long s_out,
                                       int win_r0, int win_c0) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int u = blockIdx.y;
  const int b = blockIdx.z;
  if (v >= N || u >= M) return;
  double acc = 0.0;
  for (int l = 0; l < L; ++l) {
    const double2 z = F[((size_t)b * L + l) * sF + (size_t)u * N + v];
    const double w = (weights ? weights[(size_t)b * L + l] : 1.0) * unit2[l];
    acc = fma(w, z.x * z.x + z.y * z.y, acc);
  }
  out[(size_t)b * s_out + (size_t)(win_r0 + u) * ld_out + win_c0 + v] += acc;
}

int launch_intensity_accum_c128(const double2* F, int M, int N, long long sF, int batch_inner,
                                const double* weights, const double* unit2, double* out,
                                int ld_out, long long s_out, int win_r0, int win_c0, int n_outer,
                                cudaStream_t s) {
  if (M <= 0 || N <= 0) return LGB_OK;
  dim3 grid(cdiv(N, 128), M, n_outer);
  intensity_accum_kernel<<<grid, 128, 0, s>>>(F, M, N, sF, batch_inner, weights, unit2, out,
                                             ld_out, s_out, win_r0, win_c0);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

}  // namespace lgb
