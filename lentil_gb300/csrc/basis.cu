// Modal OPD expansion and its adjoint for phase retrieval (no lentil
// counterpart: lentil has no gradients).  OPD = sum_k c_k B_k over a basis B
// [K][P] (Zernike modes, segment piston/tip/tilt), and the coefficient
// gradient g_k = sum_p B_k[p] dL/dOPD[p].  The basis is read as FP32 (half
// the bytes of FP64, FP32 multiply-adds instead of this part's slow FP64
// pipe): both passes stream the basis once and are bound by HBM.  For the
// split-precision transforms the 1e-7 relative rounding of an FP32 product
// is far below the 16-bit operand split that follows.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

constexpr int BASIS_MAX_K = 1024;
constexpr int PROJ_BLOCKS = 76;

// out[i][p] = sum_k c[k] B[k][p] + add[i][p] (add null: 0), i < count; c
// staged in shared memory as FP32
__global__ void __launch_bounds__(256) basis_expand_kernel(const float* __restrict__ B,
                                                           const double* __restrict__ c, int K,
                                                           size_t P, const double* __restrict__ add,
                                                           int count, double* __restrict__ out) {
  __shared__ float cs[BASIS_MAX_K];
  for (int k = threadIdx.x; k < K; k += blockDim.x) cs[k] = (float)c[k];
  __syncthreads();
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P;
       p += (size_t)gridDim.x * blockDim.x) {
    // eight loads in flight per thread, two partial sums
    float a0 = 0.f, a1 = 0.f;
    int k = 0;
    for (; k + 8 <= K; k += 8) {
      float b[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) b[j] = __ldg(B + (size_t)(k + j) * P + p);
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        a0 = fmaf(cs[k + j], b[j], a0);
        a1 = fmaf(cs[k + j + 1], b[j + 1], a1);
      }
    }
    for (; k < K; ++k) a0 = fmaf(cs[k], __ldg(B + (size_t)k * P + p), a0);
    const double o = widen_float(a0 + a1);         // integer widening: no FP64 pipe
    for (int i = 0; i < count; ++i) out[(size_t)i * P + p] = add ? o + add[(size_t)i * P + p] : o;
  }
}

constexpr int PROJ_KG = 8;        // modes per block of the projection

// partial[k][chunk] = sum over pixel chunk blockIdx.x of B[k][p] g[p], for
// the PROJ_KG modes of blockIdx.y: each thread loads g[p] once for all of
// them and keeps one sum per mode; one fixed-order block reduction at the end
__global__ void __launch_bounds__(256) basis_project_partial_kernel(const float* __restrict__ B,
                                                                    const double* __restrict__ g,
                                                                    int count, int K, size_t P,
                                                                    double* __restrict__ partial) {
  __shared__ double red[8][PROJ_KG];
  const int k0 = blockIdx.y * PROJ_KG, nk = min(PROJ_KG, K - k0);
  const size_t per = (P + gridDim.x - 1) / gridDim.x;
  const size_t p0 = (size_t)blockIdx.x * per, p1 = min(P, p0 + per);
  // a thread sums only a few pixels (P / gridDim.x / blockDim.x), and a warp
  // 32 such sums: FP32 up to there, FP64 for the block's warps and the blocks
  // (this part's FP64 pipe retires about two operations a clock per SM, so
  // an FP64 shuffle reduction of every warp's sums took most of the time);
  // the gradient enters as a truncated float by integer operations
  float acc[PROJ_KG];
#pragma unroll
  for (int j = 0; j < PROJ_KG; ++j) acc[j] = 0.f;
  for (size_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    float gv = truncate_double(g[p]);              // the count planes' gradients summed
    for (int i = 1; i < count; ++i) gv += truncate_double(g[(size_t)i * P + p]);
#pragma unroll
    for (int j = 0; j < PROJ_KG; ++j)
      if (j < nk) acc[j] = fmaf(__ldg(B + (size_t)(k0 + j) * P + p), gv, acc[j]);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < PROJ_KG; ++j) {
    float v = acc[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][j] = widen_float(v);
  }
  __syncthreads();
  // the block's 8 warp sums of mode j: threads 8j .. 8j+7, a 3-level
  // shuffle tree in a fixed order
  if (threadIdx.x < 8 * PROJ_KG) {
    const int j = threadIdx.x >> 3, ww = threadIdx.x & 7;
    double t = red[ww][j];
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (ww == 0 && j < nk) partial[(size_t)(k0 + j) * gridDim.x + blockIdx.x] = t;
  }
}

// FP64 sum of n values in a fixed order by one warp: lane l adds values
// l, l+32, ..., then a shuffle tree (this part's FP64 adds have a long
// latency: a single thread walking 152 partials took ~14 us)
__device__ __forceinline__ double warp_sum_fixed(const double* __restrict__ v, int n) {
  const int lane = threadIdx.x & 31;
  double t = 0.0;
  for (int i = lane; i < n; i += 32) t += v[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  return t;
}

// out[k] = sum of mode k's partials: one warp per mode
__global__ void basis_project_final_kernel(const double* __restrict__ partial, int nblocks, int K,
                                           double* __restrict__ out) {
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (k >= K) return;                                   // (warp-uniform)
  const double t = warp_sum_fixed(partial + (size_t)k * nblocks, nblocks);
  if ((threadIdx.x & 31) == 0) out[k] = t;
}

// Squared-error loss L = sum (I - T)^2 and its gradient dL/dI = 2 (I - T) dL
// (the phase-retrieval loss), each one pass over the images, FP64: the
// per-thread sums and the fixed-order block reductions make L
// deterministic.  Enough blocks that each thread keeps only a few dependent
// FP64 operations in flight.
constexpr int SQE_MAX_BLOCKS = 2048;

__global__ void __launch_bounds__(256) sq_error_partial_kernel(const double* __restrict__ I,
                                                               const double* __restrict__ T,
                                                               size_t n,
                                                               double* __restrict__ partial) {
  __shared__ double red[8];
  double a0 = 0.0, a1 = 0.0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p + stride < n; p += 2 * stride) {              // two independent chains
    const double d0 = I[p] - T[p], d1 = I[p + stride] - T[p + stride];
    a0 = fma(d0, d0, a0);
    a1 = fma(d1, d1, a1);
  }
  if (p < n) {
    const double d = I[p] - T[p];
    a0 = fma(d, d, a0);
  }
  double acc = a0 + a1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

__global__ void sq_error_final_kernel(const double* __restrict__ partial, int nblocks,
                                      double* __restrict__ out) {
  const double t = warp_sum_fixed(partial, nblocks);    // one warp
  if (threadIdx.x == 0) *out = t;
}

__global__ void sq_error_grad_kernel(const double* __restrict__ I, const double* __restrict__ T,
                                     size_t n, const double* __restrict__ dL,
                                     double* __restrict__ dI) {
  const double s = 2.0 * *dL;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (size_t)gridDim.x * blockDim.x)
    dI[p] = s * (I[p] - T[p]);
}

}  // namespace lgb

using namespace lgb;

extern "C" size_t lgb_sq_error_workspace_size(void) { return SQE_MAX_BLOCKS * sizeof(double); }

extern "C" int lgb_sq_error(const double* I, const double* T, size_t n, double* loss,
                            void* workspace, size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_sq_error");
  LGB_REQUIRE(((I && T) || n == 0) && loss && workspace, LGB_EINVAL, "sq_error: null pointer");
  LGB_REQUIRE(workspace_bytes >= lgb_sq_error_workspace_size(), LGB_EWORKSPACE,
              "sq_error: workspace too small");
  cudaStream_t s = as_stream(stream);
  double* partial = static_cast<double*>(workspace);
  const int blocks = (int)std::max<size_t>(
      1, std::min<size_t>({(size_t)SQE_MAX_BLOCKS, (size_t)8 * sm_count(), (n + 1023) / 1024}));
  sq_error_partial_kernel<<<blocks, 256, 0, s>>>(I, T, n, partial);
  sq_error_final_kernel<<<1, 32, 0, s>>>(partial, blocks, loss);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_sq_error_grad(const double* I, const double* T, size_t n, const double* dL,
                                 double* dI, lgb_stream stream) {
  LGB_RANGE("lgb_sq_error_grad");
  if (n == 0) return LGB_OK;
  LGB_REQUIRE(I && T && dL && dI, LGB_EINVAL, "sq_error_grad: null pointer");
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((size_t)8 * sm_count(), (n + 255) / 256));
  sq_error_grad_kernel<<<blocks, 256, 0, as_stream(stream)>>>(I, T, n, dL, dI);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_basis_expand_stack(const float* basis, const double* coeffs, int K, size_t P,
                                      const double* add, int count, double* out,
                                      lgb_stream stream) {
  LGB_RANGE("lgb_basis_expand");
  LGB_REQUIRE(basis && coeffs && out, LGB_EINVAL, "basis_expand: null pointer");
  LGB_REQUIRE(K >= 1 && K <= BASIS_MAX_K, LGB_EINVAL, "basis_expand: K outside 1..1024");
  LGB_REQUIRE(count >= 1, LGB_EINVAL, "basis_expand: count < 1");
  if (P == 0) return LGB_OK;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((size_t)8 * sm_count(), (P + 255) / 256));
  basis_expand_kernel<<<blocks, 256, 0, as_stream(stream)>>>(basis, coeffs, K, P, add, count, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_basis_expand(const float* basis, const double* coeffs, int K, size_t P,
                                double* out, lgb_stream stream) {
  return lgb_basis_expand_stack(basis, coeffs, K, P, nullptr, 1, out, stream);
}

extern "C" size_t lgb_basis_project_workspace_size(int K) {
  return K > 0 ? (size_t)K * PROJ_BLOCKS * sizeof(double) : 0;
}

extern "C" int lgb_basis_project_stack(const float* basis, const double* grad, int count, int K,
                                       size_t P, double* out, void* workspace,
                                       size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_basis_project");
  LGB_REQUIRE(basis && grad && out && workspace, LGB_EINVAL, "basis_project: null pointer");
  LGB_REQUIRE(K >= 1 && K <= BASIS_MAX_K, LGB_EINVAL, "basis_project: K outside 1..1024");
  LGB_REQUIRE(count >= 1, LGB_EINVAL, "basis_project: count < 1");
  LGB_REQUIRE(workspace_bytes >= lgb_basis_project_workspace_size(K), LGB_EWORKSPACE,
              "basis_project: workspace too small");
  double* partial = static_cast<double*>(workspace);
  cudaStream_t s = as_stream(stream);
  basis_project_partial_kernel<<<dim3(PROJ_BLOCKS, cdiv(K, PROJ_KG)), 256, 0, s>>>(
      basis, grad, count, K, P, partial);
  basis_project_final_kernel<<<cdiv(K, 4), 128, 0, s>>>(partial, PROJ_BLOCKS, K, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_basis_project(const float* basis, const double* grad, int K, size_t P,
                                 double* out, void* workspace, size_t workspace_bytes,
                                 lgb_stream stream) {
  return lgb_basis_project_stack(basis, grad, 1, K, P, out, workspace, workspace_bytes, stream);
}
