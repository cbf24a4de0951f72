// Plane.fit_tilt on the GPU (lentil/plane.py:522-611).
//
// lentil builds ptt_vector, a (3S) x (H*W) matrix of the masked basis
// b = [1, r*ps_r, -c*ps_c] (r, c the centred mesh of lentil/helper.py:7-17),
// and solves one least-squares problem per mask with lstsq.  The basis is
// zero off the mask, so each problem is fully described by its 3x3 normal
// equations  A = sum_p m(p)^2 b(p) b(p)^T,  y = sum_p m(p) b(p) opd(p):
// one pass over the plane per mask, no H*W x 3 matrix.  The sums are taken
// in FP64 in a fixed order (per-block partials, then one block per mask), so
// the result is deterministic; the host solves the 3x3 systems.
//
// The tilt removal then follows lentil's two branches: one mask
//     opd - m (t1 r ps_r - t2 c ps_c)
// several masks
//     sum_s (opd - m_s (t_s1 r ps_r - t_s2 c ps_c)) m_s.
// Both kernels stream the plane once per mask: HBM-bound, 8 B of mask and
// 8 B of OPD per pixel per mask.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

constexpr int PTT_THREADS = 256;
constexpr int PTT_BLOCKS = 128;          // blocks per mask in the first pass

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of 9 values; thread 0 returns them in v.
__device__ __forceinline__ void block_sum9(double (&v)[9]) {
  __shared__ double part[PTT_THREADS / 32][9];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 9; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 9; ++k) part[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      double s = 0.0;
      for (int j = 0; j < PTT_THREADS / 32; ++j) s += part[j][k];
      v[k] = s;
    }
  }
}

// pass 1: partial[s][block][9] over a grid-stride share of the plane
__global__ void __launch_bounds__(PTT_THREADS) ptt_partial_kernel(
    const double* __restrict__ opd, const double* __restrict__ mask, int H, int W, double ps_r,
    double ps_c, double* __restrict__ partial) {
  const int s = blockIdx.y;
  const double* ms = mask + (size_t)s * H * W;
  const size_t total = (size_t)H * W;
  const double r0 = floor(H / 2.0), c0 = floor(W / 2.0);
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (size_t p = (size_t)blockIdx.x * PTT_THREADS + threadIdx.x; p < total;
       p += (size_t)gridDim.x * PTT_THREADS) {
    const double m = ms[p];
    if (m == 0.0) continue;
    const int i = (int)(p / W), j = (int)(p - (size_t)i * W);
    const double b1 = ((double)i - r0) * ps_r, b2 = -((double)j - c0) * ps_c;
    const double m2 = m * m, mo = m * opd[p];
    v[0] += m2;  v[1] += m2 * b1;      v[2] += m2 * b2;
    v[3] += m2 * b1 * b1;  v[4] += m2 * b1 * b2;  v[5] += m2 * b2 * b2;
    v[6] += mo;  v[7] += mo * b1;      v[8] += mo * b2;
  }
  block_sum9(v);
  if (threadIdx.x == 0) {
    double* dst = partial + ((size_t)s * gridDim.x + blockIdx.x) * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) dst[k] = v[k];
  }
}

// pass 2: out[s][9] = sum over blocks, one block per mask, fixed order
__global__ void __launch_bounds__(PTT_THREADS) ptt_final_kernel(const double* __restrict__ partial,
                                                               int nblocks, double* __restrict__ out) {
  const int s = blockIdx.x;
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += PTT_THREADS) {
    const double* src = partial + ((size_t)s * nblocks + b) * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] += src[k];
  }
  block_sum9(v);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 9; ++k) out[(size_t)s * 9 + k] = v[k];
}

__global__ void remove_tilt_kernel(const double* __restrict__ opd, const double* __restrict__ mask,
                                   int S, int H, int W, double ps_r, double ps_c,
                                   const double* __restrict__ t, double* __restrict__ out) {
  const size_t total = (size_t)H * W;
  const double r0 = floor(H / 2.0), c0 = floor(W / 2.0);
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p / W), j = (int)(p - (size_t)i * W);
    const double b1 = ((double)i - r0) * ps_r, b2 = -((double)j - c0) * ps_c;
    const double o = opd[p];
    if (S == 1) {
      out[p] = o - mask[p] * (t[1] * b1 + t[2] * b2);
    } else {
      double acc = 0.0;
      for (int s = 0; s < S; ++s) {
        const double m = mask[(size_t)s * total + p];
        acc += (o - m * (t[3 * s + 1] * b1 + t[3 * s + 2] * b2)) * m;
      }
      out[p] = acc;
    }
  }
}

}  // namespace lgb

using namespace lgb;

extern "C" size_t lgb_ptt_normal_workspace_size(int S) {
  if (S <= 0) return 0;
  return align_up((size_t)S * PTT_BLOCKS * 9 * sizeof(double), 256);
}

extern "C" int lgb_ptt_normal(const double* opd, const double* mask, int S, int H, int W,
                              double ps_r, double ps_c, double* out, void* workspace,
                              size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_ptt_normal");
  LGB_REQUIRE(opd && mask && out, LGB_EINVAL, "ptt_normal: null pointer");
  LGB_REQUIRE(S > 0 && H > 0 && W > 0, LGB_EINVAL, "ptt_normal: sizes must be positive");
  LGB_REQUIRE(S <= 65535, LGB_EINVAL, "ptt_normal: too many masks");
  LGB_REQUIRE(workspace && workspace_bytes >= lgb_ptt_normal_workspace_size(S), LGB_EWORKSPACE,
              "ptt_normal: workspace smaller than lgb_ptt_normal_workspace_size(S)");
  cudaStream_t s = as_stream(stream);
  double* partial = static_cast<double*>(workspace);
  ptt_partial_kernel<<<dim3(PTT_BLOCKS, S), PTT_THREADS, 0, s>>>(opd, mask, H, W, ps_r, ps_c, partial);
  LGB_CUDA(cudaGetLastError());
  ptt_final_kernel<<<S, PTT_THREADS, 0, s>>>(partial, PTT_BLOCKS, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_remove_tilt(const double* opd, const double* mask, int S, int H, int W,
                               double ps_r, double ps_c, const double* t, double* out,
                               lgb_stream stream) {
  LGB_RANGE("lgb_remove_tilt");
  LGB_REQUIRE(opd && mask && t && out, LGB_EINVAL, "remove_tilt: null pointer");
  LGB_REQUIRE(S > 0 && H > 0 && W > 0, LGB_EINVAL, "remove_tilt: sizes must be positive");
  const size_t total = (size_t)H * W;
  const int blocks = (int)std::min<size_t>((size_t)8 * sm_count(), (total + 255) / 256);
  remove_tilt_kernel<<<std::max(1, blocks), 256, 0, as_stream(stream)>>>(opd, mask, S, H, W, ps_r,
                                                                          ps_c, t, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}
