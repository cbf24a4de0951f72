// Zernike OPD generators on the GPU (lentil/zernike.py:11-234, 444-480).
//
// lgb_zernike_coordinates: lentil's coordinate system of a mask.  The origin
// is the mask centroid (shift = centroid - shape/2) unless a shift is given;
// rr, cc is the centred mesh minus the shift (lentil/helper.py:7-17);
// rho = |rr + i cc| / max over the mask, theta = angle((-rr + i cc) e^{ia})
// with a = (90 - rotate) degrees.  The centroid sums count integer pixel
// indices of the boolean mask (exact in 64-bit integers), and the maximum is
// order-independent, so the coordinates do not depend on scheduling.
//
// lgb_zernike_eval: sum_j c_j Z_j (compose) or every Z_j (basis) from a mode
// table built on the host: per mode m, the scale (coefficient x Noll
// normalisation), and the radial polynomial as (coefficient, power) terms
// in lentil's order (lentil/zernike.py:96-109).  One pass over the plane:
// HBM-bound, 24 B read and 8 B written per pixel (K x 8 B for a basis).
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

__global__ void mask_moments_kernel(const double* __restrict__ mask, int H, int W,
                                    unsigned long long* __restrict__ acc) {
  const size_t total = (size_t)H * W;
  unsigned long long n = 0, si = 0, sj = 0;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    if (mask[p] != 0.0) {
      const unsigned long long i = p / W, j = p - i * W;
      n += 1; si += i; sj += j;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    n += __shfl_xor_sync(0xffffffffu, n, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
    sj += __shfl_xor_sync(0xffffffffu, sj, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(acc + 0, n); atomicAdd(acc + 1, si); atomicAdd(acc + 2, sj);
  }
}

struct ZCoord {
  double sr, sc;        // origin shift (rows, cols)
  double ca, sa;        // cos, sin of (90 - rotate) degrees
};

__device__ __forceinline__ void zcoord_at(size_t p, int H, int W, const ZCoord& z, double& rr,
                                          double& cc) {
  const int i = (int)(p / W), j = (int)(p - (size_t)(p / W) * W);
  rr = ((double)i - floor(H / 2.0)) - z.sr;
  cc = ((double)j - floor(W / 2.0)) - z.sc;
}

__global__ void zernike_rmax_kernel(const double* __restrict__ mask, int H, int W, ZCoord z,
                                    unsigned long long* __restrict__ rmax_bits) {
  const size_t total = (size_t)H * W;
  double v = 0.0;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    if (mask[p] == 0.0) continue;
    double rr, cc;
    zcoord_at(p, H, W, z, rr, cc);
    v = fmax(v, hypot(rr, cc));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  // non-negative doubles order like their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(rmax_bits, (unsigned long long)__double_as_longlong(v));
}

__global__ void zernike_coords_kernel(int H, int W, ZCoord z,
                                      const unsigned long long* __restrict__ rmax_bits,
                                      double* __restrict__ rho, double* __restrict__ theta) {
  const size_t total = (size_t)H * W;
  const double rmax = __longlong_as_double((long long)*rmax_bits);
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    double rr, cc;
    zcoord_at(p, H, W, z, rr, cc);
    rho[p] = hypot(rr, cc) / rmax;
    // (-rr e^{ia}) + (i cc e^{ia}), each product rounded as numpy does
    const double re = __dadd_rn(__dmul_rn(-rr, z.ca), -__dmul_rn(cc, z.sa));
    const double im = __dadd_rn(__dmul_rn(-rr, z.sa), __dmul_rn(cc, z.ca));
    theta[p] = atan2(im, re);
  }
}

// r^p for a small non-negative integer p by repeated squaring: a few FP64
// multiplies where pow() runs a general log/exp evaluation on this part's
// slow FP64 pipe (relative difference from pow below 1e-14 up to p = 40)
__device__ __forceinline__ double powi(double r, int p) {
  double res = 1.0, b = r;
  while (p) {
    if (p & 1) res *= b;
    b *= b;
    p >>= 1;
  }
  return res;
}

// (cos m t, sin m t) from (cos t, sin t) by complex powering, m >= 0
__device__ __forceinline__ void trig_multiple(double c, double s, int m, double& cm, double& sm) {
  double rc = 1.0, rs = 0.0, bc = c, bs = s;
  while (m) {
    if (m & 1) {
      const double t = rc * bc - rs * bs;
      rs = rc * bs + rs * bc;
      rc = t;
    }
    const double t = bc * bc - bs * bs;
    bs = 2.0 * bc * bs;
    bc = t;
    m >>= 1;
  }
  cm = rc;
  sm = rs;
}

// mode table row: [m, scale, nterms, (coef, power) x T]; the radial terms
// are summed in lentil's order, cos(m theta) / sin(m theta) come from one
// sincos of theta per pixel (absolute difference from the direct functions
// about 1e-14 for |m| <= 40)
__global__ void zernike_eval_kernel(const double* __restrict__ rho, const double* __restrict__ theta,
                                    const double* __restrict__ mask, size_t count,
                                    const double* __restrict__ table, int K, int T,
                                    double* __restrict__ out, int basis) {
  const int row = 3 + 2 * T;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < count;
       p += (size_t)gridDim.x * blockDim.x) {
    const double mk = mask[p] != 0.0 ? 1.0 : 0.0;
    const double r = rho[p], th = theta[p];
    double c1, s1;
    sincos(th, &s1, &c1);
    double acc = 0.0;
    for (int j = 0; j < K; ++j) {
      const double* t = table + (size_t)j * row;
      const int m = (int)t[0], nt = (int)t[2];
      double R = 0.0;
      for (int k = 0; k < nt; ++k) R += t[3 + 2 * k] * powi(r, (int)t[4 + 2 * k]);
      double z = t[1] * R;
      if (m != 0) {
        double cm, sm;
        trig_multiple(c1, s1, m > 0 ? m : -m, cm, sm);
        z *= m > 0 ? cm : -sm;                            // sin(m t) = -sin(|m| t) for m < 0
      }
      z *= mk;
      if (basis) out[(size_t)j * count + p] = z;
      else acc += z;
    }
    if (!basis) out[p] = acc;
  }
}

}  // namespace lgb

using namespace lgb;

extern "C" size_t lgb_zernike_workspace_size(void) { return 256; }

extern "C" int lgb_zernike_coordinates(const double* mask, int H, int W, int auto_shift,
                                       double shift_r, double shift_c, double rotate, double* rho,
                                       double* theta, void* workspace, size_t workspace_bytes,
                                       lgb_stream stream) {
  LGB_RANGE("lgb_zernike_coordinates");
  LGB_REQUIRE(mask && rho && theta, LGB_EINVAL, "zernike_coordinates: null pointer");
  LGB_REQUIRE(H > 0 && W > 0, LGB_EINVAL, "zernike_coordinates: sizes must be positive");
  LGB_REQUIRE(workspace && workspace_bytes >= lgb_zernike_workspace_size(), LGB_EWORKSPACE,
              "zernike_coordinates: workspace smaller than lgb_zernike_workspace_size()");
  cudaStream_t s = as_stream(stream);
  unsigned long long* acc = static_cast<unsigned long long*>(workspace);   // n, sum i, sum j, rmax
  const size_t total = (size_t)H * W;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((size_t)4 * sm_count(), (total + 255) / 256));
  LGB_CUDA(cudaMemsetAsync(acc, 0, 4 * sizeof(unsigned long long), s));
  ZCoord z;
  z.sr = shift_r;
  z.sc = shift_c;
  const double a = (90.0 - rotate) * M_PI / 180.0;
  z.ca = cos(a);
  z.sa = sin(a);
  if (auto_shift) {
    // the centroid is needed on the host to form the shift: one small read back
    mask_moments_kernel<<<blocks, 256, 0, s>>>(mask, H, W, acc);
    LGB_CUDA(cudaGetLastError());
    unsigned long long h[3];
    LGB_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
    LGB_CUDA(cudaStreamSynchronize(s));
    LGB_REQUIRE(h[0] > 0, LGB_EINVAL, "zernike_coordinates: the mask has no nonzero pixel");
    const double n = (double)h[0];
    z.sr = (double)h[1] / n - H / 2.0;
    z.sc = (double)h[2] / n - W / 2.0;
  }
  zernike_rmax_kernel<<<blocks, 256, 0, s>>>(mask, H, W, z, acc + 3);
  zernike_coords_kernel<<<blocks, 256, 0, s>>>(H, W, z, acc + 3, rho, theta);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_zernike_eval(const double* rho, const double* theta, const double* mask,
                                size_t count, const double* table, int K, int T, double* out,
                                int basis, lgb_stream stream) {
  LGB_RANGE("lgb_zernike_eval");
  LGB_REQUIRE(rho && theta && mask && table && out, LGB_EINVAL, "zernike_eval: null pointer");
  LGB_REQUIRE(K > 0 && T > 0, LGB_EINVAL, "zernike_eval: empty mode table");
  if (count == 0) return LGB_OK;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((size_t)8 * sm_count(), (count + 255) / 256));
  zernike_eval_kernel<<<blocks, 256, 0, as_stream(stream)>>>(rho, theta, mask, count, table, K, T,
                                                               out, basis);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}
