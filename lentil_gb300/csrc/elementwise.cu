// HBM-bound elementwise kernels of the diffraction path:
//   K2  phasor amp*mask*exp(2 pi i opd / lambda)  (lentil/plane.py:502-507)
//   K2s the same phasor written straight into the split 16-bit, transposed
//       operand of the tensor-core MFT, for every wavelength of a batch
//   K5  clipped field overlap-add / |E|^2 insert  (lentil/field.py:231-305)
//       and the intersection product of Field.__mul__ (lentil/field.py:130-147)
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

// ---------------------------------------------------------------------------
// K2: complex128 phasor over one slice
// ---------------------------------------------------------------------------
__global__ void phasor_c128_kernel(const double* __restrict__ amp, double amp_value,
                                   const double* __restrict__ mask,
                                   const double* __restrict__ opd, double opd_value, int W,
                                   int r0, int c0, int m, int n, double two_over_lambda,
                                   double2* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= n || i >= m) return;
  const size_t p = (size_t)(r0 + i) * W + (c0 + j);
  double a = amp ? amp[p] : amp_value;
  if (mask) a *= mask[p];
  const double o = opd ? opd[p] : opd_value;
  double s, c;
  sincospi(o * two_over_lambda, &s, &c);     // exp(+2 pi i opd/lambda)
  out[(size_t)i * n + j] = make_double2(a * c, a * s);
}

// A stack of K phasors amp * exp(2 pi i opd_k / lambda) over one slice, for
// the gradient path.  FAST: the phase as a float-float product opd * 2/lambda
// reduced mod 2 half-cycles, then FP32 sincospi (about 1e-7 relative: for
// operands that are rounded to 16-bit hi/lo planes next); otherwise FP64
// sincospi as lgb_phasor.
template <bool FAST>
__global__ void phasor_stack_kernel(const double* __restrict__ amp,
                                    const double* __restrict__ opd, int H, int W, int r0, int c0,
                                    int m, int n, double two_over_lambda, float2 khalf,
                                    double2* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  const int k = blockIdx.z;
  if (j >= n || i >= m) return;
  const size_t p = (size_t)(r0 + i) * W + (c0 + j);
  const double a = amp[p];
  const double o = opd[(size_t)k * H * W + p];
  double s, c;
  if (FAST) {
    const float oh = (float)o, ol = (float)(o - (double)oh);
    const float ph = oh * khalf.x;
    float e = fmaf(oh, khalf.x, -ph);
    e = fmaf(oh, khalf.y, fmaf(ol, khalf.x, e));
    const float x = (ph - 2.f * rintf(0.5f * ph)) + e;
    float sf, cf;
    sincospif(x, &sf, &cf);
    s = sf;
    c = cf;
  } else {
    sincospi(o * two_over_lambda, &s, &c);
  }
  out[((size_t)k * m + i) * n + j] = make_double2(a * c, a * s);
}

__global__ void phasor_batch_c128_kernel(const double* __restrict__ amp,
                                         const double* __restrict__ opd, int H, int W, int r0,
                                         int c0, int m, int n,
                                         const double* __restrict__ two_over_lambda, int L,
                                         double2* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  const int b = blockIdx.z;
  if (j >= n || i >= m) return;
  const size_t p = ((size_t)b * H + r0 + i) * W + (c0 + j);
  const double a = amp[p], o = opd[p];
  for (int l = 0; l < L; ++l) {
    double s, c;
    sincospi(o * two_over_lambda[l], &s, &c);
    out[(((size_t)b * L + l) * m + i) * n + j] = make_double2(a * c, a * s);
  }
}

int launch_phasor_batch_c128(const double* amp, const double* opd, int H, int W, int r0, int c0,
                             int m, int n, const double* two_over_lambda, int L, int batch,
                             double2* out, cudaStream_t s) {
  if (m <= 0 || n <= 0) return LGB_OK;
  dim3 grid(cdiv(n, 128), m, batch);
  phasor_batch_c128_kernel<<<grid, 128, 0, s>>>(amp, opd, H, W, r0, c0, m, n, two_over_lambda,
                                                L, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// ---------------------------------------------------------------------------
// K2s: split 16-bit transposed field operand.
// Output row c (field column), K index r (field row) for the real part and
// kp + r for the imaginary part: f^T in the stage-1 B-operand layout.
// One block = 64 field rows x 32 field columns and a contiguous group of
// wavelengths (blockIdx.x = row tile * groups + group, blockIdx.z = PSF).
// Splitting the wavelength loop over blocks keeps enough blocks in flight to
// cover HBM latency; the groups of one tile are adjacent in launch order, so
// that their re-reads of amp and opd hit L2.
// Per wavelength the block's four output planes (real/imaginary x hi/lo, 32
// rows of 64 K values = 128 bytes each) are written into shared memory in
// the 128-byte-swizzled layout of a TMA box and leave as four bulk tensor
// stores issued by one thread; the TMA clips rows past n and K values past
// kp.  The tiles are double-buffered, so each wavelength needs one barrier:
// before it, the issuing thread waits until the previous wavelength's stores
// have read their tiles, which frees the buffer the next wavelength writes.
// ---------------------------------------------------------------------------
constexpr int TR = 64, TC = 32;
constexpr uint32_t FT_PLANE_BYTES = TC * TR * 2;            // 4 KB: 32 rows x 128 B
constexpr uint32_t FT_SMEM_BYTES = 2 * 4 * FT_PLANE_BYTES + 1024;   // two buffers + alignment

__device__ __forceinline__ void ft_store_4d(const CUtensorMap* map, uint32_t src, int x, int y,
                                            int z, int w) {
  asm volatile(
      "cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(src), "r"(x), "r"(y), "r"(z), "r"(w)
      : "memory");
}

// a read-once stream: no L1 allocation (the block's wavelength loop keeps
// the values in registers)
__device__ __forceinline__ double ld_stream(const double* p) {
  double v;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// 1/lambda of wavelength l of the launch as a float-float pair
__device__ __forceinline__ float2 cycles_per_metre(const SplitFieldArgs& a, int l) {
  const float2 k2 = a.khalf[a.lam_idx ? a.lam_idx[l] : l];   // 2/lambda
  return make_float2(0.5f * k2.x, 0.5f * k2.y);
}

template <bool BF16, bool PHASOR>
__global__ void __launch_bounds__(256, BF16 ? 5 : 4) split_field_T_kernel(SplitFieldArgs a, int groups,
                                                            const __grid_constant__ CUtensorMap map_hi,
                                                            const __grid_constant__ CUtensorMap map_lo) {
  extern __shared__ uint8_t ft_smem_raw[];
  __shared__ int warp_nz[8];
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(ft_smem_raw);
  const uint32_t tiles = (raw + 1023u) & ~1023u;                          // 1024-byte aligned
  uint8_t* const tile = ft_smem_raw + (tiles - raw);
  const int tid = threadIdx.x;
  const int rtile = blockIdx.x / groups, g = blockIdx.x - rtile * groups;   // row tile, group
  const int rt = rtile * TR, ct = blockIdx.y * TC;
  const int b = blockIdx.z;                                                 // PSF
  const float sf = a.maxabs ? pow2_scale_for(a.maxabs[b]) : 1.f;   // none: unscaled (bf16)

  // thread (w, lane) owns field column ct + lane and rows rt + 8w .. 8w+7:
  // each global load instruction reads 32 consecutive columns of one row,
  // and the thread's 8 values of a plane are one 16-byte chunk of its tile
  // row (chunk w of row lane, swizzled: no bank conflicts)
  const int lane = tid & 31, w = tid >> 5;
  const int L = PHASOR ? a.L : 1;
  const int per = (L + groups - 1) / groups;
  const int l0 = g * per, l1 = min(L, l0 + per);
  // the block's wavelength factors 1/lambda (a float-float pair: half of the
  // stored 2/lambda, exact), one per lane for 32 wavelengths at a time and
  // broadcast by shuffles in the loop, so that no global load waits between
  // the loop's barriers
  float2 k_lane = make_float2(0.f, 0.f);
  if (PHASOR && l0 + lane < l1) k_lane = cycles_per_metre(a, l0 + lane);
  float amp_r[8], o_hi[8], o_lo[8];
  float2 fv[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int r = rt + 8 * w + k, c = ct + lane;
    amp_r[k] = 0.f; o_hi[k] = 0.f; o_lo[k] = 0.f; fv[k] = make_float2(0.f, 0.f);
    if (r < a.m && c < a.n) {
      // the conversions are integer operations, not the FP64 pipe (every
      // wavelength group of a tile repeats them); the amplitude enters
      // linearly, so its truncated float (2^-23) is far inside the split's
      // 16 (bf16) or 22 (fp16) bits
      if (PHASOR) {
        const size_t q = ((size_t)b * a.H + (a.r0 + r)) * a.W + (a.c0 + c);
        const float2 o = split_double(ld_stream(a.opd + q));
        amp_r[k] = truncate_double(ld_stream(a.amp + q)) * sf;
        o_hi[k] = o.x;
        o_lo[k] = o.y;
      } else {
        const double2 v = a.field[((size_t)b * a.m + r) * a.n + c];
        const float2 re = split_double(v.x), im = split_double(v.y);
        fv[k] = make_float2((re.x + re.y) * sf, (im.x + im.y) * sf);
      }
    }
  }

  // nonzero flags of the block's two 32-row halves x 32 columns (warps 0-3
  // hold rows 0-31, warps 4-7 rows 32-63); the first wavelength group
  // writes them, and the last column block also zeroes the padding columns
  if (a.kflags) {
    bool nz = false;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      nz |= PHASOR ? amp_r[k] != 0.f : (fv[k].x != 0.f || fv[k].y != 0.f);
    nz = __any_sync(0xffffffffu, nz);
    if (lane == 0) warp_nz[w] = nz;
    __syncthreads();
    const int units = a.kp / 32, u = 2 * rtile + tid;
    if (g == 0 && tid < 2 && u < units) {
      uint8_t* row = a.kflags + ((size_t)b * units + u) * a.kf_pitch;
      row[blockIdx.y] = (warp_nz[4 * tid] | warp_nz[4 * tid + 1] | warp_nz[4 * tid + 2] |
                         warp_nz[4 * tid + 3]) != 0;
      if (blockIdx.y == gridDim.y - 1)
        for (int c = gridDim.y; c < a.kf_pitch; ++c) row[c] = 0;
    }
  }

  const uint32_t chunk = (uint32_t)lane * 128u + ((uint32_t)(w ^ (lane & 7)) << 4);
  for (int l = l0; l < l1; ++l) {
    if (PHASOR) {
      const int j = (l - l0) & 31;
      if (j == 0 && l != l0)                         // the next 32 wavelengths (warp-uniform)
        k_lane = l + lane < l1 ? cycles_per_metre(a, l + lane) : make_float2(0.f, 0.f);
      const float kx = __shfl_sync(0xffffffffu, k_lane.x, j);
      const float ky = __shfl_sync(0xffffffffu, k_lane.y, j);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        // t = opd / lambda cycles (float-float product), reduced to
        // [-1/2, 1/2] before the sine
        const float p = o_hi[k] * kx;
        float e = fmaf(o_hi[k], kx, -p);
        e = fmaf(o_hi[k], ky, fmaf(o_lo[k], kx, e));
        const float t = (p - rintf(p)) + e;
        float sn, cs;
        if (BF16) {
          // bf16 hi+lo keeps ~16 significant bits (error ~2^-17); the SFU
          // sine's absolute error on [-pi, pi] (~2^-21.4) is far below that
          __sincosf(t * 6.28318530717959f, &sn, &cs);
        } else {
          sincospif(2.f * t, &sn, &cs);  // fp16 hi+lo keeps ~22 bits
        }
        fv[k] = make_float2(amp_r[k] * cs, amp_r[k] * sn);
      }
    }
    uint32_t pk[4][4];                               // [plane][pair of rows]
#pragma unroll
    for (int j = 0; j < 4; ++j) {                    // rows 2j, 2j+1 split as a pair
      Split16x2<BF16>::split(fv[2 * j].x, fv[2 * j + 1].x, pk[0][j], pk[1][j]);
      Split16x2<BF16>::split(fv[2 * j].y, fv[2 * j + 1].y, pk[2][j], pk[3][j]);
    }
    // buffer l&1 was read by the stores of wavelength l-2, which the issuing
    // thread saw completed before the previous barrier
    uint8_t* const buf = tile + (l & 1) * 4 * FT_PLANE_BYTES;
#pragma unroll
    for (int pl = 0; pl < 4; ++pl)                   // re_hi, re_lo, im_hi, im_lo
      *reinterpret_cast<uint4*>(buf + pl * FT_PLANE_BYTES + chunk) =
          make_uint4(pk[pl][0], pk[pl][1], pk[pl][2], pk[pl][3]);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      const uint32_t sb = tiles + (l & 1) * 4 * FT_PLANE_BYTES;
      const int q = b * L + l;
      ft_store_4d(&map_hi, sb, rt, 0, ct, q);
      ft_store_4d(&map_lo, sb + FT_PLANE_BYTES, rt, 0, ct, q);
      ft_store_4d(&map_hi, sb + 2 * FT_PLANE_BYTES, rt, 1, ct, q);
      ft_store_4d(&map_lo, sb + 3 * FT_PLANE_BYTES, rt, 1, ct, q);
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    }
  }
  // the stores have landed before the block (and its shared memory) ends
  if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

int launch_split_field_T(const SplitFieldArgs& a, bool bf16, cudaStream_t s) {
  LGB_REQUIRE(!a.kflags || (a.kp % 32 == 0 && a.kf_pitch % 8 == 0 && a.kf_pitch >= cdiv(a.n, TC)),
              LGB_EINVAL, "split field: flag rows must hold every 32-column piece");
  const int spatial = cdiv(a.kp, TR) * cdiv(a.n, TC);
  const int psfs = a.batch;
  const int L = a.amp ? a.L : 1;
  LGB_REQUIRE(L >= 1, LGB_EINVAL, "split field: no wavelengths");
  LGB_REQUIRE(psfs <= 65535, LGB_EINVAL, "split field: too many PSFs in one launch");
  CUtensorMap map_hi, map_lo;
  int st;
  if ((st = make_field_T_store_map(&map_hi, a.hi, bf16, a.kp, a.n, psfs * L))) return st;
  if ((st = make_field_T_store_map(&map_lo, a.lo, bf16, a.kp, a.n, psfs * L))) return st;
  // Wavelength groups: each group re-reads the block's amp/opd once, and
  // the blocks run in waves of `cap` resident blocks; pick the group count
  // that minimises whole waves times the work of one block (the last wave
  // of a launch is otherwise partly empty), among counts up to 16.  A
  // block's fixed part (loading and converting amp and opd, the flags)
  // counts as five wavelengths of work: measured on the 1019 x 941 field at
  // 64 wavelengths, where 1, 2, 3, 4, 6 and 16 groups ran 0.101, 0.109,
  // 0.099, 0.112, 0.115 and 0.174 ms.  A block takes at most 32 wavelengths
  // (when 16 groups allow it), so that no block holds an SM for long: the
  // MFT's persistent CTA pairs of a launch on another stream start only
  // where an SM is free, and a late pair delays its whole launch.
  int per_sm = 0;
  auto kfn = bf16 ? (a.amp ? split_field_T_kernel<true, true> : split_field_T_kernel<true, false>)
                  : (a.amp ? split_field_T_kernel<false, true> : split_field_T_kernel<false, false>);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 256, FT_SMEM_BYTES) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const long long cap = (long long)per_sm * sm_count();
  const long long base = std::max(1LL, (long long)spatial * psfs);
  int groups = 1;
  double best = 1e300;
  for (int g = std::max(1, std::min(cdiv(L, 32), 16)); g <= std::min(L, 16); ++g) {
    const long long waves = (base * g + cap - 1) / cap;
    const double cost = (double)waves * (double)(cdiv(L, g) + 5);   // waves x work per block
    if (cost < best * (1.0 - 1e-9)) { best = cost; groups = g; }
  }
  groups = cdiv(L, cdiv(L, groups));                 // no empty trailing group
  dim3 grid(cdiv(a.kp, TR) * groups, cdiv(a.n, TC), psfs);
  kfn<<<grid, 256, FT_SMEM_BYTES, s>>>(a, groups, map_hi, map_lo);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// ---------------------------------------------------------------------------
// max |.| reductions feeding the power-of-two split scales
// ---------------------------------------------------------------------------
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void maxabs_amp_kernel(const double* __restrict__ amp, int H, int W, int r0, int c0,
                                  int m, int n, float* __restrict__ out) {
  const int b = blockIdx.y;
  float v = 0.f;
  const size_t total = (size_t)m * n;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < total;
       p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p / n), j = (int)(p % n);
    v = fmaxf(v, (float)fabs(amp[((size_t)b * H + r0 + i) * W + c0 + j]));
  }
  v = warp_max(v);
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(out + b), __float_as_int(v));
}

__global__ void maxabs_c128_kernel(const double2* __restrict__ f, int count, float* __restrict__ out) {
  float v = 0.f;
  f += (size_t)blockIdx.y * count;                 // field blockIdx.y of a batch
  out += blockIdx.y;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < count; p += gridDim.x * blockDim.x) {
    const double2 z = f[p];
    v = fmaxf(v, fmaxf((float)fabs(z.x), (float)fabs(z.y)));
  }
  v = warp_max(v);
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<int*>(out), __float_as_int(v));
}

int launch_maxabs_amp(const double* amp, int batch, int H, int W, int r0, int c0, int m, int n,
                      float* out, cudaStream_t s) {
  LGB_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * batch, s));
  const int blocks = (int)std::min<size_t>(2 * (size_t)sm_count(), cdiv(m * n, 256));
  maxabs_amp_kernel<<<dim3(blocks > 0 ? blocks : 1, batch), 256, 0, s>>>(amp, H, W, r0, c0, m, n, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

int launch_maxabs_c128_batch(const double2* f, int count, int batch, float* out, cudaStream_t s) {
  LGB_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * batch, s));
  const int blocks = std::max(1, std::min(2 * sm_count(), cdiv(count, 256)));
  maxabs_c128_kernel<<<dim3(blocks, batch), 256, 0, s>>>(f, count, out);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// ---------------------------------------------------------------------------
// FP32 intensity window (reduced into by the tensor-core epilogue) added to,
// or stored into, the float64 output image (widen_float: integer operations,
// kernels.cuh).
// ---------------------------------------------------------------------------
template <bool ADD>
__global__ void window_add_kernel(const float* __restrict__ wbuf, int M, int N, int ldw,
                                  double* __restrict__ out, int ld_out, long long out_bs,
                                  int win_r0, int win_c0) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int u = blockIdx.y, b = blockIdx.z;
  if (v >= N || u >= M) return;
  double* const o = out + (size_t)b * out_bs + (size_t)(win_r0 + u) * ld_out + win_c0 + v;
  const double x = widen_float(wbuf[((size_t)b * M + u) * ldw + v]);
  if (ADD) *o += x;
  else *o = x;
}

int launch_window_add(const float* wbuf, int M, int N, int ldw, int batch, double* out, int ld_out,
                      long long out_bs, int win_r0, int win_c0, bool add, cudaStream_t s) {
  if (M <= 0 || N <= 0 || batch <= 0) return LGB_OK;
  dim3 grid(cdiv(N, 128), M, batch);
  if (add)
    window_add_kernel<true><<<grid, 128, 0, s>>>(wbuf, M, N, ldw, out, ld_out, out_bs, win_r0, win_c0);
  else
    window_add_kernel<false><<<grid, 128, 0, s>>>(wbuf, M, N, ldw, out, ld_out, out_bs, win_r0, win_c0);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// ---------------------------------------------------------------------------
// conj(in) * scale -> out (idft2 through dft2, lentil/fourier.py:193-198)
// ---------------------------------------------------------------------------
__global__ void conj_scale_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                                  size_t count, double scale) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < count;
       p += (size_t)gridDim.x * blockDim.x) {
    const double2 z = in[p];
    out[p] = make_double2(z.x * scale, -z.y * scale);
  }
}

int launch_conj_scale(const double2* in, double2* out, size_t count, double scale, cudaStream_t s) {
  if (count == 0) return LGB_OK;
  const int blocks = (int)std::min<size_t>(4 * (size_t)sm_count(), (count + 255) / 256);
  conj_scale_kernel<<<blocks, 256, 0, s>>>(in, out, count, scale);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// ---------------------------------------------------------------------------
// K5: clipped overlap-add
// ---------------------------------------------------------------------------
template <bool INTENSITY>
__global__ void insert_kernel(const double2* __restrict__ f, int fn, int fr0, int fc0,
                              void* __restrict__ out, int on, int or0, int oc0, int rows, int cols,
                              double weight) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= cols || i >= rows) return;
  const double2 z = f[(size_t)(fr0 + i) * fn + fc0 + j];
  const size_t o = (size_t)(or0 + i) * on + oc0 + j;
  if (INTENSITY) {
    double* d = static_cast<double*>(out);
    // lentil: abs(f**2) * weight
    d[o] += (z.x * z.x + z.y * z.y) * weight;
  } else {
    double2* d = static_cast<double2*>(out);
    double2 t = d[o];
    t.x += z.x * weight;
    t.y += z.y * weight;
    d[o] = t;
  }
}

__global__ void multiply_kernel(const double2* __restrict__ a, int lda, int ar0, int ac0,
                                const double2* __restrict__ b, int ldb, int br0, int bc0,
                                double2* __restrict__ out, int om, int on) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= on || i >= om) return;
  const double2 x = lda ? a[(size_t)(ar0 + i) * lda + ac0 + j] : a[0];
  const double2 y = ldb ? b[(size_t)(br0 + i) * ldb + bc0 + j] : b[0];
  out[(size_t)i * on + j] = make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

}  // namespace lgb

using namespace lgb;

extern "C" int lgb_phasor_stack(const double* amp, const double* opd, int K, int H, int W,
                                int r0, int c0, int m, int n, double wavelength, int fast,
                                lgb_c128* out, lgb_stream stream) {
  LGB_RANGE("lgb_phasor_stack");
  LGB_REQUIRE(amp && opd && out, LGB_EINVAL, "phasor_stack: null pointer");
  LGB_REQUIRE(K > 0 && K <= 65535 && m > 0 && n > 0 && r0 >= 0 && c0 >= 0 && r0 + m <= H &&
                  c0 + n <= W, LGB_EINVAL, "phasor_stack: slice outside the plane");
  LGB_REQUIRE(wavelength > 0, LGB_EINVAL, "phasor_stack: wavelength must be positive");
  const double tol = 2.0 / wavelength;
  const float hi = (float)tol;
  const float2 kh = make_float2(hi, (float)(tol - (double)hi));
  dim3 grid(cdiv(n, 128), m, K);
  if (fast)
    phasor_stack_kernel<true><<<grid, 128, 0, as_stream(stream)>>>(
        amp, opd, H, W, r0, c0, m, n, tol, kh, reinterpret_cast<double2*>(out));
  else
    phasor_stack_kernel<false><<<grid, 128, 0, as_stream(stream)>>>(
        amp, opd, H, W, r0, c0, m, n, tol, kh, reinterpret_cast<double2*>(out));
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_phasor(const double* amp, double amp_value, const double* mask,
                          const double* opd, double opd_value, int H, int W, int r0, int c0,
                          int m, int n, double wavelength, lgb_c128* out, lgb_stream stream) {
  LGB_RANGE("lgb_phasor");
  LGB_REQUIRE(out, LGB_EINVAL, "phasor: null output");
  LGB_REQUIRE(m >= 0 && n >= 0 && r0 >= 0 && c0 >= 0, LGB_EINVAL, "phasor: negative slice");
  LGB_REQUIRE((!amp && !mask && !opd) || (r0 + m <= H && c0 + n <= W), LGB_EINVAL,
              "phasor: slice outside the plane");
  LGB_REQUIRE(wavelength != 0.0, LGB_EINVAL, "phasor: wavelength must be nonzero");
  if (m == 0 || n == 0) return LGB_OK;
  dim3 grid(cdiv(n, 128), m);
  phasor_c128_kernel<<<grid, 128, 0, as_stream(stream)>>>(amp, amp_value, mask, opd, opd_value,
                                                          W, r0, c0, m, n, 2.0 / wavelength,
                                                          reinterpret_cast<double2*>(out));
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_field_insert(const lgb_c128* f, int fm, int fn, int64_t off_r, int64_t off_c,
                                void* out, int om, int on, double weight, int intensity,
                                lgb_stream stream) {
  LGB_RANGE("lgb_field_insert");
  LGB_REQUIRE(f && out, LGB_EINVAL, "field_insert: null pointer");
  LGB_REQUIRE(fm > 0 && fn > 0 && om > 0 && on > 0, LGB_EINVAL, "field_insert: empty array");
  // lentil/field.py:259-299: upper-left corner of the shifted field in the
  // output, then clip both index ranges to the output
  int64_t fr0 = 0, fr1 = fm, fc0 = 0, fc1 = fn;
  int64_t or0 = om / 2 - fm / 2 + off_r, or1 = or0 + fm;
  int64_t oc0 = on / 2 - fn / 2 + off_c, oc1 = oc0 + fn;
  if (or0 < 0) { fr0 = -or0; or0 = 0; }
  if (or1 > om) { fr1 -= or1 - om; or1 = om; }
  if (oc0 < 0) { fc0 = -oc0; oc0 = 0; }
  if (oc1 > on) { fc1 -= oc1 - on; oc1 = on; }
  const int64_t rows = std::min(fr1 - fr0, or1 - or0), cols = std::min(fc1 - fc0, oc1 - oc0);
  if (rows <= 0 || cols <= 0) return LGB_OK;   // numpy's empty-slice add is a no-op
  dim3 grid(cdiv((int)cols, 128), (unsigned)rows);
  if (intensity)
    insert_kernel<true><<<grid, 128, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(f), fn, (int)fr0, (int)fc0, out, on, (int)or0, (int)oc0,
        (int)rows, (int)cols, weight);
  else
    insert_kernel<false><<<grid, 128, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(f), fn, (int)fr0, (int)fc0, out, on, (int)or0, (int)oc0,
        (int)rows, (int)cols, weight);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_field_multiply(const lgb_c128* a, int lda, int ar0, int ac0,
                                  const lgb_c128* b, int ldb, int br0, int bc0, lgb_c128* out,
                                  int om, int on, lgb_stream stream) {
  LGB_RANGE("lgb_field_multiply");
  LGB_REQUIRE(a && b && out, LGB_EINVAL, "field_multiply: null pointer");
  LGB_REQUIRE(om >= 0 && on >= 0, LGB_EINVAL, "field_multiply: negative shape");
  if (om == 0 || on == 0) return LGB_OK;
  dim3 grid(cdiv(on, 128), om);
  multiply_kernel<<<grid, 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const double2*>(a), lda, ar0, ac0, reinterpret_cast<const double2*>(b),
      ldb, br0, bc0, reinterpret_cast<double2*>(out), om, on);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

// ---------------------------------------------------------------------------
// K7: the element-wise halves of the adjoint (no counterpart in lentil, which
// has no gradients).  Forward I = |F|^2; given dL/dI the Wirtinger gradient
// dL/dF* = (dL/dI) F, its conjugate feeds an MFT with swapped offset/shift
// (the adjoint MFT), and dL/dopd = (2 pi / lambda) * 2 Im(g conj(f)).
// ---------------------------------------------------------------------------
namespace lgb {

__global__ void abs2_kernel(const double2* __restrict__ F, double* __restrict__ I, size_t count) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < count;
       p += (size_t)gridDim.x * blockDim.x) {
    const double2 z = F[p];
    I[p] = z.x * z.x + z.y * z.y;
  }
}

__global__ void intensity_adjoint_kernel(const double2* __restrict__ F, const double* __restrict__ gI,
                                         double2* __restrict__ Hc, size_t count) {
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < count;
       p += (size_t)gridDim.x * blockDim.x) {
    const double2 z = F[p];
    const double g = gI[p];
    Hc[p] = make_double2(g * z.x, -g * z.y);      // conj(dL/dF*) = dL/dI * conj(F)
  }
}

// out[r0+i, c0+j] += -2 * scale * Im(q[i,j] * f[i,j]),  q = conj(g)
__global__ void phasor_adjoint_kernel(const double2* __restrict__ q, const double2* __restrict__ f,
                                      int m, int n, double scale, double* __restrict__ out,
                                      int ld, int r0, int c0) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= n || i >= m) return;
  const double2 a = q[(size_t)i * n + j], b = f[(size_t)i * n + j];
  out[(size_t)(r0 + i) * ld + c0 + j] += -2.0 * scale * (a.x * b.y + a.y * b.x);
}

static int grid_for(size_t count) {
  return (int)std::max<size_t>(1, std::min<size_t>(4 * (size_t)sm_count(), (count + 255) / 256));
}

}  // namespace lgb

extern "C" int lgb_abs2(const lgb_c128* F, double* I, size_t count, lgb_stream stream) {
  LGB_RANGE("lgb_abs2");
  LGB_REQUIRE(F && I, LGB_EINVAL, "abs2: null pointer");
  if (!count) return LGB_OK;
  abs2_kernel<<<grid_for(count), 256, 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(F),
                                                              I, count);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_intensity_adjoint(const lgb_c128* F, const double* grad_I, lgb_c128* Hc,
                                     size_t count, lgb_stream stream) {
  LGB_RANGE("lgb_intensity_adjoint");
  LGB_REQUIRE(F && grad_I && Hc, LGB_EINVAL, "intensity_adjoint: null pointer");
  if (!count) return LGB_OK;
  intensity_adjoint_kernel<<<grid_for(count), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const double2*>(F), grad_I, reinterpret_cast<double2*>(Hc), count);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_phasor_adjoint(const lgb_c128* q, const lgb_c128* f, int m, int n,
                                  double wavelength, double* grad_opd, int ld, int r0, int c0,
                                  lgb_stream stream) {
  LGB_RANGE("lgb_phasor_adjoint");
  LGB_REQUIRE(q && f && grad_opd, LGB_EINVAL, "phasor_adjoint: null pointer");
  LGB_REQUIRE(wavelength != 0.0, LGB_EINVAL, "phasor_adjoint: wavelength must be nonzero");
  if (m <= 0 || n <= 0) return LGB_OK;
  dim3 grid(cdiv(n, 128), m);
  phasor_adjoint_kernel<<<grid, 128, 0, as_stream(stream)>>>(
      reinterpret_cast<const double2*>(q), reinterpret_cast<const double2*>(f), m, n,
      2.0 * M_PI / wavelength, grad_opd, ld, r0, c0);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}
