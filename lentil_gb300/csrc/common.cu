// Error reporting, device queries and the host half of the fixed-point DFT
// phase reduction.
#include "common.cuh"

#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

namespace lgb {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  char buf[512];
  snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
  cudaGetLastError();  // clear a non-sticky error so the next call starts clean
  return set_error(LGB_ECUDA, buf);
}

int sm_count() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (cache[dev] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = n > 0 ? n : 1;
  }
  return cache[dev];
}

// frac(v) * 2^64 as an unsigned 64-bit integer (v any finite double).
static uint64_t frac64(double v) {
  double f = v - std::floor(v);             // [0, 1)
  // split into two 32-bit halves so the conversion is exact to 2^-64
  double hi = std::floor(std::ldexp(f, 32));
  double lo = std::ldexp(f, 32) - hi;       // exact
  uint64_t h = (uint64_t)hi;
  uint64_t l = (uint64_t)std::llround(std::ldexp(lo, 32));
  return (h << 32) + l;                     // wraps correctly if l == 2^32
}

// frac(alpha) * 2^128, exact (alpha is a double: mantissa * 2^e).
static void frac128(double alpha, uint64_t* hi, uint64_t* lo) {
  int ex = 0;
  double fr = std::frexp(std::fabs(alpha), &ex);          // |alpha| = fr * 2^ex
  unsigned __int128 mant = (unsigned __int128)(uint64_t)std::ldexp(fr, 53);
  int sh = ex - 53 + 128;                                  // |alpha| * 2^128 = mant << sh
  unsigned __int128 v;
  if (fr == 0.0) v = 0;
  else if (sh >= 128) v = 0;                               // integer-valued: no fraction
  else if (sh >= 0) v = mant << sh;                        // wraps modulo 2^128
  else if (sh > -128) v = mant >> (-sh);
  else v = 0;
  if (alpha < 0) v = (unsigned __int128)0 - v;
  *hi = (uint64_t)(v >> 64);
  *lo = (uint64_t)v;
}

int make_phase_axis(double alpha, double shift, double offset, int len_in, int len_out,
                    PhaseAxis* ax) {
  if (!std::isfinite(alpha) || !std::isfinite(shift) || !std::isfinite(offset))
    return set_error(LGB_EINVAL, "dft2: alpha, shift and offset must be finite");
  if (std::fabs(shift) > 1e9 || std::fabs(offset) > 1e9)
    return set_error(LGB_EINVAL, "dft2: |shift| and |offset| must be below 1e9 pixels");
  const double oi = std::nearbyint(offset), si = std::nearbyint(shift);
  const double of = offset - oi, sf = shift - si;   // exact (Sterbenz)
  frac128(alpha, &ax->a_hi, &ax->a_lo);
  ax->b_sf = frac64(alpha * sf);
  ax->b_of = frac64(alpha * of);
  ax->b_c = frac64(alpha * of * sf);
  ax->x0 = (int64_t)oi - (int64_t)(len_in / 2);
  ax->y0 = -(int64_t)(len_out / 2) - (int64_t)si;
  return LGB_OK;
}

}  // namespace lgb

extern "C" const char* lgb_last_error(void) { return lgb::g_last_error.c_str(); }
extern "C" int lgb_version(void) { return (1 << 16) | 0; }

extern "C" int lgb_mempool_usage(int device, int reset_high, unsigned long long out[4]) {
  LGB_REQUIRE(out, LGB_EINVAL, "mempool_usage: null output");
  cudaMemPool_t pool;
  LGB_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  if (reset_high) {
    unsigned long long zero = 0;
    LGB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReservedMemHigh, &zero));
    LGB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
  }
  const cudaMemPoolAttr attrs[4] = {cudaMemPoolAttrReservedMemCurrent, cudaMemPoolAttrReservedMemHigh,
                                    cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrUsedMemHigh};
  for (int i = 0; i < 4; ++i) {
    unsigned long long v = 0;
    LGB_CUDA(cudaMemPoolGetAttribute(pool, attrs[i], &v));
    out[i] = (unsigned long long)v;
  }
  return LGB_OK;
}
