// Allocation-free complex128 dft2.
//
// Some callers of this library cannot allocate device memory when they call
// it: a wavefront-control or instrument loop that reserves its whole memory
// budget at start-up and may not allocate (or risk an allocation failure)
// afterwards, and code that issues work into a stream being captured into a
// CUDA graph, where cudaMalloc/cudaFree are not allowed.  lgb_dft2 needs a
// workspace for the two DFT matrices and the intermediate product; this entry
// point takes that scratch from a fixed array compiled into the library
// instead, so the caller only provides its input and output.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds LGB_NOALLOC_SCRATCH_BYTES of it until the process exits.  In
// host code the symbol is only a host-side stand-in, so its device address is
// looked up with cudaGetSymbolAddress, once per device, with that device
// current, the first time lgb_dft2_noalloc runs there (make that first call
// outside any stream capture).  Every call shares the one array and leaves its
// contents behind: calls that overlap on the GPU (different streams, no
// ordering between them) race on it.  Nothing in it needs to start at zero:
// the transform overwrites every scratch element it reads, and the status word
// at its start is cleared by each call.
//
// The plain FP64 GEMMs split K over several CTAs when the output has fewer
// tiles than the GPU has SMs; their partial products go to the part of the
// array after the transform's workspace (fewer splits when they do not fit),
// never to freshly allocated memory.
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

static __device__ __align__(256) unsigned char g_dft2_scratch[LGB_NOALLOC_SCRATCH_BYTES];

// Device address of g_dft2_scratch for the current device (looked up once).
static int scratch_address(void** out) {
  static std::mutex mu;
  static std::vector<void*> addr;
  int dev = 0;
  LGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)addr.size() <= dev) addr.resize(dev + 1, nullptr);
  if (!addr[dev]) {
    void* p = nullptr;
    LGB_CUDA(cudaGetSymbolAddress(&p, g_dft2_scratch));
    addr[dev] = p;
  }
  *out = addr[dev];
  return LGB_OK;
}

}  // namespace lgb

extern "C" int lgb_dft2_noalloc(const lgb_c128* f, int m, int n, lgb_c128* F, int M, int N,
                                double alpha_r, double alpha_c, double shift_r, double shift_c,
                                double offset_r, double offset_c, int unitary, lgb_stream stream) {
  LGB_RANGE("lgb_dft2_noalloc");
  using namespace lgb;
  LGB_REQUIRE(m > 0 && n > 0 && M > 0 && N > 0, LGB_EINVAL, "dft2_noalloc: sizes must be positive");
  const size_t need = lgb_dft2_workspace_size(m, n, M, N, LGB_FP64);
  if (need > (size_t)LGB_NOALLOC_SCRATCH_BYTES)
    return set_error(LGB_EINVAL,
                     "dft2_noalloc: this transform needs " + std::to_string(need) +
                         " bytes of scratch, more than the fixed " +
                         std::to_string((size_t)LGB_NOALLOC_SCRATCH_BYTES) +
                         " bytes; use lgb_dft2 with a caller-provided workspace");
  void* ws = nullptr;
  int st = scratch_address(&ws);
  if (st) return st;
  const size_t part_off = align_up(need, 256);
  ZgemmScratch partials{static_cast<unsigned char*>(ws) + part_off,
                        (size_t)LGB_NOALLOC_SCRATCH_BYTES - part_off};
  return dft2_batch(reinterpret_cast<const double2*>(f), 1, m, n, reinterpret_cast<double2*>(F),
                    M, N, alpha_r, alpha_c, shift_r, shift_c, offset_r, offset_c, unitary,
                    LGB_FP64, ws, need, as_stream(stream), &partials);
}
