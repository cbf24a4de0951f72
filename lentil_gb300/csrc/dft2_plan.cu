// dft2 plans (lentil/fourier.py:5-110): one transform geometry -- m x n ->
// M x N, alpha, shift, offset, unitary, precision -- with its DFT matrices
// built once and kept on the device, so that repeated transforms of that
// geometry (lentil's propagate_dft called again for the same optics, the
// forward and adjoint transforms of every phase-retrieval evaluation) do no
// matrix build and no host-to-device copy per call.
//
// Status.  The split path's bounded pipeline waits report time-outs through
// a sticky device flag of the plan.  Each execute copies the flag to pinned
// host memory behind an event; the next execute of the plan reads it only if
// that event has completed (cudaEventQuery), so an error surfaces one call
// later without any host wait in steady state.  lgb_dft2_plan_status waits
// and reports at once.  Nothing is copied or queried under stream capture.
//
// Memory.  lgb_dft2_plan_create allocates the plan's device memory itself;
// lgb_dft2_plan_create_in builds the plan in memory the caller owns (a
// caching allocator's block), so that dropping a plan needs no device-wide
// wait.  Creation issues no host wait: the phase axes are written by a
// by-value kernel, and the status words live in one pinned pool shared by
// all plans.
#include <cmath>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {
namespace {

bool split_precision(int p) { return p == LGB_SPLIT_BF16 || p == LGB_SPLIT_FP16; }

struct PlanCarve {
  char* base;
  size_t used = 0;
  explicit PlanCarve(void* b) : base(static_cast<char*>(b)) {}
  template <typename T>
  T* take(size_t count) {
    used = align_up(used, 256);
    T* p = base ? reinterpret_cast<T*>(base + used) : nullptr;
    used += count * sizeof(T);
    return p;
  }
};

__global__ void store_int_kernel(int* dst, int v) { *dst = v; }

__global__ void store_axes_kernel(PhaseAxis rows, PhaseAxis cols, PhaseAxis* dst, double* unit2) {
  dst[0] = rows;
  dst[1] = cols;
  unit2[0] = 1.0;
  unit2[1] = 1.0;
}

// Pinned status words, one per live plan, from a pool allocated once.
constexpr int STATUS_SLOTS = 16384;
struct StatusPool {
  std::mutex mu;
  int* words = nullptr;
  std::vector<int> free_slots;
};
StatusPool& status_pool() {
  static StatusPool* p = new StatusPool();   // never freed: plans may outlive statics
  return *p;
}
int* take_status_word() {
  StatusPool& P = status_pool();
  std::lock_guard<std::mutex> lock(P.mu);
  if (!P.words) {
    if (cudaHostAlloc(&P.words, STATUS_SLOTS * sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
      (void)cudaGetLastError();
      P.words = nullptr;
      return nullptr;
    }
    for (int i = STATUS_SLOTS - 1; i >= 0; --i) P.free_slots.push_back(i);
  }
  if (P.free_slots.empty()) return nullptr;
  const int i = P.free_slots.back();
  P.free_slots.pop_back();
  P.words[i] = 0;
  return P.words + i;
}
void give_status_word(int* w) {
  if (!w) return;
  StatusPool& P = status_pool();
  std::lock_guard<std::mutex> lock(P.mu);
  P.free_slots.push_back((int)(w - P.words));
}

}  // namespace
}  // namespace lgb

using namespace lgb;

struct lgb_dft2_plan_s {
  int m = 0, n = 0, M = 0, N = 0, precision = 0, kp1 = 0, kp2 = 0;
  bool left = true;              // FP64 product order: (E1 f) E2, else E1 (f E2)
  double scale = 1.0;
  void* mem = nullptr;
  size_t bytes = 0;
  int* err = nullptr;            // sticky device status of the split launches
  PhaseAxis* axes = nullptr;     // [2] rows, cols
  double* unit2 = nullptr;       // [1] = 1 (the scale is applied by the epilogue)
  double2 *E1 = nullptr, *E2 = nullptr;
  uint16_t *e1h = nullptr, *e1l = nullptr, *e2h = nullptr, *e2l = nullptr;
  int* host_err = nullptr;       // pinned copy of *err (a status-pool word)
  cudaEvent_t copied = nullptr;  // recorded after that copy
  bool copy_pending = false;
  bool owns_mem = false;
  std::mutex mu;
};

namespace {

size_t plan_carve(lgb_dft2_plan_s* P, void* base) {
  PlanCarve c(base);
  P->err = c.take<int>(4);
  P->axes = c.take<PhaseAxis>(2);
  P->unit2 = c.take<double>(2);
  if (split_precision(P->precision)) {
    const size_t mrows1 = (size_t)cdiv(P->M, 64) * 128, nrows2 = (size_t)cdiv(P->N, 128) * 256;
    P->e1h = c.take<uint16_t>(mrows1 * 2 * P->kp1);
    P->e1l = c.take<uint16_t>(mrows1 * 2 * P->kp1);
    P->e2h = c.take<uint16_t>(nrows2 * 2 * P->kp2);
    P->e2l = c.take<uint16_t>(nrows2 * 2 * P->kp2);
  } else {
    P->E1 = c.take<double2>((size_t)P->M * P->m);
    P->E2 = c.take<double2>((size_t)P->n * P->N);
  }
  return c.used;
}

struct ExecSpace {
  float* maxabs;
  uint16_t *fh, *fl, *gh, *gl;
  double2* T;
};

size_t exec_carve(const lgb_dft2_plan_s* P, int count, void* base, ExecSpace* s) {
  PlanCarve c(base);
  ExecSpace t{};
  if (split_precision(P->precision)) {
    t.maxabs = c.take<float>(std::max(count, 4));
    t.fh = c.take<uint16_t>((size_t)count * P->n * 2 * P->kp1);
    t.fl = c.take<uint16_t>((size_t)count * P->n * 2 * P->kp1);
    t.gh = c.take<uint16_t>((size_t)count * P->M * 2 * P->kp2);
    t.gl = c.take<uint16_t>((size_t)count * P->M * 2 * P->kp2);
  } else {
    t.T = c.take<double2>((size_t)count *
                          std::max((size_t)P->M * P->n, (size_t)P->m * P->N));
  }
  if (s) *s = t;
  return std::max<size_t>(c.used, 256);
}

bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    (void)cudaGetLastError();
    return true;                 // unknown: behave as under capture (no copy, no query)
  }
  return cs != cudaStreamCaptureStatusNone;
}

}  // namespace

namespace {

// Fills P's sizes; returns LGB_OK or a validation error.
int plan_setup(lgb_dft2_plan_s* P, int m, int n, int M, int N, double alpha_r, double alpha_c,
               double shift_r, double shift_c, double offset_r, double offset_c, int unitary,
               int precision, PhaseAxis* ax) {
  LGB_REQUIRE(m > 0 && n > 0 && M > 0 && N > 0, LGB_EINVAL, "dft2_plan_create: sizes must be positive");
  LGB_REQUIRE((long long)m * n < (1LL << 31) && (long long)M * N < (1LL << 31), LGB_EINVAL,
              "dft2_plan_create: array too large");
  LGB_REQUIRE(precision == LGB_FP64 || split_precision(precision), LGB_EINVAL,
              "dft2_plan_create: unknown precision");
  int st;
  if ((st = make_phase_axis(alpha_r, shift_r, offset_r, m, M, &ax[0]))) return st;
  if ((st = make_phase_axis(alpha_c, shift_c, offset_c, n, N, &ax[1]))) return st;
  P->m = m; P->n = n; P->M = M; P->N = N; P->precision = precision;
  P->kp1 = round_up(m, 32);
  P->kp2 = round_up(n, 32);
  P->scale = unitary ? std::sqrt(std::fabs(alpha_r * alpha_c)) : 1.0;
  P->left = (double)M * m * n + (double)M * n * N <= (double)m * n * N + (double)M * m * N;
  P->bytes = plan_carve(P, nullptr);
  return LGB_OK;
}

// Released plans whose last status copy may still be in flight: their event
// and pinned word are returned once the copy has landed (no host wait).
struct Parked {
  cudaEvent_t ev;
  int* word;
};
std::mutex g_parked_mu;
std::vector<Parked>* g_parked = new std::vector<Parked>();   // never freed (static-order safe)

void reap_parked() {
  std::lock_guard<std::mutex> lock(g_parked_mu);
  auto& v = *g_parked;
  for (size_t i = 0; i < v.size();) {
    const cudaError_t q = cudaEventQuery(v[i].ev);
    if (q == cudaErrorNotReady) { ++i; continue; }
    if (q != cudaSuccess) (void)cudaGetLastError();
    cudaEventDestroy(v[i].ev);
    give_status_word(v[i].word);
    v[i] = v.back();
    v.pop_back();
  }
}

void plan_release_host(lgb_dft2_plan_s* P) {
  if (P->copied && P->copy_pending) {
    std::lock_guard<std::mutex> lock(g_parked_mu);
    g_parked->push_back({P->copied, P->host_err});
  } else {
    if (P->copied) cudaEventDestroy(P->copied);
    give_status_word(P->host_err);
  }
  P->copied = nullptr;
  P->host_err = nullptr;
  reap_parked();
}

// Builds the plan in P->mem (carved), on stream s, without a host wait.
int plan_build(lgb_dft2_plan_s* P, const PhaseAxis* ax, cudaStream_t s) {
  plan_carve(P, P->mem);
  reap_parked();
  P->host_err = take_status_word();
  LGB_REQUIRE(P->host_err, LGB_ECUDA, "dft2_plan_create: no pinned status word available");
  LGB_CUDA(cudaEventCreateWithFlags(&P->copied, cudaEventDisableTiming));
  LGB_CUDA(cudaMemsetAsync(P->err, 0, 4 * sizeof(int), s));
  store_axes_kernel<<<1, 1, 0, s>>>(ax[0], ax[1], P->axes, P->unit2);
  LGB_CUDA(cudaGetLastError());
  if (split_precision(P->precision)) {
    const bool bf16 = P->precision == LGB_SPLIT_BF16;
    int st = launch_e1_block_split(P->axes, 1, P->m, P->M, P->kp1, cdiv(P->M, 64) * 128, bf16,
                                   P->e1h, P->e1l, s);
    if (!st) st = launch_e2_block_split(P->axes + 1, 1, P->n, P->N, P->kp2,
                                        cdiv(P->N, 128) * 256, bf16, P->e2h, P->e2l, s);
    return st;
  }
  int st = launch_dft_matrix_c128(ax[0], P->m, P->M, P->E1, true, s);
  if (!st) st = launch_dft_matrix_c128(ax[1], P->n, P->N, P->E2, false, s);
  return st;
}

}  // namespace

extern "C" size_t lgb_dft2_plan_size(int m, int n, int M, int N, int precision) {
  lgb_dft2_plan_s P;
  PhaseAxis ax[2];
  if (plan_setup(&P, m, n, M, N, 0.01, 0.01, 0, 0, 0, 0, 0, precision, ax)) return 0;
  return P.bytes;
}

extern "C" int lgb_dft2_plan_create_in(int m, int n, int M, int N, double alpha_r,
                                       double alpha_c, double shift_r, double shift_c,
                                       double offset_r, double offset_c, int unitary,
                                       int precision, void* memory, size_t memory_bytes,
                                       lgb_stream stream, lgb_dft2_plan* plan) {
  LGB_RANGE("lgb_dft2_plan_create_in");
  LGB_REQUIRE(plan, LGB_EINVAL, "dft2_plan_create: null plan pointer");
  *plan = nullptr;
  lgb_dft2_plan_s* P = new lgb_dft2_plan_s();
  PhaseAxis ax[2];
  int st = plan_setup(P, m, n, M, N, alpha_r, alpha_c, shift_r, shift_c, offset_r, offset_c,
                      unitary, precision, ax);
  if (!st && (!memory || ((uintptr_t)memory & 255) != 0 || memory_bytes < P->bytes))
    st = set_error(LGB_EWORKSPACE, "dft2_plan_create_in: memory must be 256-byte aligned and "
                                   "hold lgb_dft2_plan_size bytes");
  if (!st) {
    P->mem = memory;
    st = plan_build(P, ax, as_stream(stream));
  }
  if (st) {
    plan_release_host(P);
    delete P;
    return st;
  }
  *plan = P;
  return LGB_OK;
}

extern "C" int lgb_dft2_plan_create(int m, int n, int M, int N, double alpha_r, double alpha_c,
                                    double shift_r, double shift_c, double offset_r,
                                    double offset_c, int unitary, int precision,
                                    lgb_stream stream, lgb_dft2_plan* plan) {
  LGB_RANGE("lgb_dft2_plan_create");
  LGB_REQUIRE(plan, LGB_EINVAL, "dft2_plan_create: null plan pointer");
  *plan = nullptr;
  lgb_dft2_plan_s* P = new lgb_dft2_plan_s();
  PhaseAxis ax[2];
  int st = plan_setup(P, m, n, M, N, alpha_r, alpha_c, shift_r, shift_c, offset_r, offset_c,
                      unitary, precision, ax);
  if (!st) {
    cudaError_t e = cudaMalloc(&P->mem, P->bytes);
    if (e != cudaSuccess) {
      P->mem = nullptr;
      st = check_cuda(e, "cudaMalloc(dft2 plan)");
    } else {
      P->owns_mem = true;
      st = plan_build(P, ax, as_stream(stream));
    }
  }
  if (st) {
    if (P->owns_mem) { cudaStreamSynchronize(as_stream(stream)); cudaFree(P->mem); }
    plan_release_host(P);
    delete P;
    return st;
  }
  *plan = P;
  return LGB_OK;
}

extern "C" size_t lgb_dft2_plan_bytes(lgb_dft2_plan P) { return P ? P->bytes : 0; }

extern "C" size_t lgb_dft2_plan_workspace_size(lgb_dft2_plan P, int count) {
  if (!P || count <= 0) return 0;
  return exec_carve(P, count, nullptr, nullptr);
}

extern "C" int lgb_dft2_plan_execute(lgb_dft2_plan P, const lgb_c128* f, int count, lgb_c128* F,
                                     void* workspace, size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_dft2_plan_execute");
  LGB_REQUIRE(P && f && F, LGB_EINVAL, "dft2_plan_execute: null argument");
  LGB_REQUIRE(count >= 1 && count <= 65535, LGB_EINVAL, "dft2_plan_execute: count outside 1..65535");
  LGB_REQUIRE(workspace && ((uintptr_t)workspace & 255) == 0, LGB_EWORKSPACE,
              "dft2_plan_execute: workspace must be non-null and 256-byte aligned");
  LGB_REQUIRE(workspace_bytes >= lgb_dft2_plan_workspace_size(P, count), LGB_EWORKSPACE,
              "dft2_plan_execute: workspace too small");
  cudaStream_t s = as_stream(stream);
  const bool cap = capturing(s);
  const bool split = split_precision(P->precision);
  if (split && !cap) {                    // an earlier execute's status, if it has landed
    std::lock_guard<std::mutex> lock(P->mu);
    if (P->copy_pending) {
      const cudaError_t q = cudaEventQuery(P->copied);
      if (q == cudaSuccess) {
        P->copy_pending = false;
        const int h = *P->host_err;
        if (h) {
          *P->host_err = 0;
          LGB_CUDA(cudaMemsetAsync(P->err, 0, sizeof(int), s));
          return set_error(h, "device-side wait expired inside the tensor-core MFT "
                              "(an earlier execute of this dft2 plan)");
        }
      } else if (q != cudaErrorNotReady) {
        return check_cuda(q, "cudaEventQuery(dft2 plan)");
      }
    }
  }
  ExecSpace w;
  exec_carve(P, count, workspace, &w);
  const double2* fin = reinterpret_cast<const double2*>(f);
  double2* Fout = reinterpret_cast<double2*>(F);
  const int m = P->m, n = P->n, M = P->M, N = P->N;
  int st;
  if (!split) {
    const long long sf = (long long)m * n, sF = (long long)M * N;
    if (P->left) {
      const long long sT = (long long)M * n;
      if ((st = launch_zgemm(M, n, m, P->E1, m, 0, fin, n, sf, w.T, n, sT, count, 1.0, s))) return st;
      return launch_zgemm(M, N, n, w.T, n, sT, P->E2, N, 0, Fout, N, sF, count, P->scale, s);
    }
    const long long sT = (long long)m * N;
    if ((st = launch_zgemm(m, N, n, fin, n, sf, P->E2, N, 0, w.T, N, sT, count, 1.0, s))) return st;
    return launch_zgemm(M, N, m, P->E1, m, 0, w.T, N, sT, Fout, N, sF, count, P->scale, s);
  }
  const bool bf16 = P->precision == LGB_SPLIT_BF16;
  float* const maxabs = bf16 ? nullptr : w.maxabs;     // bf16: no per-field scale
  if (maxabs && (st = launch_maxabs_c128_batch(fin, m * n, count, maxabs, s))) return st;
  SplitFieldArgs fa{};
  fa.field = fin;
  fa.m = m; fa.n = n; fa.kp = P->kp1; fa.L = 1; fa.batch = count;
  fa.maxabs = maxabs;
  fa.hi = w.fh; fa.lo = w.fl;
  if ((st = launch_split_field_T(fa, bf16, s))) return st;
  SplitMftProblem p{};
  p.m = m; p.n = n; p.M = M; p.N = N; p.kp1 = P->kp1; p.kp2 = P->kp2; p.L = 1; p.batch = count;
  p.bf16 = bf16;
  p.e1_hi = P->e1h; p.e1_lo = P->e1l; p.f_hi = w.fh; p.f_lo = w.fl;
  p.e2_hi = P->e2h; p.e2_lo = P->e2l; p.g_hi = w.gh; p.g_lo = w.gl;
  p.maxabs = maxabs;
  p.epilogue = 1;
  p.unit2 = P->unit2;
  p.out = reinterpret_cast<double*>(Fout);
  p.complex_scale = P->scale;
  p.err = P->err;
  if ((st = launch_split_mft(p, s))) return st;
  if (!cap) {
    std::lock_guard<std::mutex> lock(P->mu);
    LGB_CUDA(cudaMemcpyAsync(P->host_err, P->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    LGB_CUDA(cudaEventRecord(P->copied, s));
    P->copy_pending = true;
  }
  return LGB_OK;
}

extern "C" int lgb_dft2_plan_status(lgb_dft2_plan P, lgb_stream stream) {
  LGB_REQUIRE(P, LGB_EINVAL, "dft2_plan_status: null plan");
  cudaStream_t s = as_stream(stream);
  int h = 0;
  LGB_CUDA(cudaMemcpyAsync(&h, P->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  LGB_CUDA(cudaStreamSynchronize(s));
  std::lock_guard<std::mutex> lock(P->mu);
  if (P->copy_pending && cudaEventQuery(P->copied) == cudaSuccess) P->copy_pending = false;
  if (h) {
    *P->host_err = 0;
    LGB_CUDA(cudaMemsetAsync(P->err, 0, sizeof(int), s));
    return set_error(h, "device-side wait expired inside the tensor-core MFT");
  }
  return LGB_OK;
}

extern "C" int lgb_dft2_plan_inject_status(lgb_dft2_plan P, int code, lgb_stream stream) {
  LGB_REQUIRE(P, LGB_EINVAL, "dft2_plan_inject_status: null plan");
  LGB_REQUIRE(code == LGB_OK || code == LGB_ETIMEOUT, LGB_EINVAL,
              "dft2_plan_inject_status: only LGB_OK or LGB_ETIMEOUT can be injected");
  store_int_kernel<<<1, 1, 0, as_stream(stream)>>>(P->err, code);
  LGB_CUDA(cudaGetLastError());
  return LGB_OK;
}

extern "C" int lgb_dft2_plan_destroy(lgb_dft2_plan P) {
  if (!P) return LGB_OK;
  cudaError_t e = cudaSuccess;
  if (P->owns_mem) {
    // executes may still run on any stream: wait for the device before freeing
    e = cudaDeviceSynchronize();
    cudaFree(P->mem);
  }
  plan_release_host(P);
  delete P;
  if (e != cudaSuccess) return check_cuda(e, "cudaDeviceSynchronize(dft2 plan destroy)");
  return LGB_OK;
}
