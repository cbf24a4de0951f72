// Host orchestration of the C ABI: dft2 (lentil/fourier.py:5-103) in both
// precisions, and the broadband PSF plan that fuses the user wavelength loop
// (docs/user/performance.rst:44-49) over a batch of PSFs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace lgb {

// Sub-allocator over one workspace: 256-byte aligned slices.
struct Carve {
  char* base;
  size_t used = 0;
  explicit Carve(void* b) : base(static_cast<char*>(b)) {}
  template <typename T>
  T* take(size_t count) {
    used = align_up(used, 256);
    T* p = base ? reinterpret_cast<T*>(base + used) : nullptr;
    used += count * sizeof(T);
    return p;
  }
};

static bool is_split(int precision) {
  return precision == LGB_SPLIT_BF16 || precision == LGB_SPLIT_FP16;
}

// ---------------------------------------------------------------------------
// dft2 workspace layouts
// ---------------------------------------------------------------------------
struct Dft2Fp64Space {
  int* err;
  double2 *E1, *E2, *T;
};
struct Dft2SplitSpace {
  int* err;
  PhaseAxis* axes;      // [2]
  float* maxabs;
  double* unit2;
  uint16_t *e1h, *e1l, *fh, *fl, *gh, *gl, *e2h, *e2l;
};

static size_t carve_fp64(void* ws, int count, int m, int n, int M, int N, Dft2Fp64Space* s) {
  Carve c(ws);
  Dft2Fp64Space t;
  t.err = c.take<int>(4);
  t.E1 = c.take<double2>((size_t)M * m);
  t.E2 = c.take<double2>((size_t)n * N);
  t.T = c.take<double2>((size_t)count * std::max((size_t)M * n, (size_t)m * N));
  if (s) *s = t;
  return c.used;
}

static size_t carve_split(void* ws, int count, int m, int n, int M, int N, Dft2SplitSpace* s) {
  const int kp1 = round_up(m, 32), kp2 = round_up(n, 32);
  const size_t mrows1 = (size_t)cdiv(M, 64) * 128, nrows2 = (size_t)cdiv(N, 128) * 256;
  Carve c(ws);
  Dft2SplitSpace t;
  t.err = c.take<int>(4);
  t.axes = c.take<PhaseAxis>(2);
  t.maxabs = c.take<float>(std::max(count, 4));
  t.unit2 = c.take<double>(2);
  t.e1h = c.take<uint16_t>(mrows1 * 2 * kp1);
  t.e1l = c.take<uint16_t>(mrows1 * 2 * kp1);
  t.fh = c.take<uint16_t>((size_t)count * n * 2 * kp1);
  t.fl = c.take<uint16_t>((size_t)count * n * 2 * kp1);
  t.gh = c.take<uint16_t>((size_t)count * M * 2 * kp2);
  t.gl = c.take<uint16_t>((size_t)count * M * 2 * kp2);
  t.e2h = c.take<uint16_t>(nrows2 * 2 * kp2);
  t.e2l = c.take<uint16_t>(nrows2 * 2 * kp2);
  if (s) *s = t;
  return c.used;
}

static int check_sizes(int m, int n, int M, int N) {
  LGB_REQUIRE(m > 0 && n > 0 && M > 0 && N > 0, LGB_EINVAL, "dft2: sizes must be positive");
  LGB_REQUIRE((long long)m * n < (1LL << 31) && (long long)M * N < (1LL << 31), LGB_EINVAL,
              "dft2: array too large");
  return LGB_OK;
}

}  // namespace lgb

using namespace lgb;

extern "C" size_t lgb_dft2_batch_workspace_size(int count, int m, int n, int M, int N,
                                                int precision) {
  if (count <= 0 || m <= 0 || n <= 0 || M <= 0 || N <= 0) return 0;
  return is_split(precision) ? carve_split(nullptr, count, m, n, M, N, nullptr)
                             : carve_fp64(nullptr, count, m, n, M, N, nullptr);
}

extern "C" size_t lgb_dft2_workspace_size(int m, int n, int M, int N, int precision) {
  return lgb_dft2_batch_workspace_size(1, m, n, M, N, precision);
}

extern "C" int lgb_dft2_batch(const lgb_c128* f, int count, int m, int n, lgb_c128* F, int M,
                              int N, double alpha_r, double alpha_c, double shift_r,
                              double shift_c, double offset_r, double offset_c, int unitary,
                              int precision, void* workspace, size_t workspace_bytes,
                              lgb_stream stream) {
  LGB_RANGE("lgb_dft2_batch");
  return dft2_batch(reinterpret_cast<const double2*>(f), count, m, n,
                    reinterpret_cast<double2*>(F), M, N, alpha_r, alpha_c, shift_r, shift_c,
                    offset_r, offset_c, unitary, precision, workspace, workspace_bytes,
                    as_stream(stream), nullptr);
}

int lgb::dft2_batch(const double2* fin, int count, int m, int n, double2* Fout, int M, int N,
                    double alpha_r, double alpha_c, double shift_r, double shift_c,
                    double offset_r, double offset_c, int unitary, int precision, void* workspace,
                    size_t workspace_bytes, cudaStream_t s, const ZgemmScratch* zs) {
  int st = check_sizes(m, n, M, N);
  if (st) return st;
  LGB_REQUIRE(count >= 1 && count <= 65535, LGB_EINVAL, "dft2: count outside 1..65535");
  LGB_REQUIRE(fin && Fout, LGB_EINVAL, "dft2: null input or output");
  LGB_REQUIRE(precision == LGB_FP64 || is_split(precision), LGB_EINVAL, "dft2: unknown precision");
  LGB_REQUIRE(workspace && ((uintptr_t)workspace & 255) == 0, LGB_EWORKSPACE,
              "dft2: workspace must be non-null and 256-byte aligned");
  LGB_REQUIRE(workspace_bytes >= lgb_dft2_batch_workspace_size(count, m, n, M, N, precision),
              LGB_EWORKSPACE, "dft2: workspace too small");
  PhaseAxis ar, ac;
  if ((st = make_phase_axis(alpha_r, shift_r, offset_r, m, M, &ar))) return st;
  if ((st = make_phase_axis(alpha_c, shift_c, offset_c, n, N, &ac))) return st;
  const double scale = unitary ? std::sqrt(std::fabs(alpha_r * alpha_c)) : 1.0;

  if (precision == LGB_FP64) {
    Dft2Fp64Space w;
    carve_fp64(workspace, count, m, n, M, N, &w);
    LGB_CUDA(cudaMemsetAsync(w.err, 0, sizeof(int), s));
    if ((st = launch_dft_matrix_c128(ar, m, M, w.E1, true, s))) return st;
    if ((st = launch_dft_matrix_c128(ac, n, N, w.E2, false, s))) return st;
    // (E1 f) E2 as lentil, or E1 (f E2) when that order needs fewer flops;
    // the matrices are shared by the batch (stride 0)
    const long long sf = (long long)m * n, sF = (long long)M * N;
    const double cost_left = (double)M * m * n + (double)M * n * N;
    const double cost_right = (double)m * n * N + (double)M * m * N;
    if (cost_left <= cost_right) {
      const long long sT = (long long)M * n;
      if ((st = launch_zgemm(M, n, m, w.E1, m, 0, fin, n, sf, w.T, n, sT, count, 1.0, s, zs))) return st;
      return launch_zgemm(M, N, n, w.T, n, sT, w.E2, N, 0, Fout, N, sF, count, scale, s, zs);
    }
    const long long sT = (long long)m * N;
    if ((st = launch_zgemm(m, N, n, fin, n, sf, w.E2, N, 0, w.T, N, sT, count, 1.0, s, zs))) return st;
    return launch_zgemm(M, N, m, w.E1, m, 0, w.T, N, sT, Fout, N, sF, count, scale, s, zs);
  }

  // split precision on the tensor cores: one launch pair for the whole batch
  const bool bf16 = precision == LGB_SPLIT_BF16;
  const int kp1 = round_up(m, 32), kp2 = round_up(n, 32);
  Dft2SplitSpace w;
  carve_split(workspace, count, m, n, M, N, &w);
  PhaseAxis axes[2] = {ar, ac};
  LGB_CUDA(cudaMemsetAsync(w.err, 0, sizeof(int), s));
  LGB_CUDA(cudaMemcpyAsync(w.axes, axes, sizeof(axes), cudaMemcpyHostToDevice, s));
  if ((st = launch_e1_block_split(w.axes, 1, m, M, kp1, cdiv(M, 64) * 128, bf16, w.e1h, w.e1l, s))) return st;
  if ((st = launch_e2_block_split(w.axes + 1, 1, n, N, kp2, cdiv(N, 128) * 256, bf16, w.e2h, w.e2l, s))) return st;
  // bf16 keeps FP32's exponent range: no per-field scale is needed (and a
  // power-of-two scale would change no result), so only fp16 reduces max|f|
  float* const maxabs = bf16 ? nullptr : w.maxabs;
  if (maxabs && (st = launch_maxabs_c128_batch(fin, m * n, count, maxabs, s))) return st;
  SplitFieldArgs fa{};
  fa.field = fin;
  fa.m = m; fa.n = n; fa.kp = kp1; fa.L = 1; fa.batch = count;
  fa.maxabs = maxabs;
  fa.hi = w.fh; fa.lo = w.fl;
  if ((st = launch_split_field_T(fa, bf16, s))) return st;
  const double one = 1.0;
  LGB_CUDA(cudaMemcpyAsync(w.unit2, &one, sizeof(double), cudaMemcpyHostToDevice, s));
  SplitMftProblem p{};
  p.m = m; p.n = n; p.M = M; p.N = N; p.kp1 = kp1; p.kp2 = kp2; p.L = 1; p.batch = count;
  p.bf16 = bf16;
  p.e1_hi = w.e1h; p.e1_lo = w.e1l; p.f_hi = w.fh; p.f_lo = w.fl;
  p.e2_hi = w.e2h; p.e2_lo = w.e2l; p.g_hi = w.gh; p.g_lo = w.gl;
  p.maxabs = maxabs;
  p.epilogue = 1;
  p.unit2 = w.unit2;
  p.out = reinterpret_cast<double*>(Fout);
  p.complex_scale = scale;
  p.err = w.err;
  return launch_split_mft(p, s);
}

extern "C" int lgb_dft2(const lgb_c128* f, int m, int n, lgb_c128* F, int M, int N,
                        double alpha_r, double alpha_c, double shift_r, double shift_c,
                        double offset_r, double offset_c, int unitary, int precision,
                        void* workspace, size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_dft2");
  return lgb_dft2_batch(f, 1, m, n, F, M, N, alpha_r, alpha_c, shift_r, shift_c, offset_r,
                        offset_c, unitary, precision, workspace, workspace_bytes, stream);
}

// Device status of the last dft2 that used this workspace (synchronises the
// stream): LGB_OK, or LGB_ETIMEOUT when a device-side wait expired.
extern "C" int lgb_dft2_status(void* workspace, lgb_stream stream) {
  LGB_REQUIRE(workspace, LGB_EINVAL, "dft2_status: null workspace");
  int h = 0;
  LGB_CUDA(cudaMemcpyAsync(&h, workspace, sizeof(int), cudaMemcpyDeviceToHost, as_stream(stream)));
  LGB_CUDA(cudaStreamSynchronize(as_stream(stream)));
  if (h) return set_error(h, "device-side wait expired inside the tensor-core MFT");
  return LGB_OK;
}

extern "C" int lgb_idft2(const lgb_c128* F, int m, int n, lgb_c128* f, int M, int N,
                         double alpha_r, double alpha_c, double shift_r, double shift_c,
                         int unitary, int precision, void* workspace, size_t workspace_bytes,
                         lgb_stream stream) {
  LGB_RANGE("lgb_idft2");
  // lentil/fourier.py:193-198: conj(dft2(conj(F))) / F.size.  The conjugated
  // input lives in the caller's output buffer when the shapes allow,
  // otherwise in the tail of the workspace.
  int st = check_sizes(m, n, M, N);
  if (st) return st;
  LGB_REQUIRE(F && f, LGB_EINVAL, "idft2: null input or output");
  const size_t need = lgb_dft2_workspace_size(m, n, M, N, precision);
  const size_t conj_off = align_up(need, 256);
  LGB_REQUIRE(workspace_bytes >= conj_off + sizeof(double2) * (size_t)m * n, LGB_EWORKSPACE,
              "idft2: workspace too small (lgb_idft2_workspace_size)");
  cudaStream_t s = as_stream(stream);
  double2* tmp = reinterpret_cast<double2*>(static_cast<char*>(workspace) + conj_off);
  if ((st = launch_conj_scale(reinterpret_cast<const double2*>(F), tmp, (size_t)m * n, 1.0, s))) return st;
  if ((st = lgb_dft2(reinterpret_cast<lgb_c128*>(tmp), m, n, f, M, N, alpha_r, alpha_c, shift_r,
                     shift_c, 0.0, 0.0, unitary, precision, workspace, need, stream)))
    return st;
  return launch_conj_scale(reinterpret_cast<const double2*>(f), reinterpret_cast<double2*>(f),
                           (size_t)M * N, 1.0 / ((double)m * n), s);
}

extern "C" size_t lgb_idft2_workspace_size(int m, int n, int M, int N, int precision) {
  const size_t need = lgb_dft2_workspace_size(m, n, M, N, precision);
  if (!need) return 0;
  return align_up(need, 256) + sizeof(double2) * (size_t)m * n;
}

// ===========================================================================
// broadband PSF plan
// ===========================================================================
// Per-execute operands of the split path: the phasor operand f^T, the
// stage-1 result G, the FP32 intensity window, the per-PSF field maxima and
// the device status word (first, so a workspace's status is at offset 0).
struct SplitOperands {
  int* err = nullptr;
  float* maxabs = nullptr;
  uint16_t *fh = nullptr, *fl = nullptr, *gh = nullptr, *gl = nullptr;
  float* wbuf = nullptr;
  int ldw = 0;
  uint8_t* kflags = nullptr;       // [B][kp1/32][kf_pitch] field nonzero flags
  int kf_pitch = 0;
};

static size_t carve_operands(void* base, const lgb_psf_desc& d, int kp1, int kp2, int B, int L,
                             SplitOperands* o) {
  Carve c(base);
  SplitOperands t;
  const size_t Q = (size_t)B * L;
  t.err = c.take<int>(4);
  t.maxabs = c.take<float>(B);
  t.fh = c.take<uint16_t>(Q * d.n * 2 * kp1);
  t.fl = c.take<uint16_t>(Q * d.n * 2 * kp1);
  t.gh = c.take<uint16_t>(Q * d.M * 2 * kp2);
  t.gl = c.take<uint16_t>(Q * d.M * 2 * kp2);
  t.ldw = round_up(d.N, 4);
  t.wbuf = c.take<float>((size_t)B * d.M * t.ldw);
  t.kf_pitch = kflag_pitch(kp2);
  t.kflags = c.take<uint8_t>((size_t)B * (kp1 / 32) * t.kf_pitch);
  if (o) *o = t;
  return c.used;
}
struct lgb_psf_plan_s {
  lgb_psf_desc d;
  std::vector<double> lam, ar, ac, sr, sc;
  void* mem = nullptr;
  size_t bytes = 0;
  bool owns_mem = true;            // false: caller memory (lgb_psf_plan_create_in)
  cudaStream_t stream = nullptr;   // creation stream: the plan's own memory is freed on it
  int kp1 = 0, kp2 = 0;
  // device views
  int* err = nullptr;
  double* unit2 = nullptr;         // [L]
  double* two_over_lambda = nullptr;
  float2* khalf = nullptr;         // [L]
  PhaseAxis* axes = nullptr;       // [2L]: rows then cols
  float* maxabs = nullptr;         // [batch]
  // split
  uint16_t *e1h = nullptr, *e1l = nullptr, *e2h = nullptr, *e2l = nullptr;
  SplitOperands ops;               // plan-owned operands (batch > 0)
  int tile = 0;                    // tensor-core pair-tile width: 0 = the autotuner's, 128, 256
  // optional per-kernel timing: event pairs recorded around each launch
  bool profile = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  double kernel_ms[LGB_PROFILE_SLOTS] = {0};
  int kernel_launches[LGB_PROFILE_SLOTS] = {0};
  // fp64
  double2 *E1 = nullptr, *E2 = nullptr, *f = nullptr, *T = nullptr, *F = nullptr;
};

static size_t plan_carve(lgb_psf_plan_s* P, void* base) {
  const lgb_psf_desc& d = P->d;
  const int L = d.n_wavelengths, B = d.batch;
  Carve c(base);
  P->err = c.take<int>(4);
  P->unit2 = c.take<double>(L);
  P->two_over_lambda = c.take<double>(L);
  P->khalf = c.take<float2>(L);
  P->axes = c.take<PhaseAxis>(2 * (size_t)L);
  P->maxabs = c.take<float>(B);
  if (is_split(d.precision)) {
    const size_t mrows1 = (size_t)cdiv(d.M, 64) * 128, nrows2 = (size_t)cdiv(d.N, 128) * 256;
    const size_t Q = (size_t)B * L;
    P->e1h = c.take<uint16_t>(L * mrows1 * 2 * P->kp1);
    P->e1l = c.take<uint16_t>(L * mrows1 * 2 * P->kp1);
    P->e2h = c.take<uint16_t>(L * nrows2 * 2 * P->kp2);
    P->e2l = c.take<uint16_t>(L * nrows2 * 2 * P->kp2);
    (void)Q;
    if (B > 0) {
      c.used = align_up(c.used, 256);
      const size_t sz = carve_operands(base ? static_cast<char*>(base) + c.used : nullptr, d,
                                       P->kp1, P->kp2, B, L, &P->ops);
      if (!base) P->ops = SplitOperands();
      c.used += sz;
      P->ops.err = P->err;
    }
  } else {
    const size_t Q = (size_t)B * L;
    P->E1 = c.take<double2>((size_t)L * d.M * d.m);
    P->E2 = c.take<double2>((size_t)L * d.n * d.N);
    P->f = c.take<double2>(Q * d.m * d.n);
    P->T = c.take<double2>(Q * d.M * d.n);
    P->F = c.take<double2>(Q * d.M * d.N);
  }
  return c.used;
}

// Event pair bracketing one launch (slot = kernel kind) when profiling.
static int prof_begin(lgb_psf_plan_s* P, int slot, cudaStream_t s, cudaEvent_t* e) {
  if (!P->profile) return LGB_OK;
  LGB_CUDA(cudaEventCreate(&e[0]));
  LGB_CUDA(cudaEventCreate(&e[1]));
  LGB_CUDA(cudaEventRecord(e[0], s));
  (void)slot;
  return LGB_OK;
}
static int prof_end(lgb_psf_plan_s* P, int slot, cudaStream_t s, cudaEvent_t* e) {
  if (!P->profile) return LGB_OK;
  LGB_CUDA(cudaEventRecord(e[1], s));
  P->pending.push_back({slot, {e[0], e[1]}});
  return LGB_OK;
}

static int check_desc(const lgb_psf_desc& d) {
  LGB_REQUIRE(d.H > 0 && d.W > 0 && d.m > 0 && d.n > 0 && d.M > 0 && d.N > 0, LGB_EINVAL,
              "psf_plan_create: sizes must be positive");
  LGB_REQUIRE(d.r0 >= 0 && d.c0 >= 0 && d.r0 + d.m <= d.H && d.c0 + d.n <= d.W, LGB_EINVAL,
              "psf_plan_create: field slice outside the pupil plane");
  LGB_REQUIRE(d.win_r0 >= 0 && d.win_c0 >= 0 && d.win_r0 + d.M <= d.out_rows &&
                  d.win_c0 + d.N <= d.out_cols,
              LGB_EINVAL, "psf_plan_create: window outside the output image");
  LGB_REQUIRE(d.n_wavelengths > 0 && d.wavelengths && d.alpha_r && d.alpha_c && d.shift_r &&
                  d.shift_c,
              LGB_EINVAL, "psf_plan_create: wavelength arrays required");
  LGB_REQUIRE(d.batch > 0 || (d.batch == 0 && (d.precision == LGB_SPLIT_BF16 ||
                                                d.precision == LGB_SPLIT_FP16)),
              LGB_EINVAL, "psf_plan_create: batch must be positive (0: split matrices only)");
  LGB_REQUIRE(d.precision == LGB_FP64 || is_split(d.precision), LGB_EINVAL,
              "psf_plan_create: unknown precision");
  return LGB_OK;
}

// A plan object for desc with its tables copied (no device memory yet).
static lgb_psf_plan_s* new_plan(const lgb_psf_desc& d) {
  const int L = d.n_wavelengths;
  auto P = new lgb_psf_plan_s();
  P->d = d;
  P->lam.assign(d.wavelengths, d.wavelengths + L);
  P->ar.assign(d.alpha_r, d.alpha_r + L);
  P->ac.assign(d.alpha_c, d.alpha_c + L);
  P->sr.assign(d.shift_r, d.shift_r + L);
  P->sc.assign(d.shift_c, d.shift_c + L);
  P->d.wavelengths = P->d.alpha_r = P->d.alpha_c = P->d.shift_r = P->d.shift_c = nullptr;
  P->kp1 = round_up(d.m, 32);
  P->kp2 = round_up(d.n, 32);
  P->bytes = plan_carve(P, nullptr);
  return P;
}

static void free_plan(lgb_psf_plan_s* P, cudaStream_t s) {
  if (P->owns_mem && P->mem) cudaFreeAsync(P->mem, s);
  delete P;
}

// Fill a plan whose memory is in place: tables to the device, then the DFT
// matrices of every wavelength (resident for the plan's lifetime).
static int build_plan(lgb_psf_plan_s* P, cudaStream_t s, lgb_psf_plan* plan) {
  const lgb_psf_desc& d = P->d;
  const int L = d.n_wavelengths;
  cudaError_t e = cudaSuccess;
  plan_carve(P, P->mem);

  // host tables -> device
  std::vector<PhaseAxis> axes(2 * (size_t)L);
  std::vector<double> unit2(L), tol(L);
  std::vector<float2> kh(L);
  int st = LGB_OK;
  for (int l = 0; l < L && !st; ++l) {
    st = make_phase_axis(P->ar[l], P->sr[l], d.offset_r, d.m, d.M, &axes[l]);
    if (!st) st = make_phase_axis(P->ac[l], P->sc[l], d.offset_c, d.n, d.N, &axes[L + l]);
    unit2[l] = std::fabs(P->ar[l] * P->ac[l]);
    tol[l] = 2.0 / P->lam[l];
    const float hi = (float)tol[l];
    kh[l] = make_float2(hi, (float)(tol[l] - (double)hi));
  }
  if (st) { free_plan(P, s); return st; }
  auto fail = [&](cudaError_t err, const char* what) {
    free_plan(P, s);
    return check_cuda(err, what);
  };
  if ((e = cudaMemcpyAsync(P->axes, axes.data(), sizeof(PhaseAxis) * axes.size(), cudaMemcpyHostToDevice, s))) return fail(e, "copy axes");
  if ((e = cudaMemcpyAsync(P->unit2, unit2.data(), sizeof(double) * L, cudaMemcpyHostToDevice, s))) return fail(e, "copy unit2");
  if ((e = cudaMemcpyAsync(P->two_over_lambda, tol.data(), sizeof(double) * L, cudaMemcpyHostToDevice, s))) return fail(e, "copy lambda");
  if ((e = cudaMemcpyAsync(P->khalf, kh.data(), sizeof(float2) * L, cudaMemcpyHostToDevice, s))) return fail(e, "copy khalf");
  // the wavelength tables above are pageable: make sure they were consumed
  if ((e = cudaStreamSynchronize(s))) return fail(e, "sync");

  // DFT matrices of every wavelength, resident for the plan's lifetime
  if (is_split(d.precision)) {
    const bool bf16 = d.precision == LGB_SPLIT_BF16;
    st = launch_e1_block_split(P->axes, L, d.m, d.M, P->kp1, cdiv(d.M, 64) * 128, bf16, P->e1h, P->e1l, s);
    if (!st) st = launch_e2_block_split(P->axes + L, L, d.n, d.N, P->kp2, cdiv(d.N, 128) * 256, bf16, P->e2h, P->e2l, s);
  } else {
    for (int l = 0; l < L && !st; ++l) {
      st = launch_dft_matrix_c128(axes[l], d.m, d.M, P->E1 + (size_t)l * d.M * d.m, true, s);
      if (!st) st = launch_dft_matrix_c128(axes[L + l], d.n, d.N, P->E2 + (size_t)l * d.n * d.N, false, s);
    }
  }
  if (st) { free_plan(P, s); return st; }
  *plan = P;
  return LGB_OK;
}

extern "C" int lgb_psf_plan_create(const lgb_psf_desc* desc, lgb_psf_plan* plan, lgb_stream stream) {
  LGB_RANGE("lgb_psf_plan_create");
  LGB_REQUIRE(desc && plan, LGB_EINVAL, "psf_plan_create: null argument");
  *plan = nullptr;
  int st = check_desc(*desc);
  if (st) return st;
  lgb_psf_plan_s* P = new_plan(*desc);
  cudaStream_t s = as_stream(stream);
  P->stream = s;
  cudaError_t e = cudaMallocAsync(&P->mem, P->bytes, s);
  if (e != cudaSuccess) {
    delete P;
    return check_cuda(e, "cudaMallocAsync(psf plan)");
  }
  return build_plan(P, s, plan);
}

extern "C" size_t lgb_psf_plan_size(const lgb_psf_desc* desc) {
  if (!desc || check_desc(*desc) != LGB_OK) return 0;
  lgb_psf_plan_s* P = new_plan(*desc);
  const size_t bytes = P->bytes;
  delete P;
  return bytes;
}

extern "C" int lgb_psf_plan_create_in(const lgb_psf_desc* desc, void* memory, size_t memory_bytes,
                                      lgb_psf_plan* plan, lgb_stream stream) {
  LGB_RANGE("lgb_psf_plan_create_in");
  LGB_REQUIRE(desc && plan, LGB_EINVAL, "psf_plan_create_in: null argument");
  *plan = nullptr;
  int st = check_desc(*desc);
  if (st) return st;
  LGB_REQUIRE(memory && ((uintptr_t)memory & 255) == 0, LGB_EWORKSPACE,
              "psf_plan_create_in: memory must be non-null and 256-byte aligned");
  lgb_psf_plan_s* P = new_plan(*desc);
  if (memory_bytes < P->bytes) {
    delete P;
    return set_error(LGB_EWORKSPACE, "psf_plan_create_in: memory smaller than lgb_psf_plan_size");
  }
  P->mem = memory;
  P->owns_mem = false;
  P->stream = as_stream(stream);
  return build_plan(P, P->stream, plan);
}

extern "C" size_t lgb_psf_plan_bytes(lgb_psf_plan plan) { return plan ? plan->bytes : 0; }

static int psf_execute_n(lgb_psf_plan P, int B, const int* lam_idx, int n_sel, const double* amp,
                         const double* opd, const double* weights, double* out, int accumulate,
                         lgb_stream stream, const SplitOperands* ops_in = nullptr) {
  LGB_REQUIRE(P && amp && opd && out, LGB_EINVAL, "psf_execute: null argument");
  const lgb_psf_desc& d = P->d;
  LGB_REQUIRE(B >= 1 && (ops_in || B <= d.batch), LGB_EINVAL,
              "psf_execute: count outside 1..batch");
  const SplitOperands& ops = ops_in ? *ops_in : P->ops;
  int* const errp = ops_in ? ops_in->err : P->err;
  LGB_REQUIRE(!lam_idx || (n_sel >= 1 && n_sel <= d.n_wavelengths), LGB_EINVAL,
              "psf_execute: wavelength subset size outside 1..n_wavelengths");
  LGB_REQUIRE(!lam_idx || is_split(d.precision), LGB_EUNSUPPORTED,
              "psf_execute: wavelength subsets need a split-precision plan");
  const int L = lam_idx ? n_sel : d.n_wavelengths;
  cudaStream_t s = as_stream(stream);
  int st;
  const size_t img = (size_t)d.out_rows * d.out_cols;
  // the split path stores its window into a fresh image: only the pixels
  // outside the window need zeros
  const bool window_is_image = d.M == d.out_rows && d.N == d.out_cols;
  if (!accumulate && !(is_split(d.precision) && window_is_image))
    LGB_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * img * B, s));
  LGB_CUDA(cudaMemsetAsync(errp, 0, sizeof(int), s));
  if (is_split(d.precision)) {
    const bool bf16 = d.precision == LGB_SPLIT_BF16;
    cudaEvent_t ev[2];
    // bf16: no per-PSF scale (see lgb_dft2_batch)
    float* const maxabs = bf16 ? nullptr : ops.maxabs;
    if (maxabs && (st = launch_maxabs_amp(amp, B, d.H, d.W, d.r0, d.c0, d.m, d.n, maxabs, s)))
      return st;
    SplitFieldArgs fa{};
    fa.amp = amp; fa.opd = opd;
    fa.H = d.H; fa.W = d.W; fa.r0 = d.r0; fa.c0 = d.c0;
    fa.khalf = P->khalf;
    fa.m = d.m; fa.n = d.n; fa.kp = P->kp1; fa.L = L; fa.batch = B;
    fa.maxabs = maxabs;
    fa.hi = ops.fh; fa.lo = ops.fl;
    fa.lam_idx = lam_idx;
    fa.kflags = ops.kflags; fa.kf_pitch = ops.kf_pitch;
    if ((st = prof_begin(P, LGB_PROFILE_PHASOR, s, ev))) return st;
    if ((st = launch_split_field_T(fa, bf16, s))) return st;
    if ((st = prof_end(P, LGB_PROFILE_PHASOR, s, ev))) return st;
    SplitMftProblem p{};
    p.m = d.m; p.n = d.n; p.M = d.M; p.N = d.N; p.kp1 = P->kp1; p.kp2 = P->kp2;
    p.L = L; p.batch = B; p.bf16 = bf16;
    p.lam_idx = lam_idx;
    p.L_bank = d.n_wavelengths;
    p.e1_hi = P->e1h; p.e1_lo = P->e1l; p.f_hi = ops.fh; p.f_lo = ops.fl;
    p.e2_hi = P->e2h; p.e2_lo = P->e2l; p.g_hi = ops.gh; p.g_lo = ops.gl;
    p.maxabs = maxabs;
    p.epilogue = 0;
    p.weights = weights;
    p.unit2 = P->unit2;
    p.wbuf = ops.wbuf;
    p.ldw = ops.ldw;
    p.err = errp;
    p.tile = P->tile;
    p.kflags = ops.kflags; p.kf_pitch = ops.kf_pitch;   // skip all-zero field blocks
    LGB_CUDA(cudaMemsetAsync(ops.wbuf, 0, sizeof(float) * (size_t)B * d.M * ops.ldw, s));
    cudaEvent_t mev[4];
    if (P->profile) {
      for (auto& e : mev) LGB_CUDA(cudaEventCreate(&e));
      p.events = mev;
    }
    if ((st = launch_split_mft(p, s))) return st;
    if (P->profile) {
      P->pending.push_back({LGB_PROFILE_MFT1, {mev[0], mev[1]}});
      P->pending.push_back({LGB_PROFILE_MFT2, {mev[2], mev[3]}});
    }
    if ((st = prof_begin(P, LGB_PROFILE_OTHER, s, ev))) return st;
    if ((st = launch_window_add(ops.wbuf, d.M, d.N, ops.ldw, B, out, d.out_cols, (long long)img,
                                d.win_r0, d.win_c0, accumulate != 0, s)))
      return st;
    return prof_end(P, LGB_PROFILE_OTHER, s, ev);
  }
  // plain FP64
  cudaEvent_t ev[2];
  if ((st = prof_begin(P, LGB_PROFILE_PHASOR, s, ev))) return st;
  if ((st = launch_phasor_batch_c128(amp, opd, d.H, d.W, d.r0, d.c0, d.m, d.n, P->two_over_lambda,
                                     L, B, P->f, s)))
    return st;
  if ((st = prof_end(P, LGB_PROFILE_PHASOR, s, ev))) return st;
  const long long sE1 = (long long)d.M * d.m, sE2 = (long long)d.n * d.N;
  const long long sf = (long long)d.m * d.n, sT = (long long)d.M * d.n, sF = (long long)d.M * d.N;
  for (int b = 0; b < B; ++b) {
    const size_t q0 = (size_t)b * L;
    if ((st = prof_begin(P, LGB_PROFILE_MFT1, s, ev))) return st;
    if ((st = launch_zgemm(d.M, d.n, d.m, P->E1, d.m, sE1, P->f + q0 * sf, d.n, sf, P->T + q0 * sT,
                           d.n, sT, L, 1.0, s)))
      return st;
    if ((st = prof_end(P, LGB_PROFILE_MFT1, s, ev))) return st;
    if ((st = prof_begin(P, LGB_PROFILE_MFT2, s, ev))) return st;
    if ((st = launch_zgemm(d.M, d.N, d.n, P->T + q0 * sT, d.n, sT, P->E2, d.N, sE2, P->F + q0 * sF,
                           d.N, sF, L, 1.0, s)))
      return st;
    if ((st = prof_end(P, LGB_PROFILE_MFT2, s, ev))) return st;
  }
  if ((st = prof_begin(P, LGB_PROFILE_OTHER, s, ev))) return st;
  if ((st = launch_intensity_accum_c128(P->F, d.M, d.N, sF, L, weights, P->unit2, out, d.out_cols,
                                        (long long)img, d.win_r0, d.win_c0, B, s)))
    return st;
  return prof_end(P, LGB_PROFILE_OTHER, s, ev);
}

extern "C" int lgb_psf_execute(lgb_psf_plan P, const double* amp, const double* opd,
                               const double* weights, double* out, int accumulate, lgb_stream stream) {
  LGB_RANGE("lgb_psf_execute");
  LGB_REQUIRE(P, LGB_EINVAL, "psf_execute: null plan");
  return psf_execute_n(P, P->d.batch, nullptr, 0, amp, opd, weights, out, accumulate, stream);
}

extern "C" int lgb_psf_execute_batch(lgb_psf_plan P, int count, const double* amp,
                                     const double* opd, const double* weights, double* out,
                                     int accumulate, lgb_stream stream) {
  LGB_RANGE("lgb_psf_execute_batch");
  return psf_execute_n(P, count, nullptr, 0, amp, opd, weights, out, accumulate, stream);
}

extern "C" size_t lgb_psf_execute_workspace_size(lgb_psf_plan P, int count, int n_sel) {
  if (!P || count <= 0 || n_sel <= 0 || !is_split(P->d.precision)) return 0;
  return carve_operands(nullptr, P->d, P->kp1, P->kp2, count, n_sel, nullptr);
}

extern "C" int lgb_psf_execute_ws(lgb_psf_plan P, int count, const int* lam_idx, int n_sel,
                                  const double* amp, const double* opd, const double* weights,
                                  double* out, int accumulate, void* workspace,
                                  size_t workspace_bytes, lgb_stream stream) {
  LGB_RANGE("lgb_psf_execute_ws");
  LGB_REQUIRE(P, LGB_EINVAL, "psf_execute_ws: null plan");
  LGB_REQUIRE(is_split(P->d.precision), LGB_EUNSUPPORTED,
              "psf_execute_ws: caller workspaces serve split-precision plans");
  const int L = lam_idx ? n_sel : P->d.n_wavelengths;
  LGB_REQUIRE(workspace && ((uintptr_t)workspace & 255) == 0, LGB_EWORKSPACE,
              "psf_execute_ws: workspace must be non-null and 256-byte aligned");
  LGB_REQUIRE(workspace_bytes >= lgb_psf_execute_workspace_size(P, count, L), LGB_EWORKSPACE,
              "psf_execute_ws: workspace too small");
  SplitOperands ops;
  carve_operands(workspace, P->d, P->kp1, P->kp2, count, L, &ops);
  return psf_execute_n(P, count, lam_idx, lam_idx ? n_sel : 0, amp, opd, weights, out,
                       accumulate, stream, &ops);
}

extern "C" int lgb_psf_execute_subset(lgb_psf_plan P, int count, const int* lam_idx, int n_sel,
                                      const double* amp, const double* opd, const double* weights,
                                      double* out, int accumulate, lgb_stream stream) {
  LGB_RANGE("lgb_psf_execute_subset");
  LGB_REQUIRE(lam_idx, LGB_EINVAL, "psf_execute_subset: null wavelength index");
  return psf_execute_n(P, count, lam_idx, n_sel, amp, opd, weights, out, accumulate, stream);
}

extern "C" int lgb_psf_plan_set_tile(lgb_psf_plan P, int tile) {
  LGB_REQUIRE(P, LGB_EINVAL, "psf_plan_set_tile: null plan");
  LGB_REQUIRE(tile == 0 || tile == 128 || tile == 256, LGB_EINVAL,
              "psf_plan_set_tile: tile must be 0 (tuned), 128 or 256");
  P->tile = tile;
  return LGB_OK;
}

extern "C" int lgb_psf_plan_profile(lgb_psf_plan P, int enable) {
  LGB_REQUIRE(P, LGB_EINVAL, "psf_plan_profile: null plan");
  P->profile = enable != 0;
  return LGB_OK;
}

extern "C" int lgb_psf_plan_kernel_times(lgb_psf_plan P, double* ms, int* launches, int n) {
  LGB_REQUIRE(P && ms && launches && n > 0, LGB_EINVAL, "psf_plan_kernel_times: bad argument");
  for (auto& e : P->pending) {
    LGB_CUDA(cudaEventSynchronize(e.second.second));
    float t = 0.f;
    LGB_CUDA(cudaEventElapsedTime(&t, e.second.first, e.second.second));
    P->kernel_ms[e.first] += t;
    P->kernel_launches[e.first] += 1;
    cudaEventDestroy(e.second.first);
    cudaEventDestroy(e.second.second);
  }
  P->pending.clear();
  for (int k = 0; k < n && k < LGB_PROFILE_SLOTS; ++k) {
    ms[k] = P->kernel_ms[k];
    launches[k] = P->kernel_launches[k];
    P->kernel_ms[k] = 0;
    P->kernel_launches[k] = 0;
  }
  return LGB_OK;
}

extern "C" int lgb_psf_plan_status(lgb_psf_plan P, lgb_stream stream) {
  LGB_REQUIRE(P, LGB_EINVAL, "psf_plan_status: null plan");
  int h = 0;
  LGB_CUDA(cudaMemcpyAsync(&h, P->err, sizeof(int), cudaMemcpyDeviceToHost, as_stream(stream)));
  LGB_CUDA(cudaStreamSynchronize(as_stream(stream)));
  if (h) return set_error(h, "device-side wait expired inside the tensor-core MFT");
  return LGB_OK;
}

extern "C" int lgb_psf_plan_destroy(lgb_psf_plan P) {
  if (!P) return LGB_OK;
  // stream-ordered free of the plan's own memory: no device-wide
  // synchronisation; the caller destroys a plan only after the work that
  // used it has completed (caller memory is left to the caller)
  cudaError_t e = P->owns_mem ? cudaFreeAsync(P->mem, P->stream) : cudaSuccess;
  delete P;
  if (e != cudaSuccess) return check_cuda(e, "cudaFree(psf plan)");
  return LGB_OK;
}
