/*
 * lentil_gb300 — C ABI of the GB300 (sm_103a) far-field diffraction path.
 *
 * Each entry point replaces one function of lentil 0.8.8's matrix-Fourier-
 * transform path (cited beside it).  All pointers are device pointers unless
 * the comment says "host"; arrays are C-ordered (row-major) and complex
 * values are interleaved (re, im) doubles, the memory layout of numpy's
 * complex128.  Every call is asynchronous on the given CUDA stream
 * (cudaStream_t passed as void*), returns LGB_OK (0) or an error code, and
 * never aborts the process; lgb_last_error() returns the message of the
 * calling thread's last failure.
 *
 * Precision: LGB_FP64 computes in complex128 (the plain form, parity with
 * lentil within 1e-12 peak-normalised).  LGB_SPLIT_BF16 / LGB_SPLIT_FP16 run
 * the contractions on the tcgen05 tensor cores with each operand split into
 * two 16-bit floats (hi + lo; three partial products, FP32 accumulation).
 */
#ifndef LENTIL_GB300_H
#define LENTIL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; the Python layer maps them to lentil's exception types */
#define LGB_OK 0
#define LGB_EINVAL 1        /* ValueError */
#define LGB_ETYPE 2         /* TypeError */
#define LGB_ECUDA 3         /* RuntimeError: a CUDA runtime call failed */
#define LGB_EUNSUPPORTED 4  /* NotImplementedError */
#define LGB_ETIMEOUT 5      /* a device-side wait hit its time bound */
#define LGB_EWORKSPACE 6    /* workspace pointer/size too small */

#define LGB_FP64 0
#define LGB_SPLIT_BF16 1
#define LGB_SPLIT_FP16 2

typedef struct { double re, im; } lgb_c128; /* == numpy complex128 */
typedef void* lgb_stream;                   /* == cudaStream_t */

/* Message of this thread's last failed call ("" if none). */
const char* lgb_last_error(void);
/* ABI version, (major << 16) | minor. */
int lgb_version(void);
/* Usage of a device's default stream-ordered memory pool, the pool that
 * entries given no workspace take temporary memory from (the FP64 GEMMs'
 * split-K partials): out[0..3] = reserved bytes now, reserved high-water
 * mark, used bytes now, used high-water mark.  reset_high != 0 resets both
 * high-water marks to the current values first.  A diagnostic; lentil has
 * no counterpart. */
int lgb_mempool_usage(int device, int reset_high, unsigned long long out[4]);

/* ------------------------------------------------------------------------
 * DFT matrices.  Replaces lentil/fourier.py:106-110 (_dft2_matrices, with
 * the centred coordinates of _dft2_coords, lentil/fourier.py:113-121):
 *   E1[u, r] = exp(-2 pi i alpha_r (R_r + offset_r)(U_u - shift_r))  (M x m)
 *   E2[s, v] = exp(-2 pi i alpha_c (S_s + offset_c)(V_v - shift_c))  (n x N)
 * The phase is reduced modulo one cycle in exact fixed point before the
 * FP64 sincospi.
 * ---------------------------------------------------------------------- */
int lgb_dft2_matrices(int m, int n, int M, int N, double alpha_r, double alpha_c,
                      double shift_r, double shift_c, double offset_r, double offset_c,
                      lgb_c128* E1, lgb_c128* E2, lgb_stream stream);

/* ------------------------------------------------------------------------
 * Matrix triple product DFT.  Replaces lentil/fourier.py:5-103 (dft2):
 *   F = E1 . f . E2, times sqrt(|alpha_r alpha_c|) when unitary != 0.
 * f is m x n, F is M x N (F may not alias f).  The workspace must hold
 * lgb_dft2_workspace_size(m, n, M, N, precision) bytes, 256-byte aligned.
 * ---------------------------------------------------------------------- */
size_t lgb_dft2_workspace_size(int m, int n, int M, int N, int precision);
int lgb_dft2(const lgb_c128* f, int m, int n, lgb_c128* F, int M, int N,
             double alpha_r, double alpha_c, double shift_r, double shift_c,
             double offset_r, double offset_c, int unitary, int precision,
             void* workspace, size_t workspace_bytes, lgb_stream stream);
/* Device-side status of the last dft2/idft2 run on this workspace; waits
 * for the stream.  LGB_ETIMEOUT if a tensor-core pipeline wait expired. */
int lgb_dft2_status(void* workspace, lgb_stream stream);

/* Batched dft2 (an extension; lentil's dft2 transforms one array): `count`
 * fields f[count][m][n] with one geometry -> F[count][M][N]; the DFT
 * matrices are built once and the split path transforms the whole batch in
 * one pair of tensor-core launches.  lgb_dft2 is the count == 1 case.
 * Workspace: lgb_dft2_batch_workspace_size(count, ...) bytes. */
size_t lgb_dft2_batch_workspace_size(int count, int m, int n, int M, int N, int precision);
int lgb_dft2_batch(const lgb_c128* f, int count, int m, int n, lgb_c128* F, int M, int N,
                   double alpha_r, double alpha_c, double shift_r, double shift_c,
                   double offset_r, double offset_c, int unitary, int precision,
                   void* workspace, size_t workspace_bytes, lgb_stream stream);

/* dft2 plans (an extension; lentil rebuilds its DFT matrices on every
 * call): one geometry (m, n, M, N, alpha, shift, offset, unitary,
 * precision) with its DFT matrices built at creation and kept on the
 * device (lgb_dft2_plan_bytes).  lgb_dft2_plan_execute transforms `count`
 * fields f[count][m][n] -> F[count][M][N] with no matrix build, no host
 * copy and no host wait; its workspace holds
 * lgb_dft2_plan_workspace_size(plan, count) bytes (256-byte aligned) and
 * one plan may run on several streams at once.  Status of the split path:
 * each execute copies the plan's sticky device flag to pinned host memory
 * behind an event, and the next execute returns LGB_ETIMEOUT if that copy
 * has landed and shows an expired wait (nothing is copied or queried under
 * stream capture); lgb_dft2_plan_status waits and reports at once.
 * Creation issues no host wait.  lgb_dft2_plan_create allocates the plan's
 * device memory (lgb_dft2_plan_destroy then waits for the device before
 * freeing it); lgb_dft2_plan_create_in builds it in caller-owned device
 * memory of lgb_dft2_plan_size bytes (256-byte aligned), which destroy does
 * not touch: the caller keeps it alive until the plan's executes are done. */
typedef struct lgb_dft2_plan_s* lgb_dft2_plan;
size_t lgb_dft2_plan_size(int m, int n, int M, int N, int precision);
int lgb_dft2_plan_create(int m, int n, int M, int N, double alpha_r, double alpha_c,
                         double shift_r, double shift_c, double offset_r, double offset_c,
                         int unitary, int precision, lgb_stream stream, lgb_dft2_plan* plan);
int lgb_dft2_plan_create_in(int m, int n, int M, int N, double alpha_r, double alpha_c,
                            double shift_r, double shift_c, double offset_r, double offset_c,
                            int unitary, int precision, void* memory, size_t memory_bytes,
                            lgb_stream stream, lgb_dft2_plan* plan);
size_t lgb_dft2_plan_bytes(lgb_dft2_plan plan);
size_t lgb_dft2_plan_workspace_size(lgb_dft2_plan plan, int count);
int lgb_dft2_plan_execute(lgb_dft2_plan plan, const lgb_c128* f, int count, lgb_c128* F,
                          void* workspace, size_t workspace_bytes, lgb_stream stream);
int lgb_dft2_plan_status(lgb_dft2_plan plan, lgb_stream stream);
/* Test hook for the status path: stores LGB_ETIMEOUT (or LGB_OK) into the
 * plan's device status flag, stream-ordered, as an expired pipeline wait
 * would; no kernel of the transform is involved. */
int lgb_dft2_plan_inject_status(lgb_dft2_plan plan, int code, lgb_stream stream);
int lgb_dft2_plan_destroy(lgb_dft2_plan plan);

/* ------------------------------------------------------------------------
 * Allocation-free complex128 dft2 (no counterpart in lentil: an addition of
 * this library for callers that may not allocate device memory at call time,
 * e.g. a control loop with a fixed memory budget or work issued into a
 * stream under graph capture).  Same arguments and result as lgb_dft2 with
 * precision LGB_FP64, but the scratch comes from a fixed array inside the
 * library (LGB_NOALLOC_SCRATCH_BYTES, held by every GPU that loads it) and
 * the caller passes only f and F.  Transforms needing more scratch than that
 * (lgb_dft2_workspace_size(m, n, M, N, LGB_FP64) bytes) are rejected with
 * LGB_EINVAL.  The GEMMs' split-K partial products also live in the array,
 * after that workspace: a transform whose partials do not fit splits K less
 * (or not at all), so the call never allocates device memory, not even from
 * the stream-ordered pool.  The first call on a device looks the array's address up with
 * cudaGetSymbolAddress; make it outside any stream capture.  All calls share
 * the array: calls that overlap on the GPU race.
 * ---------------------------------------------------------------------- */
#define LGB_NOALLOC_SCRATCH_BYTES (16u << 20)
int lgb_dft2_noalloc(const lgb_c128* f, int m, int n, lgb_c128* F, int M, int N,
                     double alpha_r, double alpha_c, double shift_r, double shift_c,
                     double offset_r, double offset_c, int unitary, lgb_stream stream);

/* ------------------------------------------------------------------------
 * Inverse MFT.  Replaces lentil/fourier.py:124-198 (idft2):
 *   f = conj(dft2(conj(F), alpha, shape, shift, unitary)) / F.size
 * F is m x n, f is M x N.  Workspace: lgb_idft2_workspace_size bytes.
 * ---------------------------------------------------------------------- */
size_t lgb_idft2_workspace_size(int m, int n, int M, int N, int precision);
int lgb_idft2(const lgb_c128* F, int m, int n, lgb_c128* f, int M, int N,
              double alpha_r, double alpha_c, double shift_r, double shift_c,
              int unitary, int precision, void* workspace, size_t workspace_bytes,
              lgb_stream stream);

/* ------------------------------------------------------------------------
 * Plane phasor.  Replaces the per-slice phasor of Plane.__mul__,
 * lentil/plane.py:502-507:
 *   out[i, j] = amp[r0+i, c0+j] * mask[r0+i, c0+j]
 *               * exp(2 pi i opd[r0+i, c0+j] / wavelength),   i < m, j < n
 * amp, mask, opd are H x W float64; a NULL amp / opd means the scalar
 * amp_value / opd_value (lentil's size-1 planes); a NULL mask means 1.
 * ---------------------------------------------------------------------- */
int lgb_phasor(const double* amp, double amp_value, const double* mask,
               const double* opd, double opd_value, int H, int W,
               int r0, int c0, int m, int n, double wavelength,
               lgb_c128* out, lgb_stream stream);

/* ------------------------------------------------------------------------
 * Field overlap-add.  Replaces lentil/field.py:231-305 (insert): the
 * fm x fn field whose centre sits at offset (off_r, off_c) from the centre
 * of the om x on output is added, clipped to the output, as
 *   intensity == 0 :  out += weight * f              (out complex128)
 *   intensity != 0 :  out += weight * |f|^2          (out float64)
 * ---------------------------------------------------------------------- */
int lgb_field_insert(const lgb_c128* f, int fm, int fn, int64_t off_r, int64_t off_c,
                     void* out, int om, int on, double weight, int intensity,
                     lgb_stream stream);

/* ------------------------------------------------------------------------
 * Field product over an intersection.  Replaces the data product of
 * Field._mul_array, lentil/field.py:130-147 (slices from the host-side
 * extent algebra of lentil/extent.py:127-150):
 *   out[i, j] = a[ar0+i, ac0+j] * b[br0+i, bc0+j],  i < om, j < on
 * A size-1 operand (lentil's broadcast, lentil/field.py:464-484) is passed
 * with lda == 0 (its single element is used everywhere).
 * ---------------------------------------------------------------------- */
int lgb_field_multiply(const lgb_c128* a, int lda, int ar0, int ac0,
                       const lgb_c128* b, int ldb, int br0, int bc0,
                       lgb_c128* out, int om, int on, lgb_stream stream);

/* ------------------------------------------------------------------------
 * Detector pixel MTF.  Replaces lentil/detector.py:167-222 (pixel):
 *   out = |ifft2(fft2(img) * outer(s, s))|,  s = sinc(fftfreq(N) * os),
 * evaluated as |C . img . C^T| with C the real circulant of ifft(s) (FP64).
 * img and out are N x N float64 (lentil defines it for square images only;
 * rows != cols -> LGB_EINVAL).  Workspace: lgb_pixel_workspace_size bytes.
 * ---------------------------------------------------------------------- */
size_t lgb_pixel_workspace_size(int N, int oversample);
int lgb_pixel(const double* img, int rows, int cols, int oversample, double* out,
              void* workspace, size_t workspace_bytes, lgb_stream stream);

/* ------------------------------------------------------------------------
 * Pixelation.  Replaces lentil/detector.py:225-251 (pixelate = pixel, then
 * lentil/util.py:261-349 rescale(1/os, order=3, mode='nearest',
 * unitary=True)).  out is S x S with S = lgb_pixelate_size(N, os) =
 * ceil(N * (1/os)) (lentil/util.py:323-324).  When every resample point is
 * a grid point (N a multiple of os) out = p[::os, ::os] * sum(p)/sum(that),
 * zero where the sample is zero; otherwise the cubic B-spline resampling
 * of scipy.ndimage.map_coordinates(order=3, mode='nearest') folded into one
 * banded FP64 operator per axis, out = G . p . G^T, then the same unitary
 * scale and lentil's linearly interpolated nonzero mask (util.py:333-347).
 * ---------------------------------------------------------------------- */
int lgb_pixelate_size(int N, int oversample);
int lgb_pixelate(const double* img, int rows, int cols, int oversample, double* out,
                 void* workspace, size_t workspace_bytes, lgb_stream stream);

/* ------------------------------------------------------------------------
 * Plane.fit_tilt (lentil/plane.py:522-611) without forming ptt_vector.
 * opd: [H][W]; mask: [S][H][W] (S masks; S = 1 for a 2-D mask), float64.
 * lgb_ptt_normal writes, per mask s, the normal equations of lentil's
 * least-squares fit in the basis b = [1, r*ps_r, -c*ps_c] (r, c centred
 * mesh, lentil/helper.py:7-17):
 *   out[9s .. 9s+8] = {A00 A01 A02 A11 A12 A22 y0 y1 y2},
 *   A = sum m^2 b b^T, y = sum m b opd  (deterministic FP64 sums);
 * workspace: lgb_ptt_normal_workspace_size(S) bytes.
 * lgb_remove_tilt, given t[3s..3s+2] = (piston, x, y) of every mask, writes
 * lentil's tilt-free OPD: S == 1: opd - m (t1 r ps_r - t2 c ps_c);
 * S > 1: sum_s (opd - m_s (t_s1 r ps_r - t_s2 c ps_c)) m_s.
 * ---------------------------------------------------------------------- */
size_t lgb_ptt_normal_workspace_size(int S);
int lgb_ptt_normal(const double* opd, const double* mask, int S, int H, int W, double ps_r,
                   double ps_c, double* out, void* workspace, size_t workspace_bytes,
                   lgb_stream stream);
int lgb_remove_tilt(const double* opd, const double* mask, int S, int H, int W, double ps_r,
                    double ps_c, const double* t, double* out, lgb_stream stream);

/* ------------------------------------------------------------------------
 * power_spectrum (lentil/wfe.py:8-70): white noise (N x N, the caller's
 * seeded normals) filtered by the Sidick PSD 1 / (1 + (f/f0)^exponent),
 * times sqrt(N*N) and the mask, rescaled to `rms` over its nonzero pixels.
 * lentil's grid makes this defined for square planes only.  N a power of
 * two (<= 8192): FP64 radix-2 FFTs; other N: FP64 DFT matrices.
 * workspace: lgb_power_spectrum_workspace_size(N) bytes.
 * ---------------------------------------------------------------------- */
size_t lgb_power_spectrum_workspace_size(int N);
int lgb_power_spectrum(const double* noise, const double* mask, int N, double pixelscale,
                       double rms, double half_power_freq, double exponent, double* out,
                       void* workspace, size_t workspace_bytes, lgb_stream stream);

/* ------------------------------------------------------------------------
 * Zernike generators (lentil/zernike.py:11-234, 444-480).  mask: [H][W]
 * float64, nonzero = inside.
 * lgb_zernike_coordinates: rho, theta of lentil's zernike_coordinates; the
 * origin is the mask centroid when auto_shift != 0 (one 24-byte read back
 * to the host), else (shift_r, shift_c) pixels from the centre; rotate in
 * degrees.  workspace: lgb_zernike_workspace_size() bytes.
 * lgb_zernike_eval: table (device, K rows of 3 + 2T doubles) =
 *   [m, scale, nterms, (coef, power) x T]; out = sum_j scale_j R_j(rho)
 *   ang_j(theta) mask (basis == 0, [H][W]) or every term ([K][H][W]);
 *   ang = cos(m theta) for m > 0, sin(m theta) for m < 0, 1 for m == 0.
 * ---------------------------------------------------------------------- */
size_t lgb_zernike_workspace_size(void);
int lgb_zernike_coordinates(const double* mask, int H, int W, int auto_shift, double shift_r,
                            double shift_c, double rotate, double* rho, double* theta,
                            void* workspace, size_t workspace_bytes, lgb_stream stream);
int lgb_zernike_eval(const double* rho, const double* theta, const double* mask, size_t count,
                     const double* table, int K, int T, double* out, int basis,
                     lgb_stream stream);

/* ------------------------------------------------------------------------
 * Gradient building blocks (no counterpart in lentil, which has no
 * gradients; they make the MFT path differentiable for phase retrieval).
 * For I = |F|^2 with F = dft2(f), f = amp exp(2 pi i opd / lambda):
 *   lgb_abs2:              I = |F|^2                               (count)
 *   lgb_intensity_adjoint: Hc = dL/dI * conj(F)  (conjugate of dL/dF*)
 *   then q = dft2(Hc, alpha, shape=(m, n), shift=-offset, offset=-shift)
 *   (the adjoint MFT: E1^T conj(H) E2^T), and
 *   lgb_phasor_adjoint:    grad_opd[r0+i, c0+j] += -(4 pi / lambda) Im(q f)
 * ---------------------------------------------------------------------- */
int lgb_abs2(const lgb_c128* F, double* I, size_t count, lgb_stream stream);
int lgb_intensity_adjoint(const lgb_c128* F, const double* grad_I, lgb_c128* Hc, size_t count,
                          lgb_stream stream);
int lgb_phasor_adjoint(const lgb_c128* q, const lgb_c128* f, int m, int n, double wavelength,
                       double* grad_opd, int ld, int r0, int c0, lgb_stream stream);
/* Modal OPD for phase retrieval: out[p] = sum_k coeffs[k] basis[k][p] and
 * its adjoint out[k] = sum_p basis[k][p] grad[p] (deterministic sums), with
 * an FP32 basis [K][P] (K <= 1024): both stream the basis once.  Workspace of
 * the adjoint: lgb_basis_project_workspace_size(K) bytes. */
int lgb_basis_expand(const float* basis, const double* coeffs, int K, size_t P, double* out,
                     lgb_stream stream);
size_t lgb_basis_project_workspace_size(int K);
int lgb_basis_project(const float* basis, const double* grad, int K, size_t P, double* out,
                      void* workspace, size_t workspace_bytes, lgb_stream stream);
/* The same over `count` planes at once (focus-diverse images):
 * out[i][p] = sum_k coeffs[k] basis[k][p] + add[i][p] (add may be NULL), and
 * out[k] = sum_p basis[k][p] sum_i grad[i][p]. */
int lgb_basis_expand_stack(const float* basis, const double* coeffs, int K, size_t P,
                           const double* add, int count, double* out, lgb_stream stream);
int lgb_basis_project_stack(const float* basis, const double* grad, int count, int K, size_t P,
                            double* out, void* workspace, size_t workspace_bytes,
                            lgb_stream stream);
/* Squared-error loss of phase retrieval: *loss = sum_p (I[p] - T[p])^2
 * (FP64, fixed-order reduction, written on the device; workspace
 * lgb_sq_error_workspace_size() bytes) and its gradient dI[p] =
 * 2 (I[p] - T[p]) * (*dL) with dL a device scalar (n == 0: *loss = 0, and
 * I, T, dI may be null). */
size_t lgb_sq_error_workspace_size(void);
int lgb_sq_error(const double* I, const double* T, size_t n, double* loss, void* workspace,
                 size_t workspace_bytes, lgb_stream stream);
int lgb_sq_error_grad(const double* I, const double* T, size_t n, const double* dL, double* dI,
                      lgb_stream stream);
/* K phasors amp * exp(2 pi i opd[k] / wavelength) over the slice (r0, c0,
 * m, n) of H x W planes, out[K][m][n], in one launch.  fast != 0 evaluates
 * the phase in float-float and the sine in FP32 (about 1e-7 relative, for
 * the split-precision transforms); fast == 0 matches lgb_phasor. */
int lgb_phasor_stack(const double* amp, const double* opd, int K, int H, int W, int r0, int c0,
                     int m, int n, double wavelength, int fast, lgb_c128* out,
                     lgb_stream stream);

/* ------------------------------------------------------------------------
 * Broadband PSF plan: the documented user loop
 *   for lam, w: img = propagate_dft(Wavefront(lam) * pupil, ...).insert(img, w)
 * (docs/user/performance.rst:44-49) fused for a batch of PSFs that share the
 * optics: phasor (lentil/plane.py:502-507), propagate_dft's MFT into its
 * output window (lentil/propagate.py:147-242 with lentil/fourier.py:5-103),
 * and the weighted |E|^2 overlap-add of Wavefront.insert
 * (lentil/wavefront.py:145-165, lentil/field.py:231-305).
 *
 * A plan owns device memory: the DFT matrices of every wavelength (built at
 * creation, resident until destroyed) and the per-execute intermediates for
 * `batch` PSFs.  One field per PSF: the pupil slice rows [r0, r0+m), cols
 * [c0, c0+n) with lentil's slice offset; all wavelengths land in the same
 * M x N window at (win_r0, win_c0) of the out_rows x out_cols image.
 * ---------------------------------------------------------------------- */
typedef struct lgb_psf_plan_s* lgb_psf_plan;

typedef struct {
  int H, W;                   /* pupil plane shape */
  int r0, c0, m, n;           /* field slice of the pupil plane */
  double offset_r, offset_c;  /* field offset from the plane centre */
  int M, N;                   /* MFT output window shape */
  int out_rows, out_cols;     /* output image shape */
  int win_r0, win_c0;         /* window's first row/col inside the image */
  int n_wavelengths;          /* L */
  const double* wavelengths;  /* host [L], metres */
  const double* alpha_r;      /* host [L], lentil/propagate.py:121-123 */
  const double* alpha_c;      /* host [L] */
  const double* shift_r;      /* host [L], output-pixel shift of the DC */
  const double* shift_c;      /* host [L] */
  int batch;                  /* PSFs per execute (0: matrices only, see lgb_psf_execute_ws) */
  int precision;              /* LGB_FP64 / LGB_SPLIT_BF16 / LGB_SPLIT_FP16 */
} lgb_psf_desc;

int lgb_psf_plan_create(const lgb_psf_desc* desc, lgb_psf_plan* plan, lgb_stream stream);
/* The same plan in caller-owned device memory of lgb_psf_plan_size(desc)
 * bytes (256-byte aligned; 0 for an invalid desc), e.g. a block of the
 * caller's caching allocator, so that building a plan maps no new device
 * memory once the caller holds a block that size.  lgb_psf_plan_destroy
 * leaves that memory alone: the caller keeps it alive until the plan's
 * executes are done. */
size_t lgb_psf_plan_size(const lgb_psf_desc* desc);
int lgb_psf_plan_create_in(const lgb_psf_desc* desc, void* memory, size_t memory_bytes,
                           lgb_psf_plan* plan, lgb_stream stream);
/* device bytes held by the plan */
size_t lgb_psf_plan_bytes(lgb_psf_plan plan);
/* amp, opd: [batch][H][W] float64 (amp already multiplied by the mask);
 * weights: [batch][L] float64; out: [batch][out_rows][out_cols] float64.
 * out is overwritten (accumulate == 0) or added to (accumulate != 0). */
int lgb_psf_execute(lgb_psf_plan plan, const double* amp, const double* opd,
                    const double* weights, double* out, int accumulate, lgb_stream stream);
/* As lgb_psf_execute for the first `count` (1..batch) PSFs of the arrays. */
int lgb_psf_execute_batch(lgb_psf_plan plan, int count, const double* amp, const double* opd,
                          const double* weights, double* out, int accumulate, lgb_stream stream);
/* As lgb_psf_execute_batch over a subset of the plan's wavelengths:
 * lam_idx (device int32 [n_sel]) picks the plan wavelengths used; weights is
 * [count][n_sel].  The plan's DFT matrices serve every subset, so a plan
 * built on a spectral grid is a device-resident DFT-matrix cache for
 * requests with any wavelengths of that grid.  Split-precision plans only. */
int lgb_psf_execute_subset(lgb_psf_plan plan, int count, const int* lam_idx, int n_sel,
                           const double* amp, const double* opd, const double* weights,
                           double* out, int accumulate, lgb_stream stream);
/* Caller-workspace execute: a plan created with batch == 0 holds only its
 * DFT matrices; every execute then takes its per-launch operands (f^T, G,
 * intensity window, status word) from `workspace`
 * (lgb_psf_execute_workspace_size(plan, count, n_sel) bytes, 256-byte
 * aligned), so one plan may run on several streams at once.  lam_idx may be
 * NULL (all wavelengths; n_sel ignored).  lgb_dft2_status(workspace, stream)
 * reports the device status of the launch.  Split-precision plans only. */
size_t lgb_psf_execute_workspace_size(lgb_psf_plan plan, int count, int n_sel);
int lgb_psf_execute_ws(lgb_psf_plan plan, int count, const int* lam_idx, int n_sel,
                       const double* amp, const double* opd, const double* weights, double* out,
                       int accumulate, void* workspace, size_t workspace_bytes, lgb_stream stream);
/* Device-side status of the plan's last execute; waits for the stream. */
int lgb_psf_plan_status(lgb_psf_plan plan, lgb_stream stream);
/* Optional per-kernel timing of lgb_psf_execute: while enabled, each launch
 * is bracketed by CUDA events on the execute stream; lgb_psf_plan_kernel_times
 * waits for them and returns (and resets) the summed milliseconds and launch
 * counts per slot: phasor, stage-1 MFT, stage-2 MFT, other. */
#define LGB_PROFILE_PHASOR 0
#define LGB_PROFILE_MFT1 1
#define LGB_PROFILE_MFT2 2
#define LGB_PROFILE_OTHER 3
#define LGB_PROFILE_SLOTS 4
int lgb_psf_plan_profile(lgb_psf_plan plan, int enable);
/* Pair-tile width of the plan's split launches: 0 (default) = the
 * autotuner's choice (lgb_tuner_*), 256 or 128 = that width.  A caller that
 * runs several executes at once (a server with launches in flight on other
 * streams) sets 256, the width with the best MMA throughput per SM, since
 * the narrower tile only pays when pairs would otherwise idle.  Read when an
 * execute is issued. */
int lgb_psf_plan_set_tile(lgb_psf_plan plan, int tile);
int lgb_psf_plan_kernel_times(lgb_psf_plan plan, double* ms, int* launches, int n);
/* Releases the plan's memory (stream-ordered on the creation stream); call
 * it after the plan's last execute has completed. */
int lgb_psf_plan_destroy(lgb_psf_plan plan);

/* ------------------------------------------------------------------------
 * Test of the tensor-core MFT's bounded waits (no lentil counterpart).  Every
 * mbarrier wait of the split-precision kernel is bounded in time; on expiry
 * the kernel records LGB_ETIMEOUT in the entry's device status word, retires
 * the copies and MMAs it issued and returns, and the entry's status call
 * (lgb_dft2_status, lgb_dft2_plan_status, lgb_psf_plan_status) reports it.
 * This one-shot hook makes the NEXT stage-1 split launch of the process (any
 * entry, any thread) arrive on the full barrier of K block `kblock` of work
 * item `item` without issuing that block's loads, so the barrier never
 * completes, and bounds every wait of that launch by wait_ms (0 < wait_ms
 * <= 2000) instead of the default 2 s.  The launch then runs out, reports
 * LGB_ETIMEOUT, and later launches run normally.
 * ---------------------------------------------------------------------- */
int lgb_test_stall_tma(int item, int kblock, double wait_ms);

/* ------------------------------------------------------------------------
 * Tile-shape autotuner of the split-precision MFT (extension: lentil has no
 * GPU path).  Every split launch (lgb_dft2/_batch/idft2 and plan executes)
 * runs its CTA-pair tiles 256 or 128 output columns wide.  The width is
 * chosen per launch class -- precision, m, n, M, N, epilogue and the
 * occupancy of the problem count (waves of 128-wide tiles per stage over the
 * resident CTA pairs, capped at 8) -- and cached for the process:
 *   LGB_TUNE_MEASURE (default): tuned online on the caller's own launches.
 *     The first launch of a class runs the occupancy model's width, the
 *     second the other width, each bracketed by CUDA events on its stream;
 *     a later launch that finds both finished (cudaEventQuery, no host wait)
 *     caches the faster.  Nothing is relaunched or synchronised.  Launches
 *     under stream capture use the cached or model width and time nothing.
 *   LGB_TUNE_MODEL: the occupancy model decides at once.
 * lgb_tuner_force_tile(256 | 128) makes every launch use that width (0: off).
 * lgb_tuner_entries counts decided classes; lgb_tuner_lookup returns the
 * decided width of the class of (m, n, M, N, count = PSFs x wavelengths,
 * precision, epilogue 0 = intensity / 1 = complex field) or 0;
 * lgb_tuner_last_tile the width of this thread's last split launch. */
#define LGB_TUNE_MODEL 0
#define LGB_TUNE_MEASURE 1
int lgb_tuner_set_mode(int mode);
int lgb_tuner_force_tile(int tile);
void lgb_tuner_clear(void);
int lgb_tuner_entries(void);
int lgb_tuner_lookup(int m, int n, int M, int N, int count, int precision, int epilogue);
int lgb_tuner_last_tile(void);
/* Decided classes as rows of 9 ints (the class key -- bf16, m, n, M, N,
 * epilogue, waves of stage 1, waves of stage 2 -- then the width), for a
 * cache file: export writes up to max_rows rows and returns how many classes
 * are decided; import adds rows as decided classes (widths 128 or 256). */
int lgb_tuner_export(int* rows, int max_rows);
int lgb_tuner_import(const int* rows, int n);

#ifdef __cplusplus
}
#endif

#endif /* LENTIL_GB300_H */
