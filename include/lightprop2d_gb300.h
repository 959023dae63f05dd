/*
 * lightprop2d_gb300.h -- C ABI of the GB300 (sm_103a) angular-spectrum backend.
 *
 * Every entry point maps one operation of lightprop2d's Beam2D
 * (lightprop2d/beam2d.py, version 1.0.4) onto hand-written CUDA kernels.
 *
 *   - All array arguments are DEVICE pointers to row-major N x N grids,
 *     index [iy * N + ix], iy <-> Y (rows), ix <-> X (columns), exactly the
 *     layout of Beam2D.field / Beam2D.spectrum (beam2d.py:299-308).
 *   - Complex data is interleaved complex64 (numpy / torch complex64 layout).
 *   - Spectra use the unshifted fftfreq order (DC at index 0).
 *   - Lengths are in centimetres, like the reference (beam2d.py:37-41).
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     asynchronous with respect to the host; results are ready once the
 *     stream reaches them.
 *   - Ownership: the caller owns every buffer passed in.  The transforms keep
 *     their intermediates in the caller's output grid, so the fused paths
 *     allocate nothing; the library keeps per-device twiddle tables (static
 *     device arrays) and, for the unfused comparison path only, a
 *     per-(device, stream) H grid that lp_workspace_release() frees.
 *   - Errors: every call returns an lp_status; no exception crosses the ABI.
 *     lp_last_error() returns a thread-local message for the last failure.
 *   - Supported N: powers of two from 16 to 8192.  Other N return
 *     LP_ERR_UNSUPPORTED_SIZE (the reference accepts any N through numpy).
 *   - Pointers must be 8-byte aligned (complex64); N >= 16 keeps every row
 *     16-byte aligned when the base pointer is.
 */
#ifndef LIGHTPROP2D_GB300_H
#define LIGHTPROP2D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LP_ABI_VERSION 1

typedef struct lp_cfloat {
  float re;
  float im;
} lp_cfloat;

/* complex128, numpy / torch layout (re, im interleaved), 16-byte aligned. */
typedef struct lp_cdouble {
  double re;
  double im;
} lp_cdouble;

typedef enum lp_status {
  LP_OK = 0,
  LP_ERR_INVALID_ARGUMENT = 1,  /* null pointer, bad dtype code, non-finite scalar */
  LP_ERR_UNSUPPORTED_SIZE = 2,  /* N not a power of two in [16, 8192] */
  LP_ERR_MISALIGNED = 3,        /* pointer not 8-byte aligned */
  LP_ERR_CUDA = 4,              /* a CUDA runtime call failed (see lp_last_error) */
  LP_ERR_OUT_OF_MEMORY = 5,     /* scratch allocation failed */
  LP_ERR_NOT_INITIALIZED = 6,   /* first use on a device inside stream capture */
  LP_ERR_TIMEOUT = 7,           /* a bounded device-side wait gave up (batched queue) */
  LP_ERR_INTERNAL = 8
} lp_status;

/* Element type of an optional mask argument. */
typedef enum lp_mask_type {
  LP_MASK_NONE = 0,
  LP_MASK_F32 = 1,        /* real float32 multiplier */
  LP_MASK_C64 = 2,        /* complex64 multiplier */
  LP_MASK_U8 = 3,         /* bool / uint8 (0 or 1) */
  LP_MASK_PHASE_F32 = 4,  /* float32 phase phi in radians: multiplier exp(i*phi) */
  LP_MASK_F64 = 5,        /* real float64 multiplier (numpy default dtype) */
  LP_MASK_C128 = 6,       /* complex128 multiplier, rounded to complex64 */
  /* Compact profile generators, evaluated inside the pass that applies them
   * (no N x N mask in memory).  The pointer is a device array of 2*N values:
   *   LP_MASK_SEP_F32:  float32 fx[N], fy[N];  multiplier fx[ix] * fy[iy]
   *                     (separable profiles: gaussian_beam, rectangle_hole,
   *                     square_hole, square_slits, plane_wave)
   *   LP_MASK_SPAN_I32: int32 lo[N], hi[N];    multiplier 1 if lo[ix] <= iy < hi[ix]
   *                     else 0 (round_hole); x-domain masks only.
   *   LP_MASK_SEP_C64:  complex64 fx[N], fy[N]; multiplier fx[ix] * fy[iy]
   *                     (separable complex multipliers; the chirp kernels of
   *                     the transforms for sizes that are not powers of two)
   * The host builds the tables with the reference's own float64 arithmetic
   * (lightprop2d_gb300/generators.py), so boolean edges match it exactly. */
  LP_MASK_SEP_F32 = 7,
  LP_MASK_SPAN_I32 = 8,
  LP_MASK_SEP_C64 = 9,
  LP_MASK_SEP_C128 = 10   /* complex128 fx[N], fy[N] (the *_c128 entry points only) */
} lp_mask_type;

/* Flags (bitwise OR). */
#define LP_FLAG_PHASE_FP32 0x1u         /* transfer phase kz*z in plain FP32 (comparison variant) */
#define LP_FLAG_EVANESCENT_MASK 0x2u    /* H = 0 where kx^2+ky^2 > k0^2 (reference: H = 1) */
#define LP_FLAG_ADJOINT 0x4u            /* conjugate every multiplier: the adjoint operator */
#define LP_FLAG_SPECTRUM_READONLY 0x8u  /* lp_propagate: do not write spectrum*H back */
#define LP_FLAG_DZ 0x10u                /* multiply the spectrum by -2*pi*i*kz as well (d/dz) */
#define LP_FLAG_XMASK_AFTER 0x20u       /* lp_propagate_field: apply lens/xmask after the
                                           inverse transform (propagate, then screen) */

/* ---------------------------------------------------------------- meta -- */
int lp_abi_version(void);
const char* lp_last_error(void);
const char* lp_status_string(int status);
/* 1 when N is supported, else 0. */
int lp_is_supported_n(int n);
/* One-time per-device set-up (twiddle tables).  Called implicitly by the
 * first entry point on a device; call it explicitly before capturing any of
 * these calls into a CUDA graph. */
lp_status lp_init(int device);
/* Frees every cached scratch grid (all devices and streams). */
lp_status lp_workspace_release(void);
/* Measurement hook (no counterpart in the reference): until called again with
 * count = 0, lp_propagate_field and lp_propagate record the caller's CUDA
 * events (cudaEvent_t, created on the current device) on their stream at the
 * pass boundaries of each call: events[0] before the first pass and
 * events[i] after pass i (3 passes for lp_propagate_field, 2 for
 * lp_propagate).  Thread-local. */
lp_status lp_profile_events(void** events, int count);
/* Tuning hook (no counterpart in the reference): resident CTAs per SM for the
 * persistent row (kind 0) or column (kind 1) kernels of size n; value 0
 * restores the built-in choice (as many as fit).  The TMA-staged row kernels
 * (n = 4096, 16-byte aligned input) always run one CTA per SM and ignore
 * kind 0.  Returns the count now in effect, or -1 for a bad n / kind.
 * Process-wide; set by the autotuner (lightprop2d_gb300.tune). */
int lp_tune_ctas_per_sm(int n, int kind, int value);
/* Health check (no counterpart in the reference): synchronises `stream` and
 * returns LP_ERR_TIMEOUT if a bounded device-side wait of any pass kernel
 * (a TMA copy that never landed) gave up since the last call, clearing the
 * record; LP_OK otherwise.  The pass kernels never hang: a wait that runs
 * out of iterations records the error and the kernel finishes. */
lp_status lp_async_status(void* stream);

/* ------------------------------------------------------------ transforms --
 * numpy convention: forward unnormalised, inverse scaled by 1/N^2.
 * Replaces Beam2D._fft2 / Beam2D._ifft2 (beam2d.py:207-229).
 * in == out is allowed. */
lp_status lp_fft2(const lp_cfloat* in, lp_cfloat* out, int n, int inverse,
                  void* stream);

/* -------------------------------------------------------------- propagate --
 * Beam2D.propagate(z) (beam2d.py:462-490) on the stored spectrum:
 *     spectrum *= kmask * H(z)         (written back unless SPECTRUM_READONLY)
 *     field     = ifft2(spectrum)
 * with H(z) = exp(-2*pi*i * kz * z), kz = sqrt(k0^2 - kx^2 - ky^2), k0 = 1/wl,
 * kx = fftfreq(N, area_size/N).  The phase kz*z is reduced mod 1 cycle with
 * ~48-bit (float-float) arithmetic, then exp() is taken in FP32.  Evanescent
 * points pass through (H = 1) as in the reference, unless EVANESCENT_MASK.
 * z == 0 is allowed here (H = 1); Beam2D.propagate(0) returns before calling.
 * kmask is optional (LP_MASK_NONE): Beam2D.spectral_filter (beam2d.py:366-373)
 * is this call with z = 0.  spectrum and field must be different grids. */
lp_status lp_propagate(lp_cfloat* spectrum, lp_cfloat* field, int n,
                       double area_size, double wl, double z,
                       const void* kmask, int kmask_type, uint32_t flags,
                       void* stream);

/* Fused field -> field step, one pass over HBM in and one out:
 *     u        = field_in * L(lens_f) * xmask          (x domain)
 *     S        = fft2(u) * kmask * H(z)                 (k domain, in registers)
 *     field_out= ifft2(S)        [optional: spectrum_out = S, iprofile = |field_out|^2]
 * It is Beam2D.lens(f) (beam2d.py:508-511) + coordinate_filter(f_init)
 * (:339-342) + spectral_filter(f_init) (:370-373) + propagate(z) (:484-490)
 * in one launch sequence with no intermediate field or H array in HBM.
 * lens_f == 0 means no lens.  field_in == field_out is allowed;
 * spectrum_out must differ from field_out.  Any of spectrum_out /
 * iprofile_out may be NULL.  LP_FLAG_XMASK_AFTER moves the x-domain
 * multiplier after the inverse transform (field_out = m * P(field_in)).
 * With LP_FLAG_ADJOINT the call applies the adjoint operator: conj(kmask*H)
 * in the k domain and conj(lens*xmask) on the opposite side of the
 * transforms. */
lp_status lp_propagate_field(const lp_cfloat* field_in, lp_cfloat* field_out,
                             lp_cfloat* spectrum_out, float* iprofile_out,
                             int n, double area_size, double wl, double z,
                             double lens_f, const void* xmask, int xmask_type,
                             const void* kmask, int kmask_type, uint32_t flags,
                             void* stream);

/* ------------------------------------------------------------- operators -- */
/* Beam2D.lens(f) (beam2d.py:508-511): field *= exp(i*(X^2+Y^2)*k0/(2f));
 * spectrum_out = fft2(field) (NULL: skip the transform). */
lp_status lp_lens(lp_cfloat* field, lp_cfloat* spectrum_out, int n,
                  double area_size, double wl, double f, void* stream);

/* Beam2D.coordinate_filter(f_init=mask) (beam2d.py:339-342):
 * field *= mask; spectrum_out = fft2(field) (NULL: skip the transform). */
lp_status lp_coordinate_filter(lp_cfloat* field, lp_cfloat* spectrum_out,
                               int n, const void* mask, int mask_type,
                               void* stream);

/* Beam2D.spectral_filter(f_init=mask) (beam2d.py:370-373):
 * spectrum *= mask; field_out = ifft2(spectrum). */
lp_status lp_spectral_filter(lp_cfloat* spectrum, lp_cfloat* field_out, int n,
                             const void* mask, int mask_type, void* stream);

/* Beam2D.iprofile (beam2d.py:717): out = |field|^2 as float32. */
lp_status lp_iprofile(const lp_cfloat* field, float* out, int n, void* stream);

/* ---- complex128 (complex_bits=128, the reference's default dtype,
 * beam2d.py:88, :112-113) ----
 * The same operations with complex128 grids (16-byte aligned).  Transforms
 * run in float-float arithmetic (48 significant bits) on the FP32 pipes;
 * the transfer function's Kz and phase and the lens phase are the
 * reference's float64 expressions (beam2d.py:305-308, :485-489, :508-510),
 * so results agree with its numpy complex128 path to ~1e-14 relative.
 * Values keep that precision for magnitudes in ~[1e-30, 1e30] (FP32's
 * exponent range, allowing for the N^2 gain of a transform); magnitudes
 * below 2^-126 flush to zero.  Masks: any lp_mask_type (LP_MASK_SEP_C128
 * included), promoted to complex128.  Flags: LP_FLAG_EVANESCENT_MASK, and
 * LP_FLAG_SPECTRUM_READONLY for lp_propagate_c128.  npoints as for the
 * complex64 entry points.  The first call of a size on a device builds
 * tables (and, for sizes that are not powers of two, a per-stream work grid)
 * and is refused inside stream capture (LP_ERR_NOT_INITIALIZED). */

/* lp_fft2 in complex128 (beam2d.py:207-229). */
lp_status lp_fft2_c128(const lp_cdouble* in, lp_cdouble* out, int n, int inverse,
                       void* stream);

/* Beam2D.propagate (beam2d.py:462-490) in complex128: spectrum *= H(z) *
 * kmask (unless LP_FLAG_SPECTRUM_READONLY); field = ifft2(spectrum). */
lp_status lp_propagate_c128(lp_cdouble* spectrum, lp_cdouble* field, int n, double area_size,
                            double wl, double z, const void* kmask, int kmask_type,
                            uint32_t flags, void* stream);

/* lp_propagate_field in complex128: [lens, xmask] -> fft2 -> [kmask] * H(z)
 * (spectrum_out optional) -> ifft2 -> iprofile_out (float64, optional). */
lp_status lp_propagate_field_c128(const lp_cdouble* field_in, lp_cdouble* field_out,
                                  lp_cdouble* spectrum_out, double* iprofile_out, int n,
                                  double area_size, double wl, double z, double lens_f,
                                  const void* xmask, int xmask_type, const void* kmask,
                                  int kmask_type, uint32_t flags, void* stream);

/* Beam2D.lens (beam2d.py:492-511) in complex128. */
lp_status lp_lens_c128(lp_cdouble* field, lp_cdouble* spectrum_out, int n, double area_size,
                       double wl, double f, void* stream);

/* Beam2D.coordinate_filter (beam2d.py:310-342) in complex128. */
lp_status lp_coordinate_filter_c128(lp_cdouble* field, lp_cdouble* spectrum_out, int n,
                                    const void* mask, int mask_type, void* stream);

/* Beam2D.spectral_filter (beam2d.py:344-373) in complex128. */
lp_status lp_spectral_filter_c128(lp_cdouble* spectrum, lp_cdouble* field_out, int n,
                                  const void* mask, int mask_type, void* stream);

/* spectrum *= H(z) in complex128 (the propagate phase of beam2d.py:485-489). */
lp_status lp_apply_transfer_c128(lp_cdouble* spectrum, int n, double area_size, double wl,
                                 double z, uint32_t flags, void* stream);

/* Beam2D.iprofile (beam2d.py:717) of a complex128 field: float64. */
lp_status lp_iprofile_c128(const lp_cdouble* field, double* out, int n, void* stream);
/* Intensity moments for Beam2D.centroid / D4sigma / centroid_intensity
 * (beam2d.py:669-752).  Writes 5 doubles to device memory `moments`, with
 * I = |field|^2, jx = ix - n/2, jy = iy - n/2 (grid-index offsets):
 *   [0] sum I   [1] sum jx*I   [2] sum jy*I
 *   [3] sum (jx - xc)^2 I   [4] sum (jy - yc)^2 I,   xc = [1]/[0], yc = [2]/[0]
 * so Xc = dL*[1]/[0], D4sigma_x = 4*dL*sqrt([3]/[0]).  One read pass (FP32
 * run sums about each thread's own first row, moved to the grid centre in
 * FP64) and a one-thread finish that takes the second moments about the
 * centroid, like the reference; n even; asynchronous. */
lp_status lp_beam_moments(const lp_cfloat* field, int n, double* moments, void* stream);
/* Intensity loss of the differentiable design workload (no reference
 * counterpart: the inverse-design loop built on propagate, beam2d.py:462-490).
 * Forward: *loss_sum = sum_i (|y_i|^2 - target_i)^2 over `count` points, in
 * FP64 (device memory, overwritten).  Backward (lp_intensity_mse_grad):
 * grad_y_i = (*upstream) * scale * (|y_i|^2 - target_i) * y_i, with `upstream`
 * a device float (the incoming gradient, read on the device so the call can
 * be captured in a CUDA graph) and scale = 4 / count for the mean. */
lp_status lp_intensity_mse(const lp_cfloat* y, const float* target, long long count,
                           double* loss_sum, void* stream);
lp_status lp_intensity_mse_grad(const lp_cfloat* y, const float* target, long long count,
                                const float* upstream, float scale, lp_cfloat* grad_y,
                                void* stream);
/* Gradient of a real loss with respect to an FP32 phase mask phi applied as
 * x -> x * exp(i*phi) (no reference counterpart: the backward of
 * coordinate_filter with a phase, beam2d.py:310-342, in the differentiable
 * workload): out_i = Im(conj(x_i) * g_i), with x the multiplied field and g
 * the gradient with respect to it, over `count` points. */
lp_status lp_phase_grad(const lp_cfloat* x, const lp_cfloat* g, long long count, float* out,
                        void* stream);

/* spectrum *= H(z) only (no transform): used to materialise a spectrum whose
 * propagation distance the caller kept pending. */
lp_status lp_apply_transfer(lp_cfloat* spectrum, int n, double area_size,
                            double wl, double z, uint32_t flags, void* stream);

/* ------------------------------------------------------- grid management --
 * One gather kernel each over the output grid (no spectrum: recompute it with
 * lp_fft2, as the reference does after each of these). */
/* Beam2D.expand (beam2d.py:375-404): out (n_out x n_out) is `in` padded by
 * (n_out - n_in)/2 points on every side, each pad point a copy of the nearest
 * edge point.  n_out >= n_in, even difference; in != out. */
lp_status lp_expand(const lp_cfloat* in, int n_in, lp_cfloat* out, int n_out, void* stream);
/* Beam2D.coarse (beam2d.py:434-460): out (n_in/order squared) is the mean of
 * each order x order block of `in`.  order divides n_in; in != out. */
lp_status lp_coarse(const lp_cfloat* in, int n_in, lp_cfloat* out, int order, void* stream);
/* Beam2D.crop (beam2d.py:406-432): resamples the central window
 * in[first .. first+n_keep)^2 (window axis coordinates x0 + k*dL_in) onto the
 * centred grid (j - n_out/2)*dL_out, j < n_out, by bilinear interpolation with
 * nearest-point values outside the window -- what the reference's
 * scipy.interpolate.interp2d(kind="linear") does; in != out.  Also serves
 * Beam2D.lens_image (beam2d.py:513-537), whose sample grid is the field grid
 * scaled by -l1/l2 (dL_out may then differ in sign from dL_in).  n_out <= 8192. */
lp_status lp_crop(const lp_cfloat* in, int n_in, int first, int n_keep, double x0, double dL_in,
                  lp_cfloat* out, int n_out, double dL_out, void* stream);

/* ------------------------------------------------------ mode decomposition --
 * The mode basis is n_modes x nb^2 complex64 (row m = mode m, flattened
 * row-major on an nb x nb grid), applied to the central nb x nb window of the
 * n x n field ((n - nb)/2 points in from each edge).  HBM-bound
 * matrix-vector products; coefficients are complex128 pairs in device memory. */
/* Beam2D.deconstruct_by_modes(mode="scalar") (beam2d.py:574-600):
 * coeffs[m] = sum_p modes[m][p] * window[p]  (no conjugation, as there). */
lp_status lp_modes_project(const lp_cfloat* modes, int n_modes, int nb, const lp_cfloat* field,
                           int n, double* coeffs, void* stream);
/* Beam2D.construct_by_modes (beam2d.py:650-667): field = sum_m coeffs[m]*mode_m
 * inside the window and 0 outside (the zero padding of _expand_basis,
 * beam2d.py:539-559). */
lp_status lp_modes_combine(const lp_cfloat* modes, int n_modes, int nb, const double* coeffs,
                           lp_cfloat* field, int n, void* stream);

/* ------------------------------------------------------------- batches --
 * Many beams of uneven grid sizes in ONE persistent launch.  Each beam runs
 * lens(lens_f) -> propagate(z) -> iprofile on its own grid, in place:
 *     field = ifft2( fft2(field * L) * H(z) ),  iprofile = |field|^2
 * (Beam2D.lens + Beam2D.propagate + Beam2D.iprofile per beam; no reference
 * counterpart for the batching itself).  Work items (beam, pass, tiles) are
 * pulled from a device queue by resident CTAs; a column pass waits, with a
 * bounded spin, on its beam's row pass (and so on).  Supported n: 64..4096.
 * lp_batch_run is one kernel launch that allocates nothing, so it can be
 * captured in a CUDA graph; the device counters reset themselves at the end of
 * every run. */
typedef struct lp_beam_desc {
  lp_cfloat* field;  /* n x n complex64, input and output (in place) */
  float* iprofile;   /* optional n x n float32 output |field|^2, or NULL */
  int n;
  double area_size, wl, z;
  double lens_f;     /* 0: no lens */
  uint32_t flags;    /* LP_FLAG_PHASE_FP32 | LP_FLAG_EVANESCENT_MASK */
  /* optional device array of 5 doubles, or NULL: every run sets it to the
   * intensity moments of the result (Beam2D.centroid / D4sigma,
   * beam2d.py:669-704) summed in the last pass's epilogue:
   * sum I, sum jx I, sum jy I, sum jx^2 I, sum jy^2 I, with jx = ix - n/2,
   * jy = iy - n/2 (raw moments about the grid centre; the second moments
   * about the centroid follow by subtraction) */
  double* moments;
} lp_beam_desc;

typedef struct lp_batch_options {
  int ctas_per_sm;          /* resident CTAs per SM; 0: as many as fit */
  int tiles_per_item;       /* tiles (4096 points each) per queue item; 0: 8 */
  int group_points_log2;    /* beams are scheduled in groups of ~2^k points; 0: 23 */
  long long spin_limit;     /* wait iterations (~200 ns each) before LP_ERR_TIMEOUT; 0: 2^22 */
  int debug_unsatisfiable;  /* test hook: one dependency that is never met, so the run
                               ends through the timeout path; 0 otherwise */
} lp_batch_options;

typedef struct lp_batch lp_batch;

/* Plans a batch: sorts beams (largest first), builds the work queue and
 * copies it to the device (this call allocates device memory). */
lp_status lp_batch_create(const lp_beam_desc* beams, int count,
                          const lp_batch_options* options, lp_batch** out);
/* One persistent launch over the whole batch on `stream`. */
lp_status lp_batch_run(lp_batch* batch, void* stream);
/* Synchronises `stream`, then reads and clears the batch's device error flag:
 * LP_OK, or LP_ERR_TIMEOUT when a bounded wait gave up during the last run. */
lp_status lp_batch_status(lp_batch* batch, void* stream);
/* Queue and launch shape: items, CTAs launched, resident CTAs per SM. */
lp_status lp_batch_info(const lp_batch* batch, int* n_items, int* grid,
                        int* ctas_per_sm);

/* The host part of lp_batch_create alone: checks the beams and builds the
 * work queue, with no CUDA call, so a rank can plan its shard of a beam list
 * (see batch.partition_beams) on any host.  Returns the number of queue
 * items, tiles and grid points of the plan.  No reference counterpart. */
lp_status lp_batch_plan(const lp_beam_desc* beams, int count,
                        const lp_batch_options* options, int* n_items,
                        long long* n_tiles, long long* n_points);
lp_status lp_batch_destroy(lp_batch* batch);

/* -------------------------------------------------- unfused comparison --
 * The plain FFT -> multiply -> IFFT form on the same GPU, with H materialised
 * in HBM by its own kernel, like the reference's numpy/CuPy sequence
 * (beam2d.py:485-490).  LP_FLAG_PLAIN_FP64_H builds H from a float64 Kz grid
 * in FP64 exactly like the reference; otherwise H uses the same float-float
 * phase as the fused path. */
#define LP_FLAG_PLAIN_FP64_H 0x100u
lp_status lp_plain_propagate_field(const lp_cfloat* field_in,
                                   lp_cfloat* field_out, int n,
                                   double area_size, double wl, double z,
                                   uint32_t flags, void* stream);

/* No counterpart in the reference.  The same unfused propagate as
 * lp_plain_propagate_field (float-float H; flags must be 0) for callers that
 * cannot call cudaMalloc while running -- a host application that reserved
 * nearly all device memory for its own pool, or a real-time loop that forbids
 * device allocation after start-up because cudaMalloc can block the device.
 * Its H grid lives in a fixed device array of 1024 x 1024 complex64 (8 MiB),
 * held by every device that loads the library until exit, so it allocates
 * nothing.  N above 1024 returns LP_ERR_UNSUPPORTED_SIZE.  All calls on a
 * device share that array: calls that overlap on the GPU race (serialise
 * them).  The first call on a device does its one-time set-up; make it
 * before any stream capture (a first call on a capturing stream returns
 * LP_ERR_NOT_INITIALIZED). */
lp_status lp_plain_propagate_field_noalloc(const lp_cfloat* field_in,
                                           lp_cfloat* field_out, int n,
                                           double area_size, double wl,
                                           double z, uint32_t flags,
                                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LIGHTPROP2D_GB300_H */
