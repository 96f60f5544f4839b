/*
 * nanopyx_gb300.h -- C ABI of the GB300 (sm_103a) eSRRF / SRRF engine.
 *
 * Plain pointers and sizes only: every `d_*` argument is a CUDA device
 * pointer, every `stream` argument is a cudaStream_t passed as void* (NULL =
 * the legacy default stream), every function returns an int status (NX_OK or
 * a negative NX_ERR_* code; nx_last_error() gives the message of the last
 * failure on the calling thread).  All compute calls are asynchronous on
 * `stream`; arrays are float32, C-contiguous, frames outermost.
 *
 * Each entry point names the reference routine it replaces (paths inside the
 * NanoPyx project).  The Python package nanopyx_gb300 binds these through
 * ctypes and re-exposes the reference's Liquid-Engine call surface on top.
 */
#ifndef NANOPYX_GB300_H
#define NANOPYX_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NX_ABI_VERSION 1

/* status codes */
#define NX_OK 0
#define NX_ERR_INVALID_ARG (-1)     /* bad shape / parameter (reference: ValueError) */
#define NX_ERR_UNSUPPORTED (-2)     /* valid request this library does not implement */
#define NX_ERR_OUT_OF_MEMORY (-3)   /* device allocation failed (reference: cl.MemoryError retry) */
#define NX_ERR_CUDA (-4)            /* CUDA runtime error */
#define NX_ERR_DEVICE_TIMEOUT (-5)  /* a bounded device wait ran out (kernel returned early) */
#define NX_ERR_WORKSPACE (-6)       /* workspace missing or too small */
#define NX_ERR_INDEX (-7)           /* the reference would index past its input (reference: IndexError) */

/* temporal correlations (bit mask; outputs are written in this order) */
#define NX_CORR_AVG 1
#define NX_CORR_VAR 2
#define NX_CORR_TAC2 4

typedef struct nx_esrrf_plan nx_esrrf_plan;

int nx_abi_version(void);
const char* nx_last_error(void);

/* ------------------------------------------------------------------------
 * eSRRF plan: per-(H, W, magnification, radius, sensitivity, weighting)
 * constants (FP64-derived phase tables of the RGC distance weights, the
 * clamped-edge Catmull-Rom taps) uploaded once to the device.
 * Replaces the per-call parameter set-up of
 *   src/nanopyx/core/transform/_le_radial_gradient_convergence.pyx:85-104
 * ------------------------------------------------------------------------ */
int nx_esrrf_plan_create(nx_esrrf_plan** plan, int H, int W, int magnification, float radius,
                         float sensitivity, int do_intensity_weighting);
int nx_esrrf_plan_destroy(nx_esrrf_plan* plan);

/* Tiling of a plan's fused kernel (no reference counterpart: the reference's
 * CPU loops have no tiles).  Variant 0 is the default tiling; variant 1
 * (magnifications 2, 4 and 5) runs one producer warp group fewer per CTA.
 * Batches group items by kernel instantiation, so items whose plans use
 * different variants run as different kernel classes.  set returns
 * NX_ERR_UNSUPPORTED when the variant is not instantiated for the plan's
 * (magnification, window) or the plan has no fused kernel; get returns the
 * variant or NX_ERR_UNSUPPORTED.  The results do not depend on the variant. */
int nx_esrrf_plan_set_tile_variant(nx_esrrf_plan* plan, int variant);
int nx_esrrf_plan_tile_variant(const nx_esrrf_plan* plan);

/* Host-only (no device call): the RGC distance-weight phase table a plan
 * uploads, w[py][px][j][i] for output sub-pixel phase (py, px) and half-grid
 * window offset (j, i) in [-J, J]; returns J (or a negative status).  Writes
 * nothing if `cap` (floats) is smaller than magnification^2 (2J+1)^2.
 *   src/include/_c_sr_radial_gradient_convergence.c:4-6,27-64                */
int nx_esrrf_weight_table(int magnification, float radius, float* h_out, size_t cap);

/* Per-frame RGC stack (T, H*m, W*m): the output of eSRRF_ST.run
 *   src/nanopyx/core/transform/_le_esrrf.pyx:30-33,172-196                 */
size_t nx_esrrf_st_workspace_bytes(const nx_esrrf_plan* plan, int T);
int nx_esrrf_st(const nx_esrrf_plan* plan, const float* d_in, int T, float* d_out, void* d_ws,
                size_t ws_bytes, void* stream);

/* Full eSRRF(): per timepoint block of `frames_per_timepoint` frames (0 = all),
 * the temporal correlations in `corr_mask` and, if `macro_pixel_correction`,
 * the macro-pixel correction.  d_out is (n_corr, n_timepoints, H*m, W*m).
 *   src/nanopyx/methods/esrrf/eSRRF_workflow.py:58-121
 *   src/nanopyx/core/transform/sr_temporal_correlations.py:46-75,205-221
 *   src/nanopyx/core/transform/mpcorrector.pyx:7-73                          */
size_t nx_esrrf_workspace_bytes(const nx_esrrf_plan* plan, int T, int frames_per_timepoint,
                                int corr_mask);
int nx_esrrf_run(const nx_esrrf_plan* plan, const float* d_in, int T, int frames_per_timepoint,
                 int corr_mask, int macro_pixel_correction, float* d_out, void* d_ws,
                 size_t ws_bytes, void* stream);

/* The two stages of nx_esrrf_run, for callers that time or overlap them:
 * stage 1 runs the fused frame-loop kernel (per-timepoint temporal sums into
 * the workspace), stage 2 turns them into the correlations (+ macro-pixel
 * correction).  Same workspace, same arguments.                              */
int nx_esrrf_run_stage1(const nx_esrrf_plan* plan, const float* d_in, int T,
                        int frames_per_timepoint, int corr_mask, void* d_ws, size_t ws_bytes,
                        void* stream);
int nx_esrrf_run_stage2(const nx_esrrf_plan* plan, int T, int frames_per_timepoint,
                        int corr_mask, int macro_pixel_correction, float* d_out, void* d_ws,
                        size_t ws_bytes, void* stream);

/* Failure-detection self-test (not a reference routine): one CTA waits on an
 * mbarrier that nothing arrives on, with the bounded wait every TMA wait of
 * the fused kernels uses, limited to `limit_ns` (<= 1 s).  The kernel returns
 * on its own and records the time-out in the status word of `d_ws`, so
 * nx_workspace_status() then reports NX_ERR_DEVICE_TIMEOUT and the context
 * stays usable.                                                              */
int nx_selftest_wait_timeout(void* d_ws, size_t ws_bytes, unsigned long long limit_ns,
                             void* stream);

/* Failure-detection self-test of the fused eSRRF kernel itself (not a
 * reference routine): runs nx_esrrf_st's launch with every producer/consumer
 * wait bounded by `limit_ns` (1 ms .. 1 s) and with the producers withholding
 * the `full` arrival of each CTA's first frame pass.  The consumers' bounded
 * wait runs out, the CTA raises its abort flag, every other wait of the CTA
 * gives up, the producer leader waits (bounded) for its TMA copies in flight
 * and the CTA returns; the time-out is recorded in the status word of `d_ws`
 * (nx_workspace_status -> NX_ERR_DEVICE_TIMEOUT) and the context stays usable.
 * `d_out` (T, H*m, W*m) receives whatever the aborted CTAs wrote before.     */
int nx_selftest_fused_abort(const nx_esrrf_plan* plan, const float* d_in, int T, float* d_out,
                            void* d_ws, size_t ws_bytes, unsigned long long limit_ns,
                            void* stream);

/* Throughput probe (not a reference routine): `blocks` CTAs of 256 threads
 * each run `iters` iterations of 8 independent FP32 FMA chains; returns via
 * d_sink (blocks*256 floats) so nothing is optimised away.  Used to measure
 * the FP32 FMA peak the RGC kernel is compared against.                       */
int nx_probe_ffma(float* d_sink, int blocks, int iters, void* stream);
/* Same work with Blackwell's packed FP32 FMA (f32x2): 4 chains of 2 lanes.   */
int nx_probe_ffma2(float* d_sink, int blocks, int iters, void* stream);

/* Streaming accumulation for served requests: frame blocks of one
 * reconstruction are pushed as they arrive; the device-resident accumulator
 * (nx_esrrf_accum_bytes) holds the per-pixel temporal state between pushes.
 * Finalize writes (n_corr, H*m, W*m).  Same arithmetic as nx_esrrf_run with
 * one timepoint.  (No single reference counterpart: the reference keeps the
 * whole per-frame stack in host RAM, eSRRF_workflow.py:76-112.)              */
size_t nx_esrrf_accum_bytes(const nx_esrrf_plan* plan);
size_t nx_esrrf_push_workspace_bytes(const nx_esrrf_plan* plan, int T_block);
int nx_esrrf_accum_push(const nx_esrrf_plan* plan, const float* d_block, int T_block,
                        int frames_before, void* d_accum, void* d_ws, size_t ws_bytes,
                        void* stream);
int nx_esrrf_accum_finalize(const nx_esrrf_plan* plan, const void* d_accum, int total_frames,
                            int corr_mask, int macro_pixel_correction, float* d_out, void* d_ws,
                            size_t ws_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Batched eSRRF: many independent reconstructions (uneven H, W, T, m, R,
 * correlation) and sensitivity sweeps in one persistent launch per kernel
 * class (m, window), each CTA taking (stack, tile, timepoint, frame chunk)
 * units from a shared work list.  create() plans the work, bind() uploads the
 * work lists into the caller's workspace (synchronises `stream`; not
 * capturable; creates one side stream per kernel class after the first),
 * launch() issues kernels only -- each class's kernel, finalisation and
 * macro-pixel correction on its own stream, forked from and joined back into
 * `stream` by events, so class tails overlap -- and can be captured into a
 * CUDA graph and replayed while the buffers stay in place.
 * Replaces the reference's per-stack loop (eSRRF_workflow.py:76-112) and
 * the per-(R, s) loop of the parameter sweep (core/analysis/parameter_sweep.py:33-37).
 * ------------------------------------------------------------------------ */
typedef struct nx_esrrf_item {
  const nx_esrrf_plan* plan;   /* H, W, magnification, radius, weighting, sensitivity */
  const float* d_in;           /* (T, H, W) */
  int T;
  int frames_per_timepoint;    /* 0 = all frames */
  int corr_mask;               /* NX_CORR_*; NX_CORR_AVG when n_sens > 0 */
  int macro_pixel_correction;
  int n_sens;                  /* 0: the plan's sensitivity; 1..4: AVG at each of sens[] */
  float sens[4];
  int frames_per_unit;         /* frames per work unit (0: heuristic) */
  float* d_out;                /* (n_corr or n_sens, n_timepoints, H*m, W*m) */
} nx_esrrf_item;

typedef struct nx_esrrf_batch nx_esrrf_batch;
int nx_esrrf_batch_create(nx_esrrf_batch** batch, const nx_esrrf_item* items, int n_items);
size_t nx_esrrf_batch_workspace_bytes(const nx_esrrf_batch* batch);
int nx_esrrf_batch_bind(nx_esrrf_batch* batch, void* d_ws, size_t ws_bytes, void* stream);
int nx_esrrf_batch_launch(const nx_esrrf_batch* batch, void* stream);
int nx_esrrf_batch_destroy(nx_esrrf_batch* batch);

/* Device status word check (synchronises `stream`): returns NX_OK or
 * NX_ERR_DEVICE_TIMEOUT if a kernel of a previous call on this workspace
 * recorded a bounded-wait timeout.                                          */
int nx_workspace_status(const void* d_ws, void* stream);

/* ------------------------------------------------------------------------
 * Standalone Liquid-Engine ops of the path
 * ------------------------------------------------------------------------ */

/* Catmull-Rom ShiftAndMagnify; per-frame shifts (length T, device arrays).
 *   src/nanopyx/core/transform/_le_interpolation_catmull_rom.pyx:17,143-160
 *   src/include/_c_interpolation_catmull_rom.c:6-52
 * d_out is (T, (int)(H*mag_row), (int)(W*mag_col)).                        */
int nx_cr_shift_magnify(const float* d_in, int T, int H, int W, const float* d_shift_row,
                        const float* d_shift_col, float mag_row, float mag_col, float* d_out,
                        void* stream);

/* Roberts-Cross gradients (gradient_col, gradient_row), each (T, H, W).
 *   src/nanopyx/core/transform/_le_roberts_cross_gradients.pyx:67-83
 *   src/include/_c_gradients.c:53-73                                        */
int nx_roberts_cross(const float* d_in, int T, int H, int W, float* d_gc, float* d_gr,
                     void* stream);

/* Radial Gradient Convergence on given 2m-magnified gradients
 * (T, 2*rowsM, 2*colsM) and m-magnified image (T, rowsM, colsM).
 *   src/nanopyx/core/transform/_le_radial_gradient_convergence.pyx:28,79-115
 *   src/include/_c_sr_radial_gradient_convergence.c:4-90                    */
int nx_rgc(const float* d_gc_interp, const float* d_gr_interp, const float* d_img_interp, int T,
           int rowsM, int colsM, int magnification, float radius, float sensitivity,
           int do_intensity_weighting, int pad_edges, float* d_out, void* stream);

/* SRRF radiality: d_img (T, h, w), d_img_interp (T, h*m, w*m) -> (T, h*m, w*m).
 *   src/nanopyx/core/transform/_le_radiality.pyx:86-125
 *   src/include/_c_sr_radiality.c:6-51, src/include/_c_gradients.c:3-25     */
size_t nx_radiality_workspace_bytes(int T, int h, int w);
int nx_radiality(const float* d_img, const float* d_img_interp, int T, int h, int w,
                 int magnification, float ring_radius, int border, int positivity_constraint,
                 int do_intensity_weighting, float* d_out, void* d_ws, size_t ws_bytes,
                 void* stream);

/* SRRF(): magnified intensity, radiality and per-frame macro-pixel
 * correction in one call, d_img (T, h, w) -> d_out (T, h*m, w*m).
 *   src/nanopyx/methods/srrf/SRRF_workflow.py:9-76                          */
size_t nx_srrf_workspace_bytes(int T, int h, int w, int magnification);
int nx_srrf(const float* d_img, int T, int h, int w, int magnification, float ring_radius,
            int border, int positivity_constraint, int do_intensity_weighting,
            int macro_pixel_correction, float* d_out, void* d_ws, size_t ws_bytes, void* stream);

/* eSRRF temporal correlation of a stack (T, n_pixels) -> (n_pixels).
 *   src/nanopyx/core/transform/sr_temporal_correlations.py:46-75,205-221    */
int nx_temporal_correlation(const float* d_stack, int T, long long n_pixels, int correlation,
                            float* d_out, void* stream);

/* SRRF temporal correlation orders 0 (max), 1 (mean), -1 (pairwise product
 * sum), 2/3/4 (ACRF, without lag-time integration).
 *   src/nanopyx/core/transform/sr_temporal_correlations.py:4-43,78-202      */
int nx_srrf_temporal_correlation(const float* d_stack, int T, long long n_pixels, int order,
                                 float* d_out, void* stream);

/* SRRF ACRF of order 2, 3 or 4 WITH lag-time integration (the reference's
 * do_integrate_lag_times=1 branch): per level the lag products, then the
 * frames re-binned in place by `order`, until at most `order` binned frames
 * remain; the result is the last level's correlation (float32, the
 * reference's operation order).  The workspace holds a working copy of the
 * stack (the input is not modified).  Frame counts at which the reference's
 * binning reads past its last frame (orders 3 and 4) return NX_ERR_INDEX
 * before anything is launched, as the reference raises IndexError.
 *   src/nanopyx/core/transform/sr_temporal_correlations.py:111-121,159-200  */
size_t nx_srrf_acrf_workspace_bytes(int T, long long n_pixels);
int nx_srrf_acrf_integrated(const float* d_stack, int T, long long n_pixels, int order,
                            float* d_out, void* d_ws, size_t ws_bytes, void* stream);

/* Fourier interpolation (the use_fht=True path of eSRRF_ST): every frame
 * (T, H, W) -> (T, H*m, W*m), mirror padding to a power-of-two square,
 * zero-padded spectrum, rescale onto the frame's [min, max], central crop;
 * frames over 256 px a side in overlapping 256-pixel tiles blended with Hann
 * windows.  The plan holds the tile layout, the interpolation operators of
 * every padded size (float64, rounded once) and the blending weights; the
 * transform runs as batched FP32 GEMMs.
 *   src/nanopyx/core/transform/interpolation.py:22-290 (fht_space_interpolation)
 *   src/nanopyx/core/transform/_le_esrrf.pyx:183-188                          */
typedef struct nx_fht_plan nx_fht_plan;
int nx_fht_plan_create(nx_fht_plan** plan, int H, int W, int magnification);
/* Variants: NX_FHT_TILED is the plan above (interpolation.py: half spectrum
 * along x, 256-pixel tiles).  NX_FHT_FULL_SPECTRUM is the older
 * _interpolation.pyx form that ErrorMap uses (error_map.pyx:16,52-55): the
 * whole image as one mirrored square, the full complex spectrum on both axes
 * (fft2, centred block, ifft2, real part), float32 rescale.
 *   src/nanopyx/core/transform/_interpolation.pyx:106-200                     */
#define NX_FHT_TILED 0
#define NX_FHT_FULL_SPECTRUM 1
int nx_fht_plan_create_ex(nx_fht_plan** plan, int H, int W, int magnification, int variant);
int nx_fht_plan_destroy(nx_fht_plan* plan);
size_t nx_fht_workspace_bytes(const nx_fht_plan* plan, int T);
int nx_fht_interpolate(const nx_fht_plan* plan, const float* d_in, int T, float* d_out, void* d_ws,
                       size_t ws_bytes, void* stream);

/* eSRRF-3D of a (T, S, H, W) stack into d_out (S*mz, H*mxy, W*mxy): per frame
 * the 3-D gradients, Catmull-Rom x mxy in every slice (slices repeated mz
 * times, as the reference's z step does), the 3-D RGC inside the margins to
 * the power `sensitivity`, times the intensity when do_intensity_weighting;
 * then the frames' mean (mode 0) or standard deviation (mode 1).  radius_z =
 * radius * PSF_ratio / voxel_ratio.  Voxels outside the margins are 0.
 *   src/nanopyx/core/transform/_le_esrrf3d.pyx:35-140
 *   src/include/_c_sr_radial_gradient_convergence.c:92-204
 *   src/include/_c_gradients.c:75-116                                        */
size_t nx_esrrf3d_workspace_bytes(int S, int H, int W, int magnification_xy,
                                  int magnification_z, int mode);
int nx_esrrf3d_st(const float* d_in, int T, int S, int H, int W, int magnification_xy,
                  int magnification_z, double radius, double radius_z, float sensitivity,
                  int mode, int do_intensity_weighting, float* d_out, void* d_ws,
                  size_t ws_bytes, void* stream);

/* Parameter-sweep scoring (src/nanopyx/core/analysis/parameter_sweep.py:99-139).
 *
 * Gaussian blur with scipy.ndimage.gaussian_filter's definition, as ErrorMap
 * applies it (src/nanopyx/core/transform/error_map.pyx:72-77,127-146): axis 0
 * then axis 1, radius int(4 sigma + 0.5), mode 'reflect'; sigma <= 1e-15
 * leaves the image as it is.  With affine != 0 the input is first mapped to
 * alpha * x + beta (float32).  d_in and d_out (H, W) must not overlap.        */
size_t nx_gaussian_blur_workspace_bytes(int H, int W);
int nx_gaussian_blur(const float* d_in, int H, int W, double sigma, int affine, float alpha,
                     float beta, float* d_out, void* d_ws, size_t ws_bytes, void* stream);
/* The same for n images at once, each with its own sigma (host array) and,
 * when alpha/beta (host arrays) are given, its own affine map: output image i
 * (of d_out, (n, H, W)) is the blur of input image src_index[i] of d_in
 * (i itself when src_index is NULL; indices must lie inside d_in).  Up to 32
 * images per launch; the Brent searches of several error maps share one.   */
size_t nx_gaussian_blur_batch_workspace_bytes(int H, int W, int n);
int nx_gaussian_blur_batch(const float* d_in, int H, int W, int n, const int* src_index,
                           const double* sigma, const float* alpha, const float* beta,
                           float* d_out, void* d_ws, size_t ws_bytes, void* stream);
/* flags: NX_BLUR_FLOAT64_SUMS accumulates every pass in float64 and rounds it
 * to float32 (scipy's own arithmetic for float32 arrays: exact for the
 * near-identity blurs whose difference from the image is the signal).       */
#define NX_BLUR_FLOAT64_SUMS 1
int nx_gaussian_blur_batch_ex(const float* d_in, int H, int W, int n, const int* src_index,
                              const double* sigma, const float* alpha, const float* beta,
                              int flags, float* d_out, void* d_ws, size_t ws_bytes,
                              void* stream);

/* Float64 moment sums of `batch` images d_x (batch, n) against one image
 * d_y (n): per image sum x, sum y, sum x^2, sum x y, sum y^2 and
 * sum (x - y)^2 (the difference rounded to float32 first) into
 * d_sums (batch, 6), device memory.  Deterministic.                         */
size_t nx_moment_sums_workspace_bytes(int batch);
int nx_moment_sums(const float* d_x, const float* d_y, long long n, int batch, double* d_sums,
                   void* d_ws, size_t ws_bytes, void* stream);

/* Fourier ring correlation sums of `pairs` image pairs
 * (src/nanopyx/core/analysis/frc.pyx:108-143,150-179,181-198): in pair q the
 * N x N windows at (r0, c0) of d_img1 + q stride and d_img2 + q stride (row
 * pitch `pitch` floats) are Tukey(0.25)-tapered and Fourier transformed; for
 * every ring radius r = 1 .. N/2 - 2 the reference's sample positions on the
 * centred spectra are bilinearly interpolated and summed in float64:
 * d_sums[q][r] = (sum a1 a2 + b1 b2, sum a1^2 + b1^2, sum a2^2 + b2^2,
 * samples), device memory of pairs x (N/2 - 1) x 4 doubles (row 0 zero).
 * N even, 6 .. 8192; up to 8 pairs per FFT launch.                          */
typedef struct nx_frc_plan nx_frc_plan;
int nx_frc_plan_create(nx_frc_plan** plan, int N);
int nx_frc_plan_destroy(nx_frc_plan* plan);
int nx_frc_rings(const nx_frc_plan* plan);
size_t nx_frc_workspace_bytes(const nx_frc_plan* plan, int pairs);
int nx_frc_ring_sums(const nx_frc_plan* plan, const float* d_img1, const float* d_img2, int pairs,
                     long long stride, int pitch, int r0, int c0, double* d_sums, void* d_ws,
                     size_t ws_bytes, void* stream);

/* Decorrelation analysis (src/nanopyx/core/analysis/decorr.pyx:23-393).
 * nx_decorr_prepare: the (h, w) image with its 20-pixel border rolled off
 * towards the mean outside the circle of radius w/2 - 20
 * (src/nanopyx/core/transform/edges.pyx:9-49), placed in the N x N square
 * (N the power of two >= max(h, w)) at rows 0 .. h-1 and columns (N-w)/2 ..,
 * the rest filled with its first pixel (decorr.pyx:64-99).
 * nx_decorr_coefs: for B N x N images -- d_base[z], or d_base - d_sub[z]
 * (the high-pass differences) when d_sub is given -- the centred spectrum
 * (DC term zeroed when zero_dc), d_cr[z] = sum over the inscribed disc of
 * |F|^2, and d_coef[z] (2 n_r doubles): per radial bin of the band
 * [crmin, crmax] the sum of re^2/|F| + im^2/|F| and of the normalised power,
 * over the reference's walk of the centred square (decorr.pyx:120-200).
 * Uses an nx_frc_plan of size N for the transforms.                        */
size_t nx_decorr_prepare_workspace_bytes(int h, int w);
int nx_decorr_prepare(const float* d_img, int h, int w, float* d_out, int N, void* d_ws,
                      size_t ws_bytes, void* stream);
size_t nx_decorr_coefs_workspace_bytes(const nx_frc_plan* plan, int B, int n_r);
int nx_decorr_coefs(const nx_frc_plan* plan, const float* d_base, const float* d_sub, int B,
                    int zero_dc, float crmin, float crmax, int n_r, double* d_cr,
                    double* d_coef, void* d_ws, size_t ws_bytes, void* stream);

/* Macro-pixel correction in place on (S, rowsM, colsM).
 *   src/nanopyx/core/transform/mpcorrector.pyx:7-73                         */
size_t nx_macro_pixel_workspace_bytes(int S, int magnification);
int nx_macro_pixel_correct(float* d_img, int S, int rowsM, int colsM, int magnification,
                           void* d_ws, size_t ws_bytes, void* stream);

/* Macro-pixel correction that allocates nothing -- no counterpart in the
 * reference.  For callers that may not allocate device memory while they run
 * (real-time acquisition loops that reserve everything at start-up, hosts whose
 * own allocator owns the GPU): same result as nx_macro_pixel_correct, with the
 * scratch in a 256 KiB device array owned by the library (held on every GPU
 * that loads it, until exit).  A call needs
 * max(S,1) * m^2 * min(64, max(1, rowsM / m)) * 4 bytes of it (S * m^2 <= 1024
 * once rowsM >= 64 m); a larger call returns NX_ERR_INVALID_ARG and launches
 * nothing.  The first call on a device resolves the array's address and, under
 * lazy module loading, loads the library's kernels there and reserves the
 * array (it may then fail with NX_ERR_OUT_OF_MEMORY): make it at start-up,
 * before the allocation-free phase and before any stream capture.  Calls that
 * overlap on the GPU race on the array; do not call again after a reset of
 * the device in the same process.                                           */
int nx_macro_pixel_correct_static(float* d_img, int S, int rowsM, int colsM, int magnification,
                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NANOPYX_GB300_H */
