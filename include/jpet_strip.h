/* jpet_strip.h -- C ABI of the GB300-native 2D strip-PET list-mode TOF MLEM.
 *
 * This library replaces the reference's GPU backend for the strip scanner,
 *   template <typename F> void PET2D::Strip::GPU::Reconstruction::run(
 *       Scanner<F,S>&, Response<F>*, int n_responses, Output& rho,
 *       int n_iteration_blocks, int n_iterations_in_block, output, progress,
 *       int device, int n_blocks, int n_threads_per_block, device_name)
 *   (grey277/j-pet-mlem src/2d/strip/cuda/reconstruction.h:32-44,
 *    implementation src/2d/strip/cuda/reconstruction.cu:31-113),
 * and runs the iteration of the reference's CPU path
 *   PET2D::Strip::Reconstruction<F, GaussianKernel<F>>::operator()
 *   (src/2d/strip/reconstruction.h:108-154, bb_update :220-298)
 * on the GPU.  Every entry point takes plain pointers and sizes, returns a status
 * code (0 = success, < 0 = error class below) and never aborts the process;
 * jpet_strip_last_error() gives the message of the last failure on a handle.
 *
 * Threading: a handle is used by one host thread at a time; different handles
 * may be used concurrently.  Work is issued on the handle's CUDA stream.
 * All host buffers are caller-owned; all device memory is owned by the handle
 * unless an entry point says otherwise.
 */
#ifndef JPET_STRIP_H
#define JPET_STRIP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JPET_STRIP_ABI_VERSION 1

/* status codes */
#define JPET_OK 0
#define JPET_ERR_ARGUMENT (-1)   /* invalid argument (null pointer, bad size, bad mode) */
#define JPET_ERR_CUDA (-2)       /* a CUDA runtime call failed */
#define JPET_ERR_MEMORY (-3)     /* device or host allocation failed */
#define JPET_ERR_STATE (-4)      /* call out of order (e.g. iterate before set_events) */
#define JPET_ERR_TIMEOUT (-5)    /* reserved: no entry point returns it (no device-side waits) */
#define JPET_ERR_UNSUPPORTED (-6)/* option not built into this library */

typedef struct jpet_strip jpet_strip_t;

/* Scanner geometry: the arguments of Scanner's constructor in its order
 * (src/2d/strip/scanner.h:39-49), lengths in the caller's unit (mm in the
 * reference's examples).  Values are rounded to float exactly as the reference's
 * Scanner<float, short> stores them. */
typedef struct jpet_strip_geom {
  double radius;              /* R: distance of each strip from the centre line (-r) */
  double scintillator_length; /* L: strip length (-l) */
  int32_t n_y_pixels;         /* image rows (--n-y-pixels), <= 32767 */
  int32_t n_z_pixels;         /* image columns (--n-z-pixels), <= 32767 */
  double pixel_height;        /* -p */
  double pixel_width;         /* -p */
  double sigma_z;             /* --s-z */
  double sigma_dl;            /* --s-dl */
} jpet_strip_geom;

/* kernel / update semantics */
#define JPET_MODE_CPU_REFERENCE 0 /* GaussianKernel, no sensitivity: reconstruction.h:220-298 */
#define JPET_MODE_GPU_REFERENCE 1 /* AnalyticKernel, denominator weighted by the 5-point
                                     pixel sensitivity: warp_granularity.cuh:19-155 */
/* accumulation precision (fast kernel; the exact kernel and the GPU-reference
 * mode accumulate in FP32) */
#define JPET_PRECISION_FP32 0        /* FP32 evaluation, FP32 shared-memory tile sums, FP32 image */
#define JPET_PRECISION_COMPENSATED 1 /* FP32 evaluation; every shared-memory tile addition
                                        also adds its exact rounding error (TwoSum) to a
                                        compensation tile; tiles go into an FP32 image whose
                                        atomic additions' rounding errors (TwoSum of the value
                                        each atomic found), with the tile compensations, go
                                        into an FP32 compensation image added at the end */
#define JPET_PRECISION_FP64_DEN 2    /* as COMPENSATED, plus per-event denominators reduced
                                        in FP64 (the only FP64 arithmetic of the modes) */
#define JPET_PRECISION_FIXED 3       /* deterministic image: each pixel's contribution of a
                                        batch of events (FAST) or of one event (ROWS) rounded
                                        once to 2^-22 of an event (unbiased dither), summed as
                                        integers per tile and with 64-bit integer atomics over
                                        tiles, converted to FP32 once */

/* iteration kernel */
#define JPET_VARIANT_FAST 0  /* default, every precision: batch-union kernel -- batches of
                                <= 8 similar events share one lane-to-pixel map, rho is read
                                and the back-projection written once per batch, exp2-form
                                kernel with packed f32x2, per-row coefficients regenerated
                                on chip */
#define JPET_VARIANT_EXACT 1 /* every pixel evaluated in the reference's operation order */
#define JPET_VARIANT_WARP 2  /* one warp per event, shared-memory atomics */
#define JPET_VARIANT_ROWS 3  /* row-owned kernel: image rows owned by warps, one event at a
                                time per row, per-row coefficients precomputed at set-up */

/* register-cache shape of the ROWS kernel: G lanes per image row x passes of
 * 256/G event rows x sweeps of 2G columns (0 = chosen from the event boxes) */
#define JPET_RASTER_AUTO 0
#define JPET_RASTER_8x1x1 1 /* <= 32 rows, <= 15 columns */
#define JPET_RASTER_8x1x2 2 /* <= 32 rows, <= 31 columns */
#define JPET_RASTER_4x1x2 3 /* <= 64 rows, <= 15 columns */
#define JPET_RASTER_4x1x3 4 /* <= 64 rows, <= 23 columns */
#define JPET_RASTER_4x1x4 5 /* <= 64 rows, <= 31 columns */
#define JPET_RASTER_4x2x4 6 /* <= 128 rows, <= 31 columns */
#define JPET_RASTER_2x1x6 7 /* <= 64 rows, <= 23 columns, 2 lanes per row */

typedef struct jpet_strip_opts {
  int32_t device;       /* CUDA device ordinal (-D / --cuda-device) */
  int32_t mode;         /* JPET_MODE_* */
  int32_t precision;    /* JPET_PRECISION_* */
  int32_t tile_w;       /* image tile width in pixels, 0 = chosen by the tuner */
  int32_t tile_h;       /* image tile height in pixels, 0 = chosen by the tuner */
  int32_t block_threads;/* threads per CTA of the iteration kernel, 0 = default (256 for
                           the FAST kernel: 8 events per batch; 128 for the ROWS kernel;
                           both take 128 or 256; 256 otherwise) */
  int32_t variant;      /* JPET_VARIANT_*; the GPU-reference mode always runs EXACT */
  int32_t raster_shape; /* JPET_RASTER_*; events outside the shape take the exact path */
  int32_t reserved[8];  /* must be zero */
} jpet_strip_opts;

/* Per-iteration counters (the reference's ReconstructionStats,
 * src/2d/strip/reconstruction_stats.h:7-89, counted on the device). */
typedef struct jpet_strip_counters {
  int64_t n_events;          /* events processed in the last iteration */
  int64_t n_pixels;          /* bounding-box pixels of those events */
  int64_t n_kernel_calls;    /* in-ellipse kernel evaluations (n_kernel_calls) */
  int64_t n_contributing;    /* events with a positive denominator */
  int64_t n_oversize;        /* events handled by the large-box path */
  int64_t n_tiles;           /* non-empty image tiles */
  int64_t n_chunks;          /* work items of the iteration kernel */
  int64_t iterations_done;   /* iterations run since the last set_image */
  int64_t n_exact_path;      /* events the fast kernel handed to the reference-order
                                rasteriser (box outside its register-cache shape) */
} jpet_strip_counters;

/* Version of this ABI (JPET_STRIP_ABI_VERSION). */
int jpet_strip_abi_version(void);

/* Fills *opts with defaults (device 0, CPU-reference mode, FP32, tuned tiles). */
void jpet_strip_default_opts(jpet_strip_opts* opts);

/* Creates a handle: validates the geometry, selects the device, allocates the
 * image buffers and computes the sensitivity maps.  Replaces the set-up part of
 * GPU::Reconstruction::run (cuda/reconstruction.cu:54-74). */
int jpet_strip_create(const jpet_strip_geom* geom, const jpet_strip_opts* opts,
                      jpet_strip_t** out);

/* Destroys a handle and frees its device memory.  Safe on NULL. */
int jpet_strip_destroy(jpet_strip_t* h);

/* Message of the last failed call on h (or of the last failed create when h is
 * NULL); never NULL. */
const char* jpet_strip_last_error(const jpet_strip_t* h);

/* Uses the given CUDA stream (a cudaStream_t) for all later work; NULL = the
 * handle's own stream.  The caller keeps ownership of an external stream. */
int jpet_strip_set_stream(jpet_strip_t* h, void* cuda_stream);

/* Uploads events from host memory in the reference's Response layout: AoS
 * float triples (z_u, z_d, dl) (src/2d/strip/response.h:13-20), n >= 0.
 * Copies, converts to SoA on the device and prepares the per-event data the
 * iterations reuse (replaces GPU::ResponsesSOA, cuda/gpu_events_soa.h:9-51). */
int jpet_strip_set_events(jpet_strip_t* h, const float* responses_aos, int64_t n);

/* Same from three host SoA arrays. */
int jpet_strip_set_events_soa(jpet_strip_t* h, const float* z_u, const float* z_d,
                              const float* dl, int64_t n);

/* Same from device-resident SoA arrays (read during this call only). */
int jpet_strip_set_events_device(jpet_strip_t* h, const float* d_z_u,
                                 const float* d_z_d, const float* d_dl, int64_t n);

/* Sets the current image rho from host memory, float[n_y * n_z] row-major,
 * index y * n_z + z (src/2d/geometry/pixel.h:29).  The image after create is
 * all ones (reconstruction.h:59). */
int jpet_strip_set_image(jpet_strip_t* h, const float* rho);

/* Same from device memory. */
int jpet_strip_set_image_device(jpet_strip_t* h, const float* d_rho);

/* Runs n MLEM iterations on the device: rho <- sum_e K rho / sum K rho
 * (reconstruction.h:108-154).  Asynchronous on the handle's stream; errors of
 * the launches are reported, errors of the execution by the next synchronising
 * call. */
int jpet_strip_iterate(jpet_strip_t* h, int n);

/* Copies the current image to host memory (synchronises the stream). */
int jpet_strip_get_image(jpet_strip_t* h, float* rho);

/* Device pointer of the current image (valid until the next iterate/set_image). */
int jpet_strip_image_device(jpet_strip_t* h, const float** d_rho);

/* Sensitivity image to host memory: kind 0 = scanner sensitivity at pixel
 * centres (reconstruction.h:67-73), kind 1 = 5-point pixel sensitivity
 * (scanner.h:174-185, written by the reference GPU path as output(-1, ...)). */
int jpet_strip_get_sensitivity(jpet_strip_t* h, int kind, float* out);

/* Counters of the last iteration (synchronises the stream). */
int jpet_strip_get_counters(jpet_strip_t* h, jpet_strip_counters* out);

/* Synchronises the handle's stream and reports any asynchronous error. */
int jpet_strip_synchronize(jpet_strip_t* h);

/* Poisson list-mode negative log-likelihood of the current events and its
 * gradients (no counterpart in the reference, which has no likelihood code):
 *   L = sum_p s_p rho_p - sum_e log(sum_{p in E_e} K_e(p; sigma) rho_p)
 * with the reference's Gaussian kernel including its normalisation
 * (gaussian_kernel.h:27-79) at the kernel widths (sigma_z, sigma_dl), and the
 * support E_e = the event's 3-sigma ellipse for the handle's own widths, held
 * fixed.  d_rho: device float[n_y*n_z] (NULL = the current image); d_sens: device
 * sensitivity s (NULL = point sensitivity, kind 0); d_grad_rho: device
 * float[n_y*n_z] receiving dL/drho, or NULL.  loss, grad_sigma[2] (dL/dsigma_z,
 * dL/dsigma_dl) and n_skipped (events with a zero denominator, left out) are
 * host pointers, each may be NULL.  Synchronises the stream.  Needs the
 * CPU-reference mode. */
int jpet_strip_nll_grad(jpet_strip_t* h, double sigma_z, double sigma_dl, const float* d_rho,
                        const float* d_sens, double* loss, float* d_grad_rho,
                        double* grad_sigma, int64_t* n_skipped);

/* One MLEM iteration that allocates no device memory (no counterpart in the
 * reference).  For callers that may not allocate device memory, or may not let
 * a library do so: a process that must not allocate once it is acquiring data,
 * or an application that owns every device allocation and hands out only input
 * and output buffers.  d_responses_aos: device AoS (z_u, z_d, dl) float
 * triples, n <= 1048576 (larger n is rejected with JPET_ERR_ARGUMENT);
 * d_rho_in / d_rho_out: device float[n_y*n_z] images; the output is cleared by
 * the call, so it may overlap neither the input image nor the responses
 * (rejected with JPET_ERR_ARGUMENT).  Work runs on cuda_stream (a cudaStream_t, NULL = the
 * default stream) in the reference's CPU float semantics and operation order;
 * no handle is involved.  It evaluates every box pixel in that order and adds
 * with global float atomics: on a GB300, 18 ms per iteration of 1048576 events
 * at 2 mm pixels (sigma 10 / 42 mm), about 17 times the time of a handle's
 * default kernel, which prepares its events into buffers it allocates.  The per-event working data live in one fixed 24 MiB
 * device array of the library, which every GPU that loads the library keeps
 * until the process exits; calls share it, so calls that overlap on the GPU
 * (different streams or unordered host threads) race, while calls ordered on
 * one stream do not.  Every call looks up the array's address with the
 * caller's device current (so a call after cudaDeviceReset is safe); the first
 * call on a device also loads the library's device code there, so make it
 * before any stream capture.
 * Errors: jpet_strip_last_error(NULL). */
int jpet_strip_iterate_noalloc(const jpet_strip_geom* geom, const float* d_responses_aos,
                               int64_t n, const float* d_rho_in, float* d_rho_out,
                               void* cuda_stream);

/* The full reference GPU entry point over host buffers: uploads the events,
 * starts from rho (in/out, float[n_y*n_z]), runs n_blocks * n_iterations_in_block
 * iterations and calls output(iteration, image, user) at the iterations the
 * reference reports (cuda/reconstruction.cu:99-110) and output(-1, sensitivity)
 * first (.cu:63-70); progress(completed, finished, user) around every
 * iteration (.cu:82,96,112).  Either callback may be NULL.  The image passed to
 * output is host memory owned by the library, valid during the call. */
typedef void (*jpet_strip_output_fn)(int iteration, const float* image, int n_z,
                                     int n_y, void* user);
typedef void (*jpet_strip_progress_fn)(int completed, int finished, void* user);
int jpet_strip_run(const jpet_strip_geom* geom, const jpet_strip_opts* opts,
                   const float* responses_aos, int64_t n, float* rho, int n_blocks,
                   int n_iterations_in_block, jpet_strip_output_fn output,
                   jpet_strip_progress_fn progress, void* user, char* device_name,
                   size_t device_name_len);

/* The reference iteration at double on the GPU (Reconstruction<double,
 * GaussianKernel<double>>, reconstruction.h:108-154): the FP64 yardstick for
 * accuracy studies at full event counts.  n_iterations iterations of the
 * device AoS responses from d_rho (in/out, double[n_y*n_z]); d_work is a
 * second double[n_y*n_z] buffer.  Counters of the last iteration are optional.
 * Runs on cuda_stream and is complete on return.  No counterpart in the
 * reference's GPU code. */
int jpet_strip_reference_fp64(const jpet_strip_geom* geom, const float* d_responses_aos,
                              int64_t n, double* d_rho, double* d_work, int32_t n_iterations,
                              int64_t* kernel_calls, int64_t* contributing, void* cuda_stream);

/* ---- batched reconstructions ---------------------------------------------
 * No counterpart in the reference (one event set per process): n independent
 * reconstructions (own geometry, widths, events, images) whose iterations run
 * together, one CUDA graph launch per jpet_strip_batch_iterate call.  Every
 * instance is a handle of its own (jpet_strip_batch_instance) for images,
 * counters and sensitivity maps; batches run the FP32 row-owned kernel in the
 * CPU-reference mode. */
typedef struct jpet_strip_batch jpet_strip_batch_t;
typedef struct jpet_strip_batch_plan {
  int32_t raster_shape;          /* JPET_RASTER_* the instance runs (0 = automatic) */
  int32_t block_threads;         /* CTA size (0 = default) */
  double tuned_ms_per_iteration; /* best time on the tuning prefix, -1 = not timed */
  int64_t tuned_events;          /* events of the tuning prefix */
  int32_t candidates;            /* plans timed for this instance (0 = cached plan) */
  int32_t tile;                  /* square tile side in pixels (0 = from the window budget) */
} jpet_strip_batch_plan;

/* opts (NULL = defaults) apply to every instance; device = opts->device. */
int jpet_strip_batch_create(int32_t n, const jpet_strip_geom* geoms, const jpet_strip_opts* opts,
                            jpet_strip_batch_t** out);
int jpet_strip_batch_destroy(jpet_strip_batch_t* b);
const char* jpet_strip_batch_last_error(const jpet_strip_batch_t* b);
int jpet_strip_batch_size(const jpet_strip_batch_t* b);
/* The handle of instance i (owned by the batch; do not destroy it). */
int jpet_strip_batch_instance(jpet_strip_batch_t* b, int32_t i, jpet_strip_t** h);
/* AoS responses of instance i, host memory (on_device = 0) or device memory. */
int jpet_strip_batch_set_events(jpet_strip_batch_t* b, int32_t i, const float* aos, int64_t n,
                                int32_t on_device);
/* Autotuner: for every instance, times its automatic register shape and the
 * next larger one with 128- and 256-thread CTAs and two tile sides (the
 * largest square tile the CTA's window budget allows, and half of it) on the
 * first max_tune_events events (<= 0: 262144) and keeps the fastest; plans are
 * cached by grid, pixel size, widths and event-count octave.  Re-bins the
 * events with the chosen plan and resets every image to uniform 1. */
int jpet_strip_batch_tune(jpet_strip_batch_t* b, int64_t max_tune_events);
int jpet_strip_batch_plan_of(const jpet_strip_batch_t* b, int32_t i, jpet_strip_batch_plan* p);
/* n iterations of every instance: one graph launch (captured on first use for
 * each n), complete on return. */
int jpet_strip_batch_iterate(jpet_strip_batch_t* b, int32_t n);
/* Kernels per batched iteration after the first iterate (0 before). */
int jpet_strip_batch_launches_per_iteration(const jpet_strip_batch_t* b);

/* ---- event generator (the phantom tool's Monte Carlo on the GPU) ----------
 * Replaces the emission loop of src/2d/strip/phantom_cmd.cpp:136-444 /
 * src/common/phantom_monte_carlo.h:33-109 over the regions of
 * src/2d/geometry/phantom.h:137-181 ("ellipse x y a b angle intensity",
 * "rectangle x y a b intensity", "point x y intensity"). */
#define JPET_REGION_ELLIPSE 0   /* centre (x, y) = (z, y), semi-axes a, b, rotation */
#define JPET_REGION_RECTANGLE 1 /* centre (x, y), half sizes a, b */
#define JPET_REGION_POINT 2     /* (x, y) */
typedef struct jpet_strip_region {
  int32_t kind;      /* JPET_REGION_* */
  int32_t reserved;  /* must be zero */
  double x, y, a, b; /* mm */
  double angle_deg;  /* ellipse rotation in degrees */
  double intensity;
} jpet_strip_region;

#define JPET_GEN_DETECTED 1 /* n counts detected events (the reference's --detected);
                               otherwise n counts emissions over (-pi/2, pi/2) */
#define JPET_GEN_ADDITIVE 2 /* regions add up instead of earlier ones masking later ones */

/* Count images of the phantom tool (phantom_cmd.cpp:249-352): int32[n_y*n_z]
 * each (NULL = not wanted) on a grid of geom's n_z x n_y pixels of size
 * pixel_width whose lower-left corner is -(n_z, n_y) * pixel_width / 2 +
 * (origin_x, origin_y) (--image-origin); row 0 is the lowest y.  emitted:
 * emission points of every emission counted; detected: emission points of the
 * detected events; naive: the points recovered from the smeared responses.
 * tan_map (--tan-bins, phantom_cmd.cpp:243-253,339-345): int32[tan_bins * n_y *
 * n_z], index (plane * n_y + row) * n_z + column, the naive points binned also
 * by their tangent into tan_bins planes over +-1.1 L / 2R.  The naive and tan
 * bins follow the reference's float arithmetic (response.h:22-37,
 * pixel_grid.h:59-64, voxel_grid.h:109-118).
 * Device pointers for jpet_strip_generate, host pointers for
 * jpet_strip_generate_host; the device images are accumulated into, the host
 * ones overwritten. */
typedef struct jpet_strip_gen_images {
  int32_t* emitted;
  int32_t* detected;
  int32_t* naive;
  double origin_x, origin_y;
  int32_t tan_bins; /* planes of tan_map (0 = no map) */
  int32_t reserved;
  int32_t* tan_map;
  /* --full (phantom_cmd.cpp:206-232,300-333): per written event, in the order
   * of the responses, the exact (unsmeared) response (z_u, z_d, dl: 3 floats)
   * and the emission event (x, y, sin phi, cos phi: 4 floats, the layout of
   * PET2D::Event); room for `capacity` events each, NULL = not wanted */
  float* exact_responses;
  float* events;
} jpet_strip_gen_images;

/* Writes the detected, smeared responses (z_u, z_d, dl) as float triples to
 * the device buffer d_out_aos (room for `capacity` events) in a deterministic
 * order fixed by (regions, scanner, seed).  geom supplies radius,
 * scintillator_length, sigma_z and sigma_dl (the pixel fields are unused).
 * *n_written receives the number of events written: n with
 * JPET_GEN_DETECTED, else the detected among the first n emissions.  Work
 * runs on cuda_stream (NULL = the default stream) and is complete on return.
 * Errors: jpet_strip_last_error(NULL).  No counterpart in the reference's
 * GPU code (its phantom tool runs on the CPU). */
int jpet_strip_generate(const jpet_strip_geom* geom, const jpet_strip_region* regions,
                        int32_t n_regions, int64_t n, uint64_t seed, int32_t flags,
                        float* d_out_aos, int64_t capacity, int64_t* n_written,
                        const jpet_strip_gen_images* images, void* cuda_stream);
/* The same into host memory on device `device` (the library allocates and
 * frees the device buffers); for callers without a CUDA runtime of their own,
 * such as the phantom command-line tool. */
int jpet_strip_generate_host(const jpet_strip_geom* geom, const jpet_strip_region* regions,
                             int32_t n_regions, int64_t n, uint64_t seed, int32_t flags,
                             float* out_aos, int64_t capacity, int64_t* n_written,
                             const jpet_strip_gen_images* images, int32_t device);

/* Kernel map of the phantom tool's --tan-bins output (phantom_cmd.cpp:396-436):
 * float[tan_bins * n_y * n_z] into host memory `out`, index (plane * n_y + row)
 * * n_z + column, the analytic kernel (analytic_kernel.h:28-74) of an event at
 * each voxel centre (z, y, tangent of the plane) evaluated at the emission
 * point (kernel_x, kernel_y) (--kernel-point), times 4 R pixel^2 dtan sec and,
 * when divide_by_sensitivity (the reference's --detected), divided by the
 * scanner sensitivity at the kernel point.  Grid and tangent planes as for
 * jpet_strip_gen_images; geom supplies the scanner, the grid and the sigmas.
 * Runs on device `device` and is complete on return. */
int jpet_strip_tan_kernel_map(const jpet_strip_geom* geom, int32_t tan_bins, double kernel_x,
                              double kernel_y, double origin_x, double origin_y,
                              int32_t divide_by_sensitivity, float* out, int32_t device);

#ifdef __cplusplus
}
#endif
#endif
