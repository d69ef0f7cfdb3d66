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
#define JPET_ERR_TIMEOUT (-5)    /* a bounded device-side wait gave up */
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
                                        compensation tile; tile sum + compensation go into
                                        an FP64 image (compensated, Kahan-style, per tile) */
#define JPET_PRECISION_FP64_DEN 2    /* as COMPENSATED, plus per-event denominators reduced
                                        in FP64 */
#define JPET_PRECISION_FIXED 3       /* deterministic tiles: each contribution rounded once to
                                        2^-22 of an event (unbiased per-event dither) and
                                        summed with integer shared atomics; FP64 image */

/* iteration kernel */
#define JPET_VARIANT_FAST 0  /* exp2-form kernel, packed f32x2, register-cached K*rho (default) */
#define JPET_VARIANT_EXACT 1 /* every pixel evaluated in the reference's operation order */

typedef struct jpet_strip_opts {
  int32_t device;       /* CUDA device ordinal (-D / --cuda-device) */
  int32_t mode;         /* JPET_MODE_* */
  int32_t precision;    /* JPET_PRECISION_* */
  int32_t tile_w;       /* image tile width in pixels, 0 = chosen by the tuner */
  int32_t tile_h;       /* image tile height in pixels, 0 = chosen by the tuner */
  int32_t block_threads;/* threads per CTA of the iteration kernel, 0 = tuned */
  int32_t variant;      /* JPET_VARIANT_*; the GPU-reference mode always runs EXACT */
  int32_t reserved[9];  /* must be zero */
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
 * d_rho_in / d_rho_out: different device float[n_y*n_z] images; the output is
 * cleared by the call.  Work runs on cuda_stream (a cudaStream_t, NULL = the
 * default stream) in the reference's CPU float semantics and operation order;
 * no handle is involved.  The per-event working data live in one fixed 24 MiB
 * device array of the library, which every GPU that loads the library keeps
 * until the process exits; calls share it, so calls that overlap on the GPU
 * (different streams or unordered host threads) race, while calls ordered on
 * one stream do not.  The first call on a device looks up the array's address
 * with that device current; make that first call before any stream capture.
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

#ifdef __cplusplus
}
#endif
#endif
