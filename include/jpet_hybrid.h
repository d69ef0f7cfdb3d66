/* C ABI of the GB300 3D hybrid list-mode MLEM (barrel LORs x strip TOF along z).
 *
 * Replaces the reference's GPU entry point for the 3D hybrid reconstruction,
 *   PET3D::Hybrid::GPU::Reconstruction::run   (src/3d/hybrid/cuda/reconstruction.h:41-58,
 *                                              src/3d/hybrid/cuda/reconstruction.cu:36-187)
 * whose kernel is src/3d/hybrid/cuda/reconstruction/warp_granularity.cuh:28-178, and
 * the CPU set-up around it that 3d_hybrid_reconstruction runs first
 * (src/3d/hybrid/reconstruction_cmd.cpp:462-541): Reconstruction::calculate_weight,
 * calculate_sensitivity / set_sensitivity_to_one, normalize_geometry_weights and
 * translate_to_frame with the bounding-box filter (src/3d/hybrid/reconstruction.h:
 * 101-162, 218-274).  One iteration is Reconstruction::operator()
 * (reconstruction.h:276-446) in each of its three forms: one plane half with the
 * 2D sensitivity (one system matrix, no --sensitivity), one system matrix per
 * plane half with the 3D sensitivity (n_planes_half > 1), and one plane half
 * with an external 3D sensitivity (--sensitivity).  In the last two the voxels
 * of plane iz read the weights and sensitivity of plane |iz - depth| (depth =
 * n_planes_half or the sensitivity's depth); for plane 0 the reference's index
 * is one plane past its arrays, and it is clamped to the last plane here.
 *
 * Plain C: pointers, sizes and the structs below, whose layouts are those of the
 * reference's own types with F = float, S = short and a 64-bit size_t, so that a
 * caller holding the reference's arrays can pass them as they are.  All entry
 * points return JPET_OK or a negative JPET_ERR_* code of jpet_strip.h;
 * jpet_hybrid_last_error gives the message.  The work of a handle runs on its
 * CUDA stream; calls on one handle must not overlap.
 */
#ifndef JPET_HYBRID_H
#define JPET_HYBRID_H

#include <stddef.h>
#include <stdint.h>

#include "jpet_strip.h"

#ifdef __cplusplus
extern "C" {
#endif

/* PET2D::LineSegment<float> (src/2d/geometry/line_segment.h:87-93). */
typedef struct jpet_lor_segment {
  float start_x, start_y, end_x, end_y;
  float mid_x, mid_y;
  float direction_x, direction_y;
  float normal_x, normal_y;
  float length;
  float distance_from_origin;
} jpet_lor_segment;

/* PET2D::Pixel<short> (src/2d/geometry/pixel.h:18). */
typedef struct jpet_pixel {
  int16_t x, y;
} jpet_pixel;

/* PET3D::Hybrid::Scanner::Response (src/3d/hybrid/scanner.h:71-76): the LOR
 * (first, second) as read, z at the first detector, z at the second, and the
 * difference of the two path lengths. */
typedef struct jpet_hybrid_response {
  int16_t lor_first, lor_second;
  float z_up, z_dn, dl;
} jpet_hybrid_response;

/* Reconstruction::FrameEvent (src/3d/hybrid/reconstruction.h:53-63): the event
 * in its LOR's frame, the half-open range of pixel infos and of planes it
 * touches.  The pads are the compiler's alignment padding of the reference
 * struct (48 bytes). */
typedef struct jpet_hybrid_frame_event {
  int16_t lor_first, lor_second;
  float up, right, tan, sec;
  uint32_t pad0;
  uint64_t pixel_info_begin, pixel_info_end;
  int16_t plane_begin, plane_end;
  uint32_t pad1;
} jpet_hybrid_frame_event;

/* Host arrays of PET2D::Barrel::GeometrySOA<float, short>
 * (src/2d/barrel/geometry_soa.h:268-283), the voxel grid
 * (PET3D::VoxelGrid over PET2D::PixelGrid, src/3d/geometry/voxel_grid.h:22-26,
 * src/2d/geometry/pixel_grid.h:22-30) and the scanner values the reconstruction
 * reads (sigma_z(), sigma_dl(), length).  Lengths in the reference's unit. */
typedef struct jpet_hybrid_geom {
  int32_t n_detectors;                     /* n_lors = (n + 1) n / 2, n <= 32767 */
  int64_t n_pixel_infos;                   /* < 2^31 */
  const jpet_lor_segment* lor_segments;    /* [n_lors] */
  const float* lor_widths;                 /* [n_lors] (used by computed weights) */
  const jpet_pixel* pixels;                /* [n_pixel_infos], each inside the grid */
  const float* pixel_positions;            /* [n_pixel_infos], ascending within a LOR */
  const float* pixel_weights;              /* [n_planes_half * n_pixel_infos] (given weights,
                                              plane-major as GeometrySOA stores them), or NULL */
  const uint64_t* lor_pixel_info_begin;    /* [n_lors] */
  const uint64_t* lor_pixel_info_end;      /* [n_lors] */
  int32_t n_columns, n_rows;               /* pixel grid */
  float pixel_size;
  float lower_left_x, lower_left_y;        /* PixelGrid::lower_left */
  int32_t n_planes;                        /* voxels along z */
  float z_left;                            /* VoxelGrid::z_left */
  float sigma_z, sigma_dl;                 /* TOF widths of the strip kernel */
  float length;                            /* scanner length */
  int32_t n_planes_half;                   /* GeometrySOA::n_planes_half: 0 or 1 = one plane
                                              half; > 1 = one system matrix per plane half
                                              (the command loads n_planes / 2 of them) */
} jpet_hybrid_geom;

/* Where the pixel weights come from. */
#define JPET_HYBRID_WEIGHTS_COMPUTED 0   /* calculate_weight (reconstruction.h:218-238): the
                                            command without --system */
#define JPET_HYBRID_WEIGHTS_GIVEN 1      /* geom->pixel_weights as loaded (--system); normalized */
#define JPET_HYBRID_WEIGHTS_NORMALIZED 2 /* geom->pixel_weights already normalized: used as
                                            they are (what GPU::Reconstruction::run receives) */
/* Where the 2D sensitivity comes from. */
#define JPET_HYBRID_SENSITIVITY_COMPUTED 0 /* calculate_sensitivity (reconstruction.h:240-251),
                                              summed in pixel-info order */
#define JPET_HYBRID_SENSITIVITY_ONE 1      /* set_sensitivity_to_one (--sens-to-one) */
#define JPET_HYBRID_SENSITIVITY_GIVEN 2    /* opts->sensitivity_map, float[n_rows * n_columns] */
#define JPET_HYBRID_SENSITIVITY_GIVEN_3D 3 /* opts->sensitivity_map, the external 3D sensitivity
                                              (--sensitivity): float[depth][n_rows][n_columns],
                                              depth = n_planes_half if > 1, else n_planes / 2 */
/* With n_planes_half > 1 the sensitivity is 3D (depth n_planes_half): COMPUTED sums
 * each plane half's weights (reconstruction.h:240-251), ONE fills it, GIVEN_3D
 * takes it; the weights must be given (GIVEN or NORMALIZED). */

typedef struct jpet_hybrid_opts {
  int32_t device;              /* CUDA device ordinal */
  int32_t weights;             /* JPET_HYBRID_WEIGHTS_* */
  int32_t sensitivity;         /* JPET_HYBRID_SENSITIVITY_* */
  const float* sensitivity_map;/* host sensitivity for SENSITIVITY_GIVEN / GIVEN_3D */
  int32_t block_threads;       /* CTA size of the iteration kernel (0 = default, multiple of 32) */
  int32_t reserved;
} jpet_hybrid_opts;

typedef struct jpet_hybrid_counters {
  int64_t used_events;   /* events of the last iteration (Statistics::used_events) */
  int64_t used_pixels;   /* pixel infos visited (Statistics::used_pixels) */
  int64_t used_voxels;   /* voxels visited (Statistics::used_voxels) */
  int64_t contributing;  /* events with a positive denominator */
} jpet_hybrid_counters;

typedef struct jpet_hybrid jpet_hybrid_t;

/* Defaults: device 0, computed weights and sensitivity, default CTA. */
void jpet_hybrid_default_opts(jpet_hybrid_opts* opts);

/* Uploads the geometry, computes or takes the weights and the sensitivity and
 * normalizes the weights (reconstruction.h:218-274, on the device; the
 * sensitivity is summed per pixel in pixel-info order, as the reference does).
 * The image after create is all ones (reconstruction.h:71-90). */
int jpet_hybrid_create(const jpet_hybrid_geom* geom, const jpet_hybrid_opts* opts,
                       jpet_hybrid_t** out);
int jpet_hybrid_destroy(jpet_hybrid_t* h);
/* Message of the last failed call on h (or of the last failed create when h is NULL). */
const char* jpet_hybrid_last_error(const jpet_hybrid_t* h);
/* Uses the given cudaStream_t for later work (NULL = the handle's own stream). */
int jpet_hybrid_set_stream(jpet_hybrid_t* h, void* cuda_stream);

/* Host responses: translate_to_frame and the bounding-box filter on the device
 * (reconstruction.h:101-162, as operator<< keeps events, :190-212); kept events
 * stay in input order.  The pixel-info range ends one past std::upper_bound as
 * in the reference; where that passes the geometry's last pixel info it is
 * clamped (the reference reads past its array there).  Responses whose LOR
 * index is not below n_lors are dropped (the reference reads past its arrays). */
int jpet_hybrid_set_responses(jpet_hybrid_t* h, const jpet_hybrid_response* responses, int64_t n);
/* Same from device memory. */
int jpet_hybrid_set_responses_device(jpet_hybrid_t* h, const jpet_hybrid_response* d_responses,
                                     int64_t n);
/* Host frame events as GPU::Reconstruction::run receives them; each is checked
 * (LOR index, info range within the geometry, planes within the grid). */
int jpet_hybrid_set_frame_events(jpet_hybrid_t* h, const jpet_hybrid_frame_event* events,
                                 int64_t n);
/* Number of events held; with out != NULL also copies them (host, n entries). */
int jpet_hybrid_get_frame_events(jpet_hybrid_t* h, jpet_hybrid_frame_event* out, int64_t* n);

/* Image in the reference's voxel order, index x + n_columns (y + n_rows z)
 * (voxel_grid.h:54-56), host float[n_columns * n_rows * n_planes]. */
int jpet_hybrid_set_image(jpet_hybrid_t* h, const float* rho);
int jpet_hybrid_get_image(jpet_hybrid_t* h, float* rho);
/* The sensitivity (host float[depth * n_columns * n_rows], depth 1 for the 2D
 * sensitivity) and the normalized pixel weights (host
 * float[n_planes_half * n_pixel_infos]). */
int jpet_hybrid_get_sensitivity(jpet_hybrid_t* h, float* sens);
int jpet_hybrid_get_weights(jpet_hybrid_t* h, float* weights);

/* n MLEM iterations on the device (asynchronous on the handle's stream). */
int jpet_hybrid_iterate(jpet_hybrid_t* h, int n);
/* Counters of the last iteration (synchronises). */
int jpet_hybrid_get_counters(jpet_hybrid_t* h, jpet_hybrid_counters* out);
int jpet_hybrid_synchronize(jpet_hybrid_t* h);

/* The reference GPU entry point over host buffers (cuda/reconstruction.cu:36-187):
 * geometry with normalized weights, the sensitivity (2D, or 3D of depth
 * n_planes_half for a multi-plane geometry), frame events, and rho
 * (in/out, reference voxel order); runs n_blocks * n_iterations_in_block
 * iterations, skipping those below start_iteration, and calls
 * output(iteration, image, user) where the reference does (after the first 5
 * iterations and the 10th, 15th, 20th, 30th, 50th and 100th of the first
 * block, and after every block) and progress(completed, finished, user)
 * around every iteration.  device_name (may be NULL) receives the device's name. */
typedef void (*jpet_hybrid_output_fn)(int iteration, const float* image, void* user);
int jpet_hybrid_run(const jpet_hybrid_geom* geom, const float* sensitivity,
                    const jpet_hybrid_frame_event* events, int64_t n_events, float* rho,
                    int n_blocks, int n_iterations_in_block, int start_iteration,
                    jpet_hybrid_output_fn output, jpet_strip_progress_fn progress, void* user,
                    int device, char* device_name, size_t device_name_len);

#ifdef __cplusplus
}
#endif
#endif
