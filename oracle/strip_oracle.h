/* CPU restatement of the reference's 2D strip-PET list-mode MLEM path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py load this library, and only to verify results or as
 * the timed CPU baseline; the product never links or calls it.
 *
 * Every function restates one reference function, in the reference's own
 * floating-point evaluation order, so that a single-threaded run is
 * bit-identical to the reference's CPU float path (checked against the
 * reference binary built by build_ref.sh and against the committed golden
 * images in tests/golden/).  Citations are file:line in grey277/j-pet-mlem.
 */
#ifndef JPET_STRIP_ORACLE_H
#define JPET_STRIP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scanner parameters in the argument order of Scanner's constructor
 * (src/2d/strip/scanner.h:39-49), centre at the origin. */
typedef struct orc_geom {
  double radius;
  double scintillator_length;
  int32_t n_y_pixels;
  int32_t n_z_pixels;
  double pixel_height;
  double pixel_width;
  double sigma_z;
  double sigma_dl;
} orc_geom;

/* Statistics of one iteration (the reference's ReconstructionStats counters,
 * src/2d/strip/reconstruction_stats.h:7-89). */
typedef struct orc_stats {
  int64_t n_events;         /* events processed */
  int64_t n_pixels;         /* bounding-box pixels visited */
  int64_t n_kernel_calls;   /* in-ellipse kernel evaluations */
  int64_t n_contributing;   /* events with a positive denominator */
} orc_stats;

/* --- per-function restatements (float, F = float as in src/common/types.h:6) --- */
void orc_response_tan_y_z_f(float R, float z_u, float z_d, float dl,
                            float* tan, float* y, float* z);
void orc_kernel_constants_f(float sigma_z, float sigma_dl, float* inv_pow_sigma_z,
                            float* inv_pow_sigma_dl, float* c0);
void orc_ellipse_bb_f(float sigma_z, float sigma_dl, float tan, float* sec,
                      float* A, float* B, float* C, float* bb_y, float* bb_z);
float orc_bb_y_d(double A, double C, double B_2);
float orc_bb_z_d(double A, double C, double B_2);
double orc_bb_y_dd(double A, double C, double B_2);
double orc_bb_z_dd(double A, double C, double B_2);
float orc_gaussian_kernel_f(float sigma_z, float sigma_dl, float y, float tan,
                            float sec, float R, float dz, float dy);
double orc_gaussian_kernel_d(double sigma_z, double sigma_dl, double y, double tan,
                             double sec, double R, double dz, double dy);
double orc_analytic_kernel_d(double sigma_z, double sigma_dl, double y, double tan,
                             double sec, double R, double dz, double dy);
float orc_analytic_kernel_f(float sigma_z, float sigma_dl, float y, float tan,
                            float sec, float R, float dz, float dy);
void orc_pixel_at_d(const orc_geom* g, double z, double y, int32_t* px, int32_t* py);
void orc_pixel_center_d(const orc_geom* g, int32_t px, int32_t py, double* z, double* y);
double orc_sensitivity_d(const orc_geom* g, double z, double y);
float orc_sensitivity_f(const orc_geom* g, float z, float y);
float orc_pixel_sensitivity_f(const orc_geom* g, int32_t px, int32_t py);
void orc_to_projection_space_tan_d(double R, double y, double z, double tan,
                                   double* z_u, double* z_d, double* dl);

/* Sensitivity images, float32[n_y][n_z].
 * kind 0: point sensitivity at pixel centres (reconstruction.h:67-73).
 * kind 1: 5-point pixel sensitivity (scanner.h:174-185, cuda/reconstruction.cu:115-126). */
void orc_sensitivity_map_f(const orc_geom* g, int kind, float* out);
/* Naive image and tangent-binned map of smeared responses in the phantom
 * tool's float arithmetic (phantom_cmd.cpp:241-253,339-352). */
void orc_naive_bins_f(const orc_geom* g, const float* ev, int64_t n, double ox, double oy,
                      int32_t bins, int32_t* naive, int32_t* tan_map);
/* The phantom tool's --tan-bins kernel map (phantom_cmd.cpp:396-430). */
void orc_tan_kernel_map_f(const orc_geom* g, int32_t bins, double kx, double ky, double ox,
                          double oy, int32_t divide, float* out);

/* Bounding box of one event after clamping (reconstruction.h:223-246);
 * returns in-ellipse pixel count; box = [tl_x, br_x) x [tl_y, br_y). */
int32_t orc_event_box_f(const orc_geom* g, float z_u, float z_d, float dl,
                        int32_t* tl_x, int32_t* tl_y, int32_t* br_x, int32_t* br_y);

/* One or more MLEM iterations of the reference CPU float path
 * (reconstruction.h:108-154 with bb_update :220-298).
 * events: AoS float32 triples (z_u, z_d, dl), n events.
 * rho: float32[n_y*n_z], in/out.  n_threads <= 0 means all OpenMP threads.
 * Per-thread private images summed in thread order, as the reference does. */
int orc_mlem_f(const orc_geom* g, const float* events, int64_t n, float* rho,
               int n_iterations, int n_threads, orc_stats* stats);

/* The same algorithm instantiated at double (Reconstruction<double,...>);
 * events are widened from float32; rho is float64. */
int orc_mlem_d(const orc_geom* g, const float* events, int64_t n, double* rho,
               int n_iterations, int n_threads, orc_stats* stats);

/* The reference GPU kernel's semantics (cuda/reconstruction/warp_granularity.cuh:19-155):
 * AnalyticKernel (analytic_kernel.h:28-62) and a denominator weighted by the
 * 5-point pixel sensitivity; the back-projection is not divided by it.
 * pixel_sensitivity: float32[n_y*n_z] or NULL to compute kind 1 internally.
 * Accumulates in double per event (an oracle, not a bit-exact restatement). */
int orc_mlem_gpuref(const orc_geom* g, const float* events, int64_t n, float* rho,
                    int n_iterations, int n_threads, const float* pixel_sensitivity);

/* Poisson list-mode negative log-likelihood in FP64 and its gradient.
 *   L(rho, sigma) = sum_p s_p rho_p - sum_e log(sum_{p in E_e} K_e(p; sigma) rho_p)
 * K is the Gaussian kernel (gaussian_kernel.h:51-79) with its normalisation
 * constant c0(sigma) included.  The support E_e is the 3-sigma ellipse computed
 * with (support_sigma_z, support_sigma_dl), held fixed under differentiation.
 * s: float32[n_y*n_z] (NULL = point sensitivity, kind 0).
 * grad_rho: float64[n_y*n_z] or NULL; grad_sigma: float64[2] (d/d sigma_z, d/d sigma_dl) or NULL.
 * Events with an empty support or a zero denominator are skipped and counted. */
double orc_nll_grad(const orc_geom* g, double support_sigma_z, double support_sigma_dl,
                    const float* events, int64_t n, const float* rho, const float* s,
                    double* grad_rho, double* grad_sigma, int n_threads,
                    int64_t* n_skipped);

/* ---- 3D hybrid reconstruction (src/3d/hybrid/reconstruction.h) ----------------
 * Float instantiation with S = short, one plane half (n_planes_half = 1) and the
 * 2D sensitivity: the reference command's default flow (reconstruction_cmd.cpp:
 * 462-541) without --sensitivity. */

/* PET2D::LineSegment<float> fields in declaration order (line_segment.h:87-93). */
typedef struct orc_segment {
  float start_x, start_y, end_x, end_y, mid_x, mid_y, dir_x, dir_y, normal_x, normal_y;
  float length, distance_from_origin;
} orc_segment;

/* PET2D::Pixel<short> (pixel.h:18). */
typedef struct orc_pixel {
  int16_t x, y;
} orc_pixel;

/* Hybrid Scanner::Response (3d/hybrid/scanner.h:71-76): LOR (first, second),
 * z_up, z_dn, dl. */
typedef struct orc_hybrid_response {
  int16_t first, second;
  float z_up, z_dn, dl;
} orc_hybrid_response;

/* Reconstruction::FrameEvent (reconstruction.h:53-63) with F = float, S = short
 * and 64-bit size_t: the explicit pads are the compiler's alignment padding. */
typedef struct orc_frame_event {
  int16_t first, second;
  float up, right, tan, sec;
  uint32_t pad0;
  uint64_t info_begin, info_end;
  int16_t plane_begin, plane_end;
  uint32_t pad1;
} orc_frame_event;

/* GeometrySOA arrays (2d/barrel/geometry_soa.h:268-283), the voxel grid
 * (3d/geometry/voxel_grid.h:22-26 over pixel_grid.h:22-30) and the scanner
 * quantities Reconstruction reads (sigma_z(), sigma_dl(), length). */
typedef struct orc_hybrid {
  int32_t n_detectors;          /* n_lors = (n + 1) n / 2 */
  int64_t n_pixel_infos;
  const orc_segment* segments;  /* [n_lors] */
  const float* lor_widths;      /* [n_lors] */
  const orc_pixel* pixels;      /* [n_pixel_infos] */
  const float* positions;       /* [n_pixel_infos], ascending within each LOR */
  const uint64_t* info_begin;   /* [n_lors] */
  const uint64_t* info_end;     /* [n_lors] */
  int32_t n_columns, n_rows, n_planes;
  float pixel_size, lower_left_x, lower_left_y, z_left;
  float sigma_z, sigma_dl, length;
  /* GeometrySOA::n_planes_half (geometry_soa.h:283): planes of weights, each
   * n_pixel_infos long (plane-major); > 1: the multi-plane system matrix */
  int32_t n_planes_half;
  /* depth of the sensitivity image (reconstruction.h:80-85): n_planes_half when
   * > 1, else n_planes / 2 with an external 3D sensitivity, else 1 */
  int32_t sens_depth;
} orc_hybrid;

void orc_hybrid_calculate_weight(const orc_hybrid* g, float* weights);
void orc_hybrid_calculate_sensitivity(const orc_hybrid* g, const float* weights, float* sens);
void orc_hybrid_normalize(const orc_hybrid* g, float* weights, const float* sens);
int orc_hybrid_translate(const orc_hybrid* g, const orc_hybrid_response* r, const float* weights,
                         orc_frame_event* e);
int64_t orc_hybrid_translate_all(const orc_hybrid* g, const orc_hybrid_response* r, int64_t n,
                                 const float* weights, orc_frame_event* out);
int orc_hybrid_mlem(const orc_hybrid* g, const float* weights, const float* sens,
                    const orc_frame_event* ev, int64_t n, float* rho, int n_iterations,
                    int n_threads, int64_t* counters);

#ifdef __cplusplus
}
#endif
#endif
