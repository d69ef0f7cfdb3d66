/* CPU restatement of the reference's 2D strip-PET list-mode MLEM path.
 * TEST INFRASTRUCTURE ONLY (see strip_oracle.h): loaded by tests/, smoke() and
 * the CPU-baseline leg of bench.py; never by the product.
 *
 * Compiled with -ffp-contract=off and without fast-math so the float
 * instantiation keeps the reference's evaluation order and rounding (the
 * reference builds as ISO C++11, where GCC does not contract FMAs). */
#define _GNU_SOURCE
#include "strip_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#else
static int omp_get_max_threads(void) { return 1; }
static int omp_get_thread_num(void) { return 0; }
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_1_PI
#define M_1_PI 0.31830988618379067154
#endif

#define REAL float
#define SFX _f
#define SQRT sqrtf
#define EXP expf
#define ATAN atanf
#include "strip_oracle_mlem.inc"
#include "hybrid_oracle.inc"
#undef REAL
#undef SFX
#undef SQRT
#undef EXP
#undef ATAN

#define REAL double
#define SFX _d
#define SQRT sqrt
#define EXP exp
#define ATAN atan
#include "strip_oracle_mlem.inc"
#undef REAL
#undef SFX
#undef SQRT
#undef EXP
#undef ATAN

/* ---------------- per-function entry points (known-answer tests) ---------------- */

void orc_response_tan_y_z_f(float R, float z_u, float z_d, float dl, float* tan,
                            float* y, float* z) {
  tan_y_z_f(R, z_u, z_d, dl, tan, y, z);
}

void orc_kernel_constants_f(float sigma_z, float sigma_dl, float* ipz, float* ipd,
                            float* c0) {
  orc_kernel_f k;
  kernel_init_f(sigma_z, sigma_dl, &k);
  *ipz = k.ipz;
  *ipd = k.ipd;
  *c0 = k.c0;
}

void orc_ellipse_bb_f(float sigma_z, float sigma_dl, float tan, float* sec, float* A,
                      float* B, float* C, float* bb_y, float* bb_z) {
  orc_kernel_f k;
  kernel_init_f(sigma_z, sigma_dl, &k);
  ellipse_bb_f(&k, tan, sec, A, B, C, bb_y, bb_z);
}

/* GaussianKernel::bb_y / bb_z (gaussian_kernel.h:159-160). */
float orc_bb_y_d(double A, double C, double B_2) { return (float)(3 / sqrt(A - (B_2 / C))); }
float orc_bb_z_d(double A, double C, double B_2) { return (float)(3 / sqrt(C - (B_2 / A))); }
double orc_bb_y_dd(double A, double C, double B_2) { return 3 / sqrt(A - (B_2 / C)); }
double orc_bb_z_dd(double A, double C, double B_2) { return 3 / sqrt(C - (B_2 / A)); }

float orc_gaussian_kernel_f(float sigma_z, float sigma_dl, float y, float tan, float sec,
                            float R, float dz, float dy) {
  orc_kernel_f k;
  kernel_init_f(sigma_z, sigma_dl, &k);
  return gauss_f(&k, y, tan, sec, R, dz, dy);
}

double orc_gaussian_kernel_d(double sigma_z, double sigma_dl, double y, double tan,
                             double sec, double R, double dz, double dy) {
  orc_kernel_d k;
  kernel_init_d(sigma_z, sigma_dl, &k);
  return gauss_d(&k, y, tan, sec, R, dz, dy);
}

double orc_analytic_kernel_d(double sigma_z, double sigma_dl, double y, double tan,
                             double sec, double R, double dz, double dy) {
  orc_kernel_d k;
  kernel_init_d(sigma_z, sigma_dl, &k);
  return analytic_d(&k, y, tan, sec, R, dz, dy);
}

float orc_analytic_kernel_f(float sigma_z, float sigma_dl, float y, float tan, float sec,
                            float R, float dz, float dy) {
  orc_kernel_f k;
  kernel_init_f(sigma_z, sigma_dl, &k);
  return analytic_f(&k, y, tan, sec, R, dz, dy);
}

/* Scanner::pixel_at (scanner.h:142-144), double instantiation as in scanner_test.cpp. */
void orc_pixel_at_d(const orc_geom* g, double z, double y, int32_t* px, int32_t* py) {
  orc_scanner_d s;
  scanner_init_d(g, &s);
  *px = to_short_d((z - s.tl_z) / s.pixel_width);
  *py = to_short_d((s.tl_y - y) / s.pixel_height);
}

/* Scanner::pixel_center (scanner.h:136-139). */
void orc_pixel_center_d(const orc_geom* g, int32_t px, int32_t py, double* z, double* y) {
  orc_scanner_d s;
  scanner_init_d(g, &s);
  *z = s.tl_z_half_w + (int16_t)px * s.pixel_width;
  *y = s.tl_y_half_h - (int16_t)py * s.pixel_height;
}

double orc_sensitivity_d(const orc_geom* g, double z, double y) {
  orc_scanner_d s;
  scanner_init_d(g, &s);
  return sens_d(&s, z, y);
}

float orc_sensitivity_f(const orc_geom* g, float z, float y) {
  orc_scanner_f s;
  scanner_init_f(g, &s);
  return sens_f(&s, z, y);
}

float orc_pixel_sensitivity_f(const orc_geom* g, int32_t px, int32_t py) {
  orc_scanner_f s;
  scanner_init_f(g, &s);
  return pixel_sens_f(&s, (int16_t)px, (int16_t)py);
}

/* Scanner::to_projection_space_tan (scanner.h:107-113). */
void orc_to_projection_space_tan_d(double R, double y, double z, double tan,
                                   double* z_u, double* z_d, double* dl) {
  *z_u = z + (R - y) * tan;
  *z_d = z - (R + y) * tan;
  *dl = -2 * y * sqrt(tan * tan + 1);
}

void orc_sensitivity_map_f(const orc_geom* g, int kind, float* out) {
  orc_scanner_f s;
  scanner_init_f(g, &s);
  for (int y = 0; y < s.n_y; ++y)
    for (int x = 0; x < s.n_z; ++x) {
      float v;
      if (kind == 0) {
        float cx = s.tl_z_half_w + (int16_t)x * s.pixel_width;
        float cy = s.tl_y_half_h - (int16_t)y * s.pixel_height;
        v = sens_f(&s, cx, cy);
      } else {
        v = pixel_sens_f(&s, (int16_t)x, (int16_t)y);
      }
      out[y * s.n_z + x] = v;
    }
}

/* The phantom tool's float grids (phantom_cmd.cpp:241-253): PixelGrid lower-left
 * corner Point<F>(-s n_z / 2, -s n_y / 2) + origin, pixel size F(s); tangent
 * planes of VariableVoxelSizeVoxelGrid(pixel_grid, -max_tan, bins,
 * max_tan / bins * 2) with max_tan = (F)1.1 L / (2 R) (scanner fields float). */
typedef struct {
  float x0, y0, s, tan_left, tan_size;
} tan_grid_f;

static tan_grid_f tan_grid_init(const orc_geom* g, int bins, double ox, double oy) {
  tan_grid_f t;
  t.s = (float)g->pixel_width;
  t.x0 = (float)(-g->pixel_width * g->n_z_pixels / 2) + (float)ox;
  t.y0 = (float)(-g->pixel_width * g->n_y_pixels / 2) + (float)oy;
  float max_tan = (float)1.1 * (float)g->scintillator_length / (2 * (float)g->radius);
  t.tan_left = -max_tan;
  t.tan_size = bins > 0 ? max_tan / bins * 2 : 0.0f;
  return t;
}

/* Naive image and tangent-binned map of smeared responses (phantom_cmd.cpp:
 * 339-352): from_projection_space_tan (scanner.h:122-127, response.h:22-37),
 * PixelGrid::pixel_at (pixel_grid.h:59-64) and
 * VariableVoxelSizeVoxelGrid::voxel_at (voxel_grid.h:109-118), all in float;
 * voxel index (plane * n_y + row) * n_z + column (voxel.h:27-29).  naive and
 * tan_map (bins > 0) may be NULL; both are accumulated into. */
void orc_naive_bins_f(const orc_geom* g, const float* ev, int64_t n, double ox, double oy,
                      int32_t bins, int32_t* naive, int32_t* tan_map) {
  const tan_grid_f t = tan_grid_init(g, bins, ox, oy);
  const float R = (float)g->radius;
  const int nz = g->n_z_pixels, ny = g->n_y_pixels;
  for (int64_t i = 0; i < n; ++i) {
    float tan, y, z;
    tan_y_z_f(R, ev[3 * i], ev[3 * i + 1], ev[3 * i + 2], &tan, &y, &z);
    float fc = floorf((z - t.x0) / t.s), fr = floorf((y - t.y0) / t.s);
    if (!(fc >= 0 && fc < nz && fr >= 0 && fr < ny)) continue;
    int64_t pix = (int64_t)fr * nz + (int64_t)fc;
    if (naive) naive[pix] += 1;
    if (tan_map && bins > 0) {
      float fp = floorf((tan - t.tan_left) / t.tan_size);
      if (fp >= 0 && fp < bins) tan_map[(int64_t)fp * ny * nz + pix] += 1;
    }
  }
}

/* The --tan-bins kernel map (phantom_cmd.cpp:396-430), float: for every voxel
 * the tangent of the plane centre (voxel_grid.h:105-107), sec, the pixel
 * centre (pixel_grid.h:54-57), AnalyticKernel at the kernel point
 * (analytic_kernel.h:65-74), the volume element 4 R pixel^2 dtan sqrt(1+tan^2)
 * and the inverse sensitivity at the kernel point when divide (the
 * reference's --detected). */
void orc_tan_kernel_map_f(const orc_geom* g, int32_t bins, double kx_d, double ky_d, double ox,
                          double oy, int32_t divide, float* out) {
  const tan_grid_f t = tan_grid_init(g, bins, ox, oy);
  orc_kernel_f k;
  kernel_init_f((float)g->sigma_z, (float)g->sigma_dl, &k);
  orc_scanner_f sc;
  scanner_init_f(g, &sc);
  const float kx = (float)kx_d, ky = (float)ky_d, R = (float)g->radius;
  const float inv_sens = divide ? 1 / sens_f(&sc, kx, ky) : (float)1;
  const float llcx = t.x0 + t.s / 2, llcy = t.y0 + t.s / 2;
  const float bin_volume = t.s * t.s * t.tan_size;
  const int nz = g->n_z_pixels, ny = g->n_y_pixels;
  for (int z = 0; z < bins; ++z) {
    float tan = ((int16_t)z + (float)0.5) * t.tan_size + t.tan_left;
    float sec = sqrtf(1 + tan * tan);
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nz; ++x) {
        float cx = llcx + (int16_t)x * t.s, cy = llcy + (int16_t)y * t.s;
        float kv = analytic_f(&k, cy, tan, sec, R, kx - cx, ky - cy);
        float volume_elem = 4 * R * bin_volume * sqrtf(1 + tan * tan);
        out[((int64_t)z * ny + y) * nz + x] = kv * volume_elem * inv_sens;
      }
  }
}

int32_t orc_event_box_f(const orc_geom* g, float z_u, float z_d, float dl, int32_t* tl_x,
                        int32_t* tl_y, int32_t* br_x, int32_t* br_y) {
  orc_scanner_f s;
  orc_kernel_f k;
  orc_box_f b;
  scanner_init_f(g, &s);
  kernel_init_f(s.sigma_z, s.sigma_dl, &k);
  event_box_f(&s, &k, z_u, z_d, dl, &b);
  *tl_x = b.tl_x;
  *tl_y = b.tl_y;
  *br_x = b.br_x;
  *br_y = b.br_y;
  int32_t count = 0;
  for (int iy = b.tl_y; iy < b.br_y; ++iy)
    for (int iz = b.tl_x; iz < b.br_x; ++iz) {
      float px = s.tl_z_half_w + (int16_t)iz * s.pixel_width;
      float py = s.tl_y_half_h - (int16_t)iy * s.pixel_height;
      float dy = py - b.y, dz = px - b.z;
      if ((b.A * dy * dy) + (b.B * dy * dz) + (b.C * dz * dz) <= 9) ++count;
    }
  return count;
}

int orc_mlem_f(const orc_geom* g, const float* events, int64_t n, float* rho,
               int n_iterations, int n_threads, orc_stats* stats) {
  return mlem_f(g, events, n, rho, n_iterations, n_threads, stats);
}

int orc_mlem_d(const orc_geom* g, const float* events, int64_t n, double* rho,
               int n_iterations, int n_threads, orc_stats* stats) {
  return mlem_d(g, events, n, rho, n_iterations, n_threads, stats);
}

/* ---------------- reference GPU-kernel semantics ---------------- */

int orc_mlem_gpuref(const orc_geom* g, const float* events, int64_t n, float* rho,
                    int n_iterations, int n_threads, const float* pixel_sensitivity) {
  orc_scanner_f s;
  orc_kernel_f k;
  scanner_init_f(g, &s);
  kernel_init_f(s.sigma_z, s.sigma_dl, &k);
  const int64_t n_pix = (int64_t)s.n_y * s.n_z;
  float* sens = (float*)malloc((size_t)n_pix * sizeof(float));
  if (!sens) return -1;
  if (pixel_sensitivity)
    memcpy(sens, pixel_sensitivity, (size_t)n_pix * sizeof(float));
  else
    orc_sensitivity_map_f(g, 1, sens);
  int T = n_threads > 0 ? n_threads : omp_get_max_threads();
  double* images = (double*)malloc((size_t)T * n_pix * sizeof(double));
  if (!images) {
    free(sens);
    return -1;
  }
  for (int it = 0; it < n_iterations; ++it) {
    memset(images, 0, (size_t)T * n_pix * sizeof(double));
#pragma omp parallel for schedule(dynamic, 64) num_threads(T)
    for (int64_t e = 0; e < n; ++e) {
      double* out = images + (int64_t)omp_get_thread_num() * n_pix;
      orc_box_f b;
      event_box_f(&s, &k, events[3 * e], events[3 * e + 1], events[3 * e + 2], &b);
      double den = 0;
      for (int iy = b.tl_y; iy < b.br_y; ++iy)
        for (int iz = b.tl_x; iz < b.br_x; ++iz) {
          float px = s.tl_z_half_w + (int16_t)iz * s.pixel_width;
          float py = s.tl_y_half_h - (int16_t)iy * s.pixel_height;
          float dy = py - b.y, dz = px - b.z;
          if ((b.A * dy * dy) + (b.B * dy * dz) + (b.C * dz * dz) <= 9) {
            int64_t pi = (int64_t)iy * s.n_z + iz;
            float kv = analytic_f(&k, b.y, b.tan, b.sec, s.radius, dz, dy);
            den += (double)(kv * rho[pi]) * sens[pi];
          }
        }
      if (!(den > 0)) continue;
      double inv = 1.0 / den;
      for (int iy = b.tl_y; iy < b.br_y; ++iy)
        for (int iz = b.tl_x; iz < b.br_x; ++iz) {
          float px = s.tl_z_half_w + (int16_t)iz * s.pixel_width;
          float py = s.tl_y_half_h - (int16_t)iy * s.pixel_height;
          float dy = py - b.y, dz = px - b.z;
          if ((b.A * dy * dy) + (b.B * dy * dz) + (b.C * dz * dz) <= 9) {
            int64_t pi = (int64_t)iy * s.n_z + iz;
            float kv = analytic_f(&k, b.y, b.tan, b.sec, s.radius, dz, dy);
            out[pi] += (double)(kv * rho[pi]) * inv;
          }
        }
    }
    for (int64_t i = 0; i < n_pix; ++i) {
      double acc = 0;
      for (int t = 0; t < T; ++t) acc += images[(int64_t)t * n_pix + i];
      rho[i] = (float)acc;
    }
  }
  free(images);
  free(sens);
  return 0;
}

/* ---------------- FP64 Poisson list-mode NLL and gradient ---------------- */

double orc_nll_grad(const orc_geom* g, double support_sigma_z, double support_sigma_dl,
                    const float* events, int64_t n, const float* rho, const float* s_map,
                    double* grad_rho, double* grad_sigma, int n_threads,
                    int64_t* n_skipped) {
  orc_scanner_d s;
  orc_kernel_d ks; /* support ellipse constants */
  scanner_init_d(g, &s);
  kernel_init_d(support_sigma_z, support_sigma_dl, &ks);
  const double sz = g->sigma_z, sdl = g->sigma_dl;
  const double ipz = 1 / (sz * sz), ipd = 1 / (sdl * sdl);
  const double c0 = 1 / (2 * M_PI * M_PI) * sqrt(ipz * ipz * ipd);
  const int64_t n_pix = (int64_t)s.n_y * s.n_z;
  int T = n_threads > 0 ? n_threads : omp_get_max_threads();
  double* gimg = NULL;
  if (grad_rho) {
    gimg = (double*)calloc((size_t)T * n_pix, sizeof(double));
    if (!gimg) return NAN;
  }
  double loss = 0, gsz = 0, gsdl = 0;
  int64_t skipped = 0;
#pragma omp parallel for schedule(dynamic, 64) num_threads(T) \
    reduction(+ : loss, gsz, gsdl, skipped)
  for (int64_t e = 0; e < n; ++e) {
    orc_box_d b;
    event_box_d(&s, &ks, events[3 * e], events[3 * e + 1], events[3 * e + 2], &b);
    const double R = s.radius, sec = b.sec, tan = b.tan, y = b.y;
    const double sec_sq = sec * sec;
    double den = 0, dden_z = 0, dden_dl = 0;
    for (int pass = 0; pass < 2; ++pass) {
      double inv = (pass == 1) ? 1 / den : 0;
      for (int iy = b.tl_y; iy < b.br_y; ++iy)
        for (int iz = b.tl_x; iz < b.br_x; ++iz) {
          double px = s.tl_z_half_w + (int16_t)iz * s.pixel_width;
          double py = s.tl_y_half_h - (int16_t)iy * s.pixel_height;
          double dy = py - y, dz = px - b.z;
          if (!((b.A * dy * dy) + (b.B * dy * dz) + (b.C * dz * dz) <= 9)) continue;
          int64_t pi = (int64_t)iy * s.n_z + iz;
          double yp = dy + y;
          double ap = -(yp - R) * sec_sq, aq = -(yp + R) * sec_sq,
                 ar = -2 * yp * sec * tan;
          double bpq = dz - dy * tan, br = -2 * dy * sec;
          double Pa = ap * ap + aq * aq, Qa = ar * ar;
          double Pb = 2 * bpq * bpq, Qb = br * br;
          double aMa = Pa * ipz + Qa * ipd, bMb = Pb * ipz + Qb * ipd;
          double K = c0 / sqrt(aMa) * exp(-0.5 * bMb);
          double r = rho[pi];
          if (pass == 0) {
            den += K * r;
            double dlogK_dipz = 1 / ipz - 0.5 * Pa / aMa - 0.5 * Pb;
            double dlogK_dipd = 0.5 / ipd - 0.5 * Qa / aMa - 0.5 * Qb;
            dden_z += K * r * dlogK_dipz * (-2 / (sz * sz * sz));
            dden_dl += K * r * dlogK_dipd * (-2 / (sdl * sdl * sdl));
          } else if (gimg) {
            gimg[(int64_t)omp_get_thread_num() * n_pix + pi] -= K * inv;
          }
        }
      if (pass == 0 && !(den > 0)) {
        skipped += 1;
        break;
      }
      if (pass == 0) {
        loss -= log(den);
        gsz -= dden_z / den;
        gsdl -= dden_dl / den;
        if (!gimg) break;
      }
    }
  }
  float* s_point = NULL;
  if (!s_map) {
    s_point = (float*)malloc((size_t)n_pix * sizeof(float));
    if (!s_point) {
      free(gimg);
      return NAN;
    }
    orc_sensitivity_map_f(g, 0, s_point);
  }
  for (int64_t i = 0; i < n_pix; ++i) {
    double sp = s_map ? s_map[i] : s_point[i];
    loss += sp * rho[i];
    if (grad_rho) {
      double acc = sp;
      for (int t = 0; t < T; ++t) acc += gimg[(int64_t)t * n_pix + i];
      grad_rho[i] = acc;
    }
  }
  if (grad_sigma) {
    grad_sigma[0] = gsz;
    grad_sigma[1] = gsdl;
  }
  if (n_skipped) *n_skipped = skipped;
  free(s_point);
  free(gimg);
  return loss;
}
