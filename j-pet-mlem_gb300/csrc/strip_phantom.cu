// Seeded list-mode event generator for the strip scanner on the GPU (the
// phantom tool's Monte Carlo, src/2d/strip/phantom_cmd.cpp:136-444,
// src/common/phantom_monte_carlo.h:33-109).
//
// Every candidate emission has a 64-bit index; its random numbers are the
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011) at counter
// (index, draw) under the caller's 64-bit seed, so the event stream depends
// only on (regions, scanner, seed) and not on the launch shape.  A candidate:
//
//  1. picks a region with probability weight / total weight (ellipse and
//     rectangle: intensity x area, point: intensity; phantom.h:120-133,183-191);
//  2. draws a uniform point in it: ellipse r = sqrt(U), theta = 2 pi U, scaled
//     by the semi-axes and rotated (ellipse.h:83-91); rectangle uniform in
//     [x - a, x + a] x [y - b, y + b] (rectangle.h:20-51); point exact.  Unless
//     the regions are additive, a point inside an earlier-listed region is not
//     an emission (phantom.h:193-204: the reference redraws, which gives the
//     same distribution of emissions);
//  3. draws the direction angle uniform in (-phi_max, phi_max): pi/2 when
//     emissions are counted (phantom.h:213), atan(L / 2R) when detected events
//     are counted (every detected event has |tan| < L / 2R, so the accepted
//     events have the same distribution);
//  4. projects onto the strips, z_u = z + (R - y) tan, z_d = z - (R + y) tan,
//     dl = -2 y sqrt(1 + tan^2) (scanner.h:107-113), and is detected iff
//     |z_u|, |z_d| < L/2 on the exact values (scanner.h:208-213);
//  5. adds N(0, sigma_z) to z_u, z_d and N(0, sigma_dl) to dl (scanner.h:257-267,
//     Box-Muller normals), with no second acceptance test.
//
// Detected events are written in candidate order (a count pass, a scan over
// blocks and an ordered write pass with block-wide prefix sums), so the output
// is deterministic as well.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/jpet_strip.h"
#include "strip_device.cuh"
#include "strip_internal.h"

namespace jpet {
namespace {

struct GenRegion {
  int32_t kind;
  double x, y, a, b;
  double s, c;     // rotation
  double A, B, C;  // ellipse: A dx^2 + 2 C dx dy + B dy^2 <= 1
  double cdf;      // cumulative normalised weight
};

struct GenParams {
  double R, L, sigma_z, sigma_dl, phi_max;
  uint32_t key0, key1;
  int32_t n_regions, additive;
};

constexpr int kGenThreads = 256;
constexpr int kGenRounds = 16;
constexpr int kGenPerBlock = kGenThreads * kGenRounds;
constexpr int kGenMaxRegions = 256;

__device__ __forceinline__ void philox_round(uint32_t (&x)[4], uint32_t k0, uint32_t k1) {
  const uint32_t m0 = 0xD2511F53u, m1 = 0xCD9E8D57u;
  const uint32_t hi0 = __umulhi(m0, x[0]), lo0 = m0 * x[0];
  const uint32_t hi1 = __umulhi(m1, x[2]), lo1 = m1 * x[2];
  const uint32_t y0 = hi1 ^ x[1] ^ k0, y2 = hi0 ^ x[3] ^ k1;
  x[0] = y0;
  x[1] = lo1;
  x[2] = y2;
  x[3] = lo0;
}

// Philox4x32-10: ten rounds, the key advanced by the Weyl constants between rounds
__device__ __forceinline__ void philox(uint32_t (&x)[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    philox_round(x, k0, k1);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// 53-bit uniform in [0, 1)
__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
  return (static_cast<double>(a >> 5) * 67108864.0 + static_cast<double>(b >> 6)) *
         (1.0 / 9007199254740992.0);
}

struct Candidate {
  bool emitted, detected;
  float zu, zd, dl;
  double px, py;        // emission point
  float ex_zu, ex_zd, ex_dl;  // exact (unsmeared) response
  float dir_x, dir_y;   // emission direction (sin phi, cos phi)
};

// Optional count images of the phantom tool (phantom_cmd.cpp:249-258,289-352):
// a PixelGrid with its lower-left corner at -(n_z, n_y) s / 2 + origin, pixel
// (floor((z - x0) / s), floor((y - y0) / s)), index row * n_z + column.
struct GenImages {
  int32_t* emitted;   // emission points of all emissions counted
  int32_t* detected;  // emission points of the detected events
  int32_t* naive;     // points recovered from the smeared responses
  int32_t* tan_map;   // the same, binned also by tangent
  float* exact;       // exact responses of the written events (3 floats each)
  float* events;      // their emission events (x, y, dx, dy)
  double x0, y0, s;
  int32_t n_z, n_y, tan_bins;
  // the grid in the reference's float: lower-left corner, pixel size, 2R, the
  // first tangent plane's lower edge and the plane width
  float fx0, fy0, fs, two_r, tan_left, tan_size;
};

// Naive point of a smeared response and its bins, in float without
// contraction as the reference's host code computes them:
// Response::calculate_tan_y_z (response.h:22-37), PixelGrid::pixel_at
// (pixel_grid.h:59-64), VariableVoxelSizeVoxelGrid::voxel_at (voxel_grid.h:109-118).
__device__ __forceinline__ void naive_add(const GenImages& im, float zu, float zd, float dl) {
  const float t = __fdiv_rn(__fsub_rn(zu, zd), im.two_r);
  const float y = __fmul_rn(-0.5f, __fdiv_rn(dl, __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(t, t)))));
  const float z = __fmul_rn(0.5f, __fadd_rn(__fadd_rn(zu, zd), __fmul_rn(__fmul_rn(2.0f, y), t)));
  const float col = floorf(__fdiv_rn(__fsub_rn(z, im.fx0), im.fs));
  const float row = floorf(__fdiv_rn(__fsub_rn(y, im.fy0), im.fs));
  if (!(col >= 0.0f && col < static_cast<float>(im.n_z) && row >= 0.0f &&
        row < static_cast<float>(im.n_y)))
    return;
  const int pix = static_cast<int>(row) * im.n_z + static_cast<int>(col);
  if (im.naive) atomicAdd(&im.naive[pix], 1);
  if (im.tan_map) {
    const float plane = floorf(__fdiv_rn(__fsub_rn(t, im.tan_left), im.tan_size));
    if (plane >= 0.0f && plane < static_cast<float>(im.tan_bins))
      atomicAdd(&im.tan_map[static_cast<size_t>(plane) * im.n_y * im.n_z + pix], 1);
  }
}

__device__ __forceinline__ void image_add(int32_t* img, const GenImages& im, double z, double y) {
  if (!img) return;
  const double cz = floor((z - im.x0) / im.s), cy = floor((y - im.y0) / im.s);
  if (cz >= 0.0 && cz < im.n_z && cy >= 0.0 && cy < im.n_y)
    atomicAdd(&img[static_cast<int>(cy) * im.n_z + static_cast<int>(cz)], 1);
}

__device__ Candidate gen_candidate(const GenParams& p, const GenRegion* __restrict__ regs,
                                   uint64_t index) {
  const uint32_t lo = static_cast<uint32_t>(index), hi = static_cast<uint32_t>(index >> 32);
  uint32_t r0[4] = {lo, hi, 0u, 0u};
  uint32_t r1[4] = {lo, hi, 1u, 0u};
  philox(r0, p.key0, p.key1);
  philox(r1, p.key0, p.key1);
  Candidate out{false, false, 0.f, 0.f, 0.f, 0.0, 0.0, 0.f, 0.f, 0.f, 0.f, 0.f};
  // region by cumulative weight (phantom.h:183-191: the first cdf >= u)
  const double u_reg = u53(r0[0], r0[1]);
  int k = 0;
  while (k < p.n_regions - 1 && u_reg > regs[k].cdf) ++k;
  const GenRegion& rg = regs[k];
  const double u1 = u53(r0[2], r0[3]), u2 = u53(r1[0], r1[1]);
  double px, py;
  if (rg.kind == JPET_REGION_ELLIPSE) {
    const double rr = sqrt(u1);
    double st, ct;
    sincospi(2.0 * u2, &st, &ct);
    const double ex = rg.a * rr * ct, ey = rg.b * rr * st;
    px = rg.c * ex - rg.s * ey + rg.x;
    py = rg.s * ex + rg.c * ey + rg.y;
  } else if (rg.kind == JPET_REGION_RECTANGLE) {
    px = rg.x + rg.a * (2.0 * u1 - 1.0);
    py = rg.y + rg.b * (2.0 * u2 - 1.0);
  } else {
    px = rg.x;
    py = rg.y;
  }
  if (!p.additive) {
    for (int i = 0; i < k; ++i) {
      const GenRegion& q = regs[i];
      const double dx = px - q.x, dy = py - q.y;
      bool inside;
      if (q.kind == JPET_REGION_ELLIPSE)
        inside = q.A * dx * dx + 2.0 * q.C * dx * dy + q.B * dy * dy <= 1.0;
      else if (q.kind == JPET_REGION_RECTANGLE)
        inside = fabs(dx) <= q.a && fabs(dy) <= q.b;
      else
        inside = dx == 0.0 && dy == 0.0;
      if (inside) return out;
    }
  }
  out.emitted = true;
  out.px = px;
  out.py = py;
  const double phi = p.phi_max * (2.0 * u53(r1[2], r1[3]) - 1.0);
  const double t = tan(phi);
  const double zu = px + (p.R - py) * t;
  const double zd = px - (p.R + py) * t;
  const double dl = -2.0 * py * sqrt(t * t + 1.0);
  const double half = 0.5 * p.L;
  if (!(fabs(zu) < half && fabs(zd) < half)) return out;
  out.detected = true;
  out.ex_zu = static_cast<float>(zu);
  out.ex_zd = static_cast<float>(zd);
  out.ex_dl = static_cast<float>(dl);
  {
    double sp, cp;
    sincos(phi, &sp, &cp);
    out.dir_x = static_cast<float>(sp);
    out.dir_y = static_cast<float>(cp);
  }
  // Box-Muller on two pairs of uniforms (1 - U in (0, 1]) gives the normals
  uint32_t r2[4] = {lo, hi, 2u, 0u};
  uint32_t r3[4] = {lo, hi, 3u, 0u};
  philox(r2, p.key0, p.key1);
  philox(r3, p.key0, p.key1);
  const double m0 = sqrt(-2.0 * log(1.0 - u53(r2[0], r2[1])));
  const double m1 = sqrt(-2.0 * log(1.0 - u53(r3[0], r3[1])));
  double s0, c0, s1, c1;
  sincospi(2.0 * u53(r2[2], r2[3]), &s0, &c0);
  sincospi(2.0 * u53(r3[2], r3[3]), &s1, &c1);
  out.zu = static_cast<float>(zu + p.sigma_z * m0 * c0);
  out.zd = static_cast<float>(zd + p.sigma_z * m0 * s0);
  out.dl = static_cast<float>(dl + p.sigma_dl * m1 * c1);
  return out;
}

// Block-wide exclusive prefix of a flag (kGenThreads threads); returns the
// thread's rank and the block total.
__device__ __forceinline__ int block_rank(bool flag, int* s_warp, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, flag);
  const int in_warp = __popc(m & ((1u << lane) - 1u));
  if (lane == 0) s_warp[warp] = __popc(m);
  __syncthreads();
  int before = 0, sum = 0;
#pragma unroll
  for (int w = 0; w < kGenThreads / 32; ++w) {
    const int v = s_warp[w];
    before += (w < warp) ? v : 0;
    sum += v;
  }
  __syncthreads();
  total = sum;
  return before + in_warp;
}

template <bool WRITE>
__global__ void __launch_bounds__(kGenThreads) gen_kernel(
    GenParams p, const GenRegion* __restrict__ regs_g, uint64_t cand0, int2* block_counts,
    const long long* __restrict__ block_base, long long limit, int count_emissions,
    long long capacity, unsigned long long* taken, float* __restrict__ out, GenImages im) {
  __shared__ GenRegion regs[kGenMaxRegions];
  __shared__ int s_warp[2][kGenThreads / 32];
  for (int i = threadIdx.x; i < p.n_regions; i += blockDim.x) regs[i] = regs_g[i];
  __syncthreads();
  long long e_base = 0, d_base = 0;
  if (WRITE) {
    e_base = block_base[2 * blockIdx.x];
    d_base = block_base[2 * blockIdx.x + 1];
  }
  int n_emit = 0, n_det = 0;
  for (int r = 0; r < kGenRounds; ++r) {
    const uint64_t idx = cand0 + (static_cast<uint64_t>(blockIdx.x) * kGenRounds + r) * kGenThreads +
                         threadIdx.x;
    const Candidate c = gen_candidate(p, regs, idx);
    if (WRITE) {
      int te, td;
      const int re = block_rank(c.emitted, s_warp[0], te);
      const int rd = block_rank(c.detected, s_warp[1], td);
      const long long ei = e_base + re, di = d_base + rd;
      const bool take = c.detected && (count_emissions ? ei < limit : di < limit);
      if (take && di < capacity) {
        out[3 * di] = c.zu;
        out[3 * di + 1] = c.zd;
        out[3 * di + 2] = c.dl;
        if (im.exact) {
          im.exact[3 * di] = c.ex_zu;
          im.exact[3 * di + 1] = c.ex_zd;
          im.exact[3 * di + 2] = c.ex_dl;
        }
        if (im.events) {
          im.events[4 * di] = static_cast<float>(c.px);
          im.events[4 * di + 1] = static_cast<float>(c.py);
          im.events[4 * di + 2] = c.dir_x;
          im.events[4 * di + 3] = c.dir_y;
        }
      }
      if (c.emitted && (count_emissions ? ei < limit : di < limit)) {
        image_add(im.emitted, im, c.px, c.py);
        if (take) {
          image_add(im.detected, im, c.px, c.py);
          if (im.naive || im.tan_map) naive_add(im, c.zu, c.zd, c.dl);
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, take);
      if ((threadIdx.x & 31) == 0 && m) atomicAdd(taken, static_cast<unsigned long long>(__popc(m)));
      e_base += te;
      d_base += td;
    } else {
      n_emit += c.emitted;
      n_det += c.detected;
    }
  }
  if (!WRITE) {
    int te, td;
    for (int o = 16; o > 0; o >>= 1) {
      n_emit += __shfl_xor_sync(0xffffffffu, n_emit, o);
      n_det += __shfl_xor_sync(0xffffffffu, n_det, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
      s_warp[0][warp] = n_emit;
      s_warp[1][warp] = n_det;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      te = td = 0;
      for (int w = 0; w < kGenThreads / 32; ++w) {
        te += s_warp[0][w];
        td += s_warp[1][w];
      }
      block_counts[blockIdx.x] = make_int2(te, td);
    }
  }
}

constexpr double kPi = 3.14159265358979323846;

}  // namespace
}  // namespace jpet

using namespace jpet;

// The phantom tool's float grids (phantom_cmd.cpp:241-253): PixelGrid with its
// lower-left corner at float(-s n / 2) + float(origin), and the tangent planes
// of VariableVoxelSizeVoxelGrid(-max_tan, bins, max_tan / bins * 2) with
// max_tan = 1.1 L / 2R.
namespace jpet {
namespace {
struct TanGrid {
  float x0, y0, s, tan_left, tan_size;
};
TanGrid tan_grid(const jpet_strip_geom& g, int bins, double origin_x, double origin_y) {
  TanGrid t;
  t.s = static_cast<float>(g.pixel_width);
  t.x0 = static_cast<float>(-g.pixel_width * g.n_z_pixels / 2) + static_cast<float>(origin_x);
  t.y0 = static_cast<float>(-g.pixel_width * g.n_y_pixels / 2) + static_cast<float>(origin_y);
  const float max_tan = 1.1f * static_cast<float>(g.scintillator_length) /
                        (2.0f * static_cast<float>(g.radius));
  t.tan_left = -max_tan;
  t.tan_size = bins > 0 ? max_tan / static_cast<float>(bins) * 2.0f : 0.0f;
  return t;
}

// One thread per voxel of the kernel map (phantom_cmd.cpp:402-430) in the
// reference's float order: tangent of the plane centre, sec, the voxel centre,
// AnalyticKernel at the kernel point, times the volume element 4 R bin_volume
// sec and the inverse sensitivity.
__global__ void __launch_bounds__(256) tan_kernel_map_kernel(DevGeom g, int32_t n_z, int32_t n_y,
                                                             int32_t bins, TanGrid tg, float kx,
                                                             float ky, float vol4r, float inv_sens,
                                                             float* __restrict__ out) {
  const size_t n = static_cast<size_t>(n_z) * n_y * bins;
  const float llcx = __fadd_rn(tg.x0, __fmul_rn(tg.s, 0.5f));
  const float llcy = __fadd_rn(tg.y0, __fmul_rn(tg.s, 0.5f));
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % n_z);
    const int y = static_cast<int>((i / n_z) % n_y);
    const int z = static_cast<int>(i / (static_cast<size_t>(n_z) * n_y));
    const float tan = __fadd_rn(__fmul_rn(__fadd_rn(static_cast<float>(z), 0.5f), tg.tan_size),
                                tg.tan_left);
    const float sec = __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(tan, tan)));
    const float cx = __fadd_rn(llcx, __fmul_rn(static_cast<float>(x), tg.s));
    const float cy = __fadd_rn(llcy, __fmul_rn(static_cast<float>(y), tg.s));
    const float k = analytic_exact(g, cy, tan, sec, __fsub_rn(kx, cx), __fsub_rn(ky, cy));
    out[i] = __fmul_rn(__fmul_rn(k, __fmul_rn(vol4r, sec)), inv_sens);
  }
}

__global__ void sensitivity_at_kernel(DevGeom g, float px, float py, float* out) {
  *out = scanner_sensitivity(g, px, py);
}
}  // namespace
}  // namespace jpet

extern "C" {

int jpet_strip_generate(const jpet_strip_geom* geom, const jpet_strip_region* regions,
                        int32_t n_regions, int64_t n, uint64_t seed, int32_t flags,
                        float* d_out_aos, int64_t capacity, int64_t* n_written,
                        const jpet_strip_gen_images* images, void* cuda_stream) {
  if (n_written) *n_written = 0;
  if (!geom || !regions || n_regions <= 0 || n_regions > kGenMaxRegions || n < 0 ||
      (n > 0 && !d_out_aos) || capacity < 0) {
    set_call_error("jpet_strip_generate: invalid argument");
    return JPET_ERR_ARGUMENT;
  }
  const bool detected = (flags & JPET_GEN_DETECTED) != 0;
  if (detected && capacity < n) {
    set_call_error("jpet_strip_generate: capacity below the requested detected events");
    return JPET_ERR_ARGUMENT;
  }
  if (!(geom->radius > 0) || !(geom->scintillator_length > 0) || !(geom->sigma_z >= 0) ||
      !(geom->sigma_dl >= 0)) {
    set_call_error("jpet_strip_generate: invalid scanner");
    return JPET_ERR_ARGUMENT;
  }
  // regions: weights, cumulative distribution (phantom.h:120-133), rotations
  std::vector<GenRegion> regs(n_regions);
  double total = 0.0;
  for (int i = 0; i < n_regions; ++i) {
    const jpet_strip_region& r = regions[i];
    GenRegion& g = regs[i];
    g.kind = r.kind;
    g.x = r.x;
    g.y = r.y;
    g.a = r.a;
    g.b = r.b;
    const double ang = r.angle_deg * kPi / 180.0;
    g.s = std::sin(ang);
    g.c = std::cos(ang);
    double w;
    if (r.kind == JPET_REGION_ELLIPSE) {
      if (!(r.a > 0) || !(r.b > 0)) {
        set_call_error("jpet_strip_generate: ellipse semi-axes must be positive");
        return JPET_ERR_ARGUMENT;
      }
      g.A = g.c * g.c / (r.a * r.a) + g.s * g.s / (r.b * r.b);
      g.B = g.s * g.s / (r.a * r.a) + g.c * g.c / (r.b * r.b);
      g.C = g.s * g.c * (1.0 / (r.a * r.a) - 1.0 / (r.b * r.b));
      w = r.intensity * kPi * r.a * r.b;
    } else if (r.kind == JPET_REGION_RECTANGLE) {
      if (!(r.a > 0) || !(r.b > 0)) {
        set_call_error("jpet_strip_generate: rectangle half sizes must be positive");
        return JPET_ERR_ARGUMENT;
      }
      g.A = g.B = g.C = 0.0;
      w = r.intensity * 4.0 * r.a * r.b;
    } else if (r.kind == JPET_REGION_POINT) {
      g.A = g.B = g.C = 0.0;
      w = r.intensity;
    } else {
      set_call_error("jpet_strip_generate: unknown region kind");
      return JPET_ERR_ARGUMENT;
    }
    if (!(w >= 0) || !std::isfinite(w)) {
      set_call_error("jpet_strip_generate: region weights must be finite and non-negative");
      return JPET_ERR_ARGUMENT;
    }
    total += w;
    g.cdf = total;
  }
  if (!(total > 0)) {
    set_call_error("jpet_strip_generate: total region weight is zero");
    return JPET_ERR_ARGUMENT;
  }
  for (auto& g : regs) g.cdf /= total;
  if (n == 0) return JPET_OK;

  GenImages im{};
  if (images && (images->tan_bins < 0 || (images->tan_bins > 0) != (images->tan_map != nullptr))) {
    set_call_error("jpet_strip_generate: tan_map needs tan_bins > 0 and the reverse");
    return JPET_ERR_ARGUMENT;
  }
  if (images && !(images->emitted || images->detected || images->naive || images->tan_map)) {
    im.exact = images->exact_responses;
    im.events = images->events;
  }
  if (images && (images->emitted || images->detected || images->naive || images->tan_map)) {
    if (geom->n_z_pixels <= 0 || geom->n_y_pixels <= 0 || !(geom->pixel_width > 0)) {
      set_call_error("jpet_strip_generate: count images need n_z, n_y and the pixel size");
      return JPET_ERR_ARGUMENT;
    }
    im.emitted = images->emitted;
    im.detected = images->detected;
    im.naive = images->naive;
    im.tan_map = images->tan_map;
    im.tan_bins = images->tan_bins;
    im.exact = images->exact_responses;
    im.events = images->events;
    im.s = geom->pixel_width;
    im.n_z = geom->n_z_pixels;
    im.n_y = geom->n_y_pixels;
    im.x0 = -im.s * im.n_z / 2.0 + images->origin_x;
    im.y0 = -im.s * im.n_y / 2.0 + images->origin_y;
    const TanGrid tg = tan_grid(*geom, im.tan_bins, images->origin_x, images->origin_y);
    im.fx0 = tg.x0;
    im.fy0 = tg.y0;
    im.fs = tg.s;
    im.two_r = 2.0f * static_cast<float>(geom->radius);
    im.tan_left = tg.tan_left;
    im.tan_size = tg.tan_size;
  }
  GenParams p;
  p.R = geom->radius;
  p.L = geom->scintillator_length;
  p.sigma_z = geom->sigma_z;
  p.sigma_dl = geom->sigma_dl;
  p.phi_max = detected ? std::atan(p.L / (2.0 * p.R)) : 0.5 * kPi;
  p.key0 = static_cast<uint32_t>(seed);
  p.key1 = static_cast<uint32_t>(seed >> 32);
  p.n_regions = n_regions;
  p.additive = (flags & JPET_GEN_ADDITIVE) ? 1 : 0;

  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const int blocks = 1024;  // 4 Mi candidates per pass
  GenRegion* d_regs = nullptr;
  int2* d_counts = nullptr;
  long long* d_base = nullptr;
  unsigned long long* d_taken = nullptr;
  auto release = [&]() {
    cudaFree(d_regs);
    cudaFree(d_counts);
    cudaFree(d_base);
    cudaFree(d_taken);
  };
  auto fail = [&](cudaError_t e, const char* what) {
    set_call_error(std::string("jpet_strip_generate: ") + what + ": " + cudaGetErrorString(e));
    release();
    return JPET_ERR_CUDA;
  };
  cudaError_t e = cudaMalloc(&d_regs, regs.size() * sizeof(GenRegion));
  if (e == cudaSuccess) e = cudaMalloc(&d_counts, blocks * sizeof(int2));
  if (e == cudaSuccess) e = cudaMalloc(&d_base, 2 * blocks * sizeof(long long));
  if (e == cudaSuccess) e = cudaMalloc(&d_taken, sizeof(unsigned long long));
  if (e != cudaSuccess) return fail(e, "cudaMalloc");
  e = cudaMemcpyAsync(d_regs, regs.data(), regs.size() * sizeof(GenRegion),
                      cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_taken, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return fail(e, "copy regions");
  std::vector<int2> counts(blocks);
  std::vector<long long> base(2 * blocks);
  long long emitted = 0, det = 0;
  uint64_t cand0 = 0;
  const long long limit = n;
  int idle_passes = 0;
  while ((detected ? det : emitted) < limit) {
    gen_kernel<false><<<blocks, kGenThreads, 0, s>>>(p, d_regs, cand0, d_counts, nullptr, 0, 0,
                                                     0, nullptr, nullptr, GenImages{});
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(e, "count kernel");
    e = cudaMemcpyAsync(counts.data(), d_counts, blocks * sizeof(int2), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(e, "count pass");
    long long e_run = emitted, d_run = det;
    for (int b = 0; b < blocks; ++b) {
      base[2 * b] = e_run;
      base[2 * b + 1] = d_run;
      e_run += counts[b].x;
      d_run += counts[b].y;
    }
    e = cudaMemcpyAsync(d_base, base.data(), 2 * blocks * sizeof(long long),
                        cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fail(e, "copy block offsets");
    gen_kernel<true><<<blocks, kGenThreads, 0, s>>>(p, d_regs, cand0, nullptr, d_base, limit,
                                                    detected ? 0 : 1, capacity, d_taken,
                                                    d_out_aos, im);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the offsets are reused next pass
    if (e != cudaSuccess) return fail(e, "write pass");
    if ((detected ? d_run - det : e_run - emitted) == 0) {
      if (++idle_passes > 64) {
        set_call_error("jpet_strip_generate: the regions give no events");
        release();
        return JPET_ERR_ARGUMENT;
      }
    } else {
      idle_passes = 0;
    }
    emitted = e_run;
    det = d_run;
    cand0 += static_cast<uint64_t>(blocks) * kGenPerBlock;
  }
  unsigned long long taken = 0;
  e = cudaMemcpy(&taken, d_taken, sizeof(taken), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(e, "copy counter");
  release();
  if (static_cast<long long>(taken) > capacity) {
    set_call_error("jpet_strip_generate: capacity below the detected events");
    return JPET_ERR_ARGUMENT;
  }
  if (n_written) *n_written = static_cast<int64_t>(taken);
  return JPET_OK;
}

int jpet_strip_generate_host(const jpet_strip_geom* geom, const jpet_strip_region* regions,
                             int32_t n_regions, int64_t n, uint64_t seed, int32_t flags,
                             float* out_aos, int64_t capacity, int64_t* n_written,
                             const jpet_strip_gen_images* images, int32_t device) {
  if (n_written) *n_written = 0;
  if (n < 0 || capacity < 0 || (n > 0 && !out_aos)) {
    set_call_error("jpet_strip_generate_host: invalid argument");
    return JPET_ERR_ARGUMENT;
  }
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    set_call_error(std::string("jpet_strip_generate_host: cudaSetDevice: ") +
                   cudaGetErrorString(e));
    return JPET_ERR_CUDA;
  }
  const int64_t cap = std::max<int64_t>(std::min(capacity, n), 1);
  float* d_out = nullptr;
  int32_t* d_img[4] = {nullptr, nullptr, nullptr, nullptr};
  int32_t* h_img[4] = {images ? images->emitted : nullptr, images ? images->detected : nullptr,
                       images ? images->naive : nullptr, images ? images->tan_map : nullptr};
  const size_t n_pix = static_cast<size_t>(std::max(geom ? geom->n_y_pixels : 0, 0)) *
                       static_cast<size_t>(std::max(geom ? geom->n_z_pixels : 0, 0));
  const size_t n_el[4] = {n_pix, n_pix, n_pix,
                          n_pix * static_cast<size_t>(images ? std::max(images->tan_bins, 0) : 0)};
  float* d_exact = nullptr;
  float* d_events = nullptr;
  auto release = [&]() {
    cudaFree(d_out);
    cudaFree(d_exact);
    cudaFree(d_events);
    for (auto* q : d_img) cudaFree(q);
  };
  e = cudaMalloc(&d_out, static_cast<size_t>(cap) * 3 * sizeof(float));
  if (e == cudaSuccess && images && images->exact_responses)
    e = cudaMalloc(&d_exact, static_cast<size_t>(cap) * 3 * sizeof(float));
  if (e == cudaSuccess && images && images->events)
    e = cudaMalloc(&d_events, static_cast<size_t>(cap) * 4 * sizeof(float));
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
    if (!h_img[k]) continue;
    e = cudaMalloc(&d_img[k], std::max<size_t>(n_el[k], 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemset(d_img[k], 0, n_el[k] * sizeof(int32_t));
  }
  if (e != cudaSuccess) {
    set_call_error(std::string("jpet_strip_generate_host: ") + cudaGetErrorString(e));
    release();
    return JPET_ERR_MEMORY;
  }
  jpet_strip_gen_images dim{};
  if (images) {
    dim = *images;
    dim.emitted = d_img[0];
    dim.detected = d_img[1];
    dim.naive = d_img[2];
    dim.tan_map = d_img[3];
    dim.exact_responses = d_exact;
    dim.events = d_events;
  }
  int64_t written = 0;
  int rc = jpet_strip_generate(geom, regions, n_regions, n, seed, flags, d_out, cap, &written,
                               images ? &dim : nullptr, nullptr);
  if (rc == JPET_OK) {
    e = cudaMemcpy(out_aos, d_out, static_cast<size_t>(written) * 3 * sizeof(float),
                   cudaMemcpyDeviceToHost);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
      if (h_img[k]) e = cudaMemcpy(h_img[k], d_img[k], n_el[k] * sizeof(int32_t),
                                   cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && d_exact)
      e = cudaMemcpy(images->exact_responses, d_exact,
                     static_cast<size_t>(written) * 3 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && d_events)
      e = cudaMemcpy(images->events, d_events, static_cast<size_t>(written) * 4 * sizeof(float),
                     cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      set_call_error(std::string("jpet_strip_generate_host: copy: ") + cudaGetErrorString(e));
      rc = JPET_ERR_CUDA;
    }
  }
  release();
  if (rc == JPET_OK && n_written) *n_written = written;
  return rc;
}

int jpet_strip_tan_kernel_map(const jpet_strip_geom* geom, int32_t tan_bins, double kernel_x,
                              double kernel_y, double origin_x, double origin_y,
                              int32_t divide_by_sensitivity, float* out, int32_t device) {
  if (!geom || !out || tan_bins <= 0 || geom->n_z_pixels <= 0 || geom->n_y_pixels <= 0 ||
      !(geom->pixel_width > 0) || !(geom->radius > 0) || !(geom->scintillator_length > 0) ||
      !(geom->sigma_z > 0) || !(geom->sigma_dl > 0)) {
    set_call_error("jpet_strip_tan_kernel_map: invalid argument");
    return JPET_ERR_ARGUMENT;
  }
  const size_t n = static_cast<size_t>(geom->n_z_pixels) * geom->n_y_pixels * tan_bins;
  cudaError_t e = cudaSetDevice(device);
  float* d_out = nullptr;
  float* d_sens = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&d_out, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&d_sens, sizeof(float));
  const DevGeom g = make_dev_geom(*geom);
  const TanGrid tg = tan_grid(*geom, tan_bins, origin_x, origin_y);
  const float kx = static_cast<float>(kernel_x), ky = static_cast<float>(kernel_y);
  float inv_sens = 1.0f;
  if (e == cudaSuccess && divide_by_sensitivity) {
    sensitivity_at_kernel<<<1, 1>>>(g, kx, ky, d_sens);
    float sens = 0.0f;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&sens, d_sens, sizeof(float), cudaMemcpyDeviceToHost);
    inv_sens = 1.0f / sens;
  }
  // 4 R pixel^2 dtan (phantom_cmd.cpp:409-421), float left to right
  const float vol4r = 4.0f * static_cast<float>(geom->radius) * (tg.s * tg.s * tg.tan_size);
  if (e == cudaSuccess) {
    const size_t blocks = std::min<size_t>((n + 255) / 256, 152 * 16);
    tan_kernel_map_kernel<<<static_cast<unsigned>(blocks), 256>>>(
        g, geom->n_z_pixels, geom->n_y_pixels, tan_bins, tg, kx, ky, vol4r, inv_sens, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d_out, n * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d_out);
  cudaFree(d_sens);
  if (e != cudaSuccess) {
    set_call_error(std::string("jpet_strip_tan_kernel_map: ") + cudaGetErrorString(e));
    return JPET_ERR_CUDA;
  }
  return JPET_OK;
}

}  // extern "C"
