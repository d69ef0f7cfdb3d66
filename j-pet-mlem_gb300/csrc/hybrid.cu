// GB300 3D hybrid list-mode MLEM (include/jpet_hybrid.h): barrel LORs in x-y,
// the strip TOF kernel along each LOR and z.
//
// Replaces PET3D::Hybrid::GPU::Reconstruction::run and its kernel
// (src/3d/hybrid/cuda/reconstruction.cu:36-187,
// src/3d/hybrid/cuda/reconstruction/warp_granularity.cuh:28-178) and moves the
// CPU set-up the reference command runs first onto the device
// (src/3d/hybrid/reconstruction.h:101-162 frame events, 218-274 weights and
// sensitivity).
//
// Device layout.  The image is held pixel-major with the planes of a pixel
// contiguous, index (x + n_columns y) n_planes + z, so that the voxels of one
// event -- a run of planes for each pixel info on its LOR -- are contiguous
// runs in memory; the reference's plane-major order (voxel_grid.h:54-56) is used
// only at the boundary (set_image / get_image).
//
// Iteration kernel: one CTA per event.  The threads compute the event's
// per-pixel constants of the strip kernel (the terms that do not depend on z)
// into shared memory, then walk the pixel-info x plane voxels flattened, one
// CTA-wide step of consecutive voxels at a time, so that neighbouring threads
// touch neighbouring planes of one pixel.  Each thread keeps the weights
// K(z, up) w_pixel rho of its first voxels in shared memory for the
// back-projection, which adds weight / denominator with one global float
// atomic per voxel; the denominator is reduced across the CTA.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/jpet_hybrid.h"

namespace {

thread_local std::string g_hybrid_error = "no error";

template <typename T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      n = 0;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// Constants of the kernels: GaussianKernel's (gaussian_kernel.h:27-33) and the grid's.
struct HybConst {
  float ipz, ipd, c0;   // 1/sigma_z^2, 1/sigma_dl^2, normalisation
  float ps, z_left;     // voxel size, VoxelGrid::z_left
  float llcx, llcy;     // PixelGrid::lower_left_center
  float L2;             // length / 2 (GaussianKernel::sensitivity)
  float exp_bpq;        // -log2(e) / sigma_z^2: exponent coefficient of (dz - dy tan)^2
  int32_t n_columns, n_rows, n_planes;
  int32_t n_lors;
  int64_t n_infos;
  int32_t n_planes_half;  // planes of weights (> 1: one system matrix per plane half)
  int32_t sens_depth;     // planes of the sensitivity image (1: the 2D sensitivity)
};

// Forms of the denominator loop (reconstruction.h:327-357):
constexpr int kSens2D = 0;      // one plane half, 2D sensitivity
constexpr int kMultiPlane = 1;  // weights and sensitivity of plane |iz - n_planes_half|
constexpr int kSens3D = 2;      // one plane half, sensitivity of plane |iz - depth|

// The plane of the weights / sensitivity that plane iz reads: |iz - depth|.
// The reference's index reaches depth itself for plane 0 (and for the last
// plane of an odd count), one plane past its arrays; clamped to depth - 1.
__device__ __forceinline__ int abs_plane(int iz, int depth) {
  const int a = iz > depth ? iz - depth : depth - iz;
  return a < depth ? a : depth - 1;
}

// Sizes of the iteration kernel (compile-time; -D overrides for tuning sweeps).
#ifndef JPET_HYBRID_THREADS
#define JPET_HYBRID_THREADS 128
#endif
#ifndef JPET_HYBRID_CACHE_STEPS
#define JPET_HYBRID_CACHE_STEPS 32
#endif
constexpr int kThreads = JPET_HYBRID_THREADS;     // CTA size: one event per CTA at a time
constexpr int kSteps = JPET_HYBRID_CACHE_STEPS;   // voxel weights a thread keeps for the back-projection
constexpr int kPix = 256;                         // pixel infos per chunk
constexpr int kWarpsPerCta = kThreads / 32;
constexpr float kPi = 3.14159265358979323846f;

__device__ __forceinline__ int64_t lor_index(int16_t first, int16_t second) {
  return static_cast<int64_t>(static_cast<int32_t>(first) * (first + 1) / 2 + second);
}

// float -> short as the reference's x86-64 build converts (truncation to int32,
// out of range and NaN give INT32_MIN, low 16 bits kept).
__device__ __forceinline__ int16_t to_short(float v) {
  int32_t i = (v > -2147483648.0f && v < 2147483648.0f) ? __float2int_rz(v) : INT32_MIN;
  return static_cast<int16_t>(static_cast<uint32_t>(i) & 0xffffu);
}

// Pixel centre (pixel_grid.h:54-57), explicit rounding (no contraction).
__device__ __forceinline__ void pixel_center(const HybConst& c, int x, int y, float& cx,
                                             float& cy) {
  cx = __fadd_rn(c.llcx, __fmul_rn(static_cast<float>(x), c.ps));
  cy = __fadd_rn(c.llcy, __fmul_rn(static_cast<float>(y), c.ps));
}

// ---- set-up: weights, sensitivity, normalisation --------------------------------

// Reconstruction::calculate_weight (reconstruction.h:218-238): one warp per LOR.
__global__ void weights_kernel(const float4* __restrict__ seg, const float* __restrict__ widths,
                               const int2* __restrict__ pix, const uint64_t* __restrict__ ib,
                               const uint64_t* __restrict__ ie, float* __restrict__ w,
                               HybConst c, double sqrt_2pi) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  const int16_t* p16 = reinterpret_cast<const int16_t*>(pix);
  for (int64_t l = warp; l < c.n_lors; l += n_warps) {
    const float4 s2 = seg[3 * l + 2];  // normal_x, normal_y, length, distance_from_origin
    const float sigma_w = __fmul_rn(0.3f, widths[l]);
    const double gauss_norm_w = 1.0 / (static_cast<double>(sigma_w) * sqrt_2pi);
    const float inv_sigma2_w = __fdiv_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, sigma_w), sigma_w));
    for (uint64_t i = ib[l] + lane; i < ie[l]; i += 32) {
      float cx, cy;
      pixel_center(c, p16[2 * i], p16[2 * i + 1], cx, cy);
      const float d = __fsub_rn(__fadd_rn(__fmul_rn(cx, s2.x), __fmul_rn(cy, s2.y)), s2.w);
      const float e = expf(__fmul_rn(__fmul_rn(-d, d), inv_sigma2_w));
      w[i] = __double2float_rn(gauss_norm_w * static_cast<double>(e));
    }
  }
}

// Sort keys of calculate_sensitivity: pixel index of every pixel info, and a
// check that every pixel lies inside the grid.
__global__ void pixel_keys_kernel(const int16_t* __restrict__ p16, int64_t n, HybConst c,
                                  int32_t* __restrict__ keys, int32_t* __restrict__ vals,
                                  int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int x = p16[2 * i], y = p16[2 * i + 1];
    const bool in = x >= 0 && x < c.n_columns && y >= 0 && y < c.n_rows;
    if (!in) atomicExch(bad, 1);
    keys[i] = in ? x + c.n_columns * y : 0;
    vals[i] = static_cast<int32_t>(i);
  }
}

// calculate_sensitivity (reconstruction.h:240-251): the infos of each pixel,
// in ascending info order after the stable sort, summed from zero in that
// order -- the reference's order of additions into sensitivity[pixel].
__global__ void sensitivity_sum_kernel(const int32_t* __restrict__ keys,
                                       const int32_t* __restrict__ vals, int64_t n,
                                       const float* __restrict__ w, float* __restrict__ sens) {
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < n;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int32_t k = keys[j];
    if (j > 0 && keys[j - 1] == k) continue;
    float s = 0.0f;
    for (int64_t q = j; q < n && keys[q] == k; ++q) s = __fadd_rn(s, w[vals[q]]);
    sens[k] = s;
  }
}

// LOR of every pixel info (-1 for infos outside every LOR's range).
__global__ void lor_of_info_kernel(const uint64_t* __restrict__ ib, const uint64_t* __restrict__ ie,
                                   int32_t n_lors, int32_t* __restrict__ lor_of) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  for (int64_t l = warp; l < n_lors; l += n_warps)
    for (uint64_t i = ib[l] + lane; i < ie[l]; i += 32) lor_of[i] = static_cast<int32_t>(l);
}

// After the stable sort by pixel, two infos of one pixel and one LOR are
// adjacent: flags a LOR that lists a pixel twice.
__global__ void unique_pixels_kernel(const int32_t* __restrict__ keys,
                                     const int32_t* __restrict__ vals, int64_t n,
                                     const int32_t* __restrict__ lor_of, int* __restrict__ bad) {
  for (int64_t j = 1 + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < n;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (keys[j] != keys[j - 1]) continue;
    const int32_t a = lor_of[vals[j]], b = lor_of[vals[j - 1]];
    if (a >= 0 && a == b) atomicExch(bad, 1);
  }
}

// normalize_geometry_weights (reconstruction.h:253-272), every plane half:
// weight (info, plane) / sensitivity (pixel, plane).
__global__ void normalize_kernel(const int16_t* __restrict__ p16, int64_t n, HybConst c,
                                 const float* __restrict__ sens, float* __restrict__ w) {
  const int64_t n_px = static_cast<int64_t>(c.n_columns) * c.n_rows;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int x = p16[2 * i], y = p16[2 * i + 1];
    for (int plane = 0; plane < c.n_planes_half; ++plane)
      w[i + n * plane] = __fdiv_rn(w[i + n * plane], sens[x + c.n_columns * y + n_px * plane]);
  }
}

__global__ void fill_kernel(float* p, int64_t n, float v) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = v;
}

// ---- frame events -------------------------------------------------------------

__device__ __forceinline__ uint64_t lower_bound_f(const float* a, uint64_t lo, uint64_t hi,
                                                  float v) {
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (a[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ uint64_t upper_bound_f(const float* a, uint64_t lo, uint64_t hi,
                                                  float v) {
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (v < a[mid]) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// Reconstruction::translate_to_frame (reconstruction.h:101-147) with
// Response::calculate_tan_y_z (src/2d/strip/response.h:22-37) and
// GaussianKernel::ellipse_bb (gaussian_kernel.h:108-128), then
// bb_intersects_grid_with_positive_weight (reconstruction.h:151-162).  Every
// operation is rounded explicitly in the reference's order, so the frame event
// and its ranges are the reference's own.
__global__ void translate_kernel(const jpet_hybrid_response* __restrict__ r, int64_t n,
                                 const float4* __restrict__ seg, const int16_t* __restrict__ p16,
                                 const float* __restrict__ pos, const float* __restrict__ w,
                                 const uint64_t* __restrict__ ib, const uint64_t* __restrict__ ie,
                                 HybConst c, jpet_hybrid_frame_event* __restrict__ out,
                                 uint8_t* __restrict__ keep) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const jpet_hybrid_response q = r[i];
    jpet_hybrid_frame_event e{};
    e.lor_first = q.lor_first;
    e.lor_second = q.lor_second;
    const int64_t l = lor_index(q.lor_first, q.lor_second);
    if (q.lor_first < 0 || q.lor_second < 0 || l < 0 || l >= c.n_lors) {
      out[i] = e;
      keep[i] = 0;
      continue;
    }
    const float R = __fdiv_rn(seg[3 * l + 2].z, 2.0f);
    const float two_R = __fmul_rn(2.0f, R);
    const float t = __fdiv_rn(__fsub_rn(q.z_up, q.z_dn), two_R);
    const float y = __fmul_rn(-0.5f, __fdiv_rn(q.dl, __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(t, t)))));
    const float z = __fmul_rn(0.5f, __fadd_rn(__fadd_rn(q.z_up, q.z_dn),
                                              __fmul_rn(__fmul_rn(2.0f, y), t)));
    const float tan_sq = __fmul_rn(t, t);
    const float sec = __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(t, t)));
    const float A = __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(4.0f, sec), sec), c.ipd),
                              __fmul_rn(__fmul_rn(2.0f, tan_sq), c.ipz));
    const float B = __fmul_rn(__fmul_rn(-4.0f, t), c.ipz);
    const float C = __fmul_rn(2.0f, c.ipz);
    const float hb = __fdiv_rn(B, 2.0f);
    const float B_2 = __fmul_rn(hb, hb);
    const float half_up = __fdiv_rn(3.0f, __fsqrt_rn(__fsub_rn(A, __fdiv_rn(B_2, C))));
    const float half_right = __fdiv_rn(3.0f, __fsqrt_rn(__fsub_rn(C, __fdiv_rn(B_2, A))));
    e.tan = t;
    e.up = y;
    e.right = z;
    e.sec = sec;
    const float z_lo = __fsub_rn(z, half_right), z_hi = __fadd_rn(z, half_right);
    const int16_t p_lo = to_short(__fdiv_rn(__fsub_rn(z_lo, c.z_left), c.ps));
    const int16_t p_hi = to_short(__fdiv_rn(__fsub_rn(z_hi, c.z_left), c.ps));
    const int16_t zero = 0;
    e.plane_begin = (zero < p_lo) ? p_lo : zero;  // std::max((S)0, plane(z_left))
    const int16_t pe = static_cast<int16_t>(p_hi + 1);
    const int16_t np = static_cast<int16_t>(c.n_planes);
    e.plane_end = (np < pe) ? np : pe;  // std::min
    const float y_up = __fadd_rn(y, half_up), y_dn = __fsub_rn(y, half_up);
    const float t_up = __fdiv_rn(__fadd_rn(y_up, R), two_R);
    const float t_dn = __fdiv_rn(__fadd_rn(y_dn, R), two_R);
    uint64_t end = upper_bound_f(pos, ib[l], ie[l], t_up) + 1;
    if (end > static_cast<uint64_t>(c.n_infos)) end = static_cast<uint64_t>(c.n_infos);
    e.pixel_info_end = end;
    e.pixel_info_begin = lower_bound_f(pos, ib[l], ie[l], t_dn);
    bool k = !(e.plane_end <= 0 || e.plane_begin >= c.n_planes);
    if (k) {
      k = false;
      for (uint64_t j = e.pixel_info_begin; j < e.pixel_info_end; ++j) {
        const int x = p16[2 * j], yy = p16[2 * j + 1];
        if (x >= 0 && x < c.n_columns && yy >= 0 && yy < c.n_rows && w[j] > 0.0f) {
          k = true;
          break;
        }
      }
    }
    out[i] = e;
    keep[i] = k ? 1 : 0;
  }
}

// Checks caller-given frame events and sums the reference's statistics
// (used_pixels, used_voxels: reconstruction.h:311-324) over them.
__global__ void event_stats_kernel(const jpet_hybrid_frame_event* __restrict__ ev, int64_t n,
                                   const uint64_t* __restrict__ ib,
                                   const uint64_t* __restrict__ ie, HybConst c,
                                   unsigned long long* __restrict__ stats, int* __restrict__ bad) {
  unsigned long long px = 0, vx = 0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const jpet_hybrid_frame_event e = ev[i];
    const int64_t l = lor_index(e.lor_first, e.lor_second);
    // the range lies within the LOR's pixel infos and the one past its end, as
    // translate_to_frame makes it; planes within the grid
    bool ok = e.lor_first >= 0 && e.lor_second >= 0 && l >= 0 && l < c.n_lors &&
              e.pixel_info_begin <= e.pixel_info_end &&
              e.pixel_info_end <= static_cast<uint64_t>(c.n_infos) &&
              (e.plane_begin >= e.plane_end || (e.plane_begin >= 0 && e.plane_end <= c.n_planes));
    if (ok && e.pixel_info_begin < e.pixel_info_end)
      ok = e.pixel_info_begin >= ib[l] && e.pixel_info_end <= ie[l] + 1;
    if (!ok) {
      atomicExch(bad, 1);
      continue;
    }
    const unsigned long long np = e.pixel_info_end - e.pixel_info_begin;
    const int planes = e.plane_end - e.plane_begin;
    px += np;
    vx += np * static_cast<unsigned long long>(planes > 0 ? planes : 0);
  }
  for (int o = 16; o > 0; o >>= 1) {
    px += __shfl_xor_sync(0xffffffffu, px, o);
    vx += __shfl_xor_sync(0xffffffffu, vx, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&stats[0], px);
    atomicAdd(&stats[1], vx);
  }
}

// ---- image layout -----------------------------------------------------------

// reference order (x + nc (y + nr z)) -> device order ((x + nc y) np + z)
__global__ void to_device_layout(const float* __restrict__ in, float* __restrict__ out,
                                 int64_t n_px, int32_t np) {
  const int64_t n = n_px * np;
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < n;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t p = j / np, z = j - p * np;
    out[j] = in[p + z * n_px];
  }
}
__global__ void to_reference_layout(const float* __restrict__ in, float* __restrict__ out,
                                    int64_t n_px, int32_t np) {
  const int64_t n = n_px * np;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t z = i / n_px, p = i - z * n_px;
    out[i] = in[p * np + z];
  }
}

// ---- iteration ----------------------------------------------------------------

struct EvC {
  float up, right, tan, sec, R;
  float z0;  // centre of the event's first plane (voxel_grid.h:40-42)
  int32_t plane_begin;
};

// ex2.approx of the hardware; exp(x) = 2^(x log2 e).
__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// rcp.approx of the hardware (relative error below 2^-23).
__device__ __forceinline__ float rcp(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Per-pixel terms of GaussianKernel::operator() and ::sensitivity that do not
// depend on z (gaussian_kernel.h:51-79,140-150) for pixel info i of the event.
// Forms other than kSens2D keep in pa.w the info index (kMultiPlane: its weight
// is the plane's) or the pixel weight times pi (kSens3D), and in pb.z the
// pixel index (the sensitivity is the plane's).
template <int SM>
__device__ __forceinline__ void pixel_terms(const HybConst& c, const EvC& e, float4 s1,
                                            const int16_t* __restrict__ p16,
                                            const float* __restrict__ w,
                                            const float* __restrict__ sens, uint64_t i,
                                            float4& pa, float4& pb) {
  const int x = p16[2 * i], y = p16[2 * i + 1];
  float cx, cy;
  pixel_center(c, x, y, cx, cy);
  // LineSegment::projection_relative_middle (line_segment.h:82-84)
  const float up = __fadd_rn(__fmul_rn(__fsub_rn(cx, s1.x), s1.z),
                             __fmul_rn(__fsub_rn(cy, s1.y), s1.w));
  const float dy = __fsub_rn(up, e.up);
  const float yp = __fadd_rn(dy, e.up);
  const float sec_sq = __fmul_rn(e.sec, e.sec);
  const float ap = __fmul_rn(-__fsub_rn(yp, e.R), sec_sq);
  const float aq = __fmul_rn(-__fadd_rn(yp, e.R), sec_sq);
  const float ar = __fmul_rn(__fmul_rn(__fmul_rn(-2.0f, yp), e.sec), e.tan);
  const float a_ic_a = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(ap, c.ipz), ap),
                                           __fmul_rn(__fmul_rn(aq, c.ipz), aq)),
                                 __fmul_rn(__fmul_rn(ar, c.ipd), ar));
  const float ebe = __fdiv_rn(c.c0, __fsqrt_rn(a_ic_a));
  const float br = __fmul_rn(__fmul_rn(-2.0f, dy), e.sec);
  const float brr = __fmul_rn(__fmul_rn(br, c.ipd), br);
  const int pix = x + c.n_columns * y;
  // the exponent's z-independent part -log2(e) (r ipd r) / 2 and the pixel
  // weight times pi (the frame sensitivity's 1/pi) are folded in here
  const float wv = SM == kMultiPlane ? __int_as_float(static_cast<int>(i)) : w[i] * kPi;
  const float sv = SM == kSens2D ? sens[pix] : __int_as_float(pix);
  pa = make_float4(dy, ebe, brr * (-0.5f * 1.4426950408889634f), wv);
  pb = make_float4(__frcp_rn(__fsub_rn(e.R, up)), __frcp_rn(__fadd_rn(e.R, up)), sv,
                   __int_as_float(pix * c.n_planes));
}

// The pixel weight (times pi) and the sensitivity a voxel of plane col uses.
template <int SM>
__device__ __forceinline__ float voxel_pixel_weight(const HybConst& c, const float4 pa, int col,
                                                    const float* __restrict__ w) {
  if (SM != kMultiPlane) return pa.w;
  const int ap = abs_plane(col, c.n_planes_half);
  return __ldg(&w[static_cast<int64_t>(ap) * c.n_infos + __float_as_int(pa.w)]) * kPi;
}
template <int SM>
__device__ __forceinline__ float voxel_sens(const HybConst& c, const float4 pb, int col,
                                            const float* __restrict__ sens) {
  if (SM == kSens2D) return pb.z;
  const int ap = abs_plane(col, SM == kMultiPlane ? c.n_planes_half : c.sens_depth);
  return __ldg(&sens[static_cast<int64_t>(ap) * c.n_columns * c.n_rows + __float_as_int(pb.z)]);
}

// Arctangent of y / x in (-pi, pi]: reduction to r = min(|x|, |y|) / max(|x|, |y|)
// in [0, 1], atan(r) = r P(r^2) with P of degree 8 fitted by csrc/fit_atan.py
// (maximum absolute error 1e-7 on [0, 1] in float arithmetic), then the
// octant and sign reflections.  Branch-free.
__device__ __forceinline__ float atan2_poly(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float r = fminf(ax, ay) * rcp(fmaxf(ax, ay));
  const float s = r * r;
  float p = 2.456588438e-03f;
  p = fmaf(p, s, -1.440078672e-02f);
  p = fmaf(p, s, 3.978023678e-02f);
  p = fmaf(p, s, -7.234767079e-02f);
  p = fmaf(p, s, 1.049889922e-01f);
  p = fmaf(p, s, -1.416121572e-01f);
  p = fmaf(p, s, 1.998590529e-01f);
  p = fmaf(p, s, -3.333259821e-01f);
  p = fmaf(p, s, 9.999998808e-01f);
  p *= r;
  p = (ay > ax) ? 1.57079632679489662f - p : p;
  p = (x < 0.0f) ? kPi - p : p;
  return copysignf(p, y);
}

// weight = GaussianKernel::normalized(...) * pixel weight * rho of voxel
// (pixel, plane col), reconstruction.h:327-363, with the plane's terms
// dz = z - right, lp = L/2 + z, lm = L/2 - z.  exp(-b_ic_b / 2) is
// 2^(exp_bpq (dz - dy tan)^2 + pa.z); the frame sensitivity's
// atan(a) - atan(b) (gaussian_kernel.h:140-150) is evaluated as
// atan2(a - b, 1 + a b), the same angle for every a, b; a non-positive kernel
// value gives weight 0 as in the reference (reconstruction.h:335-341).
template <int SM>
__device__ __forceinline__ float plane_weight(const HybConst& c, const EvC& e, const float4 pa,
                                              const float4 pb, float dz, float lp, float lm,
                                              int col, const float* __restrict__ rho,
                                              const float* __restrict__ w) {
  const float bpq = fmaf(-pa.x, e.tan, dz);
  const float K = pa.y * ex2(fmaf(bpq * bpq, c.exp_bpq, pa.z));
  const float a = fminf(lm * pb.x, lp * pb.y);
  const float bb = fmaxf(-lp * pb.x, -lm * pb.y);
  const float ang = atan2_poly(a - bb, fmaf(a, bb, 1.0f));
  const float v = (K * voxel_pixel_weight<SM>(c, pa, col, w)) * rcp(ang) *
                  __ldg(&rho[__float_as_int(pb.w) + col]);
  return ang < 0.0f ? 0.0f : v;
}

// The same for the event's k-th plane, z = z0 + k pixel_size.
template <int SM>
__device__ __forceinline__ float voxel_weight(const HybConst& c, const EvC& e, const float4 pa,
                                              const float4 pb, int k,
                                              const float* __restrict__ rho,
                                              const float* __restrict__ w) {
  const float z = fmaf(static_cast<float>(k), c.ps, e.z0);
  return plane_weight<SM>(c, e, pa, pb, z - e.right, c.L2 + z, c.L2 - z, e.plane_begin + k,
                          rho, w);
}

// Advances a thread's (pixel, plane) position by one CTA-wide step of the
// flattened walk: kThreads voxels = q pixels and r planes.
__device__ __forceinline__ void walk(int& i, int& k, int q, int r, int npl) {
  k += r;
  i += q;
  if (k >= npl) {
    k -= npl;
    ++i;
  }
}

// Multiplicity of info i's voxels in the back-projection.  The reference keeps
// the kernel values in a voxel-indexed image (reconstruction.h:339,361,368)
// and back-projects every occurrence of a voxel with the value written last.
// Pixels of one LOR are distinct, so the only repeated pixel is the info one
// past the LOR's end that the range takes in (reconstruction.h:134-140): when
// it repeats the pixel of info dup, info dup contributes nothing and the last
// info twice.
__device__ __forceinline__ float multiplicity(int64_t i, int dup, int64_t last) {
  return dup < 0 ? 1.0f : (i == dup ? 0.0f : (i == last ? 2.0f : 1.0f));
}

// One CTA per event.  The pixel terms of up to kPix infos go to shared
// memory.  Thread tid takes plane tid % npl of the pixels tid / npl,
// tid / npl + G, ... (G = kThreads / npl groups), so neighbouring threads touch
// neighbouring planes of one pixel and every z-dependent term is computed once
// per event; each thread keeps its first kSteps weights in shared memory for
// the back-projection.  Events with more than kPix infos or kThreads planes are
// walked flattened, chunk by chunk, and recomputed in the back-projection.
template <int SM>
__global__ void __launch_bounds__(kThreads)
    iterate_kernel(const jpet_hybrid_frame_event* __restrict__ ev, int64_t n,
                   const float4* __restrict__ seg, const int16_t* __restrict__ p16,
                   const float* __restrict__ w, const float* __restrict__ sens,
                   const float* __restrict__ rho, float* __restrict__ out, HybConst c,
                   unsigned long long* __restrict__ n_positive) {
  __shared__ float4 pa[kPix];  // dy, element_before_exp, exponent term, pixel weight * pi
  __shared__ float4 pb[kPix];  // 1/(R - up), 1/(R + up), sensitivity, base index (int bits)
  __shared__ float cache[kSteps * kThreads];  // weights of each thread's first kSteps voxels
  __shared__ float red_den[kWarpsPerCta];
  __shared__ int red_dup[kWarpsPerCta];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint32_t* p32 = reinterpret_cast<const uint32_t*>(p16);
  unsigned long long positive = 0;
  for (int64_t ei = blockIdx.x; ei < n; ei += gridDim.x) {
    const jpet_hybrid_frame_event fe = ev[ei];
    const int npl = fe.plane_end - fe.plane_begin;
    const int64_t nin = static_cast<int64_t>(fe.pixel_info_end - fe.pixel_info_begin);
    if (npl <= 0 || nin <= 0) continue;
    const int64_t l = lor_index(fe.lor_first, fe.lor_second);
    const float4 s1 = seg[3 * l + 1];  // mid_x, mid_y, direction_x, direction_y
    EvC e;
    e.up = fe.up;
    e.right = fe.right;
    e.tan = fe.tan;
    e.sec = fe.sec;
    e.R = __fdiv_rn(seg[3 * l + 2].z, 2.0f);
    e.plane_begin = fe.plane_begin;
    e.z0 = __fadd_rn(__fmul_rn(__fadd_rn(static_cast<float>(fe.plane_begin), 0.5f), c.ps),
                     c.z_left);
    const uint32_t last_pixel = p32[fe.pixel_info_end - 1];
    // main path: at most kPix infos and kThreads planes; thread tid holds
    // plane k of pixel group g (G groups of npl threads)
    const bool one_chunk = nin <= kPix && npl <= kThreads;
    const int G = one_chunk ? kThreads / npl : 1;
    const int g0 = tid / npl, kk = tid - g0 * npl;
    const bool active = g0 < G;
    const int col = e.plane_begin + kk;
    const float z = fmaf(static_cast<float>(kk), c.ps, e.z0);
    const float dz = z - e.right, lp = c.L2 + z, lm = c.L2 - z;
    // fallback: the flattened walk, kThreads voxels = q pixels and r planes per step
    const int q = kThreads / npl, r = kThreads - q * npl;
    const int i0 = g0, k0 = kk;
    int dup = -1;  // info whose pixel the range's last info repeats (-1: none)
    float den = 0.0f;
    if (one_chunk) {
      const int ni = static_cast<int>(nin);
      __syncthreads();
      for (int j = tid; j < ni; j += kThreads) {
        const int64_t info = static_cast<int64_t>(fe.pixel_info_begin) + j;
        pixel_terms<SM>(c, e, s1, p16, w, sens, info, pa[j], pb[j]);
        if (j < ni - 1 && p32[info] == last_pixel) dup = j;
      }
      __syncthreads();
      // thread = (pixel group g, plane k): groups walk the pixels g, g + G, ...;
      // the first kSteps weights are kept for the back-projection
      const int nmine = active ? (ni - g0 + G - 1) / G : 0;  // pixels of this thread
      const int ncached = nmine < kSteps ? nmine : kSteps;
      const float4* a = pa + g0;
      const float4* b = pb + g0;
      float* cp = cache + tid;
      for (int t = 0; t < ncached; ++t, a += G, b += G, cp += kThreads) {
        const float4 bv = *b;
        const float v = plane_weight<SM>(c, e, *a, bv, dz, lp, lm, col, rho, w);
        den = fmaf(v, voxel_sens<SM>(c, bv, col, sens), den);
        *cp = v;
      }
      for (int t = ncached; t < nmine; ++t, a += G, b += G) {
        const float4 bv = *b;
        den = fmaf(plane_weight<SM>(c, e, *a, bv, dz, lp, lm, col, rho, w),
                   voxel_sens<SM>(c, bv, col, sens), den);
      }
    } else {
      for (int64_t cb = 0; cb < nin; cb += kPix) {
        const int cn = static_cast<int>(nin - cb < kPix ? nin - cb : kPix);
        __syncthreads();
        for (int j = tid; j < cn; j += kThreads) {
          const int64_t info = static_cast<int64_t>(fe.pixel_info_begin) + cb + j;
          pixel_terms<SM>(c, e, s1, p16, w, sens, info, pa[j], pb[j]);
          if (cb + j < nin - 1 && p32[info] == last_pixel) dup = static_cast<int>(cb + j);
        }
        __syncthreads();
        for (int i = i0, k = k0; i < cn; walk(i, k, q, r, npl))
          den = fmaf(voxel_weight<SM>(c, e, pa[i], pb[i], k, rho, w),
                     voxel_sens<SM>(c, pb[i], e.plane_begin + k, sens), den);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      den += __shfl_xor_sync(0xffffffffu, den, o);
      dup = max(dup, __shfl_xor_sync(0xffffffffu, dup, o));
    }
    if (lane == 0) {
      red_den[wid] = den;
      red_dup[wid] = dup;
    }
    __syncthreads();
    den = 0.0f;
    dup = -1;
#pragma unroll
    for (int j = 0; j < kWarpsPerCta; ++j) {
      den += red_den[j];
      dup = max(dup, red_dup[j]);
    }
    if (!(den > 0.0f)) continue;
    positive += (tid == 0);
    const float inv = __frcp_rn(den);
    if (one_chunk) {
      const int ni = static_cast<int>(nin);
      const int nmine = active ? (ni - g0 + G - 1) / G : 0;
      const int ncached = nmine < kSteps ? nmine : kSteps;
      const float4* a = pa + g0;
      const float4* b = pb + g0;
      const float* cp = cache + tid;
      float* o = out + col;
      if (dup < 0) {
        int t = 0;
        for (; t < ncached; ++t, b += G, cp += kThreads) {
          const float v = *cp;
          if (v != 0.0f) atomicAdd(o + __float_as_int(b->w), v * inv);
        }
        for (a += t * G; t < nmine; ++t, a += G, b += G) {
          const float4 bv = *b;
          const float v = plane_weight<SM>(c, e, *a, bv, dz, lp, lm, col, rho, w);
          if (v != 0.0f) atomicAdd(o + __float_as_int(bv.w), v * inv);
        }
      } else {
        for (int t = 0, i = g0; t < nmine; ++t, i += G, a += G, b += G, cp += kThreads) {
          const float4 bv = *b;
          const float v =
              t < ncached ? *cp : plane_weight<SM>(c, e, *a, bv, dz, lp, lm, col, rho, w);
          const float x = v * multiplicity(i, dup, ni - 1);
          if (x != 0.0f) atomicAdd(o + __float_as_int(bv.w), x * inv);
        }
      }
    } else {
      for (int64_t cb = 0; cb < nin; cb += kPix) {
        const int cn = static_cast<int>(nin - cb < kPix ? nin - cb : kPix);
        __syncthreads();
        for (int j = tid; j < cn; j += kThreads)
          pixel_terms<SM>(c, e, s1, p16, w, sens,
                          static_cast<int64_t>(fe.pixel_info_begin) + cb + j, pa[j], pb[j]);
        __syncthreads();
        for (int i = i0, k = k0; i < cn; walk(i, k, q, r, npl)) {
          const float x = voxel_weight<SM>(c, e, pa[i], pb[i], k, rho, w) *
                          multiplicity(cb + i, dup, nin - 1);
          if (x != 0.0f) atomicAdd(&out[__float_as_int(pb[i].w) + e.plane_begin + k], x * inv);
        }
      }
    }
  }
  if (tid == 0 && positive) atomicAdd(n_positive, positive);
}


}  // namespace

struct jpet_hybrid {
  jpet_hybrid_opts opts{};
  HybConst c{};
  int device = 0;
  int n_sms = 0;
  int iterate_blocks = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  std::string last_error = "no error";
  int64_t n_events = 0;
  int64_t used_pixels = 0, used_voxels = 0;
  Buf<float4> seg;           // 3 float4 per LOR (the LineSegment fields)
  Buf<float> widths, pos, w, sens, rho, out, stage;
  Buf<int2> pix_dummy;
  Buf<int16_t> pix;          // x, y per pixel info
  Buf<uint64_t> ib, ie;
  Buf<jpet_hybrid_frame_event> ev, ev_tmp;
  Buf<jpet_hybrid_response> resp;
  Buf<uint8_t> keep, temp;
  Buf<int32_t> keys, vals;
  Buf<long long> n_sel;
  Buf<unsigned long long> counters;  // [0] pixels [1] voxels [2] positive
  Buf<int> flag;
};

namespace {

int fail(jpet_hybrid* h, int code, const std::string& msg) {
  if (h) h->last_error = msg;
  else g_hybrid_error = msg;
  return code;
}

int cuda_fail(jpet_hybrid* h, cudaError_t e, const char* what) {
  return fail(h, JPET_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define HYB_CUDA(h, call, what)                     \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
  } while (0)

int grid_for(const jpet_hybrid* h, int64_t n, int threads = 256) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = static_cast<int64_t>(h->n_sms) * 8;
  return static_cast<int>(std::max<int64_t>(1, std::min(b, cap)));
}

// Kernel constants computed as GaussianKernel's constructor computes them
// (gaussian_kernel.h:27-33: float reciprocals, the normalisation in double
// from a float square root) and the grid's as PixelGrid's (pixel_grid.h:24-30).
HybConst make_const(const jpet_hybrid_geom& g) {
  HybConst c{};
  c.ipz = 1.0f / (g.sigma_z * g.sigma_z);
  c.ipd = 1.0f / (g.sigma_dl * g.sigma_dl);
  c.c0 = static_cast<float>(1.0 / (2.0 * M_PI * M_PI) *
                            static_cast<double>(std::sqrt(c.ipz * c.ipz * c.ipd)));
  c.ps = g.pixel_size;
  c.z_left = g.z_left;
  c.llcx = g.lower_left_x + g.pixel_size / 2.0f;
  c.llcy = g.lower_left_y + g.pixel_size / 2.0f;
  c.L2 = g.length / 2.0f;
  c.exp_bpq = static_cast<float>(-1.4426950408889634 * static_cast<double>(c.ipz));
  c.n_columns = g.n_columns;
  c.n_rows = g.n_rows;
  c.n_planes = g.n_planes;
  c.n_lors = static_cast<int32_t>((static_cast<int64_t>(g.n_detectors) + 1) * g.n_detectors / 2);
  c.n_infos = g.n_pixel_infos;
  c.n_planes_half = g.n_planes_half > 1 ? g.n_planes_half : 1;
  c.sens_depth = 1;
  return c;
}

int check_geom(const jpet_hybrid_geom* g) {
  if (!g) return fail(nullptr, JPET_ERR_ARGUMENT, "geometry is NULL");
  if (g->n_detectors < 1 || g->n_detectors > 32767)
    return fail(nullptr, JPET_ERR_ARGUMENT, "n_detectors must be in [1, 32767]");
  if (g->n_pixel_infos < 0 || g->n_pixel_infos >= (int64_t(1) << 31))
    return fail(nullptr, JPET_ERR_ARGUMENT, "n_pixel_infos must be in [0, 2^31)");
  if (g->n_columns < 1 || g->n_rows < 1 || g->n_planes < 1 || g->n_columns > 32767 ||
      g->n_rows > 32767 || g->n_planes > 32767)
    return fail(nullptr, JPET_ERR_ARGUMENT, "grid sizes must be in [1, 32767]");
  if (static_cast<int64_t>(g->n_columns) * g->n_rows * g->n_planes >= (int64_t(1) << 31))
    return fail(nullptr, JPET_ERR_ARGUMENT, "more than 2^31 - 1 voxels");
  if (!(g->pixel_size > 0) || !(g->sigma_z > 0) || !(g->sigma_dl > 0) || !(g->length > 0))
    return fail(nullptr, JPET_ERR_ARGUMENT, "pixel size, sigmas and length must be positive");
  if (!g->lor_segments || !g->lor_pixel_info_begin || !g->lor_pixel_info_end)
    return fail(nullptr, JPET_ERR_ARGUMENT, "LOR arrays are NULL");
  if (g->n_pixel_infos > 0 && (!g->pixels || !g->pixel_positions))
    return fail(nullptr, JPET_ERR_ARGUMENT, "pixel info arrays are NULL");
  if (g->n_planes_half < 0 || g->n_planes_half > g->n_planes)
    return fail(nullptr, JPET_ERR_ARGUMENT, "n_planes_half must be in [0, n_planes]");
  if (g->n_planes_half > 1 && g->n_pixel_infos * g->n_planes_half >= (int64_t(1) << 31))
    return fail(nullptr, JPET_ERR_ARGUMENT, "more than 2^31 - 1 weights");
  const int64_t n_lors = (static_cast<int64_t>(g->n_detectors) + 1) * g->n_detectors / 2;
  for (int64_t l = 0; l < n_lors; ++l) {
    if (g->lor_pixel_info_begin[l] > g->lor_pixel_info_end[l] ||
        g->lor_pixel_info_end[l] > static_cast<uint64_t>(g->n_pixel_infos))
      return fail(nullptr, JPET_ERR_ARGUMENT,
                  "LOR " + std::to_string(l) + ": pixel info range outside [0, n_pixel_infos]");
  }
  return JPET_OK;
}

// Stable radix sort of (pixel index, info index): the infos of each pixel in
// ascending info order.  Used to check that no LOR lists a pixel twice and, for
// the computed sensitivity, to sum each pixel's weights sequentially in that
// order (the reference's order of additions).
int sort_and_check_pixels(jpet_hybrid* h, bool sum) {
  const int64_t n = h->c.n_infos;
  const int64_t n_px = static_cast<int64_t>(h->c.n_columns) * h->c.n_rows;
  HYB_CUDA(h, cudaMemsetAsync(h->sens.p, 0, n_px * h->c.sens_depth * sizeof(float), h->stream),
           "memset");
  if (n == 0) return JPET_OK;
  Buf<int32_t> keys2, vals2, lor_of;
  struct Release {
    Buf<int32_t>* b[3];
    ~Release() {
      for (auto* x : b) x->release();
    }
  } release{{&keys2, &vals2, &lor_of}};
  HYB_CUDA(h, keys2.alloc(n), "cudaMalloc");
  HYB_CUDA(h, vals2.alloc(n), "cudaMalloc");
  HYB_CUDA(h, lor_of.alloc(n), "cudaMalloc");
  int end_bit = 1;
  while ((int64_t(1) << end_bit) < n_px) ++end_bit;
  size_t bytes = 0;
  HYB_CUDA(h, cub::DeviceRadixSort::SortPairs(nullptr, bytes, h->keys.p, keys2.p, h->vals.p,
                                              vals2.p, static_cast<int>(n), 0, end_bit,
                                              h->stream),
           "sort size");
  HYB_CUDA(h, h->temp.alloc(bytes), "cudaMalloc");
  HYB_CUDA(h, cub::DeviceRadixSort::SortPairs(h->temp.p, bytes, h->keys.p, keys2.p, h->vals.p,
                                              vals2.p, static_cast<int>(n), 0, end_bit,
                                              h->stream),
           "sort");
  HYB_CUDA(h, cudaMemsetAsync(lor_of.p, 0xff, n * sizeof(int32_t), h->stream), "memset");
  lor_of_info_kernel<<<grid_for(h, 32LL * h->c.n_lors), 256, 0, h->stream>>>(h->ib.p, h->ie.p,
                                                                           h->c.n_lors, lor_of.p);
  HYB_CUDA(h, cudaGetLastError(), "lor of info");
  HYB_CUDA(h, cudaMemsetAsync(h->flag.p, 0, sizeof(int), h->stream), "memset");
  unique_pixels_kernel<<<grid_for(h, n), 256, 0, h->stream>>>(keys2.p, vals2.p, n, lor_of.p,
                                                             h->flag.p);
  HYB_CUDA(h, cudaGetLastError(), "unique pixels");
  if (sum) {
    // one plane half after another (calculate_sensitivity sums each
    // (pixel, plane) over the infos in info order)
    for (int plane = 0; plane < h->c.n_planes_half; ++plane) {
      sensitivity_sum_kernel<<<grid_for(h, n), 256, 0, h->stream>>>(
          keys2.p, vals2.p, n, h->w.p + n * plane, h->sens.p + n_px * plane);
      HYB_CUDA(h, cudaGetLastError(), "sensitivity");
    }
  }
  int bad = 0;
  HYB_CUDA(h, cudaMemcpyAsync(&bad, h->flag.p, sizeof bad, cudaMemcpyDeviceToHost, h->stream),
           "copy");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  if (bad) return fail(h, JPET_ERR_ARGUMENT, "a LOR lists the same pixel twice");
  return JPET_OK;
}

int finish_events(jpet_hybrid* h, int64_t n) {
  h->n_events = n;
  HYB_CUDA(h, cudaMemsetAsync(h->counters.p, 0, 3 * sizeof(unsigned long long), h->stream),
           "memset");
  HYB_CUDA(h, cudaMemsetAsync(h->flag.p, 0, sizeof(int), h->stream), "memset");
  if (n > 0) {
    event_stats_kernel<<<grid_for(h, n), 256, 0, h->stream>>>(h->ev.p, n, h->ib.p, h->ie.p, h->c,
                                                              h->counters.p, h->flag.p);
    HYB_CUDA(h, cudaGetLastError(), "event check");
  }
  unsigned long long st[2];
  int bad = 0;
  HYB_CUDA(h, cudaMemcpyAsync(st, h->counters.p, sizeof st, cudaMemcpyDeviceToHost, h->stream),
           "copy");
  HYB_CUDA(h, cudaMemcpyAsync(&bad, h->flag.p, sizeof bad, cudaMemcpyDeviceToHost, h->stream),
           "copy");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  if (bad) {
    h->n_events = 0;
    return fail(h, JPET_ERR_ARGUMENT,
                "frame event with a LOR, pixel-info range or plane range outside the geometry "
                "(ranges lie within the LOR's pixel infos and the one past its end)");
  }
  h->used_pixels = static_cast<int64_t>(st[0]);
  h->used_voxels = static_cast<int64_t>(st[1]);
  return JPET_OK;
}

int translate(jpet_hybrid* h, const jpet_hybrid_response* d_resp, int64_t n) {
  HYB_CUDA(h, h->ev_tmp.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  HYB_CUDA(h, h->ev.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  HYB_CUDA(h, h->keep.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  long long kept = 0;
  if (n > 0) {
    translate_kernel<<<grid_for(h, n), 256, 0, h->stream>>>(
        d_resp, n, h->seg.p, h->pix.p, h->pos.p, h->w.p, h->ib.p, h->ie.p, h->c, h->ev_tmp.p,
        h->keep.p);
    HYB_CUDA(h, cudaGetLastError(), "translate");
    size_t bytes = 0;
    HYB_CUDA(h, cub::DeviceSelect::Flagged(nullptr, bytes, h->ev_tmp.p, h->keep.p, h->ev.p,
                                           h->n_sel.p, n, h->stream),
             "select size");
    HYB_CUDA(h, h->temp.alloc(bytes), "cudaMalloc");
    HYB_CUDA(h, cub::DeviceSelect::Flagged(h->temp.p, bytes, h->ev_tmp.p, h->keep.p, h->ev.p,
                                           h->n_sel.p, n, h->stream),
             "select");
    HYB_CUDA(h, cudaMemcpyAsync(&kept, h->n_sel.p, sizeof kept, cudaMemcpyDeviceToHost,
                                h->stream),
             "copy");
    HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  }
  return finish_events(h, kept);
}

}  // namespace

extern "C" {

void jpet_hybrid_default_opts(jpet_hybrid_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->weights = JPET_HYBRID_WEIGHTS_COMPUTED;
  o->sensitivity = JPET_HYBRID_SENSITIVITY_COMPUTED;
}

const char* jpet_hybrid_last_error(const jpet_hybrid_t* h) {
  return h ? h->last_error.c_str() : g_hybrid_error.c_str();
}

int jpet_hybrid_destroy(jpet_hybrid_t* h) {
  if (!h) return JPET_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->seg.release();
  h->widths.release();
  h->pos.release();
  h->w.release();
  h->sens.release();
  h->rho.release();
  h->out.release();
  h->stage.release();
  h->pix.release();
  h->ib.release();
  h->ie.release();
  h->ev.release();
  h->ev_tmp.release();
  h->resp.release();
  h->keep.release();
  h->temp.release();
  h->keys.release();
  h->vals.release();
  h->n_sel.release();
  h->counters.release();
  h->flag.release();
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return JPET_OK;
}

int jpet_hybrid_create(const jpet_hybrid_geom* g, const jpet_hybrid_opts* opts_in,
                       jpet_hybrid_t** out) {
  if (!out) return fail(nullptr, JPET_ERR_ARGUMENT, "out is NULL");
  *out = nullptr;
  int rc = check_geom(g);
  if (rc != JPET_OK) return rc;
  jpet_hybrid_opts opts;
  jpet_hybrid_default_opts(&opts);
  if (opts_in) opts = *opts_in;
  if (opts.weights < 0 || opts.weights > 2 || opts.sensitivity < 0 || opts.sensitivity > 3)
    return fail(nullptr, JPET_ERR_ARGUMENT, "unknown weights or sensitivity mode");
  const int planes_half = g->n_planes_half > 1 ? g->n_planes_half : 1;
  if (planes_half > 1 && opts.weights == JPET_HYBRID_WEIGHTS_COMPUTED)
    return fail(nullptr, JPET_ERR_ARGUMENT,
                "a multi-plane geometry needs given weights (one system matrix per plane half)");
  if (planes_half > 1 && opts.sensitivity == JPET_HYBRID_SENSITIVITY_GIVEN)
    return fail(nullptr, JPET_ERR_ARGUMENT,
                "a multi-plane geometry has a 3D sensitivity (JPET_HYBRID_SENSITIVITY_GIVEN_3D)");
  // planes of the sensitivity image (reconstruction.h:80-85)
  const int sens_depth = planes_half > 1 ? planes_half
                         : opts.sensitivity == JPET_HYBRID_SENSITIVITY_GIVEN_3D ? g->n_planes / 2
                                                                                : 1;
  if (sens_depth < 1)
    return fail(nullptr, JPET_ERR_ARGUMENT, "a 3D sensitivity needs at least 2 planes");
  if (opts.weights != JPET_HYBRID_WEIGHTS_COMPUTED && g->n_pixel_infos > 0 && !g->pixel_weights)
    return fail(nullptr, JPET_ERR_ARGUMENT, "given weights but pixel_weights is NULL");
  if (opts.weights == JPET_HYBRID_WEIGHTS_COMPUTED && !g->lor_widths)
    return fail(nullptr, JPET_ERR_ARGUMENT, "computed weights need lor_widths");
  if ((opts.sensitivity == JPET_HYBRID_SENSITIVITY_GIVEN ||
       opts.sensitivity == JPET_HYBRID_SENSITIVITY_GIVEN_3D) && !opts.sensitivity_map)
    return fail(nullptr, JPET_ERR_ARGUMENT, "given sensitivity but sensitivity_map is NULL");
  if (opts.block_threads != 0)
    return fail(nullptr, JPET_ERR_UNSUPPORTED, "the iteration kernel runs 128-thread CTAs");
  auto* h = new jpet_hybrid();
  h->opts = opts;
  h->device = opts.device;
  h->c = make_const(*g);
  h->c.sens_depth = sens_depth;
  auto bail = [&](int code) {
    g_hybrid_error = h->last_error;
    jpet_hybrid_destroy(h);
    return code;
  };
#define CREATE_CUDA(call, what)                               \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return bail(cuda_fail(h, e_, what)); \
  } while (0)
  CREATE_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
  CREATE_CUDA(cudaDeviceGetAttribute(&h->n_sms, cudaDevAttrMultiProcessorCount, h->device),
              "device attribute");
  CREATE_CUDA(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking), "stream");
  h->stream = h->own_stream;
  int per_sm = 0;
  CREATE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, iterate_kernel<kSens2D>,
                                                            kThreads, 0),
              "occupancy");
  h->iterate_blocks = std::max(1, per_sm) * h->n_sms;

  const int64_t n_lors = h->c.n_lors, n = h->c.n_infos;
  const int64_t n_px = static_cast<int64_t>(h->c.n_columns) * h->c.n_rows;
  const int64_t n_vox = n_px * h->c.n_planes;
  CREATE_CUDA(h->seg.alloc(3 * n_lors), "cudaMalloc");
  CREATE_CUDA(h->widths.alloc(n_lors), "cudaMalloc");
  CREATE_CUDA(h->ib.alloc(n_lors), "cudaMalloc");
  CREATE_CUDA(h->ie.alloc(n_lors), "cudaMalloc");
  CREATE_CUDA(h->pix.alloc(2 * std::max<int64_t>(n, 1)), "cudaMalloc");
  CREATE_CUDA(h->pos.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  CREATE_CUDA(h->w.alloc(std::max<int64_t>(n * planes_half, 1)), "cudaMalloc");
  CREATE_CUDA(h->keys.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  CREATE_CUDA(h->vals.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  CREATE_CUDA(h->sens.alloc(n_px * sens_depth), "cudaMalloc");
  CREATE_CUDA(h->rho.alloc(n_vox), "cudaMalloc");
  CREATE_CUDA(h->out.alloc(n_vox), "cudaMalloc");
  CREATE_CUDA(h->n_sel.alloc(1), "cudaMalloc");
  CREATE_CUDA(h->counters.alloc(3), "cudaMalloc");
  CREATE_CUDA(h->flag.alloc(1), "cudaMalloc");
  cudaStream_t s = h->stream;
  static_assert(sizeof(jpet_lor_segment) == 3 * sizeof(float4), "segment layout");
  CREATE_CUDA(cudaMemcpyAsync(h->seg.p, g->lor_segments, n_lors * sizeof(jpet_lor_segment),
                              cudaMemcpyHostToDevice, s),
              "upload");
  if (g->lor_widths)
    CREATE_CUDA(cudaMemcpyAsync(h->widths.p, g->lor_widths, n_lors * sizeof(float),
                                cudaMemcpyHostToDevice, s),
                "upload");
  CREATE_CUDA(cudaMemcpyAsync(h->ib.p, g->lor_pixel_info_begin, n_lors * sizeof(uint64_t),
                              cudaMemcpyHostToDevice, s),
              "upload");
  CREATE_CUDA(cudaMemcpyAsync(h->ie.p, g->lor_pixel_info_end, n_lors * sizeof(uint64_t),
                              cudaMemcpyHostToDevice, s),
              "upload");
  if (n > 0) {
    CREATE_CUDA(cudaMemcpyAsync(h->pix.p, g->pixels, n * sizeof(jpet_pixel),
                                cudaMemcpyHostToDevice, s),
                "upload");
    CREATE_CUDA(cudaMemcpyAsync(h->pos.p, g->pixel_positions, n * sizeof(float),
                                cudaMemcpyHostToDevice, s),
                "upload");
    if (opts.weights != JPET_HYBRID_WEIGHTS_COMPUTED)
      CREATE_CUDA(cudaMemcpyAsync(h->w.p, g->pixel_weights, n * planes_half * sizeof(float),
                                  cudaMemcpyHostToDevice, s),
                  "upload");
  }
  // pixels inside the grid, and the sort keys of the sensitivity
  CREATE_CUDA(cudaMemsetAsync(h->flag.p, 0, sizeof(int), s), "memset");
  if (n > 0) {
    pixel_keys_kernel<<<grid_for(h, n), 256, 0, s>>>(h->pix.p, n, h->c, h->keys.p, h->vals.p,
                                                     h->flag.p);
    CREATE_CUDA(cudaGetLastError(), "pixel check");
  }
  int bad = 0;
  CREATE_CUDA(cudaMemcpyAsync(&bad, h->flag.p, sizeof bad, cudaMemcpyDeviceToHost, s), "copy");
  CREATE_CUDA(cudaStreamSynchronize(s), "synchronize");
  if (bad) return bail(fail(h, JPET_ERR_ARGUMENT, "a pixel info lies outside the pixel grid"));
  if (opts.weights == JPET_HYBRID_WEIGHTS_COMPUTED && n > 0) {
    weights_kernel<<<grid_for(h, 32 * n_lors), 256, 0, s>>>(
        h->seg.p, h->widths.p, reinterpret_cast<const int2*>(h->pix.p), h->ib.p, h->ie.p, h->w.p,
        h->c, std::sqrt(2 * M_PI));
    CREATE_CUDA(cudaGetLastError(), "weights");
  }
  const int rc2 = sort_and_check_pixels(h, opts.sensitivity == JPET_HYBRID_SENSITIVITY_COMPUTED);
  if (rc2 != JPET_OK) return bail(rc2);
  if (opts.sensitivity == JPET_HYBRID_SENSITIVITY_ONE) {
    fill_kernel<<<grid_for(h, n_px * sens_depth), 256, 0, s>>>(h->sens.p, n_px * sens_depth,
                                                               1.0f);
    CREATE_CUDA(cudaGetLastError(), "fill");
  } else if (opts.sensitivity == JPET_HYBRID_SENSITIVITY_GIVEN ||
             opts.sensitivity == JPET_HYBRID_SENSITIVITY_GIVEN_3D) {
    CREATE_CUDA(cudaMemcpyAsync(h->sens.p, opts.sensitivity_map,
                                n_px * sens_depth * sizeof(float), cudaMemcpyHostToDevice, s),
                "upload");
  }
  h->keys.release();
  h->vals.release();
  if (opts.weights != JPET_HYBRID_WEIGHTS_NORMALIZED && n > 0) {
    normalize_kernel<<<grid_for(h, n), 256, 0, s>>>(h->pix.p, n, h->c, h->sens.p, h->w.p);
    CREATE_CUDA(cudaGetLastError(), "normalize");
  }
  fill_kernel<<<grid_for(h, n_vox), 256, 0, s>>>(h->rho.p, n_vox, 1.0f);
  CREATE_CUDA(cudaGetLastError(), "fill");
  CREATE_CUDA(cudaStreamSynchronize(s), "synchronize");
#undef CREATE_CUDA
  *out = h;
  return JPET_OK;
}

int jpet_hybrid_set_stream(jpet_hybrid_t* h, void* stream) {
  if (!h) return fail(nullptr, JPET_ERR_ARGUMENT, "handle is NULL");
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  return JPET_OK;
}

int jpet_hybrid_set_responses_device(jpet_hybrid_t* h, const jpet_hybrid_response* d, int64_t n) {
  if (!h) return fail(nullptr, JPET_ERR_ARGUMENT, "handle is NULL");
  if (n < 0 || (n > 0 && !d)) return fail(h, JPET_ERR_ARGUMENT, "bad responses");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  return translate(h, d, n);
}

int jpet_hybrid_set_responses(jpet_hybrid_t* h, const jpet_hybrid_response* r, int64_t n) {
  if (!h) return fail(nullptr, JPET_ERR_ARGUMENT, "handle is NULL");
  if (n < 0 || (n > 0 && !r)) return fail(h, JPET_ERR_ARGUMENT, "bad responses");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  HYB_CUDA(h, h->resp.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  if (n > 0)
    HYB_CUDA(h, cudaMemcpyAsync(h->resp.p, r, n * sizeof(jpet_hybrid_response),
                                cudaMemcpyHostToDevice, h->stream),
             "upload");
  return translate(h, h->resp.p, n);
}

int jpet_hybrid_set_frame_events(jpet_hybrid_t* h, const jpet_hybrid_frame_event* e, int64_t n) {
  if (!h) return fail(nullptr, JPET_ERR_ARGUMENT, "handle is NULL");
  if (n < 0 || (n > 0 && !e)) return fail(h, JPET_ERR_ARGUMENT, "bad frame events");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  HYB_CUDA(h, h->ev.alloc(std::max<int64_t>(n, 1)), "cudaMalloc");
  if (n > 0)
    HYB_CUDA(h, cudaMemcpyAsync(h->ev.p, e, n * sizeof(jpet_hybrid_frame_event),
                                cudaMemcpyHostToDevice, h->stream),
             "upload");
  return finish_events(h, n);
}

int jpet_hybrid_get_frame_events(jpet_hybrid_t* h, jpet_hybrid_frame_event* out, int64_t* n) {
  if (!h || !n) return fail(h, JPET_ERR_ARGUMENT, "NULL argument");
  *n = h->n_events;
  if (!out || h->n_events == 0) return JPET_OK;
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  HYB_CUDA(h, cudaMemcpyAsync(out, h->ev.p, h->n_events * sizeof(jpet_hybrid_frame_event),
                              cudaMemcpyDeviceToHost, h->stream),
           "download");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return JPET_OK;
}

int jpet_hybrid_set_image(jpet_hybrid_t* h, const float* rho) {
  if (!h || !rho) return fail(h, JPET_ERR_ARGUMENT, "NULL argument");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const int64_t n_px = static_cast<int64_t>(h->c.n_columns) * h->c.n_rows;
  const int64_t n_vox = n_px * h->c.n_planes;
  HYB_CUDA(h, h->stage.alloc(n_vox), "cudaMalloc");
  HYB_CUDA(h, cudaMemcpyAsync(h->stage.p, rho, n_vox * sizeof(float), cudaMemcpyHostToDevice,
                              h->stream),
           "upload");
  to_device_layout<<<grid_for(h, n_vox), 256, 0, h->stream>>>(h->stage.p, h->rho.p, n_px,
                                                              h->c.n_planes);
  HYB_CUDA(h, cudaGetLastError(), "layout");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return JPET_OK;
}

int jpet_hybrid_get_image(jpet_hybrid_t* h, float* rho) {
  if (!h || !rho) return fail(h, JPET_ERR_ARGUMENT, "NULL argument");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const int64_t n_px = static_cast<int64_t>(h->c.n_columns) * h->c.n_rows;
  const int64_t n_vox = n_px * h->c.n_planes;
  HYB_CUDA(h, h->stage.alloc(n_vox), "cudaMalloc");
  to_reference_layout<<<grid_for(h, n_vox), 256, 0, h->stream>>>(h->rho.p, h->stage.p, n_px,
                                                                 h->c.n_planes);
  HYB_CUDA(h, cudaGetLastError(), "layout");
  HYB_CUDA(h, cudaMemcpyAsync(rho, h->stage.p, n_vox * sizeof(float), cudaMemcpyDeviceToHost,
                              h->stream),
           "download");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return JPET_OK;
}

int jpet_hybrid_get_sensitivity(jpet_hybrid_t* h, float* sens) {
  if (!h || !sens) return fail(h, JPET_ERR_ARGUMENT, "NULL argument");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const int64_t n_px = static_cast<int64_t>(h->c.n_columns) * h->c.n_rows;
  HYB_CUDA(h, cudaMemcpyAsync(sens, h->sens.p, n_px * h->c.sens_depth * sizeof(float),
                              cudaMemcpyDeviceToHost, h->stream),
           "download");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return JPET_OK;
}

int jpet_hybrid_get_weights(jpet_hybrid_t* h, float* w) {
  if (!h || (!w && h->c.n_infos > 0)) return fail(h, JPET_ERR_ARGUMENT, "NULL argument");
  if (h->c.n_infos == 0) return JPET_OK;
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  HYB_CUDA(h, cudaMemcpyAsync(w, h->w.p, h->c.n_infos * h->c.n_planes_half * sizeof(float),
                              cudaMemcpyDeviceToHost, h->stream),
           "download");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return JPET_OK;
}

int jpet_hybrid_iterate(jpet_hybrid_t* h, int n) {
  if (!h) return fail(nullptr, JPET_ERR_ARGUMENT, "handle is NULL");
  if (n < 0) return fail(h, JPET_ERR_ARGUMENT, "negative iteration count");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const int64_t n_vox = static_cast<int64_t>(h->c.n_columns) * h->c.n_rows * h->c.n_planes;
  for (int it = 0; it < n; ++it) {
    HYB_CUDA(h, cudaMemsetAsync(h->out.p, 0, n_vox * sizeof(float), h->stream), "memset");
    HYB_CUDA(h, cudaMemsetAsync(h->counters.p + 2, 0, sizeof(unsigned long long), h->stream),
             "memset");
    if (h->n_events > 0) {
      auto* k = h->c.n_planes_half > 1 ? iterate_kernel<kMultiPlane>
                : h->c.sens_depth > 1  ? iterate_kernel<kSens3D>
                                       : iterate_kernel<kSens2D>;
      k<<<h->iterate_blocks, kThreads, 0, h->stream>>>(h->ev.p, h->n_events, h->seg.p, h->pix.p,
                                                      h->w.p, h->sens.p, h->rho.p, h->out.p,
                                                      h->c, h->counters.p + 2);
      HYB_CUDA(h, cudaGetLastError(), "iterate");
    }
    std::swap(h->rho, h->out);
  }
  return JPET_OK;
}

int jpet_hybrid_get_counters(jpet_hybrid_t* h, jpet_hybrid_counters* c) {
  if (!h || !c) return fail(h, JPET_ERR_ARGUMENT, "NULL argument");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  unsigned long long pos = 0;
  HYB_CUDA(h, cudaMemcpyAsync(&pos, h->counters.p + 2, sizeof pos, cudaMemcpyDeviceToHost,
                              h->stream),
           "download");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  c->used_events = h->n_events;
  c->used_pixels = h->used_pixels;
  c->used_voxels = h->used_voxels;
  c->contributing = static_cast<int64_t>(pos);
  return JPET_OK;
}

int jpet_hybrid_synchronize(jpet_hybrid_t* h) {
  if (!h) return fail(nullptr, JPET_ERR_ARGUMENT, "handle is NULL");
  HYB_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  HYB_CUDA(h, cudaStreamSynchronize(h->stream), "synchronize");
  return JPET_OK;
}

int jpet_hybrid_run(const jpet_hybrid_geom* geom, const float* sensitivity,
                    const jpet_hybrid_frame_event* events, int64_t n_events, float* rho,
                    int n_blocks, int n_iterations_in_block, int start_iteration,
                    jpet_hybrid_output_fn output, jpet_strip_progress_fn progress, void* user,
                    int device, char* device_name, size_t device_name_len) {
  if (!rho || !sensitivity || n_blocks < 0 || n_iterations_in_block < 0)
    return fail(nullptr, JPET_ERR_ARGUMENT, "bad argument");
  jpet_hybrid_opts o;
  jpet_hybrid_default_opts(&o);
  o.device = device;
  o.weights = JPET_HYBRID_WEIGHTS_NORMALIZED;
  // a multi-plane geometry comes with its 3D sensitivity (depth n_planes_half)
  o.sensitivity = (geom && geom->n_planes_half > 1) ? JPET_HYBRID_SENSITIVITY_GIVEN_3D
                                                    : JPET_HYBRID_SENSITIVITY_GIVEN;
  o.sensitivity_map = sensitivity;
  jpet_hybrid_t* h = nullptr;
  int rc = jpet_hybrid_create(geom, &o, &h);
  if (rc != JPET_OK) return rc;
  if (device_name && device_name_len > 0) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
      std::snprintf(device_name, device_name_len, "%s", prop.name);
    } else {
      device_name[0] = 0;
    }
  }
  auto done = [&](int code) {
    if (code != JPET_OK) g_hybrid_error = h->last_error;
    jpet_hybrid_destroy(h);
    return code;
  };
  if ((rc = jpet_hybrid_set_frame_events(h, events, n_events)) != JPET_OK) return done(rc);
  if ((rc = jpet_hybrid_set_image(h, rho)) != JPET_OK) return done(rc);
  // the reference's iteration and output schedule (cuda/reconstruction.cu:113-186)
  for (int block = 0; block < n_blocks; ++block) {
    for (int i = 0; i < n_iterations_in_block; ++i) {
      const int iteration = block * n_iterations_in_block + i;
      if (iteration < start_iteration) continue;
      if (progress) progress(iteration, 0, user);
      if ((rc = jpet_hybrid_iterate(h, 1)) != JPET_OK) return done(rc);
      if ((rc = jpet_hybrid_synchronize(h)) != JPET_OK) return done(rc);
      if (progress) progress(iteration, 1, user);
      if (!block && i < n_iterations_in_block - 1 &&
          (i < 5 || i == 9 || i == 14 || i == 19 || i == 29 || i == 49 || i == 99)) {
        if ((rc = jpet_hybrid_get_image(h, rho)) != JPET_OK) return done(rc);
        if (output) output(i + 1, rho, user);
      }
    }
    const int iteration = (block + 1) * n_iterations_in_block;
    if (iteration <= start_iteration) continue;
    if ((rc = jpet_hybrid_get_image(h, rho)) != JPET_OK) return done(rc);
    if (output) output(iteration, rho, user);
  }
  if (progress) progress(n_blocks * n_iterations_in_block, 0, user);
  if ((rc = jpet_hybrid_get_image(h, rho)) != JPET_OK) return done(rc);
  return done(JPET_OK);
}

}  // extern "C"
