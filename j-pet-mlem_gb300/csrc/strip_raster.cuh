// Warp rasteriser of one event in the reference's rounding (shared by the
// exact iteration kernel, the large-box path and the fast kernel's fallback).
#pragma once

#include <cstdint>

#include "strip_device.cuh"
#include "strip_internal.h"

namespace jpet {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// ---------------------------------------------------------------------------------
// Image accessors: a shared-memory window or the global image
// ---------------------------------------------------------------------------------

struct WindowAccess {
  const float* rho;  // shared
  float* out;        // shared
  int ox, oy, pitch;
  __device__ __forceinline__ float rho_at(int y, int x) const {
    return rho[(y - oy) * pitch + (x - ox)];
  }
  __device__ __forceinline__ void add(int y, int x, float v) const {
    atomicAdd(&out[(y - oy) * pitch + (x - ox)], v);
  }
};

struct GlobalAccess {
  const float* rho;
  float* out;
  int n_z;
  __device__ __forceinline__ float rho_at(int y, int x) const { return __ldg(&rho[y * n_z + x]); }
  __device__ __forceinline__ void add(int y, int x, float v) const {
    atomicAdd(&out[y * n_z + x], v);
  }
};

// ---------------------------------------------------------------------------------
// One event, one warp: reference-order arithmetic
// ---------------------------------------------------------------------------------
//
// The warp walks the rows of the event's clamped box (reconstruction.h:255-256).
// In each row it visits only the columns that can pass the 3-sigma test: the
// quadratic A dy^2 + B dy dz + C dz^2 <= 9 bounds dz to tan*dy +- h with
// h^2 = (9 - 4 ipd sec^2 dy^2) / (2 ipz); one extra column on each side absorbs
// rounding, and the reference's own test (in_ellipse, evaluated exactly as the
// reference rounds it) decides every visited pixel.  `group` lanes cover one
// row, so 32/group rows are processed per step.  Forward pass: den = sum K rho
// (times the pixel sensitivity in the reference-GPU semantics); backward pass
// recomputes K and adds K rho / den (reconstruction.h:290-297).

template <int SEM, class Access>
__device__ __forceinline__ void process_event(const DevGeom& g, int group, float4 ev, short4 box,
                                              const Access& acc, const float* __restrict__ sens,
                                              unsigned long long& kernel_calls,
                                              unsigned long long& contributing) {
  const int lane = threadIdx.x & 31;
  const int rows_per_step = 32 / group;
  const int gid = lane / group;
  const int gl = lane % group;
  const float z = ev.x, y = ev.y, t = ev.z, sec = ev.w;
  float A, B, C;
  ellipse_abc(g, t, sec, A, B, C);
  const float sec2_ipd4 = 4.0f * sec * sec * g.ipd;
  const float inv_2ipz = 0.5f / g.ipz;
  const float inv_pw = 1.0f / g.pixel_width;
  float den = 0.0f;
  unsigned calls = 0;
#pragma unroll 1
  for (int pass = 0; pass < 2; ++pass) {
    float inv = 0.0f;
    if (pass == 1) {
      den = warp_sum(den);
      if (!(den > 0.0f)) break;  // inv_denominator = 0: nothing to add (reconstruction.h:290)
      if (lane == 0) ++contributing;
      inv = __fdiv_rn(1.0f, den);
    }
#pragma unroll 1
    for (int row0 = box.y; row0 < box.w; row0 += rows_per_step) {
      const int iy = row0 + gid;
      const bool row_ok = iy < box.w;
      const float py = pixel_center_y(g, iy);
      const float dy = __fsub_rn(py, y);
      const float h2 = (9.0f - sec2_ipd4 * dy * dy) * inv_2ipz;
      const float h = sqrtf(fmaxf(h2, 0.0f));
      const float zc = z + t * dy - g.tl_z_half_w;
      float flo = floorf((zc - h) * inv_pw) - 1.0f;
      float fhi = ceilf((zc + h) * inv_pw) + 1.0f;
      flo = fmaxf(flo, static_cast<float>(box.x));
      fhi = fminf(fhi, static_cast<float>(box.z - 1));
      const int lo = static_cast<int>(flo);
      const int hi = (fhi >= flo) ? static_cast<int>(fhi) : lo - 1;
      // uniform trip count across the warp: the widest row of this step
      int span = row_ok ? (hi - lo + 1) : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) span = max(span, __shfl_xor_sync(kFull, span, o));
#pragma unroll 1
      for (int c0 = 0; c0 < span; c0 += group) {
        const int iz = lo + c0 + gl;
        bool take = row_ok && iz <= hi;
        float dz = 0.0f;
        if (take) {
          dz = __fsub_rn(pixel_center_z(g, iz), z);
          take = in_ellipse(A, B, C, dy, dz);
        }
        if (take) {
          float k = (SEM == kCpuReference) ? gauss_exact(g, y, t, sec, dz, dy)
                                           : analytic_exact(g, y, t, sec, dz, dy);
          float kr = __fmul_rn(k, acc.rho_at(iy, iz));
          if (pass == 0) {
            ++calls;
            den += (SEM == kCpuReference) ? kr : __fmul_rn(kr, __ldg(&sens[iy * g.n_z + iz]));
          } else {
            acc.add(iy, iz, __fmul_rn(kr, inv));
          }
        }
      }
    }
  }
  kernel_calls += calls;
}

}  // namespace
}  // namespace jpet
