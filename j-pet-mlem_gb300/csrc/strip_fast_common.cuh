// Helpers shared by the fast iteration kernels (strip_fast.cu, strip_rows.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "strip_internal.h"

namespace jpet {

// 2^x and log2(x) on the special-function unit, subnormal inputs and results
// flushed to zero (.ftz): the fast kernels evaluate them on normal values only
// (kernel ratios >= ~1e-2 and positive aMa terms), and without .ftz every call
// also pays for a range test and two rescaling multiplies.
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// 1/x within one ulp (subnormal inputs are not flushed to zero)
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

constexpr int kG = 4;          // lanes per image row
constexpr int kRPS = 32 / kG;  // rows per step
constexpr int kCols = 2 * kG;  // columns per sweep

// Shared-memory window of the fast kernel: origin rounded down to an even
// column and an even pitch, so that every pixel pair (2k, 2k+1) of a row is one
// 8-byte aligned ld.shared.v2; 64 floats of padding after the rho window keep
// the unconditional loads of the last row inside the allocation.  The pitch is
// 8 mod 16 words: the four rows served by one half-warp (4 lanes x 8 bytes
// each) then start in four different groups of 8 banks.
__host__ __device__ inline int fast_pitch(const Tiling& t) {
  int p = (t.win_w + 2 + 7) & ~7;
  return (p % 16 == 8) ? p : p + 8;
}
__host__ __device__ inline int fast_window_floats(const Tiling& t) {
  return t.win_h * fast_pitch(t) + 64;
}

struct FastLane {
  float2 jf[4], cj[4];  // per-lane pixel offsets j, j+1 and kz pw^2 j^2 per sweep
};

// Accumulation of the back-projection window.
//   kAccFloat: float shared-memory atomics (red.shared.add.f32)
//   kAccCompensated: float shared atomics that return the old value; the exact
//              rounding error of every addition (Knuth's TwoSum) is added to a
//              second, compensation window, so sum + compensation carries the
//              tile total to second order (the compensated-summation idea of
//              Kahan and Neumaier, made atomic); tiles go to an FP32 image and
//              an FP32 compensation image (flush_compensated).
//   kAccFixed: each contribution (a fraction of one event, in [0, 1]) rounded to
//              22 fractional bits with an unbiased per-event dither and added
//              with integer shared atomics; a window pixel of a chunk of <= 512
//              events then stays below 2^31, and its sum is independent of the
//              order of the additions; tiles go to a 64-bit integer image, so
//              the whole image is deterministic.
enum Acc : int { kAccFloat = 0, kAccCompensated = 1, kAccFixed = 2 };
constexpr float kFixedScale = 4194304.0f;     // 2^22
constexpr float kMagic = 12582912.0f;         // 1.5 * 2^23: float -> integer rounding

// Tile flush of the compensated modes: the tile sum v goes into the FP32 image
// with one float atomic; TwoSum of the value that atomic found and v recovers
// the addition's exact rounding error (the atomic rounds to nearest), which
// joins the tile's own compensation cv in the FP32 compensation image.
__device__ __forceinline__ void flush_compensated(float* out, float* lo, int i, float v,
                                                  float cv) {
  const float old = atomicAdd(out + i, v);
  const float sum = __fadd_rn(old, v);
  const float bp = __fsub_rn(sum, old);
  const float err = __fadd_rn(__fsub_rn(old, __fsub_rn(sum, bp)), __fsub_rn(v, bp));
  const float c = __fadd_rn(err, cv);
  if (c != 0.0f) atomicAdd(lo + i, c);
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  // integer finaliser of MurmurHash3 (public domain, Austin Appleby)
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return x;
}

}  // namespace jpet
