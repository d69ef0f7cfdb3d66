// Staging and warp-reduction helpers shared by the tile iteration kernels
// (strip_rows.cu, strip_union.cu): cp.async copies into shared memory and a
// transposed warp sum of several per-lane values.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "strip_raster.cuh"

namespace jpet {
namespace {

// 16-, 8- and 4-byte asynchronous global -> shared copies; an invalid copy
// zero-fills its destination (src-size 0) and reads nothing.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src, bool valid) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  const int n = valid ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, bool valid) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  const int n = valid ? 4 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Sum over the 32 lanes of E per-lane values, transposed: afterwards lane l
// holds the warp total of value rows_lane_event<E>(l) (lanes that differ only
// in the low bits hold the same total).
template <int E, typename T>
__device__ __forceinline__ T rows_transpose_sum(T (&v)[E]) {
  const int lane = threadIdx.x & 31;
  int n = E;
  int off = 16;
#pragma unroll
  for (int step = 0; step < 5; ++step) {
    if (n > 1) {
      const bool hi = (lane & off) != 0;
#pragma unroll
      for (int k = 0; k < E / 2; ++k) {
        if (k < n / 2) {
          const T send = hi ? v[k] : v[k + n / 2];
          const T keep = hi ? v[k + n / 2] : v[k];
          v[k] = keep + __shfl_xor_sync(kFull, send, off);
        }
      }
      n /= 2;
    } else {
      v[0] += __shfl_xor_sync(kFull, v[0], off);
    }
    off >>= 1;
  }
  return v[0];
}
// the value index lane l holds after rows_transpose_sum: its bits 4, 3, ... in turn
template <int E>
__device__ __forceinline__ int rows_lane_event(int lane) {
  return E == 8 ? ((lane >> 2) & 7) : (E == 4 ? ((lane >> 3) & 3) : ((lane >> 4) & 1));
}
template <int E>
__device__ __forceinline__ bool rows_lane_writes(int lane) {
  return (lane & (32 / E - 1)) == 0;
}

}  // namespace
}  // namespace jpet
