// Event ordering at set-up: one stable radix sort (CUB, from the CUDA toolkit's
// headers) of a 64-bit key per event, then a gather of the event records.
//
// Key, most significant first: the image tile of the box's top-left corner
// (the tile kernels' work unit; oversize boxes and empty boxes get two keys past
// the last tile, so they end up behind the tile events, in that order); tan in
// buckets of 1/8; the corner's row and column inside the tile; tan quantised to
// 12 bits.  Within a tile, consecutive events then have nearly the same box,
// slope and in-ellipse rows, which the batch-union kernel (strip_union.cu)
// relies on: its batches of similar events share one lane-to-pixel map, and a
// batch's per-row union is widest where its events' slopes differ (at the box's
// top and bottom rows).  Bucketing tan ahead of the corner trades about one
// pixel of corner spread for a much narrower slope spread where few events share
// a corner pixel.  The order is deterministic (the sort is stable and the input
// order is the caller's).
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <cstdint>

#include "strip_internal.h"

namespace jpet {
namespace {

__global__ void sort_keys_kernel(Tiling t, int64_t n, const float4* __restrict__ ev_geom,
                                 const short4* __restrict__ ev_box, uint64_t* __restrict__ keys,
                                 int32_t* __restrict__ idx) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const short4 b = ev_box[i];
  const int bw = b.z - b.x, bh = b.w - b.y;
  const uint64_t n_tiles = static_cast<uint64_t>(t.n_tiles_x) * static_cast<uint64_t>(t.n_tiles_y);
  uint64_t tile, ry = 0, rx = 0, tq = 0, tb = 0;
  if (bw <= 0 || bh <= 0) {
    tile = n_tiles + 1;
  } else if (bw > t.max_box_w || bh > t.max_box_h) {
    tile = n_tiles;
  } else {
    tile = static_cast<uint64_t>(b.y / t.tile_h) * t.n_tiles_x + static_cast<uint64_t>(b.x / t.tile_w);
    ry = static_cast<uint64_t>(b.y % t.tile_h) & 255u;
    rx = static_cast<uint64_t>(b.x % t.tile_w) & 255u;
    // fminf/fmaxf drop a NaN operand, so every tan maps into [0, 4095]
    const float q = fminf(fmaxf((ev_geom[i].z + 4.0f) * 512.0f, 0.0f), 4095.0f);
    tq = static_cast<uint64_t>(q);
    tb = tq >> 6;
  }
  keys[i] = (tile << 34) | (tb << 28) | (ry << 20) | (rx << 12) | tq;
  idx[i] = static_cast<int32_t>(i);
}

__global__ void gather_events_kernel(int64_t n_tile_events, int64_t n_over,
                                     const int32_t* __restrict__ idx,
                                     const float4* __restrict__ ev_geom,
                                     const short4* __restrict__ ev_box,
                                     float4* __restrict__ sorted_geom,
                                     short4* __restrict__ sorted_box,
                                     float4* __restrict__ over_geom,
                                     short4* __restrict__ over_box) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n_tile_events + n_over) return;
  const int32_t k = idx[i];
  if (i < n_tile_events) {
    sorted_geom[i] = ev_geom[k];
    sorted_box[i] = ev_box[k];
  } else {
    over_geom[i - n_tile_events] = ev_geom[k];
    over_box[i - n_tile_events] = ev_box[k];
  }
}

int key_bits(const Tiling& t) {
  const uint64_t top = static_cast<uint64_t>(t.n_tiles_x) * static_cast<uint64_t>(t.n_tiles_y) + 1;
  int bits = 1;
  while (bits < 30 && (top >> bits) != 0) ++bits;
  return 34 + bits;
}

}  // namespace

size_t sort_temp_bytes(int64_t n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, static_cast<const uint64_t*>(nullptr),
                                  static_cast<uint64_t*>(nullptr),
                                  static_cast<const int32_t*>(nullptr),
                                  static_cast<int32_t*>(nullptr), static_cast<int>(n), 0, 64);
  return bytes;
}

cudaError_t sort_events(const Tiling& t, int64_t n, const float4* ev_geom, const short4* ev_box,
                        uint64_t* keys, int32_t* idx, void* temp, size_t temp_bytes,
                        int64_t n_tile_events, int64_t n_over, float4* sorted_geom,
                        short4* sorted_box, float4* over_geom, short4* over_box,
                        cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
  sort_keys_kernel<<<blocks, 256, 0, s>>>(t, n, ev_geom, ev_box, keys, idx);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // keys/idx hold the input in their first n entries and receive the sorted
  // output in the next n
  size_t bytes = temp_bytes;
  e = cub::DeviceRadixSort::SortPairs(temp, bytes, keys, keys + n, idx, idx + n,
                                      static_cast<int>(n), 0, key_bits(t), s);
  if (e != cudaSuccess) return e;
  const int64_t m = n_tile_events + n_over;
  if (m <= 0) return cudaSuccess;
  gather_events_kernel<<<static_cast<unsigned>((m + 255) / 256), 256, 0, s>>>(
      n_tile_events, n_over, idx + n, ev_geom, ev_box, sorted_geom, sorted_box, over_geom,
      over_box);
  return cudaGetLastError();
}

}  // namespace jpet
