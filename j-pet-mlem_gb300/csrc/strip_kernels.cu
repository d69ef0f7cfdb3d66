// sm_103a kernels of the 2D strip-PET list-mode TOF MLEM iteration.
//
// Data layout in HBM (all row-major, pixel index y * n_z + z as in
// src/2d/geometry/pixel.h:29):
//   rho, out          float[n_y * n_z]  current and next image
//   ev_geom           float4[n]         (z, y, tan, sec) per event, sorted by tile
//   ev_box            short4[n]         clamped box (tl_x, tl_y, br_x, br_y)
//   chunks            Chunk[n_chunks]   runs of <= chunk_events events of one tile
//
// The iteration kernel gives each CTA one chunk.  The CTA stages the chunk's
// image window of rho in shared memory, rasterises every event of the chunk
// with one warp per event, accumulates the back-projection in a shared-memory
// copy of the window (shared atomics: lanes of a warp never collide because
// they touch distinct pixels of one event), and finally adds the window to the
// global image with one global atomic per non-zero pixel.
#include <cuda_runtime.h>

#include <cstdint>

#include "strip_device.cuh"
#include "strip_internal.h"
#include "strip_raster.cuh"

namespace jpet {

namespace {

// ---------------------------------------------------------------------------------
// Event preparation (once per set of events)
// ---------------------------------------------------------------------------------

// Pass 1: per-event set-up (tan, y, z, sec and the clamped box) and histograms
// of the box width and height, from which the host sizes the image windows.
// Events as three arrays (stride 1) or as AoS triples (z_u = base, z_d = base
// + 1, dl = base + 2, stride 3).  The box-size histograms take one atomic per
// distinct value in a warp (the events of a warp mostly share their box size)
// and the box pixels one atomic per block.
__global__ void __launch_bounds__(256) prep_events_kernel(
    DevGeom g, const float* __restrict__ z_u, const float* __restrict__ z_d,
    const float* __restrict__ dl, int32_t stride, int64_t n, float4* __restrict__ ev_geom,
    short4* __restrict__ ev_box, int32_t* hist_w, int32_t* hist_h,
    unsigned long long* box_pixels) {
  __shared__ unsigned long long block_pixels[8];
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  unsigned long long pixels = 0;
  int kw = -1, kh = -1;
  if (i < n) {
    const int64_t j = i * stride;
    EventSetup e = event_setup(g, z_u[j], z_d[j], dl[j]);
    ev_geom[i] = make_float4(e.z, e.y, e.tan, e.sec);
    ev_box[i] = make_short4(e.tl_x, e.tl_y, e.br_x, e.br_y);
    int bw = e.br_x - e.tl_x, bh = e.br_y - e.tl_y;
    if (bw > 0 && bh > 0) {
      pixels = static_cast<unsigned long long>(bw) * static_cast<unsigned long long>(bh);
      kw = min(bw, kHistBins - 1);
      kh = min(bh, kHistBins - 1);
    }
  }
  const unsigned mw = __match_any_sync(0xffffffffu, kw);
  if (kw >= 0 && lane == __ffs(mw) - 1) atomicAdd(&hist_w[kw], __popc(mw));
  const unsigned mh = __match_any_sync(0xffffffffu, kh);
  if (kh >= 0 && lane == __ffs(mh) - 1) atomicAdd(&hist_h[kh], __popc(mh));
  pixels = warp_sum_u64(pixels);
  if (lane == 0) block_pixels[threadIdx.x >> 5] = pixels;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) tot += block_pixels[w];
    if (tot) atomicAdd(box_pixels, tot);
  }
}

// Pass 2: tile key per event.  -1: empty box (the event contributes nothing,
// reconstruction.h:255-290); -2: box larger than the window (large-box path).
__global__ void key_events_kernel(Tiling t, int64_t n, const short4* __restrict__ ev_box,
                                  int32_t* __restrict__ ev_key, int32_t* tile_count,
                                  int32_t* n_oversize) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  short4 b = ev_box[i];
  int bw = b.z - b.x, bh = b.w - b.y;
  int32_t key;
  if (bw <= 0 || bh <= 0) {
    key = -1;
  } else if (bw > t.max_box_w || bh > t.max_box_h) {
    key = -2;
    atomicAdd(n_oversize, 1);
  } else {
    key = (b.y / t.tile_h) * t.n_tiles_x + (b.x / t.tile_w);
    atomicAdd(&tile_count[key], 1);
  }
  ev_key[i] = key;
}

__global__ void scatter_events_kernel(int64_t n, const float4* __restrict__ ev_geom,
                                      const short4* __restrict__ ev_box,
                                      const int32_t* __restrict__ ev_key,
                                      const int32_t* __restrict__ tile_offset,
                                      int32_t* tile_cursor, float4* __restrict__ sorted_geom,
                                      short4* __restrict__ sorted_box, int32_t* over_cursor,
                                      float4* __restrict__ over_geom,
                                      short4* __restrict__ over_box) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t key = ev_key[i];
  if (key >= 0) {
    int32_t pos = tile_offset[key] + atomicAdd(&tile_cursor[key], 1);
    sorted_geom[pos] = ev_geom[i];
    sorted_box[pos] = ev_box[i];
  } else if (key == -2) {
    int32_t pos = atomicAdd(over_cursor, 1);
    over_geom[pos] = ev_geom[i];
    over_box[pos] = ev_box[i];
  }
}

template <int SEM>
__global__ void __launch_bounds__(256) iterate_tiles_kernel(
    DevGeom g, Tiling t, const Chunk* __restrict__ chunks, const float4* __restrict__ ev_geom,
    const short4* __restrict__ ev_box, const float* __restrict__ rho,
    const float* __restrict__ sens, float* __restrict__ out, DevCounters* counters) {
  extern __shared__ float smem[];
  const int win = t.win_w * t.win_h;
  float* w_rho = smem;
  float* w_out = smem + win;
  const Chunk c = chunks[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  for (int r = warp; r < t.win_h; r += n_warps) {
    const int gy = c.oy + r;
    for (int col = lane; col < t.win_w; col += 32) {
      const int gx = c.ox + col;
      w_rho[r * t.win_w + col] = (gy < g.n_y && gx < g.n_z) ? rho[gy * g.n_z + gx] : 0.0f;
      w_out[r * t.win_w + col] = 0.0f;
    }
  }
  __syncthreads();
  WindowAccess acc{w_rho, w_out, c.ox, c.oy, t.win_w};
  unsigned long long calls = 0, contrib = 0;
  for (int e = warp; e < c.count; e += n_warps) {
    process_event<SEM>(g, t.group, ev_geom[c.start + e], ev_box[c.start + e], acc, sens, calls,
                       contrib);
  }
  calls = warp_sum_u64(calls);
  if (lane == 0) {
    atomicAdd(&counters->n_kernel_calls, calls);
    if (contrib) atomicAdd(&counters->n_contributing, contrib);
  }
  __syncthreads();
  for (int r = warp; r < t.win_h; r += n_warps) {
    const int gy = c.oy + r;
    for (int col = lane; col < t.win_w; col += 32) {
      const int gx = c.ox + col;
      const float v = w_out[r * t.win_w + col];
      if (v != 0.0f && gy < g.n_y && gx < g.n_z) atomicAdd(&out[gy * g.n_z + gx], v);
    }
  }
}

template <int SEM>
__global__ void __launch_bounds__(256) iterate_global_kernel(
    DevGeom g, int32_t n_events, const float4* __restrict__ ev_geom,
    const short4* __restrict__ ev_box, const float* __restrict__ rho,
    const float* __restrict__ sens, float* __restrict__ out, DevCounters* counters) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  GlobalAccess acc{rho, out, g.n_z};
  unsigned long long calls = 0, contrib = 0;
  for (int e = warp; e < n_events; e += n_warps) {
    process_event<SEM>(g, 32, ev_geom[e], ev_box[e], acc, sens, calls, contrib);
  }
  calls = warp_sum_u64(calls);
  if (lane == 0) {
    if (calls) atomicAdd(&counters->n_kernel_calls, calls);
    if (contrib) atomicAdd(&counters->n_contributing, contrib);
  }
}

// Sensitivity images (scanner.h:147-185).
__global__ void sensitivity_kernel(DevGeom g, int kind, float* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_y * g.n_z) return;
  int x = i % g.n_z, yy = i / g.n_z;
  float cz = pixel_center_z(g, x), cy = pixel_center_y(g, yy);
  float v;
  if (kind == 0) {
    v = scanner_sensitivity(g, cz, cy);
  } else {
    float hw = __fdiv_rn(g.pixel_width, 2.0f), hh = __fdiv_rn(g.pixel_height, 2.0f);
    v = __fadd_rn(
        __fadd_rn(__fadd_rn(__fadd_rn(__fdiv_rn(scanner_sensitivity(g, cz, cy), 3.0f),
                                      __fdiv_rn(scanner_sensitivity(g, __fadd_rn(cz, hw),
                                                                    __fadd_rn(cy, hh)),
                                                6.0f)),
                            __fdiv_rn(scanner_sensitivity(g, __fsub_rn(cz, hw), __fsub_rn(cy, hh)),
                                      6.0f)),
                  __fdiv_rn(scanner_sensitivity(g, __fadd_rn(cz, -hw), __fadd_rn(cy, hh)), 6.0f)),
        __fdiv_rn(scanner_sensitivity(g, __fsub_rn(cz, -hw), __fsub_rn(cy, hh)), 6.0f));
  }
  out[i] = v;
}

}  // namespace

// ---------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------

cudaError_t launch_prep_events(const DevGeom& g, const float* z_u, const float* z_d,
                               const float* dl, int32_t stride, int64_t n, float4* ev_geom,
                               short4* ev_box, int32_t* hist_w, int32_t* hist_h,
                               unsigned long long* box_pixels, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int threads = 256;
  const unsigned blocks = static_cast<unsigned>((n + threads - 1) / threads);
  prep_events_kernel<<<blocks, threads, 0, s>>>(g, z_u, z_d, dl, stride, n, ev_geom, ev_box,
                                                hist_w, hist_h, box_pixels);
  return cudaGetLastError();
}

cudaError_t launch_key_events(const Tiling& t, int64_t n, const short4* ev_box, int32_t* ev_key,
                              int32_t* tile_count, int32_t* n_oversize, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int threads = 256;
  const unsigned blocks = static_cast<unsigned>((n + threads - 1) / threads);
  key_events_kernel<<<blocks, threads, 0, s>>>(t, n, ev_box, ev_key, tile_count, n_oversize);
  return cudaGetLastError();
}

cudaError_t launch_scatter_events(int64_t n, const float4* ev_geom,
                                  const short4* ev_box, const int32_t* ev_key,
                                  const int32_t* tile_offset, int32_t* tile_cursor,
                                  float4* sorted_geom, short4* sorted_box,
                                  int32_t* over_cursor, float4* over_geom, short4* over_box,
                                  cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int threads = 256;
  const unsigned blocks = static_cast<unsigned>((n + threads - 1) / threads);
  scatter_events_kernel<<<blocks, threads, 0, s>>>(n, ev_geom, ev_box, ev_key, tile_offset,
                                                   tile_cursor, sorted_geom, sorted_box,
                                                   over_cursor, over_geom, over_box);
  return cudaGetLastError();
}

__global__ void fill_kernel(float* p, float v, int64_t n) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

cudaError_t launch_fill(float* p, float v, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  fill_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(p, v, n);
  return cudaGetLastError();
}

cudaError_t launch_iterate(const DevGeom& g, const Tiling& t, int32_t semantics,
                           const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                           const short4* ev_box, const float* rho, const float* sens,
                           float* out, DevCounters* counters, cudaStream_t s) {
  if (n_chunks <= 0) return cudaSuccess;
  const size_t smem = 2ull * t.win_w * t.win_h * sizeof(float);
  cudaError_t err;
  if (semantics == kCpuReference) {
    err = cudaFuncSetAttribute(iterate_tiles_kernel<kCpuReference>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(smem));
    if (err != cudaSuccess) return err;
    iterate_tiles_kernel<kCpuReference><<<n_chunks, t.threads, smem, s>>>(
        g, t, chunks, ev_geom, ev_box, rho, sens, out, counters);
  } else {
    err = cudaFuncSetAttribute(iterate_tiles_kernel<kGpuReference>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(smem));
    if (err != cudaSuccess) return err;
    iterate_tiles_kernel<kGpuReference><<<n_chunks, t.threads, smem, s>>>(
        g, t, chunks, ev_geom, ev_box, rho, sens, out, counters);
  }
  return cudaGetLastError();
}

cudaError_t launch_iterate_global(const DevGeom& g, int32_t semantics, int32_t n_events,
                                  const float4* ev_geom, const short4* ev_box,
                                  const float* rho, const float* sens, float* out,
                                  DevCounters* counters, cudaStream_t s) {
  if (n_events <= 0) return cudaSuccess;
  const int threads = 256;
  int blocks = (n_events + 7) / 8;
  if (blocks > 4096) blocks = 4096;
  if (semantics == kCpuReference)
    iterate_global_kernel<kCpuReference><<<blocks, threads, 0, s>>>(g, n_events, ev_geom, ev_box,
                                                                    rho, sens, out, counters);
  else
    iterate_global_kernel<kGpuReference><<<blocks, threads, 0, s>>>(g, n_events, ev_geom, ev_box,
                                                                    rho, sens, out, counters);
  return cudaGetLastError();
}

cudaError_t launch_sensitivity(const DevGeom& g, int kind, float* out, cudaStream_t s) {
  const int n = g.n_y * g.n_z;
  sensitivity_kernel<<<(n + 255) / 256, 256, 0, s>>>(g, kind, out);
  return cudaGetLastError();
}

}  // namespace jpet
