// Internal types shared by the kernels (strip_kernels.cu) and the C-ABI layer
// (strip_capi.cu).  Not part of the public interface.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace jpet {

// Scanner<float, short> and GaussianKernel<float> constants as the reference
// derives them (src/2d/strip/scanner.h:50-67, gaussian_kernel.h:27-33).
struct DevGeom {
  float radius, half_length;
  int32_t n_y, n_z;
  float pixel_width, pixel_height;
  float sigma_z, sigma_dl;
  float tl_y, tl_z, tl_y_half_h, tl_z_half_w;
  float ipz, ipd, c0;
};

// One work item of the iteration kernel: a run of events (sorted by image tile)
// whose boxes all lie inside the window [ox, ox + win_w) x [oy, oy + win_h).
struct Chunk {
  int32_t start;  // first event in the sorted event arrays
  int32_t count;  // number of events
  int32_t ox, oy; // window origin (pixel column, row)
};

// Window and tiling parameters chosen at set_events time.
struct Tiling {
  int32_t tile_w, tile_h;  // tile the events' box corner is binned by
  int32_t win_w, win_h;    // shared-memory window: tile + largest box
  int32_t max_box_w, max_box_h;  // largest box that fits the window
  int32_t n_tiles_x, n_tiles_y;
  int32_t chunk_events;    // events per chunk
  int32_t threads;         // threads per CTA
  int32_t group;           // lanes per image row in the warp rasteriser (8/16/32)
};

// Device counters, summed over one iteration.
struct DevCounters {
  unsigned long long n_pixels;
  unsigned long long n_kernel_calls;
  unsigned long long n_contributing;
};

enum Semantics : int32_t { kCpuReference = 0, kGpuReference = 1 };

constexpr int kHistBins = 4096;  // box width/height histogram bins (last bin: >= 4095)

// ---- launchers (strip_kernels.cu) -----------------------------------------------
cudaError_t launch_prep_events(const DevGeom& g, const float* z_u, const float* z_d,
                               const float* dl, int64_t n, float4* ev_geom, short4* ev_box,
                               int32_t* hist_w, int32_t* hist_h,
                               unsigned long long* box_pixels, cudaStream_t s);
cudaError_t launch_key_events(const Tiling& t, int64_t n, const short4* ev_box, int32_t* ev_key,
                              int32_t* tile_count, int32_t* n_oversize, cudaStream_t s);
cudaError_t launch_scatter_events(int64_t n, const float4* ev_geom, const short4* ev_box,
                                  const int32_t* ev_key, const int32_t* tile_offset,
                                  int32_t* tile_cursor, float4* sorted_geom, short4* sorted_box,
                                  int32_t* over_cursor, float4* over_geom, short4* over_box,
                                  cudaStream_t s);
cudaError_t launch_fill(float* p, float v, int64_t n, cudaStream_t s);
cudaError_t launch_iterate(const DevGeom& g, const Tiling& t, int32_t semantics,
                           const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                           const short4* ev_box, const float* rho, const float* sens,
                           float* out, DevCounters* counters, cudaStream_t s);
cudaError_t launch_iterate_global(const DevGeom& g, int32_t semantics, int32_t n_events,
                                  const float4* ev_geom, const short4* ev_box,
                                  const float* rho, const float* sens, float* out,
                                  DevCounters* counters, cudaStream_t s);
cudaError_t launch_sensitivity(const DevGeom& g, int kind, float* out, cudaStream_t s);

}  // namespace jpet
