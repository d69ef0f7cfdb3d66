// Internal types shared by the kernels (strip_kernels.cu) and the C-ABI layer
// (strip_capi.cu).  Not part of the public interface.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/jpet_strip.h"

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
  int32_t n_batches;  // batch-union kernel: batches of the chunk (set-up)
  int32_t n_exact;    // batch-union kernel: events rasterised in the reference's order
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
  int32_t row_stride;      // entries per event in the row table (>= max_box_h, even)
  int32_t fast_shape;      // register-cache shape of the warp-per-event kernel (FastShape)
  int32_t rows_shape;      // register-cache shape of the row-owned kernel (RowsShape)
};

// Register-cache shapes of the fast iteration kernel: 4 lanes per image row,
// 8 rows per step, each lane two adjacent pixels per sweep (8 columns per sweep).
enum FastShape : int32_t {
  kShapeS = 0,  // <= 32 rows, <= 16 columns per row
  kShapeM = 1,  // <= 64 rows, <= 24 columns per row
  kShapeL = 2,  // <= 96 rows, <= 32 columns per row
};

// Register-cache shapes of the row-owned iteration kernel, named G x RS x SW:
// G lanes per image row (32 / G rows per warp step, 8 warps, so 256 / G event
// rows per pass), RS passes, SW sweeps of 2 G columns.
enum RowsShape : int32_t {
  kRowsShape8x1x1 = 0,  // <= 32 rows, <= 15 columns per row
  kRowsShape8x1x2 = 1,  // <= 32 rows, <= 31 columns
  kRowsShape4x1x2 = 2,  // <= 64 rows, <= 15 columns
  kRowsShape4x1x3 = 3,  // <= 64 rows, <= 23 columns
  kRowsShape4x1x4 = 4,  // <= 64 rows, <= 31 columns
  kRowsShape4x2x4 = 5,  // <= 128 rows, <= 31 columns
  kRowsShape2x1x6 = 6,  // <= 64 rows (4-warp CTAs; 128 with 8), <= 23 columns
};

// Constants of the fast evaluation: the Gaussian kernel written as
//   K / K_ref = 2^(kz u^2 + ky(sec) dy^2 - 0.5 log2(aMa(py) / aMa(y)))
// with u = dz - dy tan, dy = py - y (gaussian_kernel.h:51-79 rewritten; the
// event constant K_ref cancels in K rho / sum K rho).
struct FastConst {
  float kz;        // -log2(e) * ipz
  float kdl;       // -2 log2(e) * ipd   (times sec^2 per event)
  float two_r2;    // 2 R^2
};

// Device counters, summed over one iteration.
struct DevCounters {
  unsigned long long n_pixels;
  unsigned long long n_kernel_calls;
  unsigned long long n_contributing;
  unsigned long long n_exact_path;
};

enum Semantics : int32_t { kCpuReference = 0, kGpuReference = 1 };

// Scanner<float, short> / GaussianKernel<float> constants from the C-ABI geometry
// (strip_capi.cu).
DevGeom make_dev_geom(const jpet_strip_geom& in);
// Message returned by jpet_strip_last_error(NULL) on this thread.
void set_call_error(const std::string& msg);

constexpr int kHistBins = 4096;  // box width/height histogram bins (last bin: >= 4095)

// ---- launchers (strip_kernels.cu) -----------------------------------------------
// z_u[i * stride], z_d[i * stride], dl[i * stride]: stride 1 for three arrays,
// 3 for AoS triples (z_d = z_u + 1, dl = z_u + 2)
cudaError_t launch_prep_events(const DevGeom& g, const float* z_u, const float* z_d,
                               const float* dl, int32_t stride, int64_t n, float4* ev_geom,
                               short4* ev_box, int32_t* hist_w, int32_t* hist_h,
                               unsigned long long* box_pixels, cudaStream_t s);
cudaError_t launch_key_events(const Tiling& t, int64_t n, const short4* ev_box, int32_t* ev_key,
                              int32_t* tile_count, int32_t* n_oversize, cudaStream_t s);
cudaError_t launch_scatter_events(int64_t n, const float4* ev_geom, const short4* ev_box,
                                  const int32_t* ev_key, const int32_t* tile_offset,
                                  int32_t* tile_cursor, float4* sorted_geom, short4* sorted_box,
                                  int32_t* over_cursor, float4* over_geom, short4* over_box,
                                  cudaStream_t s);
cudaError_t launch_fill(float* p, float v, int64_t n, cudaStream_t s);
// Exact in-ellipse column interval of every box row of every sorted event
// (GaussianKernel::in_ellipse evaluated in the reference's rounding),
// packed as (first column - box.x) | (width << 8); also sums the widths.
cudaError_t launch_row_tables(const DevGeom& g, const Tiling& t, int32_t n_events,
                              const float4* ev_geom, const short4* ev_box, uint16_t* rows,
                              unsigned long long* kernel_calls, cudaStream_t s);
// Second image of the compensated and fixed-point modes: the FP32 compensation
// image (the exact rounding errors of the main image's additions, summed) or
// the 64-bit fixed-point image (units of 2^-22 of an event; integer sums are
// exact and independent of their order).
struct AuxImage {
  float* lo;
  unsigned long long* q;
};
// Accumulation of the fast kernel: float shared atomics; compensated tile sums
// flushed into an FP32 image and its FP32 compensation image (optionally with
// FP64 denominators); or fixed-point tile sums flushed into a 64-bit integer
// image (deterministic).
enum FastPrecision : int32_t {
  kPrecisionFloat = 0,
  kPrecisionCompensated = 1,
  kPrecisionCompensatedDen64 = 2,
  kPrecisionFixed = 3,
};
// Per (event, row): exponent coefficients (p, q) and the packed row word
// (window offset of the row's even start column | interval parity | width << 24;
// the last entry of an event: its widest row); per event: the packed event word
// (window row of the box top | box rows << 12 | fits-the-shape << 31).
cudaError_t launch_row_coefficients(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                    int32_t n_events, const float4* ev_geom,
                                    const short4* ev_box, const uint16_t* rows, float2* pq,
                                    uint32_t* row_pk, uint32_t* ev_pk, cudaStream_t s);
// Sets the dynamic shared-memory limit of the row-owned kernel the tiling and
// precision select (once per event set; launch_iterate_rows only launches).
cudaError_t rows_prepare_kernel(const Tiling& t, int precision);
int rows_shape_for(int rows999, int width);
// rows and columns (2 G SW) an event may span in a register shape
int rows_shape_rows(int rows_shape);
int rows_sweep_cols(int rows_shape);
cudaError_t launch_iterate_rows(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                                const short4* ev_box, const uint32_t* ev_pk,
                                const uint32_t* rows, const float2* pq, const float* rho,
                                float* out, AuxImage aux, DevCounters* counters,
                                int precision, uint32_t seed, cudaStream_t s);
// Set-up order of the events (strip_sort.cu): radix sort by tile, box corner
// and tan, then a gather into the tile-sorted and oversize arrays.
size_t sort_temp_bytes(int64_t n);
cudaError_t sort_events(const Tiling& t, int64_t n, const float4* ev_geom, const short4* ev_box,
                        uint64_t* keys, int32_t* idx, void* temp, size_t temp_bytes,
                        int64_t n_tile_events, int64_t n_over, float4* sorted_geom,
                        short4* sorted_box, float4* over_geom, short4* over_box,
                        cudaStream_t s);
// Batch-union kernel (strip_union.cu): per-event constants and batches of up
// to 4 (128-thread CTAs) or 8 (256-thread CTAs) similar events per chunk
// (set-up), and the iteration over them in every accumulation mode (precision:
// a FastPrecision code; aux: the second image of the compensated and
// fixed-point modes; seed: the fixed-point dither's per-iteration seed).
size_t union_event_bytes();
size_t union_smem_bytes(const Tiling& t, int precision);
bool union_split_exponent(const DevGeom& g, const FastConst& fc);
cudaError_t union_prepare_kernel(const Tiling& t, int precision);
// union_row_words(): 16-bit words per event of the union-row and event-row
// arrays (urows: per batch, indexed by the batch word's position; erows: per
// event), written by launch_union_setup from the row table.
size_t union_row_words();
cudaError_t launch_union_setup(const DevGeom& g, const FastConst& fc, const Tiling& t,
                               Chunk* chunks, int32_t n_chunks, int32_t n_events,
                               const float4* ev_geom, const short4* ev_box, const uint16_t* rows,
                               void* ev_const, uint32_t* batches, uint16_t* urows,
                               uint16_t* erows, cudaStream_t s);
cudaError_t launch_iterate_union(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                 const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                                 const short4* ev_box, const void* ev_const,
                                 const uint16_t* erows, const uint16_t* urows,
                                 const uint32_t* batches, const float* rho, float* out,
                                 AuxImage aux, DevCounters* counters, int precision,
                                 uint32_t seed, cudaStream_t s);
cudaError_t launch_iterate_fast(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                                const short4* ev_box, const uint16_t* rows, const float* rho,
                                float* out, AuxImage aux, DevCounters* counters, int precision,
                                uint32_t seed, cudaStream_t s);
// Constants of the likelihood adjoint at the kernel sigmas (strip_adjoint.cu).
struct NllConst {
  float ipz, ipd, kz, kz_lo, inv_ipz, half_inv_ipd, dipz_dsz, dipd_dsdl;
  double ipz_d, ipd_d, kdl_d, log_c0;
};
NllConst make_nll_const(double sigma_z, double sigma_dl);
// acc[0] -= sum_e log den_e, acc[1..2] -= sum_e (d den_e / d sigma) / den_e,
// grad -= sum_e K_e / den_e
cudaError_t launch_nll_grad(const DevGeom& g, const NllConst& k, const Tiling& t,
                            const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                            const short4* ev_box, int32_t n_over, const float4* over_geom,
                            const short4* over_box, const float* rho, float* grad, double* acc,
                            unsigned long long* skipped, cudaStream_t s);
// acc[0] += sum s rho; grad += s (grad may be null)
cudaError_t launch_nll_finish(const float* sens, const float* rho, float* grad, double* acc,
                              int64_t n, cudaStream_t s);
// The image of an iteration in the compensated and fixed-point modes:
// rho = out + aux.lo (compensated) or rho = float(aux.q 2^-22) + out (fixed;
// out holds the contributions of events taken by the reference-order paths).
cudaError_t launch_combine_aux(int precision, AuxImage aux, const float* out, float* rho,
                               int64_t n, cudaStream_t s);
cudaError_t launch_iterate(const DevGeom& g, const Tiling& t, int32_t semantics,
                           const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                           const short4* ev_box, const float* rho, const float* sens,
                           float* out, DevCounters* counters, cudaStream_t s);
cudaError_t launch_iterate_global(const DevGeom& g, int32_t semantics, int32_t n_events,
                                  const float4* ev_geom, const short4* ev_box,
                                  const float* rho, const float* sens, float* out,
                                  DevCounters* counters, cudaStream_t s);
cudaError_t launch_sensitivity(const DevGeom& g, int kind, float* out, cudaStream_t s);

// ---------------------------------------------------------------------------
// Batched reconstructions (strip_batch.cu): what one handle contributes.
// ---------------------------------------------------------------------------
struct BatchInstance {
  DevGeom g;
  FastConst fc;
  Tiling t;
  const Chunk* chunks;
  const float4* ev_geom;
  const short4* ev_box;
  const uint32_t* ev_pk;
  const uint32_t* rows;
  const float2* pq;
  float* img[2];  // iteration k reads img[k & 1] and writes img[(k + 1) & 1]
  DevCounters* counters;
  const float4* over_geom;
  const short4* over_box;
  int32_t n_oversize;
  int32_t n_pix;
};
struct BatchItem {
  int32_t inst, index;  // chunk (tile kernel) or first large event (large-box kernel)
};
constexpr int kBatchOversizePerItem = 32;

cudaError_t batch_rows_prepare(int rows_shape, int threads, size_t smem, int* blocks_per_sm);
cudaError_t launch_batch_rows(int rows_shape, int threads, size_t smem, int grid,
                              const BatchInstance* insts, const BatchItem* items, int32_t n_items,
                              int32_t* next, int parity, cudaStream_t s);
size_t rows_smem_bytes(const Tiling& t, int threads, int rows_shape);
cudaError_t launch_batch_clear(const BatchInstance* insts, int32_t n_inst, int32_t max_pix,
                               int parity, cudaStream_t s);
cudaError_t launch_batch_oversize(const BatchInstance* insts, const BatchItem* items,
                                  int32_t n_items, int parity, cudaStream_t s);

}  // namespace jpet
