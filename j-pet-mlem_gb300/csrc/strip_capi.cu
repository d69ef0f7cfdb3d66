// C ABI of the GB300 strip-PET MLEM (include/jpet_strip.h): handle management,
// device memory, event preparation and binning, and the iteration loop.
//
// Replaces GPU::Reconstruction::run (src/2d/strip/cuda/reconstruction.cu:31-113)
// and its helpers (cuda/gpu_events_soa.h:9-51, util/cuda/memory.h:51-327): every
// CUDA failure becomes a status code plus a message instead of the reference's
// abort() (util/cuda/debug.h:17-27).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/jpet_strip.h"
#include "strip_internal.h"

using namespace jpet;

namespace {

thread_local std::string g_create_error = "no error";

}  // namespace

namespace jpet {
void set_call_error(const std::string& msg) { g_create_error = msg; }
}  // namespace jpet

namespace {

template <typename T>
struct DevBuf {
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

}  // namespace

struct jpet_strip {
  jpet_strip_geom geom_in{};
  jpet_strip_opts opts{};
  DevGeom g{};
  Tiling tiling{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  std::string last_error = "no error";

  DevBuf<float> rho, out, sens_point, sens_pixel;
  DevBuf<float> out_lo;              // compensation image of the compensated modes
  DevBuf<unsigned long long> out_q;  // 64-bit fixed-point image of the FIXED mode
  DevBuf<float> raw;                 // staging for uploaded events (kept for the next upload)
  DevBuf<float4> ev_geom, sorted_geom, over_geom;
  DevBuf<short4> ev_box, sorted_box, over_box;
  DevBuf<int32_t> ev_key, tile_count, tile_offset, tile_cursor, hist, small;
  DevBuf<Chunk> chunks;
  DevBuf<uint16_t> row_table;
  DevBuf<float2> row_pq;     // per-row exponent coefficients of the row-owned kernel
  DevBuf<uint32_t> row_pk;   // per-row packed window offset / parity / width
  DevBuf<uint32_t> ev_pk;    // per-event packed window row / box rows / fits
  DevBuf<uint64_t> sort_keys;     // set-up sort: keys (input, output)
  DevBuf<int32_t> sort_idx;       // set-up sort: event indices (input, output)
  DevBuf<unsigned char> sort_tmp; // set-up sort: radix-sort scratch
  DevBuf<uint32_t> batches;       // batch-union kernel: batch words per chunk
  DevBuf<unsigned char> ev_const; // batch-union kernel: per-event constants
  DevBuf<uint16_t> union_rows;    // batch-union kernel: union row words per batch
  DevBuf<uint16_t> event_rows;    // batch-union kernel: event row words per event
  FastConst fc{};
  bool use_fast = false;
  bool use_union = false;
  bool counters_valid = false;
  unsigned long long table_kernel_calls = 0;
  DevBuf<unsigned long long> box_pixels;
  DevBuf<double> nll_acc;            // loss, d/dsigma_z, d/dsigma_dl
  DevBuf<float> nll_grad_tmp;        // gradient image when the caller passes none
  DevBuf<DevCounters> counters;

  int64_t n_events = 0;
  int32_t n_sorted = 0;
  int32_t n_oversize = 0;
  int32_t n_chunks = 0;
  int32_t n_tiles_nonempty = 0;
  unsigned long long total_box_pixels = 0;
  bool events_ready = false;
  int64_t iterations_done = 0;

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    last_error = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(JPET_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  }
};

#define JPET_CUDA(h, expr, what)                 \
  do {                                           \
    cudaError_t _e = (expr);                     \
    if (_e != cudaSuccess) return (h)->cuda_fail(_e, what); \
  } while (0)

namespace {

}  // namespace

// Scanner<float, short> constructor arithmetic (src/2d/strip/scanner.h:50-67)
// and GaussianKernel<float> constants (gaussian_kernel.h:27-33), in float.
DevGeom jpet::make_dev_geom(const jpet_strip_geom& in) {
  volatile float R = static_cast<float>(in.radius);
  volatile float L = static_cast<float>(in.scintillator_length);
  volatile float ph = static_cast<float>(in.pixel_height);
  volatile float pw = static_cast<float>(in.pixel_width);
  volatile float sz = static_cast<float>(in.sigma_z);
  volatile float sdl = static_cast<float>(in.sigma_dl);
  const int16_t n_y = static_cast<int16_t>(in.n_y_pixels);
  const int16_t n_z = static_cast<int16_t>(in.n_z_pixels);
  DevGeom g{};
  g.radius = R;
  g.half_length = L / 2;
  g.n_y = n_y;
  g.n_z = n_z;
  g.pixel_width = pw;
  g.pixel_height = ph;
  g.sigma_z = sz;
  g.sigma_dl = sdl;
  volatile float size_y = n_y * ph;
  volatile float size_z = n_z * pw;
  volatile float tl_y = 0.0f + size_y / 2;
  volatile float tl_z = 0.0f - size_z / 2;
  g.tl_y = tl_y;
  g.tl_z = tl_z;
  g.tl_y_half_h = tl_y - ph / 2;
  g.tl_z_half_w = tl_z + pw / 2;
  volatile float ipz = 1 / (sz * sz);
  volatile float ipd = 1 / (sdl * sdl);
  g.ipz = ipz;
  g.ipd = ipd;
  volatile float prod = ipz * ipz;
  prod = prod * ipd;
  g.c0 = static_cast<float>(1 / (2 * M_PI * M_PI) * std::sqrt(static_cast<float>(prod)));
  return g;
}

namespace {

int validate_geom(const jpet_strip_geom* geom, std::string& msg) {
  if (!geom) {
    msg = "geometry is NULL";
    return JPET_ERR_ARGUMENT;
  }
  if (geom->n_y_pixels <= 0 || geom->n_z_pixels <= 0 || geom->n_y_pixels > 32767 ||
      geom->n_z_pixels > 32767) {
    msg = "n_y_pixels and n_z_pixels must be in [1, 32767]";
    return JPET_ERR_ARGUMENT;
  }
  if (static_cast<int64_t>(geom->n_y_pixels) * geom->n_z_pixels > (1ll << 30)) {
    msg = "image too large";
    return JPET_ERR_ARGUMENT;
  }
  if (!(geom->pixel_height > 0) || !(geom->pixel_width > 0) || !(geom->sigma_z > 0) ||
      !(geom->sigma_dl > 0) || !(geom->radius > 0) || !(geom->scintillator_length > 0)) {
    msg = "radius, length, pixel sizes and sigmas must be positive";
    return JPET_ERR_ARGUMENT;
  }
  return JPET_OK;
}

// Window sizing: the largest box dimension that covers all but a tiny tail of
// the events (the tail takes the global-memory path), then the largest square
// tile whose window (tile + box) fits the shared-memory budget.
void choose_tiling(const jpet_strip_opts& o, const std::vector<int32_t>& hw,
                   const std::vector<int32_t>& hh, int64_t n_nonempty, int n_sms, int n_y,
                   int n_z, Tiling& t) {
  // window pixels per array (rho, out): 12288 (~100 KiB per CTA, 2 CTAs per SM)
  // for 256-thread CTAs; 6144 (~55 KiB, 4 CTAs per SM) for the row-owned
  // kernel's 128-thread CTAs and for the batch-union kernel (~76 KiB with its
  // batch records, ~100 KiB with the compensation window, 2 CTAs of 256
  // threads per SM)
  const bool fast = o.mode == JPET_MODE_CPU_REFERENCE &&
                    (o.variant == JPET_VARIANT_FAST || o.variant == JPET_VARIANT_ROWS);
  const bool union_k = fast && o.variant == JPET_VARIANT_FAST;
  const bool rows4 = fast && o.block_threads != 256;
  const int budget_px = (rows4 || union_k) ? 6144 : 12288;
  auto pct = [&](const std::vector<int32_t>& h, double keep) {
    int64_t tail = static_cast<int64_t>(std::floor((1.0 - keep) * n_nonempty));
    int64_t acc = 0;
    for (int b = kHistBins - 1; b > 0; --b) {
      acc += h[b];
      if (acc > tail) return b;
    }
    return 1;
  };
  int mw = std::min(255, std::max(1, pct(hw, 0.99999)));
  int mh = std::min(1024, std::max(1, pct(hh, 0.99999)));
  // shrink the box limits until at least an 8x8 tile fits
  while ((mw + 8) * (mh + 8) > budget_px) {
    if (mw >= mh) mw = mw * 7 / 8; else mh = mh * 7 / 8;
  }
  int tw = o.tile_w > 0 ? o.tile_w : 0, th = o.tile_h > 0 ? o.tile_h : 0;
  if (tw == 0 || th == 0) {
    int side = 8;
    while ((mw + 2 * side) * (mh + 2 * side) <= budget_px && side < 64) side *= 2;
    if (tw == 0) tw = side;
    if (th == 0) th = side;
  }
  tw = std::min(tw, n_z);
  th = std::min(th, n_y);
  while ((mw + tw) * (mh + th) > budget_px && (tw > 1 || th > 1)) {
    if (tw >= th && tw > 1) tw = std::max(1, tw / 2); else th = std::max(1, th / 2);
  }
  t.tile_w = tw;
  t.tile_h = th;
  t.max_box_w = mw;
  t.max_box_h = mh;
  t.win_w = tw + mw;
  t.win_h = th + mh;
  t.n_tiles_x = (n_z + tw - 1) / tw;
  t.n_tiles_y = (n_y + th - 1) / th;
  // events per chunk of the batch-union kernel: the largest of 2048, 1024 and
  // 512 that still leaves at least 16 chunks per resident CTA (2 per SM).
  // Larger chunks mean fewer chunk prologues and window flushes (2e7 events at
  // 2 mm: 13.50, 13.06, 12.88 ms per iteration with 512, 1024, 2048), but
  // fewer chunks leave SMs idle at the end of the launch (event sets of ~8e5:
  // 4.2e8, 4.0e8, 3.6e8 event-iterations/s).  The other kernels and the
  // fixed-point mode (whose integer window sums must stay below 2^31) use 512.
  t.chunk_events = 512;
  if (union_k && o.precision != JPET_PRECISION_FIXED) {
    const int64_t min_chunks = 16LL * 2 * std::max(n_sms, 1);
    t.chunk_events = 2048;
    while (t.chunk_events > 512 && n_nonempty / t.chunk_events < min_chunks)
      t.chunk_events /= 2;
  }
  // the FP32 batch-union kernel (FAST variant) defaults to 256-thread CTAs
  // (8 events per batch); the row-owned kernel to 128
  t.threads = o.block_threads > 0 ? o.block_threads : (union_k ? 256 : (rows4 ? 128 : 256));
  t.group = 32;
  // one spare entry per event for its widest row; a multiple of 8 entries so
  // that every event's table starts on a 16-byte boundary
  t.row_stride = (mh + 1 + 7) & ~7;
  // register-cache shape of the fast kernel from the rows of 99.9% of the boxes
  // (fast_width_shape adds the widest in-ellipse row)
  const int rows999 = pct(hh, 0.999);
  t.fast_shape = rows999 <= 32 ? kShapeS : (rows999 <= 64 ? kShapeM : kShapeL);
  t.rows_shape = kRowsShape4x1x3;
}

// The widest in-ellipse row is 2 * 3 sigma_z / sqrt(2) / pixel (+ rounding).
int widest_row(const DevGeom& g) {
  const double half = 3.0 * g.sigma_z / std::sqrt(2.0) / g.pixel_width;
  return 2 * static_cast<int>(half) + 3;
}
int fast_width_shape(const DevGeom& g) {
  const int w = widest_row(g);
  return w <= 16 ? kShapeS : (w <= 24 ? kShapeM : kShapeL);
}

// JPET_PRECISION_* -> the fast kernels' accumulation mode
int precision_code(int precision) {
  return precision == JPET_PRECISION_COMPENSATED ? kPrecisionCompensated
         : precision == JPET_PRECISION_FP64_DEN  ? kPrecisionCompensatedDen64
         : precision == JPET_PRECISION_FIXED     ? kPrecisionFixed
                                                 : kPrecisionFloat;
}

int prepare_events(jpet_strip* h, const float* d_zu, const float* d_zd, const float* d_dl,
                   int64_t n, int32_t stride = 1) {
  cudaStream_t s = h->stream;
  h->events_ready = false;
  h->n_events = n;
  h->n_sorted = h->n_oversize = h->n_chunks = h->n_tiles_nonempty = 0;
  h->total_box_pixels = 0;
  if (n > (int64_t)INT32_MAX - 1)
    return h->fail(JPET_ERR_ARGUMENT, "at most %d events per handle", INT32_MAX - 1);
  JPET_CUDA(h, h->hist.alloc(2 * kHistBins), "cudaMalloc(histogram)");
  JPET_CUDA(h, h->box_pixels.alloc(1), "cudaMalloc(counter)");
  JPET_CUDA(h, h->small.alloc(4), "cudaMalloc(counter)");
  if (n > 0) {
    JPET_CUDA(h, h->ev_geom.alloc(n), "cudaMalloc(events)");
    JPET_CUDA(h, h->ev_box.alloc(n), "cudaMalloc(events)");
    JPET_CUDA(h, h->ev_key.alloc(n), "cudaMalloc(events)");
  }
  JPET_CUDA(h, cudaMemsetAsync(h->hist.p, 0, 2 * kHistBins * sizeof(int32_t), s), "memset");
  JPET_CUDA(h, cudaMemsetAsync(h->box_pixels.p, 0, sizeof(unsigned long long), s), "memset");
  JPET_CUDA(h, cudaMemsetAsync(h->small.p, 0, 4 * sizeof(int32_t), s), "memset");
  JPET_CUDA(h, launch_prep_events(h->g, d_zu, d_zd, d_dl, stride, n, h->ev_geom.p, h->ev_box.p,
                                  h->hist.p, h->hist.p + kHistBins, h->box_pixels.p, s),
            "prep_events launch");
  std::vector<int32_t> hist(2 * kHistBins);
  JPET_CUDA(h, cudaMemcpyAsync(hist.data(), h->hist.p, hist.size() * sizeof(int32_t),
                               cudaMemcpyDeviceToHost, s), "copy histogram");
  JPET_CUDA(h, cudaMemcpyAsync(&h->total_box_pixels, h->box_pixels.p,
                               sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
            "copy counter");
  JPET_CUDA(h, cudaStreamSynchronize(s), "prep_events");
  std::vector<int32_t> hw(hist.begin(), hist.begin() + kHistBins);
  std::vector<int32_t> hh(hist.begin() + kHistBins, hist.end());
  int64_t nonempty = 0;
  for (int b = 1; b < kHistBins; ++b) nonempty += hw[b];
  int n_sms = 0;
  JPET_CUDA(h, cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, h->device),
            "cudaDeviceGetAttribute");
  choose_tiling(h->opts, hw, hh, nonempty, n_sms, h->g.n_y, h->g.n_z, h->tiling);
  h->tiling.fast_shape = std::max(h->tiling.fast_shape, fast_width_shape(h->g));
  {
    int64_t tail = static_cast<int64_t>(std::floor(0.001 * nonempty)), acc_h = 0;
    int rows999 = 1;
    for (int b = kHistBins - 1; b > 0; --b) {
      acc_h += hh[b];
      if (acc_h > tail) { rows999 = b; break; }
    }
    h->tiling.rows_shape = h->opts.raster_shape > 0
                               ? h->opts.raster_shape - 1
                               : rows_shape_for(rows999, widest_row(h->g) - 1);
  }
  const Tiling& t = h->tiling;
  const int32_t n_tiles = t.n_tiles_x * t.n_tiles_y;
  JPET_CUDA(h, h->tile_count.alloc(n_tiles), "cudaMalloc(tiles)");
  JPET_CUDA(h, h->tile_offset.alloc(n_tiles), "cudaMalloc(tiles)");
  JPET_CUDA(h, h->tile_cursor.alloc(n_tiles), "cudaMalloc(tiles)");
  JPET_CUDA(h, cudaMemsetAsync(h->tile_count.p, 0, n_tiles * sizeof(int32_t), s), "memset");
  JPET_CUDA(h, cudaMemsetAsync(h->tile_cursor.p, 0, n_tiles * sizeof(int32_t), s), "memset");
  JPET_CUDA(h, launch_key_events(t, n, h->ev_box.p, h->ev_key.p, h->tile_count.p, h->small.p, s),
            "key_events launch");
  std::vector<int32_t> count(n_tiles);
  int32_t n_over = 0;
  JPET_CUDA(h, cudaMemcpyAsync(count.data(), h->tile_count.p, n_tiles * sizeof(int32_t),
                               cudaMemcpyDeviceToHost, s), "copy tile counts");
  JPET_CUDA(h, cudaMemcpyAsync(&n_over, h->small.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s),
            "copy counter");
  JPET_CUDA(h, cudaStreamSynchronize(s), "key_events");
  // exclusive scan over tiles and chunk list (full chunks first, then the
  // partial tail chunks by decreasing size, so the longest work starts first)
  std::vector<int32_t> offset(n_tiles);
  std::vector<Chunk> full, partial;
  int32_t acc = 0;
  for (int32_t k = 0; k < n_tiles; ++k) {
    offset[k] = acc;
    const int32_t c = count[k];
    if (c > 0) ++h->n_tiles_nonempty;
    const int32_t ox = (k % t.n_tiles_x) * t.tile_w, oy = (k / t.n_tiles_x) * t.tile_h;
    for (int32_t s0 = 0; s0 < c; s0 += t.chunk_events) {
      Chunk ch{acc + s0, std::min(t.chunk_events, c - s0), ox, oy};
      (ch.count == t.chunk_events ? full : partial).push_back(ch);
    }
    acc += c;
  }
  std::stable_sort(partial.begin(), partial.end(),
                   [](const Chunk& a, const Chunk& b) { return a.count > b.count; });
  full.insert(full.end(), partial.begin(), partial.end());
  h->n_sorted = acc;
  h->n_oversize = n_over;
  h->n_chunks = static_cast<int32_t>(full.size());
  JPET_CUDA(h, h->chunks.alloc(std::max<size_t>(full.size(), 1)), "cudaMalloc(chunks)");
  if (!full.empty())
    JPET_CUDA(h, cudaMemcpyAsync(h->chunks.p, full.data(), full.size() * sizeof(Chunk),
                                 cudaMemcpyHostToDevice, s), "copy chunks");
  JPET_CUDA(h, cudaMemcpyAsync(h->tile_offset.p, offset.data(), n_tiles * sizeof(int32_t),
                               cudaMemcpyHostToDevice, s), "copy tile offsets");
  JPET_CUDA(h, h->sorted_geom.alloc(std::max(acc, 1)), "cudaMalloc(sorted events)");
  JPET_CUDA(h, h->sorted_box.alloc(std::max(acc, 1)), "cudaMalloc(sorted events)");
  JPET_CUDA(h, h->over_geom.alloc(std::max(n_over, 1)), "cudaMalloc(large events)");
  JPET_CUDA(h, h->over_box.alloc(std::max(n_over, 1)), "cudaMalloc(large events)");
  if (n > 0) {
    // tile, then box corner inside the tile, then tan (strip_sort.cu)
    const size_t tmp = sort_temp_bytes(n);
    JPET_CUDA(h, h->sort_keys.alloc(2 * static_cast<size_t>(n)), "cudaMalloc(sort keys)");
    JPET_CUDA(h, h->sort_idx.alloc(2 * static_cast<size_t>(n)), "cudaMalloc(sort indices)");
    JPET_CUDA(h, h->sort_tmp.alloc(std::max<size_t>(tmp, 1)), "cudaMalloc(sort scratch)");
    JPET_CUDA(h, sort_events(t, n, h->ev_geom.p, h->ev_box.p, h->sort_keys.p, h->sort_idx.p,
                             h->sort_tmp.p, tmp, acc, n_over, h->sorted_geom.p, h->sorted_box.p,
                             h->over_geom.p, h->over_box.p, s),
              "event sort");
  }
  h->use_fast = h->opts.mode == JPET_MODE_CPU_REFERENCE && h->opts.variant != JPET_VARIANT_EXACT;
  h->use_union = h->use_fast && h->opts.variant == JPET_VARIANT_FAST;
  h->table_kernel_calls = 0;
  if (h->use_fast && acc > 0) {
    JPET_CUDA(h, h->row_table.alloc(static_cast<size_t>(acc) * t.row_stride),
              "cudaMalloc(row table)");
    JPET_CUDA(h, cudaMemsetAsync(h->box_pixels.p, 0, sizeof(unsigned long long), s), "memset");
    JPET_CUDA(h, launch_row_tables(h->g, t, acc, h->sorted_geom.p, h->sorted_box.p,
                                   h->row_table.p, h->box_pixels.p, s),
              "row_table launch");
    if (h->use_union) {
      JPET_CUDA(h, h->batches.alloc(static_cast<size_t>(acc)), "cudaMalloc(batches)");
      JPET_CUDA(h, h->ev_const.alloc(static_cast<size_t>(acc) * union_event_bytes()),
                "cudaMalloc(event constants)");
      JPET_CUDA(h, h->union_rows.alloc(static_cast<size_t>(acc) * union_row_words()),
                "cudaMalloc(union rows)");
      JPET_CUDA(h, h->event_rows.alloc(static_cast<size_t>(acc) * union_row_words()),
                "cudaMalloc(event rows)");
      JPET_CUDA(h, launch_union_setup(h->g, h->fc, t, h->chunks.p, h->n_chunks, acc,
                                      h->sorted_geom.p, h->sorted_box.p, h->row_table.p,
                                      h->ev_const.p, h->batches.p, h->union_rows.p,
                                      h->event_rows.p, s),
                "batch formation launch");
      JPET_CUDA(h, union_prepare_kernel(t, precision_code(h->opts.precision)),
                "batch-union kernel attributes");
    } else if (h->opts.variant == JPET_VARIANT_FAST || h->opts.variant == JPET_VARIANT_ROWS) {
      JPET_CUDA(h, h->row_pq.alloc(static_cast<size_t>(acc) * t.row_stride),
                "cudaMalloc(row coefficients)");
      JPET_CUDA(h, h->row_pk.alloc(static_cast<size_t>(acc) * t.row_stride),
                "cudaMalloc(row words)");
      JPET_CUDA(h, h->ev_pk.alloc(static_cast<size_t>(acc)), "cudaMalloc(event words)");
      JPET_CUDA(h, launch_row_coefficients(h->g, h->fc, t, acc, h->sorted_geom.p,
                                           h->sorted_box.p, h->row_table.p, h->row_pq.p,
                                           h->row_pk.p, h->ev_pk.p, s),
                "row coefficient launch");
      JPET_CUDA(h, rows_prepare_kernel(t, precision_code(h->opts.precision)),
                "row-owned kernel attributes");
    }
    JPET_CUDA(h, cudaMemcpyAsync(&h->table_kernel_calls, h->box_pixels.p,
                                 sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
              "copy counter");
  }
  JPET_CUDA(h, cudaStreamSynchronize(s), "prepare events");
  // unsorted copies and sort buffers are no longer needed
  h->ev_geom.release();
  h->ev_box.release();
  h->ev_key.release();
  h->sort_keys.release();
  h->sort_idx.release();
  h->sort_tmp.release();
  h->events_ready = true;
  h->counters_valid = false;
  return JPET_OK;
}

int upload_and_prepare(jpet_strip* h, const float* zu, const float* zd, const float* dl,
                       const float* aos, int64_t n) {
  if (n < 0) return h->fail(JPET_ERR_ARGUMENT, "negative event count");
  if (n > 0 && !aos && (!zu || !zd || !dl)) return h->fail(JPET_ERR_ARGUMENT, "NULL event array");
  if (n == 0) return prepare_events(h, nullptr, nullptr, nullptr, 0);
  JPET_CUDA(h, h->raw.alloc(3 * static_cast<size_t>(n)), "cudaMalloc(events)");
  float* d_zu = h->raw.p;
  float* d_zd = h->raw.p + n;
  float* d_dl = h->raw.p + 2 * n;
  cudaStream_t s = h->stream;
  if (aos) {
    // one contiguous copy of the AoS triples; the preparation kernel reads
    // them with stride 3 (the reference transposes to SoA on the host,
    // cuda/gpu_events_soa.h:15-44)
    JPET_CUDA(h, cudaMemcpyAsync(h->raw.p, aos, 3 * static_cast<size_t>(n) * sizeof(float),
                                 cudaMemcpyHostToDevice, s),
              "copy events");
    return prepare_events(h, h->raw.p, h->raw.p + 1, h->raw.p + 2, n, 3);
  } else {
    const size_t bytes = static_cast<size_t>(n) * sizeof(float);
    JPET_CUDA(h, cudaMemcpyAsync(d_zu, zu, bytes, cudaMemcpyHostToDevice, s), "copy z_u");
    JPET_CUDA(h, cudaMemcpyAsync(d_zd, zd, bytes, cudaMemcpyHostToDevice, s), "copy z_d");
    JPET_CUDA(h, cudaMemcpyAsync(d_dl, dl, bytes, cudaMemcpyHostToDevice, s), "copy dl");
  }
  return prepare_events(h, d_zu, d_zd, d_dl, n);
}

}  // namespace

// ---- access for the batch (strip_batch.cu) --------------------------------------
namespace jpet {

int handle_batch_view(jpet_strip* h, BatchInstance* v, std::string& why) {
  if (!h->events_ready) {
    why = "events not set";
    return JPET_ERR_STATE;
  }
  if (!h->use_fast || h->opts.variant != JPET_VARIANT_ROWS ||
      h->opts.precision != JPET_PRECISION_FP32) {
    why = "batched instances run the FP32 row-owned kernel (CPU-reference mode, ROWS variant)";
    return JPET_ERR_UNSUPPORTED;
  }
  v->g = h->g;
  v->fc = h->fc;
  v->t = h->tiling;
  v->chunks = h->chunks.p;
  v->ev_geom = h->sorted_geom.p;
  v->ev_box = h->sorted_box.p;
  v->ev_pk = h->ev_pk.p;
  v->rows = h->row_pk.p;
  v->pq = h->row_pq.p;
  v->img[0] = h->rho.p;
  v->img[1] = h->out.p;
  v->counters = h->counters.p;
  v->over_geom = h->over_geom.p;
  v->over_box = h->over_box.p;
  v->n_oversize = h->n_oversize;
  v->n_pix = static_cast<int32_t>(h->g.n_y) * h->g.n_z;
  return JPET_OK;
}

int32_t handle_n_chunks(const jpet_strip* h) { return h->n_chunks; }
int handle_device(const jpet_strip* h) { return h->device; }

// After n batched iterations: the latest image is in img[n & 1].
void handle_batch_done(jpet_strip* h, int n) {
  if (n & 1) std::swap(h->rho, h->out);
  h->iterations_done += n;
  h->counters_valid = true;
}

int handle_reprepare(jpet_strip* h, int raster_shape, int block_threads, int tile,
                     const float* d_zu, const float* d_zd, const float* d_dl, int64_t n) {
  h->opts.raster_shape = raster_shape;
  h->opts.block_threads = block_threads;
  h->opts.tile_w = h->opts.tile_h = tile;
  return prepare_events(h, d_zu, d_zd, d_dl, n);
}

const char* handle_error(const jpet_strip* h) { return h->last_error.c_str(); }

}  // namespace jpet

extern "C" {

int jpet_strip_abi_version(void) { return JPET_STRIP_ABI_VERSION; }

void jpet_strip_default_opts(jpet_strip_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
}

int jpet_strip_create(const jpet_strip_geom* geom, const jpet_strip_opts* opts,
                      jpet_strip_t** out) {
  if (!out) {
    g_create_error = "output handle pointer is NULL";
    return JPET_ERR_ARGUMENT;
  }
  *out = nullptr;
  std::string msg;
  int rc = validate_geom(geom, msg);
  if (rc != JPET_OK) {
    g_create_error = msg;
    return rc;
  }
  jpet_strip_opts o;
  jpet_strip_default_opts(&o);
  if (opts) o = *opts;
  if (o.mode != JPET_MODE_CPU_REFERENCE && o.mode != JPET_MODE_GPU_REFERENCE) {
    g_create_error = "unknown mode";
    return JPET_ERR_ARGUMENT;
  }
  if (o.variant != JPET_VARIANT_FAST && o.variant != JPET_VARIANT_EXACT &&
      o.variant != JPET_VARIANT_WARP && o.variant != JPET_VARIANT_ROWS) {
    g_create_error = "unknown kernel variant";
    return JPET_ERR_ARGUMENT;
  }
  if (o.mode == JPET_MODE_CPU_REFERENCE &&
      (o.variant == JPET_VARIANT_FAST || o.variant == JPET_VARIANT_ROWS) &&
      o.block_threads != 0 && o.block_threads != 128 && o.block_threads != 256) {
    g_create_error = "the row-owned kernel runs 128- or 256-thread CTAs";
    return JPET_ERR_ARGUMENT;
  }
  if (o.raster_shape < JPET_RASTER_AUTO || o.raster_shape > JPET_RASTER_2x1x6) {
    g_create_error = "unknown rasterisation shape";
    return JPET_ERR_ARGUMENT;
  }
  if (o.precision != JPET_PRECISION_FP32 && o.precision != JPET_PRECISION_COMPENSATED &&
      o.precision != JPET_PRECISION_FP64_DEN && o.precision != JPET_PRECISION_FIXED) {
    g_create_error = "unknown precision mode";
    return JPET_ERR_ARGUMENT;
  }
  if (o.precision != JPET_PRECISION_FP32 &&
      (o.mode != JPET_MODE_CPU_REFERENCE || o.variant == JPET_VARIANT_EXACT)) {
    g_create_error = "compensated precision modes need the fast kernel and the CPU-reference mode";
    return JPET_ERR_UNSUPPORTED;
  }
  int n_dev = 0;
  cudaError_t e = cudaGetDeviceCount(&n_dev);
  if (e != cudaSuccess || n_dev <= 0) {
    g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return JPET_ERR_CUDA;
  }
  if (o.device < 0 || o.device >= n_dev) {
    g_create_error = "device ordinal out of range";
    return JPET_ERR_ARGUMENT;
  }
  e = cudaSetDevice(o.device);
  if (e != cudaSuccess) {
    g_create_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return JPET_ERR_CUDA;
  }
  jpet_strip* h = new (std::nothrow) jpet_strip();
  if (!h) {
    g_create_error = "host allocation failed";
    return JPET_ERR_MEMORY;
  }
  h->geom_in = *geom;
  h->opts = o;
  h->device = o.device;
  h->g = make_dev_geom(*geom);
  h->fc.kz = -1.4426950408889634f * h->g.ipz;
  h->fc.kdl = -2.0f * 1.4426950408889634f * h->g.ipd;
  h->fc.two_r2 = 2.0f * h->g.radius * h->g.radius;
  e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    g_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    delete h;
    return JPET_ERR_CUDA;
  }
  h->stream = h->own_stream;
  const size_t n_pix = static_cast<size_t>(h->g.n_y) * h->g.n_z;
  const bool comp = o.precision == JPET_PRECISION_COMPENSATED ||
                    o.precision == JPET_PRECISION_FP64_DEN;
  if ((comp && h->out_lo.alloc(n_pix) != cudaSuccess) ||
      (o.precision == JPET_PRECISION_FIXED && h->out_q.alloc(n_pix) != cudaSuccess) ||
      h->rho.alloc(n_pix) != cudaSuccess || h->out.alloc(n_pix) != cudaSuccess ||
      h->sens_point.alloc(n_pix) != cudaSuccess || h->sens_pixel.alloc(n_pix) != cudaSuccess ||
      h->counters.alloc(1) != cudaSuccess) {
    g_create_error = "cudaMalloc(images) failed";
    jpet_strip_destroy(h);
    return JPET_ERR_MEMORY;
  }
  if (launch_fill(h->rho.p, 1.0f, n_pix, h->stream) != cudaSuccess ||
      launch_sensitivity(h->g, 0, h->sens_point.p, h->stream) != cudaSuccess ||
      launch_sensitivity(h->g, 1, h->sens_pixel.p, h->stream) != cudaSuccess ||
      cudaMemsetAsync(h->counters.p, 0, sizeof(DevCounters), h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess) {
    g_create_error = std::string("initialisation kernels failed: ") +
                     cudaGetErrorString(cudaGetLastError());
    jpet_strip_destroy(h);
    return JPET_ERR_CUDA;
  }
  *out = h;
  return JPET_OK;
}

int jpet_strip_destroy(jpet_strip_t* h) {
  if (!h) return JPET_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->rho.release();
  h->out.release();
  h->out_lo.release();
  h->out_q.release();
  h->sens_point.release();
  h->sens_pixel.release();
  h->raw.release();
  h->ev_geom.release();
  h->sorted_geom.release();
  h->over_geom.release();
  h->ev_box.release();
  h->sorted_box.release();
  h->over_box.release();
  h->ev_key.release();
  h->tile_count.release();
  h->tile_offset.release();
  h->tile_cursor.release();
  h->hist.release();
  h->small.release();
  h->chunks.release();
  h->row_table.release();
  h->row_pq.release();
  h->row_pk.release();
  h->ev_pk.release();
  h->sort_keys.release();
  h->sort_idx.release();
  h->sort_tmp.release();
  h->batches.release();
  h->ev_const.release();
  h->union_rows.release();
  h->event_rows.release();
  h->box_pixels.release();
  h->nll_acc.release();
  h->nll_grad_tmp.release();
  h->counters.release();
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return JPET_OK;
}

const char* jpet_strip_last_error(const jpet_strip_t* h) {
  return h ? h->last_error.c_str() : g_create_error.c_str();
}

int jpet_strip_set_stream(jpet_strip_t* h, void* stream) {
  if (!h) return JPET_ERR_ARGUMENT;
  h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
  return JPET_OK;
}

int jpet_strip_set_events(jpet_strip_t* h, const float* aos, int64_t n) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (n > 0 && !aos) return h->fail(JPET_ERR_ARGUMENT, "NULL event array");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  return upload_and_prepare(h, nullptr, nullptr, nullptr, aos, n);
}

int jpet_strip_set_events_soa(jpet_strip_t* h, const float* zu, const float* zd,
                              const float* dl, int64_t n) {
  if (!h) return JPET_ERR_ARGUMENT;
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  return upload_and_prepare(h, zu, zd, dl, nullptr, n);
}

int jpet_strip_set_events_device(jpet_strip_t* h, const float* zu, const float* zd,
                                 const float* dl, int64_t n) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (n < 0) return h->fail(JPET_ERR_ARGUMENT, "negative event count");
  if (n > 0 && (!zu || !zd || !dl)) return h->fail(JPET_ERR_ARGUMENT, "NULL event array");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  return prepare_events(h, zu, zd, dl, n);
}

int jpet_strip_set_image(jpet_strip_t* h, const float* rho) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (!rho) return h->fail(JPET_ERR_ARGUMENT, "NULL image");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const size_t bytes = static_cast<size_t>(h->g.n_y) * h->g.n_z * sizeof(float);
  JPET_CUDA(h, cudaMemcpyAsync(h->rho.p, rho, bytes, cudaMemcpyHostToDevice, h->stream),
            "copy image");
  JPET_CUDA(h, cudaStreamSynchronize(h->stream), "copy image");
  h->iterations_done = 0;
  return JPET_OK;
}

int jpet_strip_set_image_device(jpet_strip_t* h, const float* d_rho) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (!d_rho) return h->fail(JPET_ERR_ARGUMENT, "NULL image");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const size_t bytes = static_cast<size_t>(h->g.n_y) * h->g.n_z * sizeof(float);
  JPET_CUDA(h, cudaMemcpyAsync(h->rho.p, d_rho, bytes, cudaMemcpyDeviceToDevice, h->stream),
            "copy image");
  h->iterations_done = 0;
  return JPET_OK;
}

int jpet_strip_iterate(jpet_strip_t* h, int n) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (n < 0) return h->fail(JPET_ERR_ARGUMENT, "negative iteration count");
  if (!h->events_ready) return h->fail(JPET_ERR_STATE, "set_events has not succeeded");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t s = h->stream;
  const size_t n_pix = static_cast<size_t>(h->g.n_y) * h->g.n_z;
  const float* sens = h->sens_pixel.p;
  for (int it = 0; it < n; ++it) {
    JPET_CUDA(h, cudaMemsetAsync(h->out.p, 0, n_pix * sizeof(float), s), "clear image");
    JPET_CUDA(h, cudaMemsetAsync(h->counters.p, 0, sizeof(DevCounters), s), "clear counters");
    const bool aux_img = h->opts.precision != JPET_PRECISION_FP32;
    const AuxImage aux{h->out_lo.p, h->out_q.p};
    if (h->out_lo.p)
      JPET_CUDA(h, cudaMemsetAsync(h->out_lo.p, 0, n_pix * sizeof(float), s), "clear image");
    if (h->out_q.p)
      JPET_CUDA(h, cudaMemsetAsync(h->out_q.p, 0, n_pix * sizeof(unsigned long long), s),
                "clear image");
    if (h->use_fast) {
      const int prec = precision_code(h->opts.precision);
      const uint32_t seed = 0x9E3779B9u * static_cast<uint32_t>(h->iterations_done + 1);
      if (h->use_union) {
        JPET_CUDA(h, launch_iterate_union(h->g, h->fc, h->tiling, h->chunks.p, h->n_chunks,
                                          h->sorted_geom.p, h->sorted_box.p, h->ev_const.p,
                                          h->event_rows.p, h->union_rows.p, h->batches.p,
                                          h->rho.p, h->out.p, aux, h->counters.p, prec, seed,
                                          s),
                  "iteration kernel launch");
      } else if (h->opts.variant == JPET_VARIANT_WARP) {
        JPET_CUDA(h, launch_iterate_fast(h->g, h->fc, h->tiling, h->chunks.p, h->n_chunks,
                                         h->sorted_geom.p, h->sorted_box.p, h->row_table.p,
                                         h->rho.p, h->out.p, aux, h->counters.p, prec,
                                         seed, s),
                  "iteration kernel launch");
      } else {
        JPET_CUDA(h, launch_iterate_rows(h->g, h->fc, h->tiling, h->chunks.p, h->n_chunks,
                                         h->sorted_geom.p, h->sorted_box.p, h->ev_pk.p,
                                         h->row_pk.p, h->row_pq.p, h->rho.p, h->out.p,
                                         aux, h->counters.p, prec, seed, s),
                  "iteration kernel launch");
      }
    } else {
      JPET_CUDA(h, launch_iterate(h->g, h->tiling, h->opts.mode, h->chunks.p, h->n_chunks,
                                  h->sorted_geom.p, h->sorted_box.p, h->rho.p, sens, h->out.p,
                                  h->counters.p, s),
                "iteration kernel launch");
    }
    JPET_CUDA(h, launch_iterate_global(h->g, h->opts.mode, h->n_oversize, h->over_geom.p,
                                       h->over_box.p, h->rho.p, sens, h->out.p, h->counters.p, s),
              "large-box kernel launch");
    if (aux_img)
      JPET_CUDA(h, launch_combine_aux(precision_code(h->opts.precision), aux, h->out.p, h->out.p,
                                      n_pix, s),
                "combine kernel launch");
    std::swap(h->rho, h->out);
    ++h->iterations_done;
    h->counters_valid = true;
  }
  return JPET_OK;
}

int jpet_strip_get_image(jpet_strip_t* h, float* rho) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (!rho) return h->fail(JPET_ERR_ARGUMENT, "NULL image");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const size_t bytes = static_cast<size_t>(h->g.n_y) * h->g.n_z * sizeof(float);
  JPET_CUDA(h, cudaMemcpyAsync(rho, h->rho.p, bytes, cudaMemcpyDeviceToHost, h->stream),
            "copy image");
  JPET_CUDA(h, cudaStreamSynchronize(h->stream), "iteration");
  return JPET_OK;
}

int jpet_strip_image_device(jpet_strip_t* h, const float** d_rho) {
  if (!h || !d_rho) return JPET_ERR_ARGUMENT;
  *d_rho = h->rho.p;
  return JPET_OK;
}

int jpet_strip_get_sensitivity(jpet_strip_t* h, int kind, float* out) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (!out || (kind != 0 && kind != 1)) return h->fail(JPET_ERR_ARGUMENT, "bad sensitivity kind");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  const size_t bytes = static_cast<size_t>(h->g.n_y) * h->g.n_z * sizeof(float);
  JPET_CUDA(h, cudaMemcpyAsync(out, kind == 0 ? h->sens_point.p : h->sens_pixel.p, bytes,
                               cudaMemcpyDeviceToHost, h->stream), "copy sensitivity");
  JPET_CUDA(h, cudaStreamSynchronize(h->stream), "copy sensitivity");
  return JPET_OK;
}

int jpet_strip_get_counters(jpet_strip_t* h, jpet_strip_counters* out) {
  if (!h || !out) return JPET_ERR_ARGUMENT;
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  DevCounters c{};
  JPET_CUDA(h, cudaMemcpyAsync(&c, h->counters.p, sizeof(c), cudaMemcpyDeviceToHost, h->stream),
            "copy counters");
  JPET_CUDA(h, cudaStreamSynchronize(h->stream), "copy counters");
  std::memset(out, 0, sizeof(*out));
  out->n_events = h->n_events;
  out->n_pixels = static_cast<int64_t>(h->total_box_pixels);
  out->n_kernel_calls = static_cast<int64_t>(c.n_kernel_calls) +
                        (h->use_fast && h->counters_valid
                             ? static_cast<int64_t>(h->table_kernel_calls) : 0);
  out->n_contributing = static_cast<int64_t>(c.n_contributing);
  out->n_oversize = h->n_oversize;
  out->n_tiles = h->n_tiles_nonempty;
  out->n_chunks = h->n_chunks;
  out->iterations_done = h->iterations_done;
  out->n_exact_path = static_cast<int64_t>(c.n_exact_path);
  return JPET_OK;
}

int jpet_strip_synchronize(jpet_strip_t* h) {
  if (!h) return JPET_ERR_ARGUMENT;
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  JPET_CUDA(h, cudaStreamSynchronize(h->stream), "stream");
  return JPET_OK;
}

int jpet_strip_nll_grad(jpet_strip_t* h, double sigma_z, double sigma_dl, const float* d_rho,
                        const float* d_sens, double* loss, float* d_grad_rho,
                        double* grad_sigma, int64_t* n_skipped) {
  if (!h) return JPET_ERR_ARGUMENT;
  if (!(sigma_z > 0) || !(sigma_dl > 0))
    return h->fail(JPET_ERR_ARGUMENT, "kernel sigmas must be positive");
  if (!h->events_ready) return h->fail(JPET_ERR_STATE, "set_events has not succeeded");
  if (h->opts.mode != JPET_MODE_CPU_REFERENCE)
    return h->fail(JPET_ERR_UNSUPPORTED, "the likelihood uses the Gaussian kernel (CPU-reference mode)");
  JPET_CUDA(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t s = h->stream;
  const size_t n_pix = static_cast<size_t>(h->g.n_y) * h->g.n_z;
  JPET_CUDA(h, h->nll_acc.alloc(4), "cudaMalloc(likelihood)");
  float* grad = d_grad_rho;
  if (!grad) {
    JPET_CUDA(h, h->nll_grad_tmp.alloc(n_pix), "cudaMalloc(gradient)");
    grad = h->nll_grad_tmp.p;
  }
  const float* rho = d_rho ? d_rho : h->rho.p;
  const float* sens = d_sens ? d_sens : h->sens_point.p;
  JPET_CUDA(h, cudaMemsetAsync(h->nll_acc.p, 0, 4 * sizeof(double), s), "memset");
  JPET_CUDA(h, cudaMemsetAsync(grad, 0, n_pix * sizeof(float), s), "memset");
  const NllConst k = make_nll_const(sigma_z, sigma_dl);
  JPET_CUDA(h, launch_nll_grad(h->g, k, h->tiling, h->chunks.p, h->n_chunks, h->sorted_geom.p,
                               h->sorted_box.p, h->n_oversize, h->over_geom.p, h->over_box.p, rho,
                               grad, h->nll_acc.p,
                               reinterpret_cast<unsigned long long*>(h->nll_acc.p + 3), s),
            "likelihood kernel launch");
  JPET_CUDA(h, launch_nll_finish(sens, rho, grad, h->nll_acc.p, static_cast<int64_t>(n_pix), s),
            "likelihood finish launch");
  double host[4];
  JPET_CUDA(h, cudaMemcpyAsync(host, h->nll_acc.p, sizeof(host), cudaMemcpyDeviceToHost, s),
            "copy likelihood");
  JPET_CUDA(h, cudaStreamSynchronize(s), "likelihood");
  if (loss) *loss = host[0];
  if (grad_sigma) {
    grad_sigma[0] = host[1];
    grad_sigma[1] = host[2];
  }
  unsigned long long sk;
  std::memcpy(&sk, &host[3], sizeof(sk));
  if (n_skipped) *n_skipped = static_cast<int64_t>(sk);
  return JPET_OK;
}

int jpet_strip_run(const jpet_strip_geom* geom, const jpet_strip_opts* opts,
                   const float* responses, int64_t n, float* rho, int n_blocks,
                   int n_iterations_in_block, jpet_strip_output_fn output,
                   jpet_strip_progress_fn progress, void* user, char* device_name,
                   size_t device_name_len) {
  if (!rho || n_blocks < 0 || n_iterations_in_block < 0 || (n > 0 && !responses)) {
    g_create_error = "invalid argument to jpet_strip_run";
    return JPET_ERR_ARGUMENT;
  }
  jpet_strip_t* h = nullptr;
  int rc = jpet_strip_create(geom, opts, &h);
  if (rc != JPET_OK) return rc;
  auto done = [&](int code) {
    if (code != JPET_OK) g_create_error = h->last_error;
    jpet_strip_destroy(h);
    return code;
  };
  if (device_name && device_name_len > 0) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, h->device) == cudaSuccess) {
      std::snprintf(device_name, device_name_len, "%s", prop.name);
    } else {
      device_name[0] = 0;
    }
  }
  const int n_z = h->g.n_z, n_y = h->g.n_y;
  std::vector<float> host(static_cast<size_t>(n_z) * n_y);
  // output(-1, sensitivity) first (cuda/reconstruction.cu:63-70)
  if (output) {
    if ((rc = jpet_strip_get_sensitivity(h, 1, host.data())) != JPET_OK) return done(rc);
    output(-1, host.data(), n_z, n_y, user);
  }
  if ((rc = jpet_strip_set_image(h, rho)) != JPET_OK) return done(rc);
  if ((rc = jpet_strip_set_events(h, responses, n)) != JPET_OK) return done(rc);
  for (int block = 0; block < n_blocks; ++block) {
    for (int i = 0; i < n_iterations_in_block; ++i) {
      const int iteration = block * n_iterations_in_block + i;
      if (progress) progress(iteration, 0, user);
      if ((rc = jpet_strip_iterate(h, 1)) != JPET_OK) return done(rc);
      if (progress) {
        if ((rc = jpet_strip_synchronize(h)) != JPET_OK) return done(rc);
        progress(iteration, 1, user);
      }
      // first 5 iterations and 10, 15, 20, 30, 50, 100 (cuda/reconstruction.cu:99-104)
      if (!block && i < n_iterations_in_block - 1 &&
          (i < 5 || i == 9 || i == 14 || i == 19 || i == 29 || i == 49 || i == 99)) {
        if ((rc = jpet_strip_get_image(h, rho)) != JPET_OK) return done(rc);
        if (output) output(i + 1, rho, n_z, n_y, user);
      }
    }
    if ((rc = jpet_strip_get_image(h, rho)) != JPET_OK) return done(rc);
    if (output) output((block + 1) * n_iterations_in_block, rho, n_z, n_y, user);
  }
  if (progress) progress(n_blocks * n_iterations_in_block, 0, user);
  return done(JPET_OK);
}

}  // extern "C"
