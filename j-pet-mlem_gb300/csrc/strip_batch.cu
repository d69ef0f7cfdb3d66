// Many independent reconstructions in one graph launch (no counterpart in the
// reference, which reconstructs one event set per process).
//
// Every instance is an ordinary handle: its events are binned into tiles and
// chunks, its row tables and coefficients built, by jpet_strip_set_events*.
// The batch then lists the work of all instances as (instance, chunk) items,
// grouped by register shape and CTA size, largest chunks first, and captures
// one CUDA graph per iteration count: per iteration one kernel that clears
// every instance's output image and counters, one persistent work-queue kernel
// per group (CTAs take items from a counter until none is left), and one
// kernel for the events too large for any tile.  Images alternate between each
// handle's two buffers; after an odd number of iterations the handles swap them
// so that each handle's image is the latest, and the instance table on the
// device is rewritten to match.
//
// The autotuner times candidate (register shape, CTA size, tile) plans per instance
// on a prefix of its events with the single-handle iteration and keeps the
// fastest; plans are cached by geometry, widths and event-count octave, so
// instances of the same kind are timed once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/jpet_strip.h"
#include "strip_internal.h"

namespace jpet {
int handle_batch_view(jpet_strip* h, BatchInstance* v, std::string& why);
int32_t handle_n_chunks(const jpet_strip* h);
int handle_device(const jpet_strip* h);
void handle_batch_done(jpet_strip* h, int n);
int handle_reprepare(jpet_strip* h, int raster_shape, int block_threads, int tile,
                     const float* d_zu, const float* d_zd, const float* d_dl, int64_t n);
const char* handle_error(const jpet_strip* h);
}  // namespace jpet

using namespace jpet;

namespace {

struct Group {
  int shape, threads;
  size_t smem;
  int grid;
  int32_t first_item, n_items;
};

struct RawEvents {
  float* d = nullptr;  // SoA: z_u[n], z_d[n], dl[n]
  int64_t n = 0;
};

using TuneKey = std::tuple<int, int, int, int, int, int>;

__global__ void aos_to_soa_kernel(const float* __restrict__ aos, int64_t n, float* __restrict__ soa) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  soa[i] = aos[3 * i];
  soa[n + i] = aos[3 * i + 1];
  soa[2 * n + i] = aos[3 * i + 2];
}

}  // namespace

struct jpet_strip_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error = "no error";
  std::vector<jpet_strip_t*> h;
  std::vector<RawEvents> raw;
  std::vector<jpet_strip_batch_plan> plan;
  std::vector<BatchInstance> host_insts;
  BatchInstance* d_insts = nullptr;
  BatchItem* d_items = nullptr;
  int32_t* d_next = nullptr;
  std::vector<Group> groups;
  int32_t first_over = 0, n_over = 0;
  int32_t max_pix = 0;
  bool built = false;
  std::map<int, cudaGraphExec_t> graphs;
  std::map<TuneKey, std::tuple<int, int, int>> tune_cache;  // shape, CTA threads, tile

  int fail(int code, const std::string& m) {
    last_error = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(JPET_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }
  void drop_plan() {
    drop_graphs();
    cudaFree(d_insts);
    cudaFree(d_items);
    cudaFree(d_next);
    d_insts = nullptr;
    d_items = nullptr;
    d_next = nullptr;
    groups.clear();
    built = false;
  }
};

namespace {

#define BATCH_CUDA(b, expr, what)                       \
  do {                                                  \
    cudaError_t _e = (expr);                            \
    if (_e != cudaSuccess) return (b)->cuda_fail(_e, what); \
  } while (0)

int build(jpet_strip_batch* b) {
  b->drop_plan();
  const int n_inst = static_cast<int>(b->h.size());
  b->host_insts.assign(n_inst, BatchInstance{});
  b->max_pix = 0;
  std::string why;
  for (int i = 0; i < n_inst; ++i) {
    const int rc = handle_batch_view(b->h[i], &b->host_insts[i], why);
    if (rc != JPET_OK) return b->fail(rc, "instance " + std::to_string(i) + ": " + why);
    b->max_pix = std::max(b->max_pix, b->host_insts[i].n_pix);
  }
  // work items, grouped by (shape, CTA size); in each group the largest chunks first
  std::map<std::pair<int, int>, std::vector<std::pair<int32_t, BatchItem>>> by_group;
  std::vector<BatchItem> over;
  for (int i = 0; i < n_inst; ++i) {
    const BatchInstance& v = b->host_insts[i];
    const int32_t nc = handle_n_chunks(b->h[i]);
    std::vector<Chunk> ch(nc);
    if (nc > 0)
      BATCH_CUDA(b, cudaMemcpy(ch.data(), v.chunks, nc * sizeof(Chunk), cudaMemcpyDeviceToHost),
                 "copy chunk list");
    auto& list = by_group[{v.t.rows_shape, v.t.threads}];
    for (int32_t k = 0; k < nc; ++k) list.push_back({ch[k].count, BatchItem{i, k}});
    for (int32_t e = 0; e < v.n_oversize; e += kBatchOversizePerItem) over.push_back({i, e});
  }
  std::vector<BatchItem> items;
  int sms = 0;
  BATCH_CUDA(b, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device),
             "device attribute");
  for (auto& kv : by_group) {
    auto& list = kv.second;
    std::stable_sort(list.begin(), list.end(),
                     [](const auto& a, const auto& c) { return a.first > c.first; });
    Group g{kv.first.first, kv.first.second, 0, 0, static_cast<int32_t>(items.size()),
            static_cast<int32_t>(list.size())};
    for (const auto& it : list) {
      items.push_back(it.second);
      const BatchInstance& v = b->host_insts[it.second.inst];
      g.smem = std::max(g.smem, rows_smem_bytes(v.t, g.threads, g.shape));
    }
    int bps = 0;
    BATCH_CUDA(b, batch_rows_prepare(g.shape, g.threads, g.smem, &bps), "kernel attributes");
    if (bps <= 0) return b->fail(JPET_ERR_UNSUPPORTED, "a batch group does not fit on an SM");
    g.grid = std::max(1, std::min(sms * bps, g.n_items));
    b->groups.push_back(g);
  }
  b->first_over = static_cast<int32_t>(items.size());
  b->n_over = static_cast<int32_t>(over.size());
  items.insert(items.end(), over.begin(), over.end());
  BATCH_CUDA(b, cudaMalloc(&b->d_insts, std::max(1, n_inst) * sizeof(BatchInstance)),
             "cudaMalloc(batch)");
  BATCH_CUDA(b, cudaMalloc(&b->d_items, std::max<size_t>(1, items.size()) * sizeof(BatchItem)),
             "cudaMalloc(batch)");
  BATCH_CUDA(b, cudaMalloc(&b->d_next, std::max<size_t>(1, b->groups.size()) * sizeof(int32_t)),
             "cudaMalloc(batch)");
  BATCH_CUDA(b, cudaMemcpy(b->d_insts, b->host_insts.data(), n_inst * sizeof(BatchInstance),
                           cudaMemcpyHostToDevice), "copy instances");
  if (!items.empty())
    BATCH_CUDA(b, cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(BatchItem),
                             cudaMemcpyHostToDevice), "copy work items");
  b->built = true;
  return JPET_OK;
}

int capture(jpet_strip_batch* b, int n, cudaGraphExec_t* exec) {
  cudaGraph_t graph = nullptr;
  BATCH_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal),
             "begin capture");
  cudaError_t e = cudaSuccess;
  const int32_t n_inst = static_cast<int32_t>(b->h.size());
  for (int k = 0; k < n && e == cudaSuccess; ++k) {
    const int parity = k & 1;
    e = launch_batch_clear(b->d_insts, n_inst, b->max_pix, parity, b->stream);
    if (e == cudaSuccess && !b->groups.empty())
      e = cudaMemsetAsync(b->d_next, 0, b->groups.size() * sizeof(int32_t), b->stream);
    for (size_t gi = 0; gi < b->groups.size() && e == cudaSuccess; ++gi) {
      const Group& g = b->groups[gi];
      e = launch_batch_rows(g.shape, g.threads, g.smem, g.grid, b->d_insts,
                            b->d_items + g.first_item, g.n_items, b->d_next + gi, parity,
                            b->stream);
    }
    if (e == cudaSuccess)
      e = launch_batch_oversize(b->d_insts, b->d_items + b->first_over, b->n_over, parity,
                                b->stream);
  }
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) return b->cuda_fail(e, "graph capture");
  return JPET_OK;
}

}  // namespace

extern "C" {

int jpet_strip_batch_create(int32_t n, const jpet_strip_geom* geoms, const jpet_strip_opts* opts,
                            jpet_strip_batch_t** out) {
  if (!out || n <= 0 || !geoms) {
    set_call_error("jpet_strip_batch_create: invalid argument");
    return JPET_ERR_ARGUMENT;
  }
  *out = nullptr;
  jpet_strip_opts o;
  jpet_strip_default_opts(&o);
  if (opts) o = *opts;
  if (o.mode != JPET_MODE_CPU_REFERENCE ||
      (o.variant != JPET_VARIANT_FAST && o.variant != JPET_VARIANT_ROWS) ||
      o.precision != JPET_PRECISION_FP32) {
    set_call_error("jpet_strip_batch_create: batches run the FP32 row-owned kernel "
                   "(CPU-reference mode, FAST or ROWS variant)");
    return JPET_ERR_UNSUPPORTED;
  }
  // every instance is a handle of the row-owned kernel
  o.variant = JPET_VARIANT_ROWS;
  auto* b = new jpet_strip_batch();
  b->device = o.device;
  cudaError_t e = cudaSetDevice(o.device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    set_call_error(std::string("jpet_strip_batch_create: ") + cudaGetErrorString(e));
    delete b;
    return JPET_ERR_CUDA;
  }
  b->h.assign(n, nullptr);
  b->raw.assign(n, RawEvents{});
  b->plan.assign(n, jpet_strip_batch_plan{});
  for (int i = 0; i < n; ++i) {
    const int rc = jpet_strip_create(&geoms[i], &o, &b->h[i]);
    if (rc == JPET_OK) jpet_strip_set_stream(b->h[i], b->stream);
    if (rc != JPET_OK) {
      jpet_strip_batch_destroy(b);
      return rc;
    }
    b->plan[i].raster_shape = o.raster_shape;
    b->plan[i].block_threads = o.block_threads;
  }
  *out = b;
  return JPET_OK;
}

int jpet_strip_batch_destroy(jpet_strip_batch_t* b) {
  if (!b) return JPET_OK;
  cudaSetDevice(b->device);
  b->drop_plan();
  for (auto* x : b->h)
    if (x) jpet_strip_destroy(x);
  for (auto& r : b->raw) cudaFree(r.d);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return JPET_OK;
}

const char* jpet_strip_batch_last_error(const jpet_strip_batch_t* b) {
  return b ? b->last_error.c_str() : "NULL batch";
}

int jpet_strip_batch_size(const jpet_strip_batch_t* b) {
  return b ? static_cast<int>(b->h.size()) : 0;
}

int jpet_strip_batch_instance(jpet_strip_batch_t* b, int32_t i, jpet_strip_t** h) {
  if (!b || !h || i < 0 || i >= static_cast<int32_t>(b->h.size())) return JPET_ERR_ARGUMENT;
  *h = b->h[i];
  return JPET_OK;
}

int jpet_strip_batch_set_events(jpet_strip_batch_t* b, int32_t i, const float* aos, int64_t n,
                                int32_t on_device) {
  if (!b) return JPET_ERR_ARGUMENT;
  if (i < 0 || i >= static_cast<int32_t>(b->h.size()) || n < 0 || (n > 0 && !aos))
    return b->fail(JPET_ERR_ARGUMENT, "jpet_strip_batch_set_events: invalid argument");
  BATCH_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
  b->drop_plan();
  RawEvents& r = b->raw[i];
  cudaFree(r.d);
  r.d = nullptr;
  r.n = n;
  if (n > 0) {
    // keep a device SoA copy so that the tuner can re-bin the events
    const size_t bytes = static_cast<size_t>(n) * 3 * sizeof(float);
    BATCH_CUDA(b, cudaMalloc(&r.d, bytes), "cudaMalloc(events)");
    float* staging = nullptr;
    const float* src = aos;
    if (!on_device) {
      BATCH_CUDA(b, cudaMalloc(&staging, bytes), "cudaMalloc(events)");
      cudaError_t e = cudaMemcpyAsync(staging, aos, bytes, cudaMemcpyHostToDevice, b->stream);
      if (e != cudaSuccess) {
        cudaFree(staging);
        return b->cuda_fail(e, "copy events");
      }
      src = staging;
    }
    aos_to_soa_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, b->stream>>>(src, n, r.d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(staging);
    if (e != cudaSuccess) return b->cuda_fail(e, "events to SoA");
  }
  const int rc = jpet_strip_set_events_device(b->h[i], r.d, r.d + n, r.d + 2 * n, n);
  if (rc != JPET_OK) return b->fail(rc, handle_error(b->h[i]));
  return JPET_OK;
}

int jpet_strip_batch_tune(jpet_strip_batch_t* b, int64_t max_tune_events) {
  if (!b) return JPET_ERR_ARGUMENT;
  BATCH_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
  b->drop_plan();
  if (max_tune_events <= 0) max_tune_events = 262144;
  cudaEvent_t e0, e1;
  BATCH_CUDA(b, cudaEventCreate(&e0), "event");
  BATCH_CUDA(b, cudaEventCreate(&e1), "event");
  int rc = JPET_OK;
  for (size_t i = 0; i < b->h.size() && rc == JPET_OK; ++i) {
    jpet_strip_t* h = b->h[i];
    const RawEvents& r = b->raw[i];
    BatchInstance gv{};
    {
      std::string why;
      if (handle_batch_view(h, &gv, why) != JPET_OK) {
        rc = b->fail(JPET_ERR_STATE, "instance " + std::to_string(i) + ": " + why);
        break;
      }
    }
    const int octave = r.n > 0 ? static_cast<int>(std::log2(static_cast<double>(r.n))) : 0;
    const TuneKey key{gv.g.n_y, gv.g.n_z, static_cast<int>(std::lround(gv.g.pixel_width * 100)),
                      static_cast<int>(std::lround(gv.g.sigma_z * 2)),
                      static_cast<int>(std::lround(gv.g.sigma_dl)), octave};
    const int64_t nt = std::min<int64_t>(r.n, max_tune_events);
    auto hit = b->tune_cache.find(key);
    int best_shape = 0, best_threads = 128, best_tile = 0;
    double best_ms = 1e30;
    int n_cand = 0;
    if (hit != b->tune_cache.end()) {
      std::tie(best_shape, best_threads, best_tile) = hit->second;
    } else if (nt > 0) {
      // candidates: the automatic register shape and the next larger one, 4- and
      // 8-warp CTAs, and the automatic square tile of that CTA's window budget or
      // one of half its side
      std::vector<int> shapes;
      {
        rc = handle_reprepare(h, JPET_RASTER_AUTO, 128, 0, r.d, r.d + r.n, r.d + 2 * r.n, nt);
        if (rc != JPET_OK) break;
        BatchInstance v{};
        std::string why;
        handle_batch_view(h, &v, why);
        const int auto_shape = v.t.rows_shape + 1;  // JPET_RASTER_* numbering
        shapes.push_back(auto_shape);
        if (auto_shape < JPET_RASTER_4x2x4) shapes.push_back(auto_shape + 1);
      }
      for (int shape : shapes) {
        for (int threads : {128, 256}) {
          int auto_tile = 0;
          for (int tile_pass = 0; tile_pass < 2 && rc == JPET_OK; ++tile_pass) {
            int tile = 0;
            if (tile_pass == 1) {
              tile = auto_tile / 2;
              if (tile < 8) break;
            }
            rc = handle_reprepare(h, shape, threads, tile, r.d, r.d + r.n, r.d + 2 * r.n, nt);
            if (rc != JPET_OK) break;
            if (tile_pass == 0) {
              BatchInstance v{};
              std::string why;
              handle_batch_view(h, &v, why);
              auto_tile = std::min(v.t.tile_w, v.t.tile_h);
            }
            rc = jpet_strip_iterate(h, 1);  // warm-up
            if (rc != JPET_OK) break;
            BATCH_CUDA(b, cudaEventRecord(e0, b->stream), "event");
            rc = jpet_strip_iterate(h, 3);
            if (rc != JPET_OK) break;
            BATCH_CUDA(b, cudaEventRecord(e1, b->stream), "event");
            BATCH_CUDA(b, cudaEventSynchronize(e1), "event");
            float ms = 0;
            BATCH_CUDA(b, cudaEventElapsedTime(&ms, e0, e1), "event");
            ++n_cand;
            if (ms / 3 < best_ms) {
              best_ms = ms / 3;
              best_shape = shape;
              best_threads = threads;
              best_tile = tile;
            }
          }
          if (rc != JPET_OK) break;
        }
        if (rc != JPET_OK) break;
      }
      if (rc != JPET_OK) break;
      b->tune_cache[key] = std::make_tuple(best_shape, best_threads, best_tile);
    }
    // the chosen plan on all of the instance's events, from a uniform image
    rc = handle_reprepare(h, best_shape, best_threads, best_tile, r.d, r.d + r.n, r.d + 2 * r.n,
                          r.n);
    if (rc != JPET_OK) break;
    std::vector<float> ones(static_cast<size_t>(gv.n_pix), 1.0f);
    rc = jpet_strip_set_image(h, ones.data());
    if (rc != JPET_OK) break;
    b->plan[i].raster_shape = best_shape;
    b->plan[i].block_threads = best_threads;
    b->plan[i].tile = best_tile;
    b->plan[i].tuned_ms_per_iteration = best_ms < 1e30 ? best_ms : -1.0;
    b->plan[i].tuned_events = nt;
    b->plan[i].candidates = n_cand;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != JPET_OK && b->last_error == "no error") b->last_error = "tuning failed";
  if (rc != JPET_OK) {
    for (auto* x : b->h)
      if (std::string(handle_error(x)) != "no error") {
        b->last_error = std::string("tuning: ") + handle_error(x);
        break;
      }
  }
  return rc;
}

int jpet_strip_batch_plan_of(const jpet_strip_batch_t* b, int32_t i, jpet_strip_batch_plan* p) {
  if (!b || !p || i < 0 || i >= static_cast<int32_t>(b->h.size())) return JPET_ERR_ARGUMENT;
  *p = b->plan[i];
  return JPET_OK;
}

int jpet_strip_batch_iterate(jpet_strip_batch_t* b, int32_t n) {
  if (!b) return JPET_ERR_ARGUMENT;
  if (n < 0) return b->fail(JPET_ERR_ARGUMENT, "negative iteration count");
  if (n == 0) return JPET_OK;
  BATCH_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
  if (!b->built) {
    const int rc = build(b);
    if (rc != JPET_OK) return rc;
  }
  auto it = b->graphs.find(n);
  if (it == b->graphs.end()) {
    cudaGraphExec_t exec = nullptr;
    const int rc = capture(b, n, &exec);
    if (rc != JPET_OK) return rc;
    it = b->graphs.emplace(n, exec).first;
  }
  BATCH_CUDA(b, cudaGraphLaunch(it->second, b->stream), "graph launch");
  BATCH_CUDA(b, cudaStreamSynchronize(b->stream), "batched iterations");
  for (auto* x : b->h) handle_batch_done(x, n);
  if (n & 1) {
    for (auto& v : b->host_insts) std::swap(v.img[0], v.img[1]);
    BATCH_CUDA(b, cudaMemcpy(b->d_insts, b->host_insts.data(),
                             b->host_insts.size() * sizeof(BatchInstance), cudaMemcpyHostToDevice),
               "copy instances");
  }
  return JPET_OK;
}

int jpet_strip_batch_launches_per_iteration(const jpet_strip_batch_t* b) {
  if (!b || !b->built) return 0;
  return 1 + static_cast<int>(b->groups.size()) + (b->n_over > 0 ? 1 : 0);
}

}  // extern "C"
