// One MLEM iteration that allocates no device memory.
//
// Some callers of this library may not allocate device memory themselves or
// let a library do it: a data-acquisition process that must not allocate once
// it is running, a host application that owns every device allocation through
// its own pool and hands out only input and output buffers, or a caller whose
// process has a fixed device-memory budget that cudaMalloc would break.  For
// them jpet_strip_iterate_noalloc runs one iteration (the reference CPU float
// semantics, evaluated in the reference's operation order) over the caller's
// device buffers, keeping its per-event working data in a fixed array of this
// file instead of allocated memory.
//
// The working array holds at most kNoallocMaxEvents prepared events (24 bytes
// each, 24 MiB in total) plus the iteration counters; every GPU that loads the
// library keeps it until the process exits.  All calls share it, so calls
// whose work overlaps on the GPU (different streams, or different host threads
// without ordering) race on it; calls ordered on one stream do not.  Each call
// looks up the array's device address with the caller's device current, so a
// call after a device reset uses the array of the new context; the first call
// on a device also loads this library's device code there, so make it before
// any stream capture.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/jpet_strip.h"
#include "strip_device.cuh"
#include "strip_internal.h"

namespace jpet {
namespace {

constexpr int64_t kNoallocMaxEvents = 1 << 20;

struct NoallocScratch {
  float4 geom[kNoallocMaxEvents];
  short4 box[kNoallocMaxEvents];
  DevCounters counters;
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Per-event set-up (response -> tan, y, z, sec and the clamped box) into the
// working array; boxes of events that contribute nothing stay as computed and
// are skipped by the rasteriser (empty rows or columns).
__global__ void noalloc_prep_kernel(DevGeom g, const float* __restrict__ aos, int64_t n,
                                    NoallocScratch* __restrict__ sc) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  EventSetup e = event_setup(g, aos[3 * i], aos[3 * i + 1], aos[3 * i + 2]);
  sc->geom[i] = make_float4(e.z, e.y, e.tan, e.sec);
  sc->box[i] = make_short4(e.tl_x, e.tl_y, e.br_x, e.br_y);
}

// The device address of the working array in the current device's context
// (looked up on every call: the lookup allocates nothing, and a cached address
// would dangle after a device reset).
NoallocScratch* scratch_address() {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) {
    set_call_error(std::string("jpet_strip_iterate_noalloc: cudaGetSymbolAddress: ") +
                   cudaGetErrorString(e));
    return nullptr;
  }
  return static_cast<NoallocScratch*>(p);
}

// whether the byte ranges [a, a + na) and [b, b + nb) overlap
bool overlaps(const void* a, size_t na, const void* b, size_t nb) {
  const uintptr_t pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
  return na > 0 && nb > 0 && pa < pb + nb && pb < pa + na;
}

}  // namespace
}  // namespace jpet

using namespace jpet;

extern "C" {

int jpet_strip_iterate_noalloc(const jpet_strip_geom* geom, const float* d_responses_aos,
                               int64_t n, const float* d_rho_in, float* d_rho_out,
                               void* cuda_stream) {
  if (!geom || !d_rho_in || !d_rho_out || (n > 0 && !d_responses_aos) || n < 0) {
    set_call_error("jpet_strip_iterate_noalloc: invalid argument");
    return JPET_ERR_ARGUMENT;
  }
  if (n > kNoallocMaxEvents) {
    set_call_error("jpet_strip_iterate_noalloc: at most 1048576 events per call");
    return JPET_ERR_ARGUMENT;
  }
  if (geom->n_y_pixels <= 0 || geom->n_z_pixels <= 0 || geom->n_y_pixels > 32767 ||
      geom->n_z_pixels > 32767 || !(geom->pixel_height > 0) || !(geom->pixel_width > 0) ||
      !(geom->sigma_z > 0) || !(geom->sigma_dl > 0) || !(geom->radius > 0)) {
    set_call_error("jpet_strip_iterate_noalloc: invalid geometry");
    return JPET_ERR_ARGUMENT;
  }
  const size_t img_bytes =
      static_cast<size_t>(geom->n_y_pixels) * static_cast<size_t>(geom->n_z_pixels) * sizeof(float);
  const size_t ev_bytes = static_cast<size_t>(n) * 3 * sizeof(float);
  // the output is cleared before the inputs are read: it may overlap neither
  if (overlaps(d_rho_in, img_bytes, d_rho_out, img_bytes) ||
      overlaps(d_responses_aos, ev_bytes, d_rho_out, img_bytes)) {
    set_call_error("jpet_strip_iterate_noalloc: the output image overlaps an input buffer");
    return JPET_ERR_ARGUMENT;
  }
  NoallocScratch* sc = scratch_address();
  if (!sc) return JPET_ERR_CUDA;
  cudaError_t e;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const DevGeom g = make_dev_geom(*geom);
  const size_t n_pix = static_cast<size_t>(g.n_y) * g.n_z;
  // the output accumulates: it and the counters start at zero
  e = cudaMemsetAsync(d_rho_out, 0, n_pix * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(&sc->counters, 0, sizeof(DevCounters), s);
  if (e == cudaSuccess && n > 0) {
    noalloc_prep_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(g, d_responses_aos,
                                                                             n, sc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && n > 0)
    e = launch_iterate_global(g, kCpuReference, static_cast<int32_t>(n), sc->geom, sc->box,
                              d_rho_in, nullptr, d_rho_out, &sc->counters, s);
  if (e != cudaSuccess) {
    set_call_error(std::string("jpet_strip_iterate_noalloc: ") + cudaGetErrorString(e));
    return JPET_ERR_CUDA;
  }
  return JPET_OK;
}

}  // extern "C"
