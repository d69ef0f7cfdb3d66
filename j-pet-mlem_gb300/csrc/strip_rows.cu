// Row-owned MLEM iteration kernel for the CPU-reference semantics (the ROWS
// variant; the precision modes and the batched reconstructions run it).
//
// One CTA of NW warps (4 by default, or 8) per chunk of events of one image
// tile, with the rho window and the back-projection window in shared memory, as
// the other tile kernels.  What differs is who writes a window pixel: window row
// r belongs to warp (r / R) mod NW, R = 32 / G rows per warp step (G lanes per
// row, two adjacent pixels per lane and sweep), and only that warp ever writes
// it.  All NW warps take the same batch of E events: each evaluates its own rows
// of every event (exp2-form kernel, packed f32x2 math, K rho kept in registers),
// writes its partial forward sums to shared memory, and after one barrier per
// batch adds the NW partials in a fixed order and back-projects K rho / den into its own
// rows with plain shared-memory read-modify-write.  No shared-memory atomics
// are issued (on this GPU a float atomic on shared memory is a load plus a
// compare-and-swap loop; an integer one is native but still slower than a plain
// store).  Events are consecutive in the tile-sorted order, so the event records
// and row tables of the next batch are one contiguous range each; they are
// staged into shared memory with cp.async while the current batch computes.
//
// The kernel value is the exp2 form of the fast kernel of strip_fast.cu:
//   K / K_ref = 2^(kz u^2 + ky dy^2 - log2(aMa(py)/aMa(y)) / 2),  u = dz - dy tan
// (src/2d/strip/gaussian_kernel.h:51-79), over exactly the reference's pixels:
// the per-row column intervals of row_table_kernel (gaussian_kernel.h:131-137
// evaluated in the reference's rounding).  Events whose rows or widths exceed
// the register shape are queued and rasterised after the batches with the
// reference-order warp rasteriser (shared atomics, which no warp's plain
// stores race with at that point).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "strip_device.cuh"
#include "strip_fast_common.cuh"
#include "strip_internal.h"
#include "strip_raster.cuh"
#include "strip_async.cuh"

namespace jpet {
namespace {

constexpr int kMaxChunkEvents = 512;

// a - b for packed floats (negation is exact, so this is one rounding)
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  return __fadd2_rn(a, make_float2(-b.x, -b.y));
}

// Staging buffer of one batch: E packed event words, E packed row tables and E
// rows of exponent coefficients (float2), each part 16-byte aligned.
__host__ __device__ inline int rows_stage_tab(int e) { return (e * 4 + 15) & ~15; }
__host__ __device__ inline int rows_stage_pq(int e, int stride) {
  return rows_stage_tab(e) + e * stride * 4;
}
__host__ __device__ inline int rows_stage_bytes(int e, int stride) {
  return (rows_stage_pq(e, stride) + e * stride * 8 + 15) & ~15;
}

// One chunk of events of one tile on one CTA (the whole body of the kernel;
// the persistent batched kernel calls it once per work item).
template <int NW, int G, int RS, int SW, int E, int ACC, bool DEN64>
__device__ __forceinline__ void rows_chunk(
    const DevGeom& g, const FastConst& fc, const Tiling& t, const Chunk c,
    const float4* __restrict__ ev_geom, const short4* __restrict__ ev_box,
    const uint32_t* __restrict__ ev_pk, const uint32_t* __restrict__ rows,
    const float2* __restrict__ row_pq, const float* __restrict__ rho, float* __restrict__ out,
    AuxImage aux, DevCounters* counters, uint32_t seed) {
  constexpr int kRowsPerWarp = 32 / G;       // rows of one warp step
  constexpr int kPass = NW * kRowsPerWarp;   // event rows covered by one step of all warps
  constexpr int kSweep = 2 * G;              // columns per sweep
  static_assert((kPass & (kPass - 1)) == 0, "rows per pass must be a power of two");
  using DenT = typename std::conditional<DEN64, double, float>::type;
  extern __shared__ __align__(16) float smem[];
  __shared__ DenT den_part[2][E][NW];
  __shared__ int fb_list[kMaxChunkEvents];
  __shared__ int fb_count;

  const int pitch = fast_pitch(t);
  const int wfl = fast_window_floats(t);
  constexpr int kArrays = (ACC == kAccCompensated) ? 3 : 2;
  float* w_rho = smem;
  float* w_out = smem + wfl;
  float* w_comp = (ACC == kAccCompensated) ? smem + 2 * wfl : nullptr;
  const int stride = t.row_stride;
  const int stage_bytes = rows_stage_bytes(E, stride);
  unsigned char* stage0 = reinterpret_cast<unsigned char*>(smem + kArrays * wfl);

  const int ox = c.ox & ~1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane / G, gl = lane % G;
  const int n_batches = (c.count + E - 1) / E;

  auto stage_ev = [&](int buf) {
    return reinterpret_cast<uint32_t*>(stage0 + buf * stage_bytes);
  };
  auto stage_tab = [&](int buf) {
    return reinterpret_cast<uint32_t*>(stage0 + buf * stage_bytes + rows_stage_tab(E));
  };
  auto stage_pq = [&](int buf) {
    return reinterpret_cast<float2*>(stage0 + buf * stage_bytes + rows_stage_pq(E, stride));
  };
  auto issue_stage = [&](int b, int buf) {
    const int e0 = b * E;
    const int tid = threadIdx.x;
    if (tid < E) {
      const bool v = e0 + tid < c.count;
      cp_async4(stage_ev(buf) + tid, ev_pk + c.start + min(e0 + tid, c.count - 1), v);
    }
    const int n_tab = E * stride / 4;  // 16-byte pieces of the E row tables
    const int n_pq = E * stride / 2;   // 16-byte pieces of the E coefficient rows
    uint32_t* st = stage_tab(buf);
    float2* sp = stage_pq(buf);
    for (int k = tid; k < n_tab + n_pq; k += NW * 32) {
      if (k < n_tab) {
        const int ek = (k * 4) / stride;
        const bool v = e0 + ek < c.count;
        const size_t src = static_cast<size_t>(c.start + min(e0 + ek, c.count - 1)) * stride;
        cp_async16(st + k * 4, rows + src + (k * 4 - ek * stride), v);
      } else {
        const int kk = k - n_tab;
        const int ek = (kk * 2) / stride;
        const bool v = e0 + ek < c.count;
        const size_t src = static_cast<size_t>(c.start + min(e0 + ek, c.count - 1)) * stride;
        cp_async16(sp + kk * 2, row_pq + src + (kk * 2 - ek * stride), v);
      }
    }
    cp_async_commit();
  };

  if (threadIdx.x == 0) fb_count = 0;
  issue_stage(0, 0);
  for (int r = warp; r < t.win_h; r += NW) {
    const int gy = c.oy + r;
    for (int col = lane; col < pitch; col += 32) {
      const int gx = ox + col;
      w_rho[r * pitch + col] = (gy < g.n_y && gx < g.n_z) ? rho[gy * g.n_z + gx] : 0.0f;
      w_out[r * pitch + col] = 0.0f;
      if (ACC == kAccCompensated) w_comp[r * pitch + col] = 0.0f;
    }
  }
  for (int i = threadIdx.x; i < 64; i += NW * 32) w_rho[t.win_h * pitch + i] = 0.0f;

  // per-lane pixel offsets k, k+1 within a sweep and kz pw^2 k^2
  float2 jf[SW], cj[SW];
  {
    const float kzp2 = fc.kz * g.pixel_width * g.pixel_width;
#pragma unroll
    for (int s = 0; s < SW; ++s) {
      const float j0 = static_cast<float>(2 * gl + kSweep * s);
      jf[s] = make_float2(j0, j0 + 1.0f);
      cj[s] = make_float2(kzp2 * j0 * j0, kzp2 * (j0 + 1.0f) * (j0 + 1.0f));
    }
  }
  unsigned long long contrib = 0, exact_path = 0, dummy_calls = 0;
  cp_async_wait_all();
  __syncthreads();

  for (int b = 0; b < n_batches; ++b) {
    const int buf = b & 1;
    if (b + 1 < n_batches) issue_stage(b + 1, buf ^ 1);
    const uint32_t* se = stage_ev(buf);
    const uint32_t* st = stage_tab(buf);
    const float2* sp = stage_pq(buf);
    float2 cache[E][RS][SW];
    int base[E][RS];
    // column bound of the row's pixel pairs: a pair starting at k0 holds a
    // pixel of the event iff k0 < bound (0 for rows outside the event)
    int bound[E][RS];
    unsigned fits_mask = 0;
    DenT dsum[E];
    // ---- forward: this warp's rows of every event of the batch
#pragma unroll
    for (int j = 0; j < E; ++j) {
      // packed event word (row_coeff_kernel): window row of the box top,
      // box rows, fits-the-shape flag; zero past the chunk's end
      const uint32_t epk = se[j];
      const uint32_t* tab = st + j * stride;
      const float2* pqt = sp + j * stride;
      const bool fits = (epk >> 31) != 0;
      fits_mask |= fits ? (1u << j) : 0u;
      const int r0 = static_cast<int>(epk & 0xFFFu);
      const int nrows = static_cast<int>((epk >> 12) & 0xFFFu);
      float2 den_a = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int rs = 0; rs < RS; ++rs) {
        const int ri = ((kRowsPerWarp * warp + gid - r0) & (kPass - 1)) + kPass * rs;
        const bool rv = fits && ri < nrows;
        const int ric = rv ? ri : 0;
        // packed row word: window offset of the row's even start column (with
        // the interval's parity in bit 0) and the interval width
        const uint32_t en = tab[ric];
        const float2 pqv = pqt[ric];
        const int w = rv ? static_cast<int>(en >> 24) : 0;
        const int lead = static_cast<int>(en & 1u);  // 0 or 1 pixels before the interval
        const int end = lead + w;
        const int bse = static_cast<int>(en & 0xFFFFFEu) + 2 * gl;
        base[j][rs] = bse;
        bound[j][rs] = w > 0 ? end : 0;
        const float2 p2 = make_float2(pqv.x, pqv.x), q2 = make_float2(pqv.y, pqv.y);
#pragma unroll
        for (int s = 0; s < SW; ++s) {
          const int k0 = 2 * gl + kSweep * s;
          const float2 a = __ffma2_rn(q2, jf[s], __fadd2_rn(p2, cj[s]));
          const float2 r2 = *reinterpret_cast<const float2*>(w_rho + bse + kSweep * s);
          float2 kr = __fmul2_rn(make_float2(ex2_approx(a.x), ex2_approx(a.y)), r2);
          // only the first pixel of the row can lie before the interval
          kr.x = ((s > 0 || k0 >= lead) && k0 < end) ? kr.x : 0.0f;
          kr.y = (k0 + 1 < end) ? kr.y : 0.0f;
          cache[j][rs][s] = kr;
          den_a = __fadd2_rn(den_a, kr);
        }
      }
      if (DEN64)
        dsum[j] = static_cast<double>(den_a.x) + static_cast<double>(den_a.y);
      else
        dsum[j] = den_a.x + den_a.y;
    }
    {
      const DenT tot = rows_transpose_sum<E>(dsum);
      if (rows_lane_writes<E>(lane)) den_part[buf][rows_lane_event<E>(lane)][warp] = tot;
    }
    cp_async_wait_all();
    __syncthreads();
    // ---- denominators: lane j (mod E) adds the warps' partials of event j
    float inv_l;
    unsigned ok_mask;
    {
      const int jl = lane & (E - 1);
      DenT den = den_part[buf][jl][0];
#pragma unroll
      for (int w = 1; w < NW; ++w) den += den_part[buf][jl][w];
      const bool ok = den > DenT(0);  // inv_denominator = 0 otherwise (reconstruction.h:290)
      inv_l = ok ? __frcp_rn(static_cast<float>(den)) : 0.0f;
      ok_mask = __ballot_sync(kFull, ok && lane < E) & fits_mask;
    }
    if (threadIdx.x == 0) {
      contrib += __popc(ok_mask);
      const int n_valid = min(E, c.count - b * E);
      const unsigned valid_mask = (n_valid >= 32) ? ~0u : ((1u << n_valid) - 1u);
      unsigned fb = valid_mask & ~fits_mask;
      while (fb) {
        const int j = __ffs(fb) - 1;
        fb &= fb - 1;
        fb_list[fb_count++] = b * E + j;
        ++exact_path;
      }
    }
    // ---- back-projection into this warp's rows
#pragma unroll
    for (int j = 0; j < E; ++j) {
      // events without a positive denominator (or outside the register shape,
      // or past the chunk's end) carry K rho = 0 in every slot, or inv = 0:
      // their pass below changes no pixel, so it runs without a branch
      const float inv = __shfl_sync(kFull, inv_l, j);
      // Branch-free read-modify-write of the pixel pair: the pair is always
      // loaded (inside the window) and stored when its first pixel lies inside
      // the event's row interval (a zero contribution leaves it unchanged), so
      // no lane writes outside its event's rows.
      if (ACC == kAccFixed) {
        // q = floor(v 2^22 + U), U uniform in [0, 1) per event: E[q] = v 2^22
        const uint32_t key = hash32(static_cast<uint32_t>(c.start + b * E + j) ^ seed);
        const float dither = static_cast<float>(key >> 8) * 5.9604644775390625e-08f - 0.5f;
        const float sc = inv * kFixedScale;
        const float2 sc2 = make_float2(sc, sc), d2 = make_float2(dither, dither);
        const float2 m2 = make_float2(kMagic, kMagic);
        uint32_t* oq = reinterpret_cast<uint32_t*>(w_out);
#pragma unroll
        for (int rs = 0; rs < RS; ++rs) {
#pragma unroll
          for (int s = 0; s < SW; ++s) {
            const float2 kr = cache[j][rs][s];
            const float2 x = __fadd2_rn(__ffma2_rn(kr, sc2, d2), m2);
            const uint32_t q0 = __float_as_uint(x.x) - 0x4B400000u;
            const uint32_t q1 = __float_as_uint(x.y) - 0x4B400000u;
            uint32_t* op = oq + base[j][rs] + kSweep * s;
            const uint2 o = *reinterpret_cast<const uint2*>(op);
            // a zero contribution quantises to q = 0 (|dither| <= 0.5 rounds to
            // the magic constant, ties to even), so the pair is stored whole
            if (2 * gl + kSweep * s < bound[j][rs])
              *reinterpret_cast<uint2*>(op) = make_uint2(o.x + q0, o.y + q1);
          }
        }
      } else {
        const float2 inv2 = make_float2(inv, inv);
#pragma unroll
        for (int rs = 0; rs < RS; ++rs) {
#pragma unroll
          for (int s = 0; s < SW; ++s) {
            const float2 kr = cache[j][rs][s];
            const float2 v = __fmul2_rn(kr, inv2);
            float* op = w_out + base[j][rs] + kSweep * s;
            const float2 o = *reinterpret_cast<const float2*>(op);
            const float2 n = __fadd2_rn(o, v);
            if (ACC == kAccCompensated) {
              // TwoSum: o + v = n + err exactly
              float* cp = w_comp + base[j][rs] + kSweep * s;
              const float2 bp = fsub2(n, o);
              const float2 err = __fadd2_rn(fsub2(o, fsub2(n, bp)), fsub2(v, bp));
              const float2 co = *reinterpret_cast<const float2*>(cp);
              const float2 cn = __fadd2_rn(co, err);
              // a pixel without contribution keeps n = o and err = 0, cn = co
              if (2 * gl + kSweep * s < bound[j][rs]) {
                *reinterpret_cast<float2*>(op) = n;
                *reinterpret_cast<float2*>(cp) = cn;
              }
            } else {
              // one 8-byte store when the pair's first pixel lies inside the
              // event's row interval: a pixel without contribution gets o + 0 = o
              // (the pair lies in one row, owned by this warp, inside the pitch)
              if (2 * gl + kSweep * s < bound[j][rs]) *reinterpret_cast<float2*>(op) = n;
            }
          }
        }
      }
      __syncwarp();  // the next event's loads see this event's stores
    }
  }

  // ---- events outside the register shape: reference-order warp rasteriser
  __syncthreads();
  const int n_fb = fb_count;
  for (int k = warp; k < n_fb; k += NW) {
    const int ei = c.start + fb_list[k];
    const float4 ev = ev_geom[ei];
    const short4 box = ev_box[ei];
    if (ACC == kAccFloat) {
      WindowAccess acc{w_rho, w_out, ox, c.oy, pitch};
      process_event<kCpuReference>(g, 32, ev, box, acc, nullptr, dummy_calls, contrib);
    } else {
      GlobalAccess gacc{rho, out, g.n_z};
      process_event<kCpuReference>(g, 32, ev, box, gacc, nullptr, dummy_calls, contrib);
    }
  }
  if (lane == 0 && contrib) atomicAdd(&counters->n_contributing, contrib);
  if (threadIdx.x == 0 && exact_path) atomicAdd(&counters->n_exact_path, exact_path);
  __syncthreads();
  for (int r = warp; r < t.win_h; r += NW) {
    const int gy = c.oy + r;
    for (int col = lane; col < pitch; col += 32) {
      const int gx = ox + col;
      if (ACC == kAccFloat) {
        const float v = w_out[r * pitch + col];
        if (v != 0.0f && gy < g.n_y && gx < g.n_z) atomicAdd(&out[gy * g.n_z + gx], v);
      } else if (ACC == kAccCompensated) {
        const float v = w_out[r * pitch + col], cv = w_comp[r * pitch + col];
        if ((v != 0.0f || cv != 0.0f) && gy < g.n_y && gx < g.n_z)
          flush_compensated(out, aux.lo, gy * g.n_z + gx, v, cv);
      } else {
        const uint32_t q = reinterpret_cast<const uint32_t*>(w_out)[r * pitch + col];
        if (q != 0u && gy < g.n_y && gx < g.n_z)
          atomicAdd(&aux.q[gy * g.n_z + gx], static_cast<unsigned long long>(q));
      }
    }
  }
}

template <int NW, int G, int RS, int SW, int E, int ACC, bool DEN64>
__global__ void __launch_bounds__(NW * 32, (NW == 8 ? 2 : 4)) iterate_rows_kernel(
    DevGeom g, FastConst fc, Tiling t, const Chunk* __restrict__ chunks,
    const float4* __restrict__ ev_geom, const short4* __restrict__ ev_box,
    const uint32_t* __restrict__ ev_pk, const uint32_t* __restrict__ rows,
    const float2* __restrict__ row_pq, const float* __restrict__ rho, float* __restrict__ out,
    AuxImage aux, DevCounters* counters, uint32_t seed) {
  rows_chunk<NW, G, RS, SW, E, ACC, DEN64>(g, fc, t, chunks[blockIdx.x], ev_geom, ev_box, ev_pk,
                                           rows, row_pq, rho, out, aux, counters, seed);
}

// Shapes name the rows an event may span (kPass * RS): the warps per CTA set
// how those rows split into warp steps.
template <int NW, int G, int ROWS, int SW, int ACC, bool DEN64>
cudaError_t launch_rows_kernel(const DevGeom& g, const FastConst& fc, const Tiling& t,
                               const Chunk* chunks,
                               int32_t n_chunks, const float4* ev_geom, const short4* ev_box,
                               const uint32_t* ev_pk, const uint32_t* rows, const float2* pq,
                               const float* rho,
                               float* out, AuxImage aux, DevCounters* counters, uint32_t seed,
                               cudaStream_t s, int op) {
  constexpr int kPass = NW * (32 / G);
  constexpr int RS = (ROWS + kPass - 1) / kPass;
  constexpr int E = (RS * SW <= 4) ? 8 : (RS * SW <= 8 ? 4 : 2);
  const size_t smem = (ACC == kAccCompensated ? 3ull : 2ull) * fast_window_floats(t) * 4 +
                      2ull * rows_stage_bytes(E, t.row_stride);
  auto* k = iterate_rows_kernel<NW, G, RS, SW, E, ACC, DEN64>;
  if (op == 0)  // once per event set, not per iteration
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem));
  k<<<n_chunks, NW * 32, smem, s>>>(g, fc, t, chunks, ev_geom, ev_box, ev_pk, rows, pq, rho, out,
                                    aux, counters, seed);
  return cudaGetLastError();
}

template <int NW, int G, int ROWS, int SW>
cudaError_t launch_rows_prec(const DevGeom& g, const FastConst& fc, const Tiling& t,
                             const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                             const short4* ev_box, const uint32_t* ev_pk, const uint32_t* rows,
                              const float2* pq,
                             const float* rho, float* out, AuxImage aux, DevCounters* counters,
                             int precision, uint32_t seed, cudaStream_t s, int op) {
  switch (precision) {
    case kPrecisionCompensated:
      return launch_rows_kernel<NW, G, ROWS, SW, kAccCompensated, false>(
          g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho, out, aux, counters, seed,
          s, op);
    case kPrecisionCompensatedDen64:
      return launch_rows_kernel<NW, G, ROWS, SW, kAccCompensated, true>(
          g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho, out, aux, counters, seed,
          s, op);
    case kPrecisionFixed:
      return launch_rows_kernel<NW, G, ROWS, SW, kAccFixed, false>(
          g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho, out, aux, counters, seed,
          s, op);
    default:
      return launch_rows_kernel<NW, G, ROWS, SW, kAccFloat, false>(
          g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho, out, aux, counters, seed,
          s, op);
  }
}

// CTAs of 4 warps (the default: 4 CTAs of ~55 KiB per SM) or 8 warps
// (Tiling::threads = 256, 2 CTAs of ~100 KiB per SM)
template <int G, int ROWS, int SW>
cudaError_t launch_rows_shape(const DevGeom& g, const FastConst& fc, const Tiling& t,
                              const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                              const short4* ev_box, const uint32_t* ev_pk, const uint32_t* rows,
                              const float2* pq,
                              const float* rho, float* out, AuxImage aux, DevCounters* counters,
                              int precision, uint32_t seed, cudaStream_t s, int op) {
  if (t.threads == 256)
    return launch_rows_prec<8, G, ROWS, SW>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq,
                                            rho, out, aux, counters, precision, seed, s, op);
  return launch_rows_prec<4, G, ROWS, SW>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq,
                                          rho, out, aux, counters, precision, seed, s, op);
}

// ---- batched reconstructions ------------------------------------------------------

// Persistent CTAs take (instance, chunk) work items from a shared counter,
// largest first (the host sorts the items), and run the chunk with that
// instance's geometry, tiling, events and images.
template <int NW, int G, int RS, int SW, int E>
__global__ void __launch_bounds__(NW * 32, (NW == 8 ? 2 : 4))
    batch_rows_kernel(const BatchInstance* __restrict__ insts, const BatchItem* __restrict__ items,
                      int32_t n_items, int32_t* next, int parity) {
  __shared__ int32_t s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int32_t it = s_item;
    __syncthreads();
    if (it >= n_items) break;
    const BatchItem w = items[it];
    const BatchInstance& in = insts[w.inst];
    rows_chunk<NW, G, RS, SW, E, kAccFloat, false>(
        in.g, in.fc, in.t, in.chunks[w.index], in.ev_geom, in.ev_box, in.ev_pk, in.rows, in.pq,
        in.img[parity], in.img[parity ^ 1], AuxImage{}, in.counters, 0u);
    __syncthreads();
  }
}

template <int NW, int G, int ROWS, int SW>
struct BatchRows {
  static constexpr int kPass = NW * (32 / G);
  static constexpr int RS = (ROWS + kPass - 1) / kPass;
  static constexpr int E = (RS * SW <= 4) ? 8 : (RS * SW <= 8 ? 4 : 2);
  static auto kernel() { return batch_rows_kernel<NW, G, RS, SW, E>; }
};

template <int NW, int G, int ROWS, int SW>
cudaError_t batch_rows_dispatch(int op, size_t smem, int grid, int* bps,
                                const BatchInstance* insts, const BatchItem* items,
                                int32_t n_items, int32_t* next, int parity, cudaStream_t s) {
  auto* k = BatchRows<NW, G, ROWS, SW>::kernel();
  if (op == 0) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, k, NW * 32, smem);
  }
  k<<<grid, NW * 32, smem, s>>>(insts, items, n_items, next, parity);
  return cudaGetLastError();
}

template <int NW>
cudaError_t batch_rows_shape(int shape, int op, size_t smem, int grid, int* bps,
                             const BatchInstance* insts, const BatchItem* items, int32_t n_items,
                             int32_t* next, int parity, cudaStream_t s) {
  switch (shape) {
    case kRowsShape8x1x1:
      return batch_rows_dispatch<NW, 8, 32, 1>(op, smem, grid, bps, insts, items, n_items, next,
                                               parity, s);
    case kRowsShape8x1x2:
      return batch_rows_dispatch<NW, 8, 32, 2>(op, smem, grid, bps, insts, items, n_items, next,
                                               parity, s);
    case kRowsShape4x1x2:
      return batch_rows_dispatch<NW, 4, 64, 2>(op, smem, grid, bps, insts, items, n_items, next,
                                               parity, s);
    case kRowsShape4x1x3:
      return batch_rows_dispatch<NW, 4, 64, 3>(op, smem, grid, bps, insts, items, n_items, next,
                                               parity, s);
    case kRowsShape4x1x4:
      return batch_rows_dispatch<NW, 4, 64, 4>(op, smem, grid, bps, insts, items, n_items, next,
                                               parity, s);
    case kRowsShape2x1x6:
      return batch_rows_dispatch<NW, 2, 64, 6>(op, smem, grid, bps, insts, items, n_items, next,
                                               parity, s);
    default:
      return batch_rows_dispatch<NW, 4, 128, 4>(op, smem, grid, bps, insts, items, n_items, next,
                                                parity, s);
  }
}

__global__ void batch_clear_kernel(const BatchInstance* __restrict__ insts, int parity) {
  const BatchInstance& in = insts[blockIdx.y];
  float* out = in.img[parity ^ 1];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < in.n_pix; i += gridDim.x * blockDim.x)
    out[i] = 0.0f;
  if (blockIdx.x == 0 && threadIdx.x == 0) *in.counters = DevCounters{};
}

// Large-box events of every instance: one warp per event, reference order,
// global-memory atomics (as the single-handle large-box path).
__global__ void batch_oversize_kernel(const BatchInstance* __restrict__ insts,
                                      const BatchItem* __restrict__ items, int32_t n_items,
                                      int parity) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const BatchItem w = items[it];
    const BatchInstance& in = insts[w.inst];
    const int end = min(in.n_oversize, w.index + kBatchOversizePerItem);
    unsigned long long calls = 0, contrib = 0;
    GlobalAccess acc{in.img[parity], in.img[parity ^ 1], in.g.n_z};
    for (int e = w.index + warp; e < end; e += n_warps)
      process_event<kCpuReference>(in.g, 32, in.over_geom[e], in.over_box[e], acc, nullptr, calls,
                                   contrib);
    if (lane == 0 && contrib) atomicAdd(&in.counters->n_contributing, contrib);
    if (lane == 0 && calls) atomicAdd(&in.counters->n_kernel_calls, calls);
  }
}

}  // namespace

int rows_shape_rows(int rows_shape) {
  static const int rows[] = {32, 32, 64, 64, 64, 128, 64};
  return (rows_shape >= 0 && rows_shape <= kRowsShape2x1x6) ? rows[rows_shape] : 128;
}
int rows_sweep_cols(int rows_shape) {
  static const int cols[] = {16, 32, 16, 24, 32, 32, 24};
  return (rows_shape >= 0 && rows_shape <= kRowsShape2x1x6) ? cols[rows_shape] : 32;
}

int rows_shape_for(int rows999, int width) {
  if (rows999 <= 32 && width <= 15) return kRowsShape8x1x1;
  if (rows999 <= 32 && width <= 31) return kRowsShape8x1x2;
  if (rows999 <= 64 && width <= 15) return kRowsShape4x1x2;
  if (rows999 <= 64 && width <= 23) return kRowsShape4x1x3;
  if (rows999 <= 64) return kRowsShape4x1x4;
  return kRowsShape4x2x4;
}

static cudaError_t rows_dispatch(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                                const short4* ev_box, const uint32_t* ev_pk, const uint32_t* rows,
                              const float2* pq,
                                const float* rho, float* out, AuxImage aux,
                                DevCounters* counters, int precision, uint32_t seed,
                                cudaStream_t s, int op) {
  if (op != 0 && n_chunks <= 0) return cudaSuccess;
  if (t.chunk_events > kMaxChunkEvents || (t.row_stride & 7) != 0) return cudaErrorInvalidValue;
  switch (t.rows_shape) {
    case kRowsShape8x1x1:
      return launch_rows_shape<8, 32, 1>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho,
                                         out, aux, counters, precision, seed, s, op);
    case kRowsShape8x1x2:
      return launch_rows_shape<8, 32, 2>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho,
                                         out, aux, counters, precision, seed, s, op);
    case kRowsShape4x1x2:
      return launch_rows_shape<4, 64, 2>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho,
                                         out, aux, counters, precision, seed, s, op);
    case kRowsShape4x1x3:
      return launch_rows_shape<4, 64, 3>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho,
                                         out, aux, counters, precision, seed, s, op);
    case kRowsShape4x1x4:
      return launch_rows_shape<4, 64, 4>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho,
                                         out, aux, counters, precision, seed, s, op);
    case kRowsShape2x1x6:
      return launch_rows_shape<2, 64, 6>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho,
                                         out, aux, counters, precision, seed, s, op);
    default:
      return launch_rows_shape<4, 128, 4>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho,
                                          out, aux, counters, precision, seed, s, op);
  }
}

cudaError_t launch_iterate_rows(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                                const short4* ev_box, const uint32_t* ev_pk, const uint32_t* rows,
                                const float2* pq, const float* rho, float* out, AuxImage aux,
                                DevCounters* counters, int precision, uint32_t seed,
                                cudaStream_t s) {
  return rows_dispatch(g, fc, t, chunks, n_chunks, ev_geom, ev_box, ev_pk, rows, pq, rho, out,
                       aux, counters, precision, seed, s, 1);
}

cudaError_t rows_prepare_kernel(const Tiling& t, int precision) {
  return rows_dispatch(DevGeom{}, FastConst{}, t, nullptr, 0, nullptr, nullptr, nullptr, nullptr,
                       nullptr, nullptr, nullptr, AuxImage{}, nullptr, precision, 0u, nullptr, 0);
}

size_t rows_smem_bytes(const Tiling& t, int threads, int rows_shape) {
  const int nw = threads == 256 ? 8 : 4;
  static const int rows_of[] = {32, 32, 64, 64, 64, 128, 64};
  static const int g_of[] = {8, 8, 4, 4, 4, 4, 2};
  static const int sw_of[] = {1, 2, 2, 3, 4, 4, 6};
  const int k = (rows_shape >= 0 && rows_shape <= kRowsShape2x1x6) ? rows_shape : kRowsShape4x2x4;
  const int pass = nw * (32 / g_of[k]);
  const int rs = (rows_of[k] + pass - 1) / pass;
  const int e = (rs * sw_of[k] <= 4) ? 8 : (rs * sw_of[k] <= 8 ? 4 : 2);
  return 2ull * fast_window_floats(t) * 4 + 2ull * rows_stage_bytes(e, t.row_stride);
}

cudaError_t batch_rows_prepare(int rows_shape, int threads, size_t smem, int* blocks_per_sm) {
  if (threads == 256)
    return batch_rows_shape<8>(rows_shape, 0, smem, 0, blocks_per_sm, nullptr, nullptr, 0, nullptr,
                               0, nullptr);
  return batch_rows_shape<4>(rows_shape, 0, smem, 0, blocks_per_sm, nullptr, nullptr, 0, nullptr, 0,
                             nullptr);
}

cudaError_t launch_batch_rows(int rows_shape, int threads, size_t smem, int grid,
                              const BatchInstance* insts, const BatchItem* items, int32_t n_items,
                              int32_t* next, int parity, cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  if (threads == 256)
    return batch_rows_shape<8>(rows_shape, 1, smem, grid, nullptr, insts, items, n_items, next,
                               parity, s);
  return batch_rows_shape<4>(rows_shape, 1, smem, grid, nullptr, insts, items, n_items, next,
                             parity, s);
}

cudaError_t launch_batch_clear(const BatchInstance* insts, int32_t n_inst, int32_t max_pix,
                               int parity, cudaStream_t s) {
  if (n_inst <= 0) return cudaSuccess;
  const int bx = std::max(1, std::min(64, (max_pix + 255) / 256));
  batch_clear_kernel<<<dim3(bx, n_inst), 256, 0, s>>>(insts, parity);
  return cudaGetLastError();
}

cudaError_t launch_batch_oversize(const BatchInstance* insts, const BatchItem* items,
                                  int32_t n_items, int parity, cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  batch_oversize_kernel<<<std::min(n_items, 152 * 8), 256, 0, s>>>(insts, items, n_items, parity);
  return cudaGetLastError();
}

}  // namespace jpet
