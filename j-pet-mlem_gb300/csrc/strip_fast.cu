// Fast sm_103a MLEM iteration for the CPU-reference semantics.
//
// Two pieces:
//
// 1. row_table_kernel (once per event set): for every sorted event and every
//    row of its clamped box, the exact column interval whose pixel centres pass
//    the reference's 3-sigma test (GaussianKernel::in_ellipse,
//    src/2d/strip/gaussian_kernel.h:131-137, evaluated in the reference's
//    rounding).  The test's quadratic form is convex along a row, so the passing
//    columns are one interval; it is found from the analytic endpoints
//    tan*dy +- sqrt((9 - 4 ipd sec^2 dy^2) / (2 ipz)) and corrected by evaluating
//    the exact test around them.  Stored as 16 bits per row: first column
//    relative to the box (8 bits) and width (8 bits); the last entry of the
//    event's table holds its widest row.  The pixel set of every
//    event is therefore exactly the reference's, without any per-pixel test in
//    the iterations.
//
// 2. iterate_fast_kernel (every iteration, the JPET_VARIANT_WARP variant; the
//    default variant is the row-owned kernel of strip_rows.cu): one CTA per chunk of events of one
//    image tile, rho window and back-projection window in shared memory (as the
//    exact kernel).  One warp per event; 4 lanes per image row, 8 rows per step,
//    each lane two adjacent pixels per 8-column sweep, so that the packed f32x2
//    instructions of sm_100+ (FFMA2/FADD2/FMUL2) evaluate two pixels each.  The
//    kernel value is rewritten so that a pixel costs one exp2:
//
//      K = c0 / sqrt(aMa) * exp(-bMb / 2)                      (gaussian_kernel.h:51-79)
//      bMb = 2 ipz u^2 + 4 ipd sec^2 dy^2,  u = dz - dy tan,  dy = py - y
//      aMa = 2 ipz sec^4 (py^2 + R^2) + 4 ipd sec^2 tan^2 py^2
//      K / K_ref = 2^(kz u^2 + ky dy^2 - log2(aMa(py)/aMa(y)) / 2)
//
//    with kz = -log2(e) ipz and ky = -2 log2(e) ipd sec^2; K_ref = c0/sqrt(aMa(y))
//    is a per-event constant that cancels in K rho / sum K rho.  Along a row,
//    u = u0 + j pw for the j-th in-ellipse pixel, so the exponent is
//    P_row + Q_row j + kz pw^2 j^2 with a per-lane constant for the last term.
//    The exponent is evaluated with ex2.approx, the row prefactor with
//    lg2.approx.  K rho of every pixel stays in registers between the forward
//    sum and the back-projection (shared-memory atomics).  Events whose box does
//    not fit the register cache take the exact warp rasteriser instead.
#include <cuda_runtime.h>

#include <cstdint>

#include "strip_device.cuh"
#include "strip_internal.h"
#include "strip_fast_common.cuh"
#include "strip_raster.cuh"

namespace jpet {
namespace {

// ---------------------------------------------------------------------------------
// exact per-row intervals
// ---------------------------------------------------------------------------------

__global__ void __launch_bounds__(256) row_table_kernel(DevGeom g, int32_t n, int32_t stride,
                                                        const float4* __restrict__ ev_geom,
                                                        const short4* __restrict__ ev_box,
                                                        uint16_t* __restrict__ rows,
                                                        unsigned long long* kernel_calls) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long calls = 0;
  for (int e = warp; e < n; e += n_warps) {
    const float4 ev = ev_geom[e];
    const short4 b = ev_box[e];
    const float z = ev.x, y = ev.y, t = ev.z, sec = ev.w;
    float A, B, C;
    ellipse_abc(g, t, sec, A, B, C);
    const int nrows = b.w - b.y;
    const int bx = b.x, bz = b.z;
    int maxw = 0;
    for (int ri = lane; ri < nrows; ri += 32) {
      int first;
      const int w = row_interval(g, A, B, C, z, y, t, sec, bx, bz, b.y + ri, first);
      rows[static_cast<size_t>(e) * stride + ri] =
          static_cast<uint16_t>((first - bx) | (w << 8));
      calls += static_cast<unsigned long long>(w);
      maxw = max(maxw, w);
    }
    // the last entry of every event holds its widest row (stride > max rows)
    maxw = __reduce_max_sync(kFull, maxw);
    if (lane == 0) rows[static_cast<size_t>(e) * stride + stride - 1] = static_cast<uint16_t>(maxw);
  }
  calls = warp_sum_u64(calls);
  if (lane == 0 && calls) atomicAdd(kernel_calls, calls);
}

// ---------------------------------------------------------------------------------
// fast iteration
// ---------------------------------------------------------------------------------

// One event on one warp, straight-line code for RS row steps x SW sweeps:
// phase A computes the constants of 32 rows per pass (one row per lane), phase
// B evaluates every (row step, sweep) slot without branches (invalid pixels
// are zeroed), phase C adds K rho / den with shared-memory atomics.
// DEN64 reduces the per-lane partial denominators in FP64.
// Returns whether the event contributed (den > 0).
template <int RS, int SW, int ACC, bool DEN64>
__device__ __forceinline__ bool fast_event(const DevGeom& g, const FastConst& fc, float4 ev,
                                           short4 box, const uint32_t* ent, int nrows, int ox,
                                           int oy, int pitch, const float* w_rho, float* w_out,
                                           float* w_comp, const FastLane& fl,
                                           uint32_t dither_key) {
  constexpr int kSets = (RS * kRPS + 31) / 32;
  const int lane = threadIdx.x & 31;
  const int gid = lane / kG, gl = lane % kG;
  const float z = ev.x, y = ev.y, tn = ev.z, sec = ev.w;
  const float sec2 = sec * sec;
  const float ky = fc.kdl * sec2;
  // aMa(py) = P + Q py^2
  const float P = fc.two_r2 * sec2 * sec2 * g.ipz;
  const float Q = 2.0f * sec2 * sec2 * g.ipz + 4.0f * sec2 * tn * tn * g.ipd;
  const float lref = 0.5f * lg2_approx(fmaf(Q, y * y, P));
  const float u_base = g.tl_z_half_w - z;
  const int col0 = box.x - ox;
  const float kz2pw = 2.0f * fc.kz * g.pixel_width;

  // phase A: row constants, lane l <- rows l, l + 32, ...
  int rw[kSets], rb[kSets];
  float rpv[kSets], rqv[kSets];
#pragma unroll
  for (int k = 0; k < kSets; ++k) {
    const int ri = lane + 32 * k;
    const uint32_t en = ent[k];
    const int w = (ri < nrows) ? static_cast<int>(en >> 8) : 0;
    const int lo = col0 + static_cast<int>(en & 255u);
    const int a_off = lo & ~1;
    const int row = min(ri, nrows - 1) + box.y - oy;
    const float py = g.tl_y_half_h - static_cast<float>(box.y + ri) * g.pixel_height;
    const float dy = py - y;
    const float lf = lref - 0.5f * lg2_approx(fmaf(Q, py * py, P));
    const float ua = fmaf(static_cast<float>(ox + a_off), g.pixel_width, u_base - dy * tn);
    rw[k] = w | ((lo & 1) << 8);
    rb[k] = row * pitch + a_off;
    rpv[k] = fmaf(fc.kz * ua, ua, fmaf(ky * dy, dy, lf));
    rqv[k] = kz2pw * ua;
  }

  // phase B: forward sum over all slots
  float2 cache[RS][SW];
  float2 den_a = make_float2(0.0f, 0.0f), den_b = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int rs = 0; rs < RS; ++rs) {
    const int src = (rs * kRPS) % 32 + gid;
    const int set = (rs * kRPS) / 32;
    const int wl = __shfl_sync(kFull, rw[set], src);
    const int base = __shfl_sync(kFull, rb[set], src);
    const float p = __shfl_sync(kFull, rpv[set], src);
    const float q = __shfl_sync(kFull, rqv[set], src);
    const int lodd = (wl >> 8) & 1;
    const int d = (wl & 255) + lodd - 2 * gl;  // elements of the row left for this lane
    const bool lo_skip = (gl == 0) && lodd;
    const float* rp = w_rho + base + 2 * gl;
    const float2 p2 = make_float2(p, p), q2 = make_float2(q, q);
#pragma unroll
    for (int s = 0; s < SW; ++s) {
      const float2 a = __ffma2_rn(q2, fl.jf[s], __fadd2_rn(p2, fl.cj[s]));
      const float2 r2 = *reinterpret_cast<const float2*>(rp + kCols * s);
      float2 kr = __fmul2_rn(make_float2(ex2_approx(a.x), ex2_approx(a.y)), r2);
      const bool v0 = (kCols * s < d) && !(s == 0 && lo_skip);
      const bool v1 = (kCols * s + 1 < d);
      kr.x = v0 ? kr.x : 0.0f;
      kr.y = v1 ? kr.y : 0.0f;
      cache[rs][s] = kr;
      if (rs & 1)
        den_b = __fadd2_rn(den_b, kr);
      else
        den_a = __fadd2_rn(den_a, kr);
    }
  }
  float den;
  if (DEN64) {
    double dd = static_cast<double>(den_a.x + den_a.y) + static_cast<double>(den_b.x + den_b.y);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dd += __shfl_xor_sync(kFull, dd, o);
    den = static_cast<float>(dd);
    if (!(dd > 0.0)) return false;
  } else {
    den = warp_sum((den_a.x + den_a.y) + (den_b.x + den_b.y));
  }
  if (!(den > 0.0f)) return false;  // inv_denominator = 0 (reconstruction.h:290)
  const float inv = __fdiv_rn(1.0f, den);
  // phase C: back-projection
  if (ACC == kAccFloat) {
    const float2 inv2 = make_float2(inv, inv);
#pragma unroll
    for (int rs = 0; rs < RS; ++rs) {
      const int src = (rs * kRPS) % 32 + gid;
      const int set = (rs * kRPS) / 32;
      const int base = __shfl_sync(kFull, rb[set], src);
      float* op = w_out + base + 2 * gl;
#pragma unroll
      for (int s = 0; s < SW; ++s) {
        const float2 v = __fmul2_rn(cache[rs][s], inv2);
        if (v.x != 0.0f) atomicAdd(op + kCols * s, v.x);
        if (v.y != 0.0f) atomicAdd(op + kCols * s + 1, v.y);
      }
    }
  } else if (ACC == kAccCompensated) {
    const float2 inv2 = make_float2(inv, inv);
#pragma unroll
    for (int rs = 0; rs < RS; ++rs) {
      const int src = (rs * kRPS) % 32 + gid;
      const int set = (rs * kRPS) / 32;
      const int base = __shfl_sync(kFull, rb[set], src) + 2 * gl;
#pragma unroll
      for (int s = 0; s < SW; ++s) {
        const float2 v = __fmul2_rn(cache[rs][s], inv2);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float x = h ? v.y : v.x;
          if (x != 0.0f) {
            const int i = base + kCols * s + h;
            const float old = atomicAdd(w_out + i, x);
            // TwoSum: old + x = t + err exactly, t the value now in memory
            const float t = __fadd_rn(old, x);
            const float bp = __fsub_rn(t, old);
            const float err = __fadd_rn(__fsub_rn(old, __fsub_rn(t, bp)), __fsub_rn(x, bp));
            if (err != 0.0f) atomicAdd(w_comp + i, err);
          }
        }
      }
    }
  } else {
    // q = floor(v 2^22 + U), U uniform in [0, 1) per event: E[q] = v 2^22
    const float dither =
        static_cast<float>(hash32(dither_key) >> 8) * 5.9604644775390625e-08f - 0.5f;
    const float sc = inv * kFixedScale;
    const float2 sc2 = make_float2(sc, sc), d2 = make_float2(dither, dither);
    const float2 m2 = make_float2(kMagic, kMagic);
    uint32_t* oq = reinterpret_cast<uint32_t*>(w_out);
#pragma unroll
    for (int rs = 0; rs < RS; ++rs) {
      const int src = (rs * kRPS) % 32 + gid;
      const int set = (rs * kRPS) / 32;
      const int base = __shfl_sync(kFull, rb[set], src);
      uint32_t* op = oq + base + 2 * gl;
#pragma unroll
      for (int s = 0; s < SW; ++s) {
        const float2 x = __fadd2_rn(__ffma2_rn(cache[rs][s], sc2, d2), m2);
        const uint32_t q0 = __float_as_uint(x.x) - 0x4B400000u;
        const uint32_t q1 = __float_as_uint(x.y) - 0x4B400000u;
        if (q0 != 0u) atomicAdd(op + kCols * s, q0);
        if (q1 != 0u) atomicAdd(op + kCols * s + 1, q1);
      }
    }
  }
  return true;
}

template <int RS, int SW, int ACC, bool DEN64>
__global__ void __launch_bounds__(256) iterate_fast_kernel(
    DevGeom g, FastConst fc, Tiling t, const Chunk* __restrict__ chunks,
    const float4* __restrict__ ev_geom, const short4* __restrict__ ev_box,
    const uint16_t* __restrict__ rows, const float* __restrict__ rho, float* __restrict__ out,
    AuxImage aux, DevCounters* counters, uint32_t seed) {
  extern __shared__ __align__(16) float smem[];
  const int pitch = fast_pitch(t);
  const int wfl = fast_window_floats(t);
  float* w_rho = smem;
  float* w_out = smem + wfl;
  float* w_comp = (ACC == kAccCompensated) ? smem + 2 * wfl : nullptr;
  const Chunk c = chunks[blockIdx.x];
  const int ox = c.ox & ~1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  for (int r = warp; r < t.win_h; r += n_warps) {
    const int gy = c.oy + r;
    for (int col = lane; col < pitch; col += 32) {
      const int gx = ox + col;
      w_rho[r * pitch + col] = (gy < g.n_y && gx < g.n_z) ? rho[gy * g.n_z + gx] : 0.0f;
      w_out[r * pitch + col] = 0.0f;
      if (ACC == kAccCompensated) w_comp[r * pitch + col] = 0.0f;
    }
  }
  for (int i = threadIdx.x; i < 64; i += blockDim.x) w_rho[t.win_h * pitch + i] = 0.0f;
  __syncthreads();

  FastLane fl;
  {
    const int gl = lane % kG;
    const float kzp2 = fc.kz * g.pixel_width * g.pixel_width;
#pragma unroll
    for (int s = 0; s < SW; ++s) {
      const float j0 = static_cast<float>(2 * gl + kCols * s);
      fl.jf[s] = make_float2(j0, j0 + 1.0f);
      fl.cj[s] = make_float2(kzp2 * j0 * j0, kzp2 * (j0 + 1.0f) * (j0 + 1.0f));
    }
  }
  constexpr int kEntRegs = (RS * kRPS + 31) / 32;
  WindowAccess acc{w_rho, w_out, ox, c.oy, pitch};
  unsigned long long contrib = 0, dummy_calls = 0, exact_path = 0;
  int e = warp;
  float4 ev_next = make_float4(0.f, 0.f, 0.f, 0.f);
  short4 box_next = make_short4(0, 0, 0, 0);
  if (e < c.count) {
    ev_next = ev_geom[c.start + e];
    box_next = ev_box[c.start + e];
  }
  for (; e < c.count; e += n_warps) {
    const int ei = c.start + e;
    const float4 ev = ev_next;
    const short4 box = box_next;
    const int nrows = box.w - box.y;
    const uint16_t* rt = rows + static_cast<size_t>(ei) * t.row_stride;
    uint32_t ent[kEntRegs];
    int maxw = 0;
#pragma unroll
    for (int k = 0; k < kEntRegs; ++k) {
      const int ri = lane + 32 * k;
      ent[k] = (ri < nrows) ? rt[ri] : 0u;
      maxw = max(maxw, static_cast<int>(ent[k] >> 8));
    }
    if (e + n_warps < c.count) {  // prefetch the next event of this warp
      ev_next = ev_geom[ei + n_warps];
      box_next = ev_box[ei + n_warps];
    }
    maxw = __reduce_max_sync(kFull, maxw);
    bool ok;
    const uint32_t key = hash32(static_cast<uint32_t>(ei) ^ seed);
    if (nrows > RS * kRPS || maxw + 1 > SW * kCols) {
      ++exact_path;
      // boxes outside the register-cache shape: reference-order rasteriser;
      // in the fixed-point mode it adds to the global float image directly
      if (ACC == kAccFloat) {
        process_event<kCpuReference>(g, 32, ev, box, acc, nullptr, dummy_calls, contrib);
      } else {
        GlobalAccess gacc{rho, out, g.n_z};
        process_event<kCpuReference>(g, 32, ev, box, gacc, nullptr, dummy_calls, contrib);
      }
      continue;
    } else if (RS > 4 && nrows <= (RS / 2) * kRPS) {
      ok = fast_event<(RS > 4 ? RS / 2 : RS), SW, ACC, DEN64>(
          g, fc, ev, box, ent, nrows, ox, c.oy, pitch, w_rho, w_out, w_comp, fl, key);
    } else {
      ok = fast_event<RS, SW, ACC, DEN64>(g, fc, ev, box, ent, nrows, ox, c.oy, pitch, w_rho,
                                          w_out, w_comp, fl, key);
    }
    if (ok && lane == 0) ++contrib;
  }
  if (lane == 0 && contrib) atomicAdd(&counters->n_contributing, contrib);
  if (lane == 0 && exact_path) atomicAdd(&counters->n_exact_path, exact_path);
  __syncthreads();
  for (int r = warp; r < t.win_h; r += n_warps) {
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

template <int RS, int SW, int ACC, bool DEN64>
cudaError_t launch_fast_kernel(const DevGeom& g, const FastConst& fc, const Tiling& t,
                               const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                               const short4* ev_box, const uint16_t* rows, const float* rho,
                               float* out, AuxImage aux, DevCounters* counters, uint32_t seed,
                               cudaStream_t s) {
  const size_t smem =
      (ACC == kAccCompensated ? 3ull : 2ull) * fast_window_floats(t) * sizeof(float);
  cudaError_t err = cudaFuncSetAttribute(iterate_fast_kernel<RS, SW, ACC, DEN64>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
  if (err != cudaSuccess) return err;
  iterate_fast_kernel<RS, SW, ACC, DEN64><<<n_chunks, t.threads, smem, s>>>(
      g, fc, t, chunks, ev_geom, ev_box, rows, rho, out, aux, counters, seed);
  return cudaGetLastError();
}

template <int RS, int SW>
cudaError_t launch_fast_shape(const DevGeom& g, const FastConst& fc, const Tiling& t,
                              const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                              const short4* ev_box, const uint16_t* rows, const float* rho,
                              float* out, AuxImage aux, DevCounters* counters, int precision,
                              uint32_t seed, cudaStream_t s) {
  switch (precision) {
    case kPrecisionCompensated:
      return launch_fast_kernel<RS, SW, kAccCompensated, false>(
          g, fc, t, chunks, n_chunks, ev_geom, ev_box, rows, rho, out, aux, counters, seed, s);
    case kPrecisionCompensatedDen64:
      return launch_fast_kernel<RS, SW, kAccCompensated, true>(
          g, fc, t, chunks, n_chunks, ev_geom, ev_box, rows, rho, out, aux, counters, seed, s);
    case kPrecisionFixed:
      return launch_fast_kernel<RS, SW, kAccFixed, false>(g, fc, t, chunks, n_chunks, ev_geom,
                                                          ev_box, rows, rho, out, aux, counters,
                                                          seed, s);
    default:
      return launch_fast_kernel<RS, SW, kAccFloat, false>(g, fc, t, chunks, n_chunks, ev_geom,
                                                          ev_box, rows, rho, out, aux, counters,
                                                          seed, s);
  }
}

__global__ void combine_aux_kernel(int fixed, AuxImage aux, const float* __restrict__ out,
                                   float* __restrict__ rho, int64_t n) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (fixed)  // one rounding from the exact integer sum, then an exact power-of-2 scale
    rho[i] = __fadd_rn(__fmul_rn(__ull2float_rn(aux.q[i]), 1.0f / 4194304.0f), out[i]);
  else
    rho[i] = __fadd_rn(out[i], aux.lo[i]);
}

}  // namespace

cudaError_t launch_row_tables(const DevGeom& g, const Tiling& t, int32_t n_events,
                              const float4* ev_geom, const short4* ev_box, uint16_t* rows,
                              unsigned long long* kernel_calls, cudaStream_t s) {
  if (n_events <= 0) return cudaSuccess;
  int blocks = (n_events + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  row_table_kernel<<<blocks, 256, 0, s>>>(g, n_events, t.row_stride, ev_geom, ev_box, rows,
                                          kernel_calls);
  return cudaGetLastError();
}

// Iteration-invariant data of every (event, row) for the row-owned kernel: the
// packed row word (window offset of the sweep start, interval parity, width),
// the packed event word (window row of the box top, box rows, whether the box
// fits the register shape), and the exponent coefficients: with the window origin ox of the event's tile (rounded down
// to an even column, as the kernel's window) and a = the row's first column
// rounded down to even, the exponent of the j-th pixel from a is
// p + q j + kz pw^2 j^2 (the form of fast_event's phase A).
__global__ void __launch_bounds__(256) row_coeff_kernel(DevGeom g, FastConst fc, Tiling t,
                                                        int32_t n, int32_t stride, int pitch,
                                                        int shape_rows, int shape_cols,
                                                        const float4* __restrict__ ev_geom,
                                                        const short4* __restrict__ ev_box,
                                                        const uint16_t* __restrict__ rows,
                                                        float2* __restrict__ pq,
                                                        uint32_t* __restrict__ row_pk,
                                                        uint32_t* __restrict__ ev_pk) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  const float kz2pw = 2.0f * fc.kz * g.pixel_width;
  for (int e = warp; e < n; e += n_warps) {
    const float4 ev = ev_geom[e];
    const short4 box = ev_box[e];
    const float z = ev.x, y = ev.y, tn = ev.z, sec = ev.w;
    const float sec2 = sec * sec;
    const float ky = fc.kdl * sec2;
    const float P = fc.two_r2 * sec2 * sec2 * g.ipz;
    const float Q = 2.0f * sec2 * sec2 * g.ipz + 4.0f * sec2 * tn * tn * g.ipd;
    const float lref = 0.5f * lg2_approx(fmaf(Q, y * y, P));
    const float u_base = g.tl_z_half_w - z;
    const int ox = ((box.x / t.tile_w) * t.tile_w) & ~1;
    const int r0 = box.y - (box.y / t.tile_h) * t.tile_h;  // window row of the box top
    const int col0 = box.x - ox;
    const int nrows = box.w - box.y;
    if (lane == 0) {
      const int maxw = rows[static_cast<size_t>(e) * stride + stride - 1];
      const bool fits = nrows <= shape_rows && maxw + 1 <= shape_cols;
      ev_pk[e] = static_cast<uint32_t>(r0) | (static_cast<uint32_t>(nrows) << 12) |
                 (fits ? 0x80000000u : 0u);
      row_pk[static_cast<size_t>(e) * stride + stride - 1] = static_cast<uint32_t>(maxw);
    }
    for (int ri = lane; ri < nrows; ri += 32) {
      const uint32_t en = rows[static_cast<size_t>(e) * stride + ri];
      const int lo = col0 + static_cast<int>(en & 255u);
      const int a_off = lo & ~1;
      row_pk[static_cast<size_t>(e) * stride + ri] =
          static_cast<uint32_t>((r0 + ri) * pitch + a_off) | static_cast<uint32_t>(lo & 1) |
          ((en >> 8) << 24);
      const float py = g.tl_y_half_h - static_cast<float>(box.y + ri) * g.pixel_height;
      const float dy = py - y;
      const float lf = lref - 0.5f * lg2_approx(fmaf(Q, py * py, P));
      const float ua = fmaf(static_cast<float>(ox + a_off), g.pixel_width, u_base - dy * tn);
      pq[static_cast<size_t>(e) * stride + ri] =
          make_float2(fmaf(fc.kz * ua, ua, fmaf(ky * dy, dy, lf)), kz2pw * ua);
    }
  }
}

cudaError_t launch_row_coefficients(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                    int32_t n_events, const float4* ev_geom,
                                    const short4* ev_box, const uint16_t* rows, float2* pq,
                                    uint32_t* row_pk, uint32_t* ev_pk, cudaStream_t s) {
  if (n_events <= 0) return cudaSuccess;
  if (static_cast<int64_t>(t.win_h) * fast_pitch(t) >= (1 << 24) || t.win_h >= 4096)
    return cudaErrorInvalidValue;  // packed offsets hold 24 bits, window rows 12
  int blocks = (n_events + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  row_coeff_kernel<<<blocks, 256, 0, s>>>(g, fc, t, n_events, t.row_stride, fast_pitch(t),
                                          rows_shape_rows(t.rows_shape),
                                          rows_sweep_cols(t.rows_shape), ev_geom, ev_box, rows,
                                          pq, row_pk, ev_pk);
  return cudaGetLastError();
}

cudaError_t launch_iterate_fast(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                                const short4* ev_box, const uint16_t* rows, const float* rho,
                                float* out, AuxImage aux, DevCounters* counters, int precision,
                                uint32_t seed, cudaStream_t s) {
  if (n_chunks <= 0) return cudaSuccess;
  switch (t.fast_shape) {
    case kShapeS:
      return launch_fast_shape<4, 2>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, rows, rho, out,
                                     aux, counters, precision, seed, s);
    case kShapeM:
      return launch_fast_shape<8, 3>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, rows, rho, out,
                                     aux, counters, precision, seed, s);
    default:
      return launch_fast_shape<12, 4>(g, fc, t, chunks, n_chunks, ev_geom, ev_box, rows, rho,
                                      out, aux, counters, precision, seed, s);
  }
}

cudaError_t launch_combine_aux(int precision, AuxImage aux, const float* out, float* rho,
                               int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  combine_aux_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(
      precision == kPrecisionFixed ? 1 : 0, aux, out, rho, n);
  return cudaGetLastError();
}

}  // namespace jpet
