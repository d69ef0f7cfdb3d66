// Batch-union MLEM iteration kernel for the CPU-reference semantics (the
// default kernel of every accumulation mode), and the set-up passes that feed
// it.
//
// Events are sorted by image tile, then by tan in buckets of 1/8, their box
// corner inside the tile and tan (strip_sort.cu), so neighbouring events in a
// chunk have nearly the same box and the same in-ellipse rows.  At set-up,
// union_batches_kernel groups each chunk's events greedily into batches of up
// to E consecutive events whose
// union -- per window row, from the smallest first column (rounded down to
// even) to the largest last column -- spans at most 64 rows and 32 columns, and
// writes, per batch, each union row's start column and width and, per event
// and union row, its in-ellipse interval relative to that start.  An event
// that does not fit that rectangle on its own is rasterised in the reference's
// order instead (the exact path); union_events_kernel stores each event's
// constants (y, tan, exponent coefficients, window-relative box).
//
// The iteration kernel runs one CTA of NW warps per chunk (E = NW events per
// batch), with the rho and back-projection windows of the tile in shared
// memory.  For a batch, union row r belongs to the 4 lanes (gid) of one warp,
// lane gl owning the pixel pairs 2 gl + 8 s (s < 4) of the row from its even
// start column: the SAME pixels for every event of the batch.  So rho is read
// once per batch, each event's K rho stays in registers, and the
// back-projection adds sum_e K_e rho inv_e to each owned pixel pair with one
// shared-memory read-modify-write per batch (not per event); no pixel has two
// writers in a batch and no atomics are issued.  The per-(event, row)
// exponent coefficients and column masks of batch b + 1 are computed by all
// threads in the same straight-line block as batch b's forward sums
// (double-buffered), so a batch costs one CTA barrier (the one that publishes
// the denominators).
//
// Accumulation modes (template argument ACC, DEN64): FP32 windows flushed with
// float atomics; compensated windows (each batch's addition followed by
// Knuth's TwoSum into a compensation window, flushed into the FP32 image and
// its FP32 compensation image); FP64 denominators on top of that (lane
// partials over <= 8 pixels in FP32, the sums across lanes and warps in FP64);
// fixed-point integer windows (a batch's value rounded once to 2^-22 of an
// event with a per-batch dither, flushed into the 64-bit integer image).
//
// Kernel value (src/2d/strip/gaussian_kernel.h:51-79, rewritten as in
// strip_fast.cu): along a row the exponent of K / K_ref is p + q j + c j^2 with
// c = kz pw^2.  With j counted from the union row's even start column and
// jc = j - 16, K = 2^(p' + q' jc) * 2^(c jc^2); the second factor is the same
// for every event, row and batch, so where it stays in range (|c| 16^2 <= 80,
// e.g. 2 mm pixels at sigma_z 10: 15) it multiplies rho when rho is read
// (rho'' = rho 2^(c jc^2)) and a pixel costs one FFMA2 per pixel pair, one ex2
// per pixel and one FMUL2; otherwise (coarse pixels, where 2^(c jc^2) would
// underflow while 2^(p' + q' jc) overflows) the full exponent is evaluated,
// one FADD2 more per pair.  The coefficients p', q' are regenerated on chip for
// every batch from the event's constants and the row (no per-row coefficient
// table in memory).
//
// Chain form (the default where the row Gaussian spans several pixels,
// |c| <= 0.06, e.g. 2 mm or 1 mm pixels at sigma_z = 5 pixels): along a row
// K' = 2^(p' + q' jc) is geometric, so a lane evaluates two ex2 per event and
// row (its first pixel pair) and steps to its next pair, 8 columns on, with one
// FMUL2 by R8 = 2^(8 q') (computed once per event and row at set-up).  Every
// K' a lane forms is a product of at most four rounded factors, within ~1e-6
// of the direct value, and stays a normal float: a column of the union row is
// at most ~43 pixels from the event's row peak, where 2^(c 43^2) >= 2^-111.
// The masked K' stay in registers; the forward sum takes K' rho'' in one FFMA2
// per pair, and the back-projection forms sum_e K'_e inv_e per pair and
// multiplies by rho'' once per batch.
//
// Pixel set: exactly the reference's (gaussian_kernel.h:131-137 in its
// rounding), from the exact per-row intervals of row_table_kernel: an event's
// row interval [lo, hi) relative to the union start becomes a 32-bit column
// mask (bit j = column j of the union row), tested once per pixel.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <type_traits>

#include "strip_async.cuh"
#include "strip_device.cuh"
#include "strip_fast_common.cuh"
#include "strip_internal.h"
#include "strip_raster.cuh"

namespace jpet {
namespace {

constexpr int kURows = 64;       // union rows per batch
constexpr int kUCols = 32;       // union columns from the even start
constexpr int kUSW = 4;          // sweeps of 8 columns (4 lanes x 2 pixels)
constexpr int kUMaxChunk = 2048;     // events per chunk (batch words keep 11 bits of offset)
constexpr int kUMaxChunkFixed = 512; // fixed point: a window pixel's integer sum stays < 2^31
constexpr int kUMaxE = 8;        // largest batch
constexpr int kUWinRows = 128;   // window rows the batch former tracks (4 per lane)
// Padded per-event strides of the shared-memory batch arrays: the set-up
// threads of one union row write four different events at once, and with
// unpadded strides (multiples of 128 bytes) those writes hit the same banks.
constexpr int kUPqStride = kURows + 1;    // float4 records: events 16 bytes apart in banks
constexpr int kUMaskStride = kURows + 4;  // 32-bit masks: events 4 banks apart
constexpr int kUTabStride = kURows + 8;   // 16-bit row entries: events 16 bytes apart

// Per-event constants (union_events_kernel): K / K_ref exponent terms as in
// row_coeff_kernel, and the box relative to the tile's window origin
// (first row | rows << 8 | first column << 16).
struct UEvConst {
  float y, tn, ky, lref;
  float P, Q, ub;
  uint32_t box;
};
static_assert(sizeof(UEvConst) == 32, "two 16-byte pieces");

// Batch word: first event (offset in the chunk) | events << 11 | union rows << 15
// | union's first window row << 22.
__host__ __device__ inline uint32_t ubatch_word(int first, int cnt, int rows, int u0) {
  return static_cast<uint32_t>(first) | (static_cast<uint32_t>(cnt) << 11) |
         (static_cast<uint32_t>(rows) << 15) | (static_cast<uint32_t>(u0) << 22);
}
__device__ __forceinline__ int ub_first(uint32_t w) { return static_cast<int>(w & 2047u); }
__device__ __forceinline__ int ub_cnt(uint32_t w) { return static_cast<int>((w >> 11) & 15u); }
__device__ __forceinline__ int ub_u0(uint32_t w) { return static_cast<int>((w >> 22) & 127u); }

// Union row word (per batch and union row): start column in the window | width << 9.
__host__ __device__ inline uint16_t urow_word(int u, int wu) {
  return static_cast<uint16_t>(u | (wu << 9));
}
// Event row word (per event and union row of its batch): first in-ellipse
// column relative to the union row's start | width << 8 (0: no pixel).

template <int E>
struct UStage {
  UEvConst ev[E];
  uint16_t rows[E][kUTabStride];  // event row words of the batch's union rows
  uint16_t urows[kURows];         // union row words
};

template <int E, class DT>
struct USmem {
  UStage<E> stage[2];
  float4 pq[2][E][kUPqStride];      // {p, p, q, q}, chain form {p, q, R8, R8}
  uint32_t mask[2][E][kUMaskStride];  // columns of the union row inside the event's interval
  uint32_t urow[2][kURows];     // union start column | union width << 16
  __align__(16) DT den_part[2][E][kUMaxE];  // float, or double (FP64 denominators)
  float gfac[kUCols];           // 2^(c jc^2), jc = j - 16 (split exponent)
  float cjc[kUCols];            // c jc^2 (full exponent)
  uint32_t bw[kUMaxChunk + 4];  // the chunk's batch words and exact-path list (+ one read past the last batch)
};

template <int E>
__device__ __forceinline__ void u_issue_stage(UStage<E>& st, const UEvConst* __restrict__ evc,
                                              const uint16_t* __restrict__ erows,
                                              const uint16_t* __restrict__ urows, int bi,
                                              int first, int cnt) {
  const int tid = threadIdx.x;
  if (tid < 2 * E) {
    const int j = tid >> 1, h = tid & 1;
    const bool v = j < cnt;
    const int e = first + (v ? j : 0);
    cp_async16(reinterpret_cast<float4*>(&st.ev[j]) + h,
               reinterpret_cast<const float4*>(evc + e) + h, v);
  } else if (tid >= 2 * E && tid < 2 * E + kURows / 8) {
    const int q = tid - 2 * E;
    cp_async16(&st.urows[8 * q], urows + static_cast<size_t>(bi) * kURows + 8 * q, true);
  } else if (tid >= 32 && tid < 32 + E * (kURows / 8)) {
    const int k = tid - 32;
    const int j = k >> 3, q = k & 7;
    const bool v = j < cnt;
    const size_t src = static_cast<size_t>(first + (v ? j : 0)) * kURows + 8 * q;
    cp_async16(&st.rows[j][8 * q], erows + src, v);
  }
  cp_async_commit();
}

// Union rows and per-(event, row) records of one batch: NW / 2 threads per
// union row (consecutive lanes), each handling two events.
// Exponent forms of the iteration kernel (template argument XM).
constexpr int kXFull = 0;   // p + q jc + c jc^2 per pixel
constexpr int kXSplit = 1;  // 2^(c jc^2) folded into rho''
constexpr int kXChain = 2;  // split, and K' stepped along the row by R8

template <int E, int NW, int XM, class DT>
__device__ __forceinline__ void u_setup(const DevGeom& g, const FastConst& fc, USmem<E, DT>& S,
                                        int buf, uint32_t bw, int ox, int oy) {
  constexpr int kTPR = NW / 2;  // threads per union row
  static_assert(E == 2 * kTPR, "two events per set-up thread");
  const UStage<E>& st = S.stage[buf];
  const int u0 = ub_u0(bw);
  const int r = threadIdx.x / kTPR, sub = threadIdx.x % kTPR;
  // union row (start column, width) and the events' intervals relative to it,
  // as the batch former wrote them (rows past the union, and events past the
  // batch's count, read as 0: no pixel)
  const uint32_t ur = st.urows[r];
  const int u = static_cast<int>(ur & 511u), wu = static_cast<int>(ur >> 9);
  if (sub == 0) S.urow[buf][r] = static_cast<uint32_t>(u) | (static_cast<uint32_t>(wu) << 16);
  const float py = g.tl_y_half_h - static_cast<float>(oy + u0 + r) * g.pixel_height;
  const float colm = static_cast<float>(ox + u + 16);
  const float kz2pw = 2.0f * fc.kz * g.pixel_width;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int j = 2 * sub + k;
    const UEvConst& e = st.ev[j];
    const float dy = py - e.y;
    const float lf = e.lref - 0.5f * lg2_approx(fmaf(e.Q, py * py, e.P));
    const float ua = fmaf(colm, g.pixel_width, e.ub - dy * e.tn);
    const float p = fmaf(fc.kz * ua, ua, fmaf(e.ky * dy, dy, lf));
    const float q = kz2pw * ua;
    const uint32_t ew = st.rows[j][r];
    const int w = static_cast<int>(ew >> 8);
    const int lr = static_cast<int>(ew & 255u);  // 0 <= lr, lr + w <= wu <= 32
    // w low bits set (0 <= w <= 32): the clamped funnel shift of ~0 by 32 - w
    const uint32_t bits = __funnelshift_rc(0xFFFFFFFFu, 0u, static_cast<unsigned>(32 - w));
    if (XM == kXChain) {
      const float r8 = ex2_approx(8.0f * q);
      S.pq[buf][j][r] = make_float4(p, q, r8, r8);
    } else {
      S.pq[buf][j][r] = make_float4(p, p, q, q);
    }
    S.mask[buf][j][r] = bits << lr;
  }
}

// Forward sums of one row step with SWN active sweeps: rho'' of the owned
// pixel pairs, then every event's K rho'' (masked to its interval).
template <int E, int SWN, int RSI, int RS, bool SPLIT, class DT>
__device__ __forceinline__ void u_forward(float2 (&kr)[E][RS][kUSW], DT (&dsum)[E],
                                          const float* w_rho, const USmem<E, DT>& S, int buf,
                                          int base,
                                          int r_u, const float2 (&jc2)[kUSW], int gl) {
  float2 rr[kUSW], cq[kUSW];
#pragma unroll
  for (int s = 0; s < SWN; ++s) {
    const float2 rv = *reinterpret_cast<const float2*>(w_rho + base + 8 * s);
    if (SPLIT) {
      const float2 gv = *reinterpret_cast<const float2*>(&S.gfac[2 * gl + 8 * s]);
      rr[s] = __fmul2_rn(rv, gv);
    } else {
      rr[s] = rv;
      cq[s] = *reinterpret_cast<const float2*>(&S.cjc[2 * gl + 8 * s]);
    }
  }
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const float4 a = S.pq[buf][j][r_u];
    const uint32_t m = S.mask[buf][j][r_u] >> (2 * gl);
    const float2 p2 = make_float2(a.x, a.y), q2 = make_float2(a.z, a.w);
    float2 dd = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int s = 0; s < SWN; ++s) {
      const float2 e = SPLIT ? __ffma2_rn(q2, jc2[s], p2)
                             : __ffma2_rn(q2, jc2[s], __fadd2_rn(p2, cq[s]));
      float2 v = __fmul2_rn(make_float2(ex2_approx(e.x), ex2_approx(e.y)), rr[s]);
      v.x = (m & (1u << (8 * s))) ? v.x : 0.0f;
      v.y = (m & (2u << (8 * s))) ? v.y : 0.0f;
      kr[j][RSI][s] = v;
      dd = __fadd2_rn(dd, v);
    }
    dsum[j] += static_cast<DT>(dd.x + dd.y);
  }
}

// Forward sums of one row step in the chain form: per event two ex2 for the
// lane's first pixel pair, then one FMUL2 by R8 per further pair; the masked
// K' stay in kr and the sum takes K' rho'' with one FFMA2 per pair.
template <int E, int SWN, int RSI, int RS, class DT>
__device__ __forceinline__ void u_forward_chain(float2 (&kr)[E][RS][kUSW], DT (&dsum)[E],
                                                const float* w_rho, const USmem<E, DT>& S, int buf,
                                                int base, int r_u, float jc0, int gl) {
  float2 rr[kUSW];
#pragma unroll
  for (int s = 0; s < SWN; ++s) {
    const float2 rv = *reinterpret_cast<const float2*>(w_rho + base + 8 * s);
    const float2 gv = *reinterpret_cast<const float2*>(&S.gfac[2 * gl + 8 * s]);
    rr[s] = __fmul2_rn(rv, gv);
  }
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const float4 a = S.pq[buf][j][r_u];
    const uint32_t m = S.mask[buf][j][r_u] >> (2 * gl);
    const float e0 = fmaf(a.y, jc0, a.x);
    float2 k = make_float2(ex2_approx(e0), ex2_approx(e0 + a.y));
    const float2 r8 = make_float2(a.z, a.w);
    float2 dd;
#pragma unroll
    for (int s = 0; s < SWN; ++s) {
      if (s > 0) k = __fmul2_rn(k, r8);
      float2 v;
      v.x = (m & (1u << (8 * s))) ? k.x : 0.0f;
      v.y = (m & (2u << (8 * s))) ? k.y : 0.0f;
      kr[j][RSI][s] = v;
      dd = (s == 0) ? __fmul2_rn(v, rr[0]) : __ffma2_rn(v, rr[s], dd);
    }
    // a lane's partial over its <= 8 pixels of the row in FP32; FP64 (DEN64)
    // from the sums across lanes and warps on
    const DT pr = static_cast<DT>(dd.x + dd.y);
    dsum[j] = (RSI == 0) ? pr : dsum[j] + pr;
  }
}

// Adds a pixel pair's batch value v (sum over the batch's events of
// K rho / den) into the back-projection window, storing only where the row
// group owns the pair (own):
//   kAccFloat        plain float addition;
//   kAccCompensated  float addition whose exact rounding error (Knuth's TwoSum)
//                    joins the compensation window;
//   kAccFixed        v rounded once to 2^-22 of an event with the batch's
//                    dither (floor(v 2^22 + U), U uniform in [0, 1): unbiased)
//                    and added to the integer window (order-independent sums;
//                    a window pixel of a chunk of <= 512 events stays < 2^31,
//                    so the fixed-point mode's chunks hold at most 512).
template <int ACC>
__device__ __forceinline__ void u_accumulate(float* w_out, float* w_comp, int idx, float2 v,
                                             bool own, float dither) {
  if (ACC == kAccFixed) {
    uint2* op = reinterpret_cast<uint2*>(w_out + idx);
    const uint2 o = *op;
    const uint32_t q0 = __float2uint_rn(fmaf(v.x, kFixedScale, dither));
    const uint32_t q1 = __float2uint_rn(fmaf(v.y, kFixedScale, dither));
    if (own) *op = make_uint2(o.x + q0, o.y + q1);
  } else {
    float2* op = reinterpret_cast<float2*>(w_out + idx);
    const float2 o = *op;
    const float2 n = __fadd2_rn(o, v);
    if (ACC == kAccCompensated) {
      float2* cp = reinterpret_cast<float2*>(w_comp + idx);
      const float2 bp = __fadd2_rn(n, make_float2(-o.x, -o.y));
      const float2 nb = __fadd2_rn(n, make_float2(-bp.x, -bp.y));
      const float2 err = __fadd2_rn(__fadd2_rn(o, make_float2(-nb.x, -nb.y)),
                                    __fadd2_rn(v, make_float2(-bp.x, -bp.y)));
      const float2 cn = __fadd2_rn(*cp, err);
      if (own) {
        *op = n;
        *cp = cn;
      }
    } else if (own) {
      *op = n;
    }
  }
}

// Back-projection of one row step in the chain form: rho'' sum_e K'_e inv_e
// per owned pixel pair (rho'' read again), one read-modify-write of the pair.
template <int E, int SWN, int RSI, int RS, int ACC>
__device__ __forceinline__ void u_back_chain(const float2 (&kr)[E][RS][kUSW], float inv_l,
                                             const float* w_rho, const float* gfac,
                                             float* w_out, float* w_comp, int base, int wu,
                                             int gl, float dither) {
  // events outer, so that one event's 1/den is live at a time (lane j holds
  // event j's); the per-pair sums take the events in the same order as before
  float2 acc[kUSW];
#pragma unroll
  for (int j = 0; j < E; ++j) {
    const float v = __shfl_sync(kFull, inv_l, j);
    const float2 i2 = make_float2(v, v);
#pragma unroll
    for (int s = 0; s < SWN; ++s)
      acc[s] = (j == 0) ? __fmul2_rn(kr[0][RSI][s], i2) : __ffma2_rn(kr[j][RSI][s], i2, acc[s]);
  }
#pragma unroll
  for (int s = 0; s < SWN; ++s) {
    // loads stay inside the windows (a row's last pair ends before the next
    // row's pitch plus the 64-float padding); the store is predicated on the
    // union row's width, the only pixels this row group owns
    const float2 rv = *reinterpret_cast<const float2*>(w_rho + base + 8 * s);
    const float2 gv = *reinterpret_cast<const float2*>(gfac + 2 * gl + 8 * s);
    const bool own = 2 * gl + 8 * s < wu;
    if (ACC == kAccFloat) {
      float2* op = reinterpret_cast<float2*>(w_out + base + 8 * s);
      const float2 nv = __ffma2_rn(acc[s], __fmul2_rn(rv, gv), *op);
      if (own) *op = nv;
    } else {
      u_accumulate<ACC>(w_out, w_comp, base + 8 * s, __fmul2_rn(acc[s], __fmul2_rn(rv, gv)),
                        own, dither);
    }
  }
}

// Back-projection of one row step: sum_e K_e rho inv_e per owned pixel pair,
// one read-modify-write of the pair (inside the union row's width).
template <int E, int SWN, int RSI, int RS, int ACC>
__device__ __forceinline__ void u_back(const float2 (&kr)[E][RS][kUSW], const float2 (&inv2)[E],
                                       float* w_out, float* w_comp, int base, int wu, int gl,
                                       float dither) {
#pragma unroll
  for (int s = 0; s < SWN; ++s) {
    float2 acc = __fmul2_rn(kr[0][RSI][s], inv2[0]);
#pragma unroll
    for (int j = 1; j < E; ++j) acc = __ffma2_rn(kr[j][RSI][s], inv2[j], acc);
    if (ACC == kAccFloat) {
      if (2 * gl + 8 * s < wu) {
        float2* op = reinterpret_cast<float2*>(w_out + base + 8 * s);
        *op = __fadd2_rn(*op, acc);
      }
    } else {
      u_accumulate<ACC>(w_out, w_comp, base + 8 * s, acc, 2 * gl + 8 * s < wu, dither);
    }
  }
}

template <int E, int SWN, int RSI, int RS, int XM, class DT>
__device__ __forceinline__ void u_forward_x(float2 (&kr)[E][RS][kUSW], DT (&dsum)[E],
                                            const float* w_rho, const USmem<E, DT>& S, int buf,
                                            int base, int r_u, const float2 (&jc2)[kUSW],
                                            int gl) {
  if (XM == kXChain)
    u_forward_chain<E, SWN, RSI, RS, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2[0].x, gl);
  else
    u_forward<E, SWN, RSI, RS, XM == kXSplit, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl);
}

// One row step (RS == 1): forward sums, their transposed warp sum and the
// set-up of the next batch's records in one straight-line block per sweep
// count, so that the scheduler interleaves the set-up's loads, ex2/lg2 and the
// sum's shuffles with the evaluation.  The set-up runs even after a chunk's last
// batch (it then fills the unused buffer from stale staged data).
template <int E, int NW, int SWN, int XM, class DT>
__device__ __forceinline__ DT u_forward_setup_x(float2 (&kr)[E][1][kUSW], DT (&dsum)[E],
                                                const float* w_rho, USmem<E, DT>& S, int buf,
                                                   int base, int r_u, const float2 (&jc2)[kUSW],
                                                   int gl, const DevGeom& g,
                                                   const FastConst& fc, uint32_t bw_next,
                                                   int ox, int oy) {
  if (SWN > 0)
    u_forward_x<E, (SWN > 0 ? SWN : 1), 0, 1, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2,
                                                      gl);
  const DT tot = rows_transpose_sum<E>(dsum);
  u_setup<E, NW, XM, DT>(g, fc, S, buf ^ 1, bw_next, ox, oy);
  return tot;
}

template <int E, int NW, int XM, class DT>
__device__ __forceinline__ DT u_forward_setup_dispatch(
    int nsw, float2 (&kr)[E][1][kUSW], DT (&dsum)[E], const float* w_rho, USmem<E, DT>& S,
    int buf, int base, int r_u, const float2 (&jc2)[kUSW], int gl, const DevGeom& g,
    const FastConst& fc, uint32_t bw_next, int ox, int oy) {
  switch (nsw) {
    case 4:
      return u_forward_setup_x<E, NW, 4, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl, g, fc,
                                             bw_next, ox, oy);
    case 3:
      return u_forward_setup_x<E, NW, 3, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl, g, fc,
                                             bw_next, ox, oy);
    case 2:
      return u_forward_setup_x<E, NW, 2, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl, g, fc,
                                             bw_next, ox, oy);
    case 1:
      return u_forward_setup_x<E, NW, 1, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl, g, fc,
                                             bw_next, ox, oy);
    default:
      return u_forward_setup_x<E, NW, 0, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl, g, fc,
                                             bw_next, ox, oy);
  }
}

template <int E, int RSI, int RS, int XM, class DT>
__device__ __forceinline__ void u_forward_dispatch(int nsw, float2 (&kr)[E][RS][kUSW],
                                                   DT (&dsum)[E], const float* w_rho,
                                                   const USmem<E, DT>& S, int buf, int base, int r_u,
                                                   const float2 (&jc2)[kUSW], int gl) {
  switch (nsw) {
    case 4: u_forward_x<E, 4, RSI, RS, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl); break;
    case 3: u_forward_x<E, 3, RSI, RS, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl); break;
    case 2: u_forward_x<E, 2, RSI, RS, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl); break;
    case 1: u_forward_x<E, 1, RSI, RS, XM, DT>(kr, dsum, w_rho, S, buf, base, r_u, jc2, gl); break;
    default: break;
  }
}

template <int E, int SWN, int RSI, int RS, int XM, int ACC>
__device__ __forceinline__ void u_back_x(const float2 (&kr)[E][RS][kUSW], float inv_l,
                                         const float* w_rho, const float* gfac, float* w_out,
                                         float* w_comp, int base, int wu, int gl, float dither) {
  if (XM == kXChain) {
    u_back_chain<E, SWN, RSI, RS, ACC>(kr, inv_l, w_rho, gfac, w_out, w_comp, base, wu, gl,
                                       dither);
  } else {
    float2 inv2[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
      const float v = __shfl_sync(kFull, inv_l, j);
      inv2[j] = make_float2(v, v);
    }
    u_back<E, SWN, RSI, RS, ACC>(kr, inv2, w_out, w_comp, base, wu, gl, dither);
  }
}

// nsw is warp-uniform (a warp maximum), so the shuffles inside run converged
template <int E, int RSI, int RS, int XM, int ACC>
__device__ __forceinline__ void u_back_dispatch(int nsw, const float2 (&kr)[E][RS][kUSW],
                                                float inv_l, const float* w_rho,
                                                const float* gfac, float* w_out, float* w_comp,
                                                int base, int wu, int gl, float dither) {
  switch (nsw) {
    case 4:
      u_back_x<E, 4, RSI, RS, XM, ACC>(kr, inv_l, w_rho, gfac, w_out, w_comp, base, wu, gl,
                                       dither);
      break;
    case 3:
      u_back_x<E, 3, RSI, RS, XM, ACC>(kr, inv_l, w_rho, gfac, w_out, w_comp, base, wu, gl,
                                       dither);
      break;
    case 2:
      u_back_x<E, 2, RSI, RS, XM, ACC>(kr, inv_l, w_rho, gfac, w_out, w_comp, base, wu, gl,
                                       dither);
      break;
    case 1:
      u_back_x<E, 1, RSI, RS, XM, ACC>(kr, inv_l, w_rho, gfac, w_out, w_comp, base, wu, gl,
                                       dither);
      break;
    default: break;
  }
}

template <int NW>
constexpr int u_min_blocks() {
  return NW == 8 ? 2 : 4;
}

// Shared memory of the kernel: the rho and back-projection windows (and the
// compensation window of the compensated modes), then the batch records.
template <int NW, int ACC, bool DEN64>
size_t u_smem(const Tiling& t) {
  using DT = typename std::conditional<DEN64, double, float>::type;
  return (ACC == kAccCompensated ? 3ull : 2ull) * fast_window_floats(t) * sizeof(float) +
         sizeof(USmem<NW, DT>);
}

// ACC: kAccFloat (the FP32 iteration), kAccCompensated (tile windows with
// TwoSum compensation, flushed into the FP32 image and its FP32 compensation
// image), kAccFixed (integer tile windows flushed into the 64-bit fixed-point
// image); DEN64: per-event denominators reduced in FP64.
template <int NW, int XM, int ACC, bool DEN64>
__global__ void __launch_bounds__(NW * 32, u_min_blocks<NW>()) iterate_union_kernel(
    DevGeom g, FastConst fc, Tiling t, const Chunk* __restrict__ chunks,
    const float4* __restrict__ ev_geom, const short4* __restrict__ ev_box,
    const UEvConst* __restrict__ evc, const uint16_t* __restrict__ erows,
    const uint16_t* __restrict__ urows, const uint32_t* __restrict__ batches,
    const float* __restrict__ rho, float* __restrict__ out, AuxImage aux, uint32_t seed,
    DevCounters* counters) {
  using DT = typename std::conditional<DEN64, double, float>::type;
  constexpr int E = NW;                      // events per batch
  constexpr int kRowsPerStep = NW * 8;       // union rows per step of all warps
  constexpr int RS = kURows / kRowsPerStep;  // row steps
  constexpr int kWindows = ACC == kAccCompensated ? 3 : 2;
  extern __shared__ __align__(16) float smem[];
  const int pitch = fast_pitch(t);
  const int wfl = fast_window_floats(t);
  float* w_rho = smem;
  float* w_out = smem + wfl;
  float* w_comp = ACC == kAccCompensated ? smem + 2 * wfl : nullptr;
  USmem<E, DT>& S = *reinterpret_cast<USmem<E, DT>*>(smem + kWindows * wfl);

  const Chunk c = chunks[blockIdx.x];
  const int ox = c.ox & ~1, oy = c.oy;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, gl = lane & 3;
  const int nb = c.n_batches;
  const uint32_t* bws = batches + c.start;
  auto issue = [&](int b, int buf, uint32_t w) {
    u_issue_stage<E>(S.stage[buf], evc, erows, urows, c.start + b, c.start + ub_first(w),
                     ub_cnt(w));
  };

  if (nb > 0) issue(0, 0, bws[0]);
  if (nb > 1) issue(1, 1, bws[1]);
  for (int i = threadIdx.x; i < c.count; i += NW * 32) S.bw[i] = bws[i];
  // rho window by asynchronous copies (zero outside the image), so that its
  // loads overlap with each other and with the first batches' staging
  for (int r = warp; r < t.win_h; r += NW) {
    const int gy = oy + r;
    for (int col = lane; col < pitch; col += 32) {
      const int gx = ox + col;
      const bool in = gy < g.n_y && gx < g.n_z;
      cp_async4(&w_rho[r * pitch + col], rho + (in ? gy * g.n_z + gx : 0), in);
      w_out[r * pitch + col] = 0.0f;
      if (ACC == kAccCompensated) w_comp[r * pitch + col] = 0.0f;
    }
  }
  cp_async_commit();
  for (int i = threadIdx.x; i < 64; i += NW * 32) w_rho[t.win_h * pitch + i] = 0.0f;
  if (threadIdx.x < kUCols) {
    const float cz = fc.kz * g.pixel_width * g.pixel_width;
    const float jc = static_cast<float>(threadIdx.x) - 16.0f;
    S.cjc[threadIdx.x] = cz * jc * jc;
    S.gfac[threadIdx.x] = ex2_approx(cz * jc * jc);
  }
  float2 jc2[kUSW];
#pragma unroll
  for (int s = 0; s < kUSW; ++s) {
    const float j0 = static_cast<float>(2 * gl + 8 * s) - 16.0f;
    jc2[s] = make_float2(j0, j0 + 1.0f);
  }
  unsigned long long contrib = 0;
  cp_async_wait_all();
  __syncthreads();
  if (nb > 0) u_setup<E, NW, XM, DT>(g, fc, S, 0, S.bw[0], ox, oy);
  __syncthreads();

  for (int b = 0; b < nb; ++b) {
    const int buf = b & 1;
    const uint32_t bw = S.bw[b];
    const int cnt = ub_cnt(bw), u0 = ub_u0(bw);
    if (b + 2 < nb) issue(b + 2, buf, S.bw[b + 2]);
    // ---- forward: this warp's union rows of every event of the batch
    float2 kr[E][RS][kUSW];
    DT dsum[E];
#pragma unroll
    for (int j = 0; j < E; ++j) dsum[j] = DT(0);
    int base[RS], wu[RS], nsw[RS];
#pragma unroll
    for (int rs = 0; rs < RS; ++rs) {
      const int r_u = kRowsPerStep * rs + 8 * warp + gid;
      const uint32_t ur = S.urow[buf][r_u];
      const int wrow = min(u0 + r_u, t.win_h - 1);
      base[rs] = wrow * pitch + static_cast<int>(ur & 0xFFFFu) + 2 * gl;
      wu[rs] = static_cast<int>(ur >> 16);
      nsw[rs] = (__reduce_max_sync(kFull, static_cast<unsigned>(wu[rs])) + 7) >> 3;
    }
    // ---- forward, and the set-up of the next batch (its staged data was
    // published by the last barrier)
    DT tot;
    if constexpr (RS == 1) {
      tot = u_forward_setup_dispatch<E, NW, XM, DT>(nsw[0], kr, dsum, w_rho, S, buf, base[0],
                                                8 * warp + gid, jc2, gl, g, fc, S.bw[b + 1],
                                                ox, oy);
    } else {
      u_forward_dispatch<E, 0, RS, XM, DT>(nsw[0], kr, dsum, w_rho, S, buf, base[0],
                                           8 * warp + gid, jc2, gl);
      u_forward_dispatch<E, (RS > 1 ? 1 : 0), RS, XM, DT>(nsw[RS - 1], kr, dsum, w_rho, S, buf,
                                                      base[RS - 1],
                                                      kRowsPerStep + 8 * warp + gid, jc2, gl);
      if (b + 1 < nb) u_setup<E, NW, XM, DT>(g, fc, S, buf ^ 1, S.bw[b + 1], ox, oy);
      tot = rows_transpose_sum<E>(dsum);
    }
    if (rows_lane_writes<E>(lane)) S.den_part[buf][rows_lane_event<E>(lane)][warp] = tot;
    if (b + 2 < nb) cp_async_wait_all();
    __syncthreads();
    // ---- denominators: lane j (mod E) adds the warps' partials of event j
    float inv_l;
    {
      const int jl = lane & (E - 1);
      DT den;
      if constexpr (DEN64) {
        den = S.den_part[buf][jl][0];
#pragma unroll
        for (int w = 1; w < NW; ++w) den += S.den_part[buf][jl][w];
      } else {
        const float4* dp = reinterpret_cast<const float4*>(S.den_part[buf][jl]);
        const float4 d0 = dp[0];
        den = (d0.x + d0.y) + (d0.z + d0.w);
        if (NW == 8) {
          const float4 d1 = dp[1];
          den += (d1.x + d1.y) + (d1.z + d1.w);
        }
      }
      const bool ok = den > DT(0);  // inv_denominator = 0 otherwise (reconstruction.h:290)
      inv_l = ok ? rcp_approx(static_cast<float>(den)) : 0.0f;
      const unsigned okm = __ballot_sync(kFull, ok && lane < cnt);
      if (threadIdx.x == 0) contrib += __popc(okm);
    }
    // ---- back-projection into the owned pixel pairs (fixed-point mode: one
    // dither per batch, from the batch's position and the iteration's seed)
    float dither = 0.0f;
    if (ACC == kAccFixed) {
      const uint32_t key = hash32(static_cast<uint32_t>(c.start + b) ^ seed);
      dither = static_cast<float>(key >> 8) * 5.9604644775390625e-08f - 0.5f;
    }
    u_back_dispatch<E, 0, RS, XM, ACC>(nsw[0], kr, inv_l, w_rho, S.gfac, w_out, w_comp, base[0],
                                       wu[0], gl, dither);
    if (RS > 1)
      u_back_dispatch<E, (RS > 1 ? 1 : 0), RS, XM, ACC>(nsw[RS - 1], kr, inv_l, w_rho, S.gfac,
                                                        w_out, w_comp, base[RS - 1], wu[RS - 1],
                                                        gl, dither);
  }

  // ---- events outside the batch rectangle: reference-order warp rasteriser
  __syncthreads();
  unsigned long long dummy_calls = 0, exact_path = 0;
  const int nx = c.n_exact;
  for (int k = warp; k < nx; k += NW) {
    const int ei = c.start + static_cast<int>(S.bw[c.count - 1 - k]);
    if (ACC == kAccFloat) {
      WindowAccess acc{w_rho, w_out, ox, oy, pitch};
      process_event<kCpuReference>(g, 32, ev_geom[ei], ev_box[ei], acc, nullptr, dummy_calls,
                                   contrib);
    } else {
      // the other modes' windows hold compensated or integer sums: these events
      // add into the FP32 image directly (combined with the second image after
      // the iteration)
      GlobalAccess gacc{rho, out, g.n_z};
      process_event<kCpuReference>(g, 32, ev_geom[ei], ev_box[ei], gacc, nullptr, dummy_calls,
                                   contrib);
    }
    if (lane == 0) ++exact_path;
  }
  if (lane == 0 && contrib) atomicAdd(&counters->n_contributing, contrib);
  if (lane == 0 && exact_path) atomicAdd(&counters->n_exact_path, exact_path);
  __syncthreads();
  for (int r = warp; r < t.win_h; r += NW) {
    const int gy = oy + r;
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

// Per-event constants of the sorted events (the arithmetic of row_coeff_kernel).
__global__ void union_events_kernel(DevGeom g, FastConst fc, Tiling t, int32_t n,
                                    const float4* __restrict__ ev_geom,
                                    const short4* __restrict__ ev_box, UEvConst* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 ev = ev_geom[i];
  const short4 b = ev_box[i];
  const float y = ev.y, tn = ev.z, sec = ev.w;
  const float sec2 = sec * sec;
  UEvConst c;
  c.y = y;
  c.tn = tn;
  c.ky = fc.kdl * sec2;
  c.P = fc.two_r2 * sec2 * sec2 * g.ipz;
  c.Q = 2.0f * sec2 * sec2 * g.ipz + 4.0f * sec2 * tn * tn * g.ipd;
  c.lref = 0.5f * lg2_approx(fmaf(c.Q, y * y, c.P));
  c.ub = g.tl_z_half_w - ev.x;
  const int oy = (b.y / t.tile_h) * t.tile_h;
  const int ox = ((b.x / t.tile_w) * t.tile_w) & ~1;
  const int rows = min(b.w - b.y, 255);
  c.box = static_cast<uint32_t>(b.y - oy) | (static_cast<uint32_t>(rows) << 8) |
          (static_cast<uint32_t>(b.x - ox) << 16);
  out[i] = c;
}

// Greedy batch formation, one warp per chunk: events in sorted order join the
// current batch while the union stays inside 64 rows x 32 columns and the batch
// has fewer than max_e events.  Batch words go to batches[c.start ...]; events
// that fit no batch rectangle alone are listed from the end of the chunk's
// range (batches[c.start + c.count - 1 - k]).
__global__ void __launch_bounds__(256) union_batches_kernel(Chunk* __restrict__ chunks,
                                                            int32_t n_chunks, int32_t max_e,
                                                            const short4* __restrict__ ev_box,
                                                            const uint16_t* __restrict__ rows,
                                                            int32_t stride,
                                                            uint32_t* __restrict__ batches,
                                                            uint16_t* __restrict__ urows,
                                                            uint16_t* __restrict__ erows) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  for (int ci = wid; ci < n_chunks; ci += n_warps) {
    const Chunk c = chunks[ci];
    const int ox = c.ox & ~1, oy = c.oy;
    int ulo[4], uhi[4];
    int u0 = INT_MAX, u1 = INT_MIN, cnt = 0, bstart = 0, nb = 0, nx = 0;
    auto reset = [&]() {
      cnt = 0;
      u0 = INT_MAX;
      u1 = INT_MIN;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        ulo[k] = INT_MAX;
        uhi[k] = INT_MIN;
      }
    };
    auto emit = [&]() {
      if (cnt > 0) {
        if (lane == 0) batches[c.start + nb] = ubatch_word(bstart, cnt, u1 - u0, u0);
        // union row words of the batch, and each event's intervals relative to
        // its union rows (lane: window rows lane + 32 k; the arrays start zeroed)
        uint16_t* ub = urows + static_cast<size_t>(c.start + nb) * kURows;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int wr = lane + 32 * k, r = wr - u0;
          if (r >= 0 && r < kURows && ulo[k] != INT_MAX) {
            const int u = ulo[k] & ~1;
            ub[r] = urow_word(u, uhi[k] - u);
            for (int i = bstart; i < bstart + cnt; ++i) {
              const short4 b = ev_box[c.start + i];
              const int ri = wr - (b.y - oy);
              if (ri < 0 || ri >= b.w - b.y) continue;
              const uint32_t e = rows[static_cast<size_t>(c.start + i) * stride + ri];
              const int w = static_cast<int>(e >> 8);
              if (w == 0) continue;
              const int f = (b.x - ox) + static_cast<int>(e & 255u);
              erows[static_cast<size_t>(c.start + i) * kURows + r] =
                  static_cast<uint16_t>((f - u) | (w << 8));
            }
          }
        }
        ++nb;
      }
      reset();
    };
    reset();
    for (int i = 0; i < c.count; ++i) {
      const short4 b = ev_box[c.start + i];
      const int r0 = b.y - oy, n = b.w - b.y, bx = b.x - ox;
      const uint16_t* rt = rows + static_cast<size_t>(c.start + i) * stride;
      int f[4], w[4];
      bool alone = n <= kURows && r0 >= 0 && r0 + n <= kUWinRows;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int ri = lane + 32 * k - r0;
        const bool v = ri >= 0 && ri < n && ri < kURows;
        const uint32_t e = v ? rt[v ? ri : 0] : 0u;
        w[k] = static_cast<int>(e >> 8);
        f[k] = bx + static_cast<int>(e & 255u);
        if (w[k] > 0 && f[k] + w[k] - (f[k] & ~1) > kUCols) alone = false;
      }
      alone = __all_sync(kFull, alone);
      if (!alone) {
        emit();  // a batch is a contiguous run of events: close the open one first
        if (lane == 0) batches[c.start + c.count - 1 - nx] = static_cast<uint32_t>(i);
        ++nx;
        continue;
      }
      // would the event join the current batch?
      bool join = cnt > 0 && cnt < max_e && max(u1, r0 + n) - min(u0, r0) <= kURows;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (w[k] > 0) {
          const int lo = min(ulo[k], f[k]), hi = max(uhi[k], f[k] + w[k]);
          if (hi - (lo & ~1) > kUCols) join = false;
        }
      }
      join = __all_sync(kFull, join);
      if (!join) {
        emit();
        bstart = i;
      }
      ++cnt;
      u0 = min(u0, r0);
      u1 = max(u1, r0 + n);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (w[k] > 0) {
          ulo[k] = min(ulo[k], f[k]);
          uhi[k] = max(uhi[k], f[k] + w[k]);
        }
      }
    }
    emit();
    if (lane == 0) {
      chunks[ci].n_batches = nb;
      chunks[ci].n_exact = nx;
    }
  }
}

}  // namespace

size_t union_event_bytes() { return sizeof(UEvConst); }

size_t union_smem_bytes(const Tiling& t, int precision) {
  const bool w8 = t.threads == 256;
  switch (precision) {
    case kPrecisionCompensated:
      return w8 ? u_smem<8, kAccCompensated, false>(t) : u_smem<4, kAccCompensated, false>(t);
    case kPrecisionCompensatedDen64:
      return w8 ? u_smem<8, kAccCompensated, true>(t) : u_smem<4, kAccCompensated, true>(t);
    case kPrecisionFixed:
      return w8 ? u_smem<8, kAccFixed, false>(t) : u_smem<4, kAccFixed, false>(t);
    default:
      return w8 ? u_smem<8, kAccFloat, false>(t) : u_smem<4, kAccFloat, false>(t);
  }
}

// whether 2^(c jc^2), |jc| <= 16, may multiply rho (see the file comment)
bool union_split_exponent(const DevGeom& g, const FastConst& fc) {
  const float cz = fc.kz * g.pixel_width * g.pixel_width;
  return -cz * 256.0f <= 80.0f;
}

// whether the chain form applies: split, and the row Gaussian wide enough that
// every K' a lane steps through stays a normal float (see the file comment)
bool union_chain_exponent(const DevGeom& g, const FastConst& fc) {
  const float cz = fc.kz * g.pixel_width * g.pixel_width;
  return union_split_exponent(g, fc) && -cz <= 0.06f;
}

namespace {
template <int NW, int ACC, bool DEN64>
cudaError_t union_set_smem(int bytes) {
  cudaError_t e = cudaFuncSetAttribute(iterate_union_kernel<NW, kXFull, ACC, DEN64>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(iterate_union_kernel<NW, kXSplit, ACC, DEN64>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(iterate_union_kernel<NW, kXChain, ACC, DEN64>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}
template <int NW>
cudaError_t union_set_smem_mode(int precision, int bytes) {
  switch (precision) {
    case kPrecisionCompensated: return union_set_smem<NW, kAccCompensated, false>(bytes);
    case kPrecisionCompensatedDen64: return union_set_smem<NW, kAccCompensated, true>(bytes);
    case kPrecisionFixed: return union_set_smem<NW, kAccFixed, false>(bytes);
    default: return union_set_smem<NW, kAccFloat, false>(bytes);
  }
}

template <int NW, int ACC, bool DEN64>
void union_launch(int xm, int n_chunks, size_t smem, cudaStream_t s, const DevGeom& g,
                  const FastConst& fc, const Tiling& t, const Chunk* chunks,
                  const float4* ev_geom, const short4* ev_box, const UEvConst* evc,
                  const uint16_t* erows, const uint16_t* urows, const uint32_t* batches,
                  const float* rho, float* out, AuxImage aux, uint32_t seed,
                  DevCounters* counters) {
  auto* k = xm == kXChain   ? iterate_union_kernel<NW, kXChain, ACC, DEN64>
            : xm == kXSplit ? iterate_union_kernel<NW, kXSplit, ACC, DEN64>
                            : iterate_union_kernel<NW, kXFull, ACC, DEN64>;
  k<<<n_chunks, NW * 32, smem, s>>>(g, fc, t, chunks, ev_geom, ev_box, evc, erows, urows, batches,
                                    rho, out, aux, seed, counters);
}

template <int NW>
void union_launch_mode(int precision, int xm, int n_chunks, size_t smem, cudaStream_t s,
                       const DevGeom& g, const FastConst& fc, const Tiling& t,
                       const Chunk* chunks, const float4* ev_geom, const short4* ev_box,
                       const UEvConst* evc, const uint16_t* erows, const uint16_t* urows,
                       const uint32_t* batches, const float* rho, float* out, AuxImage aux,
                       uint32_t seed, DevCounters* counters) {
  switch (precision) {
    case kPrecisionCompensated:
      union_launch<NW, kAccCompensated, false>(xm, n_chunks, smem, s, g, fc, t, chunks, ev_geom,
                                               ev_box, evc, erows, urows, batches, rho, out, aux,
                                               seed, counters);
      break;
    case kPrecisionCompensatedDen64:
      union_launch<NW, kAccCompensated, true>(xm, n_chunks, smem, s, g, fc, t, chunks, ev_geom,
                                              ev_box, evc, erows, urows, batches, rho, out, aux,
                                              seed, counters);
      break;
    case kPrecisionFixed:
      union_launch<NW, kAccFixed, false>(xm, n_chunks, smem, s, g, fc, t, chunks, ev_geom,
                                         ev_box, evc, erows, urows, batches, rho, out, aux,
                                         seed, counters);
      break;
    default:
      union_launch<NW, kAccFloat, false>(xm, n_chunks, smem, s, g, fc, t, chunks, ev_geom,
                                         ev_box, evc, erows, urows, batches, rho, out, aux,
                                         seed, counters);
      break;
  }
}
}  // namespace

cudaError_t union_prepare_kernel(const Tiling& t, int precision) {
  const int bytes = static_cast<int>(union_smem_bytes(t, precision));
  return t.threads == 256 ? union_set_smem_mode<8>(precision, bytes)
                          : union_set_smem_mode<4>(precision, bytes);
}

cudaError_t launch_union_setup(const DevGeom& g, const FastConst& fc, const Tiling& t,
                               Chunk* chunks, int32_t n_chunks, int32_t n_events,
                               const float4* ev_geom, const short4* ev_box, const uint16_t* rows,
                               void* ev_const, uint32_t* batches, uint16_t* urows,
                               uint16_t* erows, cudaStream_t s) {
  if (n_events <= 0) return cudaSuccess;
  if (t.threads != 128 && t.threads != 256) return cudaErrorInvalidValue;
  union_events_kernel<<<(n_events + 255) / 256, 256, 0, s>>>(
      g, fc, t, n_events, ev_geom, ev_box, static_cast<UEvConst*>(ev_const));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || n_chunks <= 0) return e;
  const size_t words = static_cast<size_t>(n_events) * kURows * sizeof(uint16_t);
  e = cudaMemsetAsync(urows, 0, words, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(erows, 0, words, s);
  if (e != cudaSuccess) return e;
  int blocks = (n_chunks + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  union_batches_kernel<<<blocks, 256, 0, s>>>(chunks, n_chunks, t.threads / 32, ev_box, rows,
                                              t.row_stride, batches, urows, erows);
  return cudaGetLastError();
}

size_t union_row_words() { return kURows; }

cudaError_t launch_iterate_union(const DevGeom& g, const FastConst& fc, const Tiling& t,
                                 const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                                 const short4* ev_box, const void* ev_const,
                                 const uint16_t* erows, const uint16_t* urows,
                                 const uint32_t* batches, const float* rho, float* out,
                                 AuxImage aux, DevCounters* counters, int precision,
                                 uint32_t seed, cudaStream_t s) {
  if (n_chunks <= 0) return cudaSuccess;
  if (t.chunk_events > kUMaxChunk || (t.threads != 128 && t.threads != 256) ||
      (precision == kPrecisionFixed && t.chunk_events > kUMaxChunkFixed))
    return cudaErrorInvalidValue;
  const int xm = union_chain_exponent(g, fc) ? kXChain
                 : union_split_exponent(g, fc) ? kXSplit
                                               : kXFull;
  const auto* evc = static_cast<const UEvConst*>(ev_const);
  const size_t smem = union_smem_bytes(t, precision);
  if (t.threads == 256)
    union_launch_mode<8>(precision, xm, n_chunks, smem, s, g, fc, t, chunks, ev_geom, ev_box, evc,
                         erows, urows, batches, rho, out, aux, seed, counters);
  else
    union_launch_mode<4>(precision, xm, n_chunks, smem, s, g, fc, t, chunks, ev_geom, ev_box, evc,
                         erows, urows, batches, rho, out, aux, seed, counters);
  return cudaGetLastError();
}

}  // namespace jpet
