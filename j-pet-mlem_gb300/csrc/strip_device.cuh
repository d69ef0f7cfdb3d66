// Device-side geometry and kernel arithmetic of the 2D strip-PET MLEM.
//
// The per-event set-up (response -> tan/y/z, 3-sigma ellipse and its pixel box)
// is evaluated with explicitly rounded intrinsics (__fadd_rn, __fmul_rn,
// __fdiv_rn, __fsqrt_rn) in the reference's own operation order, so that no FMA
// contraction changes a result: the box of every event is then the box the
// reference's CPU float path computes (src/2d/strip/reconstruction.h:220-246).
#pragma once

#include <cstdint>

#include "strip_internal.h"

namespace jpet {

// x86-64 conversion semantics of the reference build for float -> short
// (src/2d/strip/scanner.h:142-144 stores float into Pixel<short>): the value is
// truncated to int32 (out-of-range and NaN give INT32_MIN) and the low 16 bits
// are kept.  Only absurd inputs (|value| >= 2^31 or NaN) reach the special case.
__device__ __forceinline__ int16_t ref_float_to_short(float v) {
  int32_t i = (v > -2147483648.0f && v < 2147483648.0f) ? __float2int_rz(v)
                                                        : INT32_MIN;
  return static_cast<int16_t>(static_cast<uint32_t>(i) & 0xffffu);
}

__device__ __forceinline__ int32_t ref_float_to_int(float v) {
  return (v > -2147483648.0f && v < 2147483648.0f) ? __float2int_rz(v) : INT32_MIN;
}

__device__ __forceinline__ int16_t short_clamp(int16_t v, int16_t lo, int16_t hi) {
  // compat::min(br, compat::max(tl, v)) with std::min/max (src/2d/geometry/pixel.h:51-54)
  int16_t m = (lo < v) ? v : lo;
  return (m < hi) ? m : hi;
}

// Per-event quantities that do not change between iterations.
struct EventSetup {
  float z, y, tan, sec;
  float A, B, C;
  int16_t tl_x, tl_y, br_x, br_y;
};

// Response::calculate_tan_y_z (src/2d/strip/response.h:22-37) followed by
// GaussianKernel::ellipse_bb (src/2d/strip/gaussian_kernel.h:108-128), the
// centre pixel (scanner.h:142-144), n_pixels_in_line (reconstruction.h:216-218)
// and the clamp of both box corners (reconstruction.h:237-246).
__device__ __forceinline__ EventSetup event_setup(const DevGeom& g, float z_u, float z_d,
                                                  float dl) {
  EventSetup e;
  float t = __fdiv_rn(__fsub_rn(z_u, z_d), __fmul_rn(2.0f, g.radius));
  float ts = __fadd_rn(1.0f, __fmul_rn(t, t));
  float y = __fmul_rn(-0.5f, __fdiv_rn(dl, __fsqrt_rn(ts)));
  float z = __fmul_rn(0.5f, __fadd_rn(__fadd_rn(z_u, z_d), __fmul_rn(__fmul_rn(2.0f, y), t)));
  float tan_sq = __fmul_rn(t, t);
  float sec = __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(t, t)));
  float A = __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(4.0f, sec), sec), g.ipd),
                      __fmul_rn(__fmul_rn(2.0f, tan_sq), g.ipz));
  float B = __fmul_rn(__fmul_rn(-4.0f, t), g.ipz);
  float C = __fmul_rn(2.0f, g.ipz);
  float hb = __fdiv_rn(B, 2.0f);
  float B_2 = __fmul_rn(hb, hb);
  float bb_y = __fdiv_rn(3.0f, __fsqrt_rn(__fsub_rn(A, __fdiv_rn(B_2, C))));
  float bb_z = __fdiv_rn(3.0f, __fsqrt_rn(__fsub_rn(C, __fdiv_rn(B_2, A))));
  int16_t cx = ref_float_to_short(__fdiv_rn(__fsub_rn(z, g.tl_z), g.pixel_width));
  int16_t cy = ref_float_to_short(__fdiv_rn(__fsub_rn(g.tl_y, y), g.pixel_height));
  int32_t half_w = ref_float_to_int(__fadd_rn(__fdiv_rn(bb_z, g.pixel_width), 0.5f));
  int32_t half_h = ref_float_to_int(__fadd_rn(__fdiv_rn(bb_y, g.pixel_height), 0.5f));
  // int arithmetic wraps like the reference's short(int) narrowing
  int16_t tlx = static_cast<int16_t>(static_cast<uint32_t>(cx) - static_cast<uint32_t>(half_w));
  int16_t tly = static_cast<int16_t>(static_cast<uint32_t>(cy) - static_cast<uint32_t>(half_h));
  int16_t brx = static_cast<int16_t>(static_cast<uint32_t>(cx) + static_cast<uint32_t>(half_w));
  int16_t bry = static_cast<int16_t>(static_cast<uint32_t>(cy) + static_cast<uint32_t>(half_h));
  int16_t mx = static_cast<int16_t>(g.n_z - 1), my = static_cast<int16_t>(g.n_y - 1);
  e.z = z;
  e.y = y;
  e.tan = t;
  e.sec = sec;
  e.A = A;
  e.B = B;
  e.C = C;
  e.tl_x = short_clamp(tlx, 0, mx);
  e.tl_y = short_clamp(tly, 0, my);
  e.br_x = short_clamp(brx, 0, mx);
  e.br_y = short_clamp(bry, 0, my);
  return e;
}

// Recomputes A, B, C of GaussianKernel::ellipse_bb from tan and sec with the
// same rounding as event_setup (used by kernels that only store z, y, tan, sec).
__device__ __forceinline__ void ellipse_abc(const DevGeom& g, float t, float sec, float& A,
                                            float& B, float& C) {
  float tan_sq = __fmul_rn(t, t);
  A = __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn(4.0f, sec), sec), g.ipd),
                __fmul_rn(__fmul_rn(2.0f, tan_sq), g.ipz));
  B = __fmul_rn(__fmul_rn(-4.0f, t), g.ipz);
  C = __fmul_rn(2.0f, g.ipz);
}

// Scanner::pixel_center (scanner.h:136-139).
__device__ __forceinline__ float pixel_center_z(const DevGeom& g, int x) {
  return __fadd_rn(g.tl_z_half_w, __fmul_rn(static_cast<float>(x), g.pixel_width));
}
__device__ __forceinline__ float pixel_center_y(const DevGeom& g, int y) {
  return __fsub_rn(g.tl_y_half_h, __fmul_rn(static_cast<float>(y), g.pixel_height));
}

// GaussianKernel::in_ellipse (gaussian_kernel.h:131-137) in the reference's order.
__device__ __forceinline__ bool in_ellipse(float A, float B, float C, float dy, float dz) {
  float q = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(A, dy), dy), __fmul_rn(__fmul_rn(B, dy), dz)),
                      __fmul_rn(__fmul_rn(C, dz), dz));
  return q <= 9.0f;
}

// GaussianKernel::multiply_inv_cor_mat (gaussian_kernel.h:152-156).
__device__ __forceinline__ float mic(const DevGeom& g, float ap, float aq, float ar, float bp,
                                     float bq, float br) {
  return __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(ap, g.ipz), bp), __fmul_rn(__fmul_rn(aq, g.ipz), bq)),
                   __fmul_rn(__fmul_rn(ar, g.ipd), br));
}

// GaussianKernel::operator()(y, tan, sec, R, distance) (gaussian_kernel.h:51-79),
// reference order; exp by the CUDA math library's expf.
__device__ __forceinline__ float gauss_exact(const DevGeom& g, float y, float t, float sec,
                                             float dz, float dy) {
  float sec_sq = __fmul_rn(sec, sec);
  float yp = __fadd_rn(dy, y);
  float ap = __fmul_rn(-__fsub_rn(yp, g.radius), sec_sq);
  float aq = __fmul_rn(-__fadd_rn(yp, g.radius), sec_sq);
  float ar = __fmul_rn(__fmul_rn(__fmul_rn(-2.0f, yp), sec), t);
  float bpq = __fsub_rn(dz, __fmul_rn(dy, t));
  float br = __fmul_rn(__fmul_rn(-2.0f, dy), sec);
  float a_ic_a = mic(g, ap, aq, ar, ap, aq, ar);
  float b_ic_b = mic(g, bpq, bpq, br, bpq, bpq, br);
  float ebe = __fdiv_rn(g.c0, __fsqrt_rn(a_ic_a));
  return __fmul_rn(ebe, expf(__fmul_rn(-0.5f, b_ic_b)));
}

// AnalyticKernel::operator() (src/2d/strip/analytic_kernel.h:28-62).
__device__ __forceinline__ float analytic_exact(const DevGeom& g, float y, float t, float sec,
                                                float dz, float dy) {
  float sec_sq = __fmul_rn(sec, sec);
  float yp = __fadd_rn(dy, y);
  float ap = __fmul_rn(-__fsub_rn(yp, g.radius), sec_sq);
  float aq = __fmul_rn(-__fadd_rn(yp, g.radius), sec_sq);
  float ar = __fmul_rn(__fmul_rn(__fmul_rn(-2.0f, yp), sec), t);
  float op = __fmul_rn(ap, t);
  float oq = __fmul_rn(aq, t);
  float orr = __fmul_rn(__fmul_rn(-yp, sec),
                        __fadd_rn(1.0f, __fmul_rn(__fmul_rn(2.0f, t), t)));
  float bpq = __fsub_rn(dz, __fmul_rn(dy, t));
  float br = __fmul_rn(__fmul_rn(-2.0f, dy), sec);
  float a_ic_a = mic(g, ap, aq, ar, ap, aq, ar);
  float b_ic_a = mic(g, bpq, bpq, br, ap, aq, ar);
  float b_ic_b = mic(g, bpq, bpq, br, bpq, bpq, br);
  float o_ic_b = mic(g, op, oq, orr, bpq, bpq, br);
  float norm = __fadd_rn(a_ic_a, __fmul_rn(2.0f, o_ic_b));
  float ebe = __fdiv_rn(g.c0, __fsqrt_rn(norm));
  float arg = __fmul_rn(-0.5f, __fsub_rn(b_ic_b, __fdiv_rn(__fmul_rn(b_ic_a, b_ic_a), norm)));
  return __fmul_rn(ebe, expf(arg));
}

// Exact column interval of box row iy whose pixel centres pass the reference's
// 3-sigma test (in_ellipse above, reference rounding).  The test's quadratic is
// convex along the row, so the passing columns form one interval; it is found
// from the analytic endpoints tan*dy +- sqrt((9 - 4 ipd sec^2 dy^2)/(2 ipz)) and
// corrected by evaluating the exact test around them.  Every loop is bounded by
// the box.  Returns the width (0 if no pixel passes) and the first column.
__device__ __forceinline__ int row_interval(const DevGeom& g, float A, float B, float C, float z,
                                            float y, float t, float sec, int bx, int bz, int iy,
                                            int& first) {
  const float dy = __fsub_rn(pixel_center_y(g, iy), y);
  auto pass = [&](int c) { return in_ellipse(A, B, C, dy, __fsub_rn(pixel_center_z(g, c), z)); };
  const float inv_pw = 1.0f / g.pixel_width;
  const float h =
      sqrtf(fmaxf((9.0f - 4.0f * sec * sec * g.ipd * dy * dy) * (0.5f / g.ipz), 0.0f)) * inv_pw;
  const float xc = (z + t * dy - g.tl_z_half_w) * inv_pw;
  const float fbx = static_cast<float>(bx), fbz = static_cast<float>(bz - 1);
  first = bx;
  if (bz <= bx) return 0;
  // the column nearest the minimum of the convex test quadratic
  int cs = static_cast<int>(fminf(fmaxf(rintf(xc), fbx), fbz));
  bool any = pass(cs);
  if (!any && cs - 1 >= bx && pass(cs - 1)) {
    cs -= 1;
    any = true;
  }
  if (!any && cs + 1 < bz && pass(cs + 1)) {
    cs += 1;
    any = true;
  }
  if (!any) return 0;
  int lo = static_cast<int>(fminf(fmaxf(ceilf(xc - h), fbx), static_cast<float>(cs)));
  if (pass(lo)) {
    while (lo > bx && pass(lo - 1)) --lo;
  } else {
    while (lo < cs && !pass(lo)) ++lo;
  }
  int hi = static_cast<int>(fminf(fmaxf(floorf(xc + h), static_cast<float>(cs)), fbz));
  if (pass(hi)) {
    while (hi < bz - 1 && pass(hi + 1)) ++hi;
  } else {
    while (hi > cs && !pass(hi)) --hi;
  }
  first = lo;
  return hi - lo + 1;
}

// Scanner::sensitivity (scanner.h:147-171), float.
__device__ __forceinline__ float scanner_sensitivity(const DevGeom& g, float px, float py) {
  float half = g.half_length;
  float L_plus = __fadd_rn(half, px);
  float L_minus = __fsub_rn(half, px);
  float R_plus = __fadd_rn(g.radius, py);
  float R_minus = __fsub_rn(g.radius, py);
  if (R_plus <= 0.0f) R_plus = 1.0f;
  if (R_minus <= 0.0f) R_minus = 1.0f;
  float a1 = __fdiv_rn(L_minus, R_minus), a2 = __fdiv_rn(L_plus, R_plus);
  float mn = (a2 < a1) ? a2 : a1;
  float b1 = __fdiv_rn(-L_plus, R_minus), b2 = __fdiv_rn(-L_minus, R_plus);
  float mx = (b1 < b2) ? b2 : b1;
  return __fmul_rn(static_cast<float>(0.31830988618379067154), __fsub_rn(atanf(mn), atanf(mx)));
}

}  // namespace jpet
