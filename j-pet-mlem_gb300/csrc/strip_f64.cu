// The reference iteration at double on the GPU: PET2D::Strip::Reconstruction
// <double, GaussianKernel<double>> (src/2d/strip/reconstruction.h:108-154,
// bb_update :220-298), the instantiation the reference's own tests use
// (kernel_test.cpp:33).  It is the FP64 yardstick of the accuracy studies at
// event counts the CPU cannot iterate: every event's set-up, box, 3-sigma test,
// kernel value, denominator and back-projection in double, one warp per event,
// lanes over the box pixels in row-major order, double atomics into the image.
// Only the summation order differs from the reference template, which at double
// is far below any float effect.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>

#include "../../include/jpet_strip.h"
#include "strip_internal.h"

namespace jpet {
namespace {

struct GeomD {
  double radius, tl_y, tl_z, tl_y_half_h, tl_z_half_w, pw, ph, ipz, ipd, c0;
  int16_t n_y, n_z;
};

// float/double -> int as the x86-64 reference build converts (cvttsd2si):
// out of range and NaN give INT32_MIN; -> short keeps the low 16 bits
__device__ __forceinline__ int32_t to_int_d(double v) {
  return (v > -2147483648.0 && v < 2147483648.0) ? static_cast<int32_t>(v) : INT32_MIN;
}
__device__ __forceinline__ int16_t to_short_d(double v) {
  return static_cast<int16_t>(static_cast<uint16_t>(static_cast<uint32_t>(to_int_d(v)) & 0xffffu));
}
__device__ __forceinline__ int16_t wrap16(int32_t v) {
  return static_cast<int16_t>(static_cast<uint16_t>(static_cast<uint32_t>(v) & 0xffffu));
}

__global__ void __launch_bounds__(256) iterate_f64_kernel(GeomD g, const float* __restrict__ aos,
                                                          int64_t n, const double* __restrict__ rho,
                                                          double* __restrict__ out,
                                                          unsigned long long* counts) {
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
  unsigned long long calls = 0, contrib = 0;
  for (int64_t e = warp0; e < n; e += n_warps) {
    const double zu = aos[3 * e], zd = aos[3 * e + 1], dl = aos[3 * e + 2];
    // Response::calculate_tan_y_z (response.h:22-37)
    const double tn = (zu - zd) / (2.0 * g.radius);
    const double y = -0.5 * (dl / sqrt(1.0 + tn * tn));
    const double z = 0.5 * (zu + zd + (2.0 * y * tn));
    // GaussianKernel::ellipse_bb (gaussian_kernel.h:108-128)
    const double sec = sqrt(1.0 + tn * tn);
    const double A = 4.0 * sec * sec * g.ipd + 2.0 * tn * tn * g.ipz;
    const double B = -4.0 * tn * g.ipz;
    const double C = 2.0 * g.ipz;
    const double b2 = (B / 2.0) * (B / 2.0);
    const double bb_y = 3.0 / sqrt(A - (b2 / C));
    const double bb_z = 3.0 / sqrt(C - (b2 / A));
    // box and clamp (reconstruction.h:216-246, scanner.h:142-144, pixel.h:51-54)
    const int16_t cx = to_short_d((z - g.tl_z) / g.pw);
    const int16_t cy = to_short_d((g.tl_y - y) / g.ph);
    const int32_t hw = to_int_d(bb_z / g.pw + 0.5), hh = to_int_d(bb_y / g.ph + 0.5);
    const int16_t mx = static_cast<int16_t>(g.n_z - 1), my = static_cast<int16_t>(g.n_y - 1);
    auto clamp16 = [](int16_t v, int16_t hi) {
      return static_cast<int16_t>(v < 0 ? 0 : (v > hi ? hi : v));
    };
    const int tlx = clamp16(wrap16(static_cast<int32_t>(cx) - hw), mx);
    const int tly = clamp16(wrap16(static_cast<int32_t>(cy) - hh), my);
    const int brx = clamp16(wrap16(static_cast<int32_t>(cx) + hw), mx);
    const int bry = clamp16(wrap16(static_cast<int32_t>(cy) + hh), my);
    const int w = brx > tlx ? brx - tlx : 0;
    const int h = bry > tly ? bry - tly : 0;
    const int npx = w * h;
    // two passes over the box in row-major order (forward sum, back-projection)
    const double sec2 = sec * sec;
    double den = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
      double inv = 0.0;
      if (pass == 1) {
        for (int o = 16; o > 0; o >>= 1) den += __shfl_xor_sync(0xffffffffu, den, o);
        if (!(den > 0.0)) break;  // inv_denominator = 0 (reconstruction.h:290)
        inv = 1.0 / den;
        if (lane == 0) ++contrib;
      }
      for (int k = lane; k < npx; k += 32) {
        const int iy = tly + k / w, iz = tlx + k % w;
        const double px = g.tl_z_half_w + static_cast<int16_t>(iz) * g.pw;
        const double py = g.tl_y_half_h - static_cast<int16_t>(iy) * g.ph;
        const double dy = py - y, dz = px - z;
        if ((A * dy * dy) + (B * dy * dz) + (C * dz * dz) <= 9.0) {
          // GaussianKernel::operator() (gaussian_kernel.h:51-79)
          const double yp = dy + y;
          const double ap = -(yp - g.radius) * sec2, aq = -(yp + g.radius) * sec2;
          const double ar = -2.0 * yp * sec * tn;
          const double bpq = dz - dy * tn, br = -2.0 * dy * sec;
          const double aia = ap * g.ipz * ap + aq * g.ipz * aq + ar * g.ipd * ar;
          const double bib = bpq * g.ipz * bpq + bpq * g.ipz * bpq + br * g.ipd * br;
          const double kv = g.c0 / sqrt(aia) * exp(-0.5 * bib);
          const int pi = iy * g.n_z + iz;
          const double kr = kv * rho[pi];
          if (pass == 0) {
            den += kr;
            ++calls;
          } else {
            atomicAdd(&out[pi], kr * inv);
          }
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) calls += __shfl_xor_sync(0xffffffffu, calls, o);
  if (lane == 0) {
    atomicAdd(&counts[0], calls);
    atomicAdd(&counts[1], contrib);
  }
}

}  // namespace
}  // namespace jpet

using namespace jpet;

extern "C" {

int jpet_strip_reference_fp64(const jpet_strip_geom* geom, const float* d_responses_aos,
                              int64_t n, double* d_rho, double* d_work, int32_t n_iterations,
                              int64_t* kernel_calls, int64_t* contributing, void* cuda_stream) {
  if (!geom || !d_rho || !d_work || n < 0 || (n > 0 && !d_responses_aos) || n_iterations < 0 ||
      geom->n_y_pixels <= 0 || geom->n_z_pixels <= 0 || geom->n_y_pixels > 32767 ||
      geom->n_z_pixels > 32767 || !(geom->pixel_width > 0) || !(geom->pixel_height > 0) ||
      !(geom->sigma_z > 0) || !(geom->sigma_dl > 0) || !(geom->radius > 0)) {
    set_call_error("jpet_strip_reference_fp64: invalid argument");
    return JPET_ERR_ARGUMENT;
  }
  // Scanner<double, short> and GaussianKernel<double> constants (scanner.h:50-67,
  // gaussian_kernel.h:27-33)
  GeomD g;
  g.radius = geom->radius;
  g.n_y = static_cast<int16_t>(geom->n_y_pixels);
  g.n_z = static_cast<int16_t>(geom->n_z_pixels);
  g.pw = geom->pixel_width;
  g.ph = geom->pixel_height;
  const double size_y = g.n_y * g.ph, size_z = g.n_z * g.pw;
  g.tl_y = 0.0 + size_y / 2;
  g.tl_z = 0.0 - size_z / 2;
  g.tl_y_half_h = g.tl_y - g.ph / 2;
  g.tl_z_half_w = g.tl_z + g.pw / 2;
  g.ipz = 1.0 / (geom->sigma_z * geom->sigma_z);
  g.ipd = 1.0 / (geom->sigma_dl * geom->sigma_dl);
  const double kPi = 3.14159265358979323846;
  g.c0 = 1.0 / (2.0 * kPi * kPi) * sqrt(g.ipz * g.ipz * g.ipd);
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const size_t n_pix = static_cast<size_t>(g.n_y) * g.n_z;
  unsigned long long* counts = nullptr;
  unsigned long long h_counts[2] = {0, 0};
  cudaError_t e = cudaMalloc(&counts, 2 * sizeof(unsigned long long));
  double* cur = d_rho;
  double* nxt = d_work;
  for (int it = 0; it < n_iterations && e == cudaSuccess; ++it) {
    e = cudaMemsetAsync(nxt, 0, n_pix * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), s);
    if (e == cudaSuccess && n > 0) {
      iterate_f64_kernel<<<152 * 8, 256, 0, s>>>(g, d_responses_aos, n, cur, nxt, counts);
      e = cudaGetLastError();
    }
    std::swap(cur, nxt);
  }
  // the result goes back to d_rho
  if (e == cudaSuccess && cur != d_rho)
    e = cudaMemcpyAsync(d_rho, cur, n_pix * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_counts, counts, sizeof(h_counts), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(counts);
  if (e != cudaSuccess) {
    set_call_error(std::string("jpet_strip_reference_fp64: ") + cudaGetErrorString(e));
    return JPET_ERR_CUDA;
  }
  if (kernel_calls) *kernel_calls = static_cast<int64_t>(h_counts[0]);
  if (contributing) *contributing = static_cast<int64_t>(h_counts[1]);
  return JPET_OK;
}

}  // extern "C"
