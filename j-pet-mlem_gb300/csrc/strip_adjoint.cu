// Adjoint of the list-mode Poisson likelihood of the strip MLEM model.
//
//   L(rho, sigma) = sum_p s_p rho_p - sum_e log( sum_{p in E_e} K_e(p; sigma) rho_p )
//   dL/drho_p     = s_p - sum_e K_e(p) / den_e
//   dL/dsigma     = - sum_e ( sum_p dK_e(p)/dsigma rho_p ) / den_e
//
// K is the reference's Gaussian kernel (src/2d/strip/gaussian_kernel.h:51-79)
// with its normalisation c0 = 1/(2 pi^2) ipz sqrt(ipd) included, so that
// d log K / d ipz = 1/ipz - Pa/(2 aMa) - u^2 and
// d log K / d ipd = 1/(2 ipd) - Qa/(2 aMa) - 2 sec^2 dy^2, with aMa = Pa ipz + Qa ipd,
// Pa = 2 sec^4 (py^2 + R^2), Qa = 4 sec^2 tan^2 py^2, u = dz - dy tan.  The support
// E_e is the event's 3-sigma ellipse for the handle's sigmas (the row tables),
// held fixed while the kernel sigmas vary.  There is no reference code for this
// path.
//
// The loss has to be a smooth function of sigma to the ~1e-9 relative level for
// central differences with h = 1e-3 mm to resolve it: every sigma-dependent
// constant is rounded differently at sigma +- h, and a float rounding of, e.g.,
// ipd shifts log K of every pixel in the same direction.  So the kernel value
// uses the accurate exp2f (not the .approx form of the MLEM kernel), the row
// prefactor -log2(aMa(py)/aMa(y))/2 - 2 log2(e) ipd sec^2 dy^2 is computed in
// FP64 from FP64 constants, the per-pixel coefficient kz = -log2(e) ipz is
// applied as a float pair (kz + kz_lo), and the event constant
// log(c0 / sqrt(aMa(y))) enters the loss in FP64.
//
// One warp per event; each row's exact in-ellipse interval is found with the
// same search as the MLEM row tables (row_interval), so the support is exactly
// the reference's.  The rows' constants are set up 32 at a time, one row per
// lane, and broadcast to the warp for the row's pixels; the constants of the
// first 128 rows are kept in registers for the second (gradient) pass.  For the
// events of the tiled chunks the rho window and a
// gradient window live in shared memory (as in the MLEM kernel); events whose
// box exceeds the windows use the global image.  Per-event log-likelihood and
// sigma-derivative terms are reduced in FP64 per CTA.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "strip_device.cuh"
#include "strip_internal.h"
#include "strip_raster.cuh"

namespace jpet {
namespace {

constexpr double kNllLog2e = 1.4426950408889634;

struct NllWindow {
  const float* rho;
  float* grad;
  int ox, oy, pitch;
  __device__ __forceinline__ int index(int y, int x) const { return (y - oy) * pitch + (x - ox); }
};

// One event on one warp: forward sums (den, d den / d sigma) and, if den > 0,
// the gradient contributions -K / den; returns the per-event terms on lane 0.
template <class Win>
__device__ __forceinline__ void nll_event(const DevGeom& g, const NllConst& k, float4 ev,
                                          short4 box, const Win& wv, double& loss, double& gz,
                                          double& gdl, unsigned long long& skipped) {
  const int lane = threadIdx.x & 31;
  const float z = ev.x, y = ev.y, tn = ev.z, sec = ev.w;
  float A, B, C;
  ellipse_abc(g, tn, sec, A, B, C);
  const float sec2 = sec * sec;
  const float pa_c = 2.0f * sec2 * sec2;     // Pa = pa_c (py^2 + R^2)
  const float qa_c = 4.0f * sec2 * tn * tn;  // Qa = qa_c py^2
  const double ama_ref_d =
      (static_cast<double>(pa_c) * (static_cast<double>(y) * y +
                                    static_cast<double>(g.radius) * g.radius)) * k.ipz_d +
      static_cast<double>(qa_c) * y * y * k.ipd_d;
  // aMa(py) / aMa(y) = 1 + qq (py - y)(py + y)
  const double qq = (pa_c * k.ipz_d + qa_c * k.ipd_d) / ama_ref_d;
  const double kdl_sec2 = k.kdl_d * sec2;
  const int nrows = box.w - box.y;
  float den = 0.0f, dz = 0.0f, ddl = 0.0f, inv = 0.0f;
  // lane l sets up row rb + l: exact interval and FP64 row term
  struct RowConst {
    int first, w;
    float arg, cz, cdl, u;
  };
  auto setup = [&](int rb) {
    RowConst c{0, 0, 0.0f, 0.0f, 0.0f, 0.0f};
    const int ri = rb + lane;
    if (ri < nrows) {
      const int iy = box.y + ri;
      c.w = row_interval(g, A, B, C, z, y, tn, sec, box.x, box.z, iy, c.first);
      const float py = g.tl_y_half_h - static_cast<float>(iy) * g.pixel_height;
      const float dy = py - y;
      const float pa = pa_c * (py * py + g.radius * g.radius), qa = qa_c * py * py;
      const float ama = pa * k.ipz + qa * k.ipd;
      const double dyd = dy;
      c.arg = static_cast<float>(-0.5 * kNllLog2e * log1p(qq * dyd * (static_cast<double>(py) + y)) +
                                 kdl_sec2 * dyd * dyd);
      c.cz = k.inv_ipz - 0.5f * pa / ama;
      c.cdl = k.half_inv_ipd - 0.5f * qa / ama - 2.0f * sec2 * dy * dy;
      c.u = g.tl_z_half_w - z - dy * tn;
    }
    return c;
  };
  // the warp sweeps the group's rows one by one with the constants broadcast
  // from their lanes: forward sums (pass 0) or gradient contributions (pass 1)
  auto sweep = [&](int pass, int rb, const RowConst& c) {
    const int n_group = min(32, nrows - rb);
    for (int r = 0; r < n_group; ++r) {
      const int wr = __shfl_sync(kFull, c.w, r);
      if (wr == 0) continue;
      const int fr = __shfl_sync(kFull, c.first, r);
      const float ra = __shfl_sync(kFull, c.arg, r);
      const float czr = __shfl_sync(kFull, c.cz, r);
      const float cdr = __shfl_sync(kFull, c.cdl, r);
      const float ur = __shfl_sync(kFull, c.u, r);
      const int iy = box.y + rb + r;
      for (int j = lane; j < wr; j += 32) {
        const int col = fr + j;
        const float u = fmaf(static_cast<float>(col), g.pixel_width, ur);
        const float kv = exp2f(fmaf(k.kz * u, u, fmaf(k.kz_lo * u, u, ra)));
        const int wi = wv.index(iy, col);
        if (pass == 0) {
          const float kr = kv * wv.rho[wi];
          den += kr;
          dz += kr * (czr - u * u);
          ddl += kr * cdr;
        } else {
          atomicAdd(&wv.grad[wi], -kv * inv);
        }
      }
    }
  };
  // the constants of up to kCachedGroups x 32 rows stay in registers between
  // the two passes; taller boxes set their rows up again in the second pass
  constexpr int kCachedGroups = 4;
  RowConst cache[kCachedGroups];
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      dz *= k.dipz_dsz;
      ddl *= k.dipd_dsdl;
      double dd = den, dzz = dz, ddd = ddl;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dd += __shfl_xor_sync(kFull, dd, o);
        dzz += __shfl_xor_sync(kFull, dzz, o);
        ddd += __shfl_xor_sync(kFull, ddd, o);
      }
      if (!(dd > 0.0)) {
        if (lane == 0) ++skipped;
        return;
      }
      if (lane == 0) {
        // log of the absolute denominator: K = K_ref K', K_ref = c0 / sqrt(aMa(y))
        loss -= log(dd) + k.log_c0 - 0.5 * log(ama_ref_d);
        gz -= dzz / dd;
        gdl -= ddd / dd;
      }
      inv = static_cast<float>(1.0 / dd);
    }
#pragma unroll 1
    for (int rb = 0; rb < nrows; rb += 32) {
      const int gi = rb >> 5;
      RowConst c;
      if (gi >= kCachedGroups || pass == 0) {
        c = setup(rb);
        if (gi < kCachedGroups) cache[gi] = c;
      } else {
        c = cache[gi];
      }
      sweep(pass, rb, c);
    }
  }
}

__device__ __forceinline__ void nll_block_reduce(double loss, double gz, double gdl,
                                                 unsigned long long sk, double* s_acc,
                                                 double* acc, unsigned long long* skipped) {
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_acc[0], loss);
    atomicAdd(&s_acc[1], gz);
    atomicAdd(&s_acc[2], gdl);
    if (sk) atomicAdd(skipped, sk);
  }
  __syncthreads();
  if (threadIdx.x < 3) atomicAdd(&acc[threadIdx.x], s_acc[threadIdx.x]);
}

__global__ void __launch_bounds__(256) nll_grad_tiles_kernel(
    DevGeom g, NllConst k, Tiling t, const Chunk* __restrict__ chunks,
    const float4* __restrict__ ev_geom, const short4* __restrict__ ev_box,
    const float* __restrict__ rho, float* __restrict__ grad, double* __restrict__ acc,
    unsigned long long* skipped) {
  extern __shared__ __align__(16) float smem[];
  const int pitch = t.win_w;
  const int win = t.win_w * t.win_h;
  float* w_rho = smem;
  float* w_grad = smem + win;
  __shared__ double s_acc[3];
  const Chunk c = chunks[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  if (threadIdx.x < 3) s_acc[threadIdx.x] = 0.0;
  for (int r = warp; r < t.win_h; r += n_warps) {
    const int gy = c.oy + r;
    for (int col = lane; col < pitch; col += 32) {
      const int gx = c.ox + col;
      w_rho[r * pitch + col] = (gy < g.n_y && gx < g.n_z) ? rho[gy * g.n_z + gx] : 0.0f;
      w_grad[r * pitch + col] = 0.0f;
    }
  }
  __syncthreads();
  NllWindow wv{w_rho, w_grad, c.ox, c.oy, pitch};
  double loss = 0.0, gz = 0.0, gdl = 0.0;
  unsigned long long sk = 0;
  for (int e = warp; e < c.count; e += n_warps)
    nll_event(g, k, ev_geom[c.start + e], ev_box[c.start + e], wv, loss, gz, gdl, sk);
  nll_block_reduce(loss, gz, gdl, sk, s_acc, acc, skipped);
  for (int r = warp; r < t.win_h; r += n_warps) {
    const int gy = c.oy + r;
    for (int col = lane; col < pitch; col += 32) {
      const int gx = c.ox + col;
      const float v = w_grad[r * pitch + col];
      if (v != 0.0f && gy < g.n_y && gx < g.n_z) atomicAdd(&grad[gy * g.n_z + gx], v);
    }
  }
}

__global__ void __launch_bounds__(256) nll_grad_global_kernel(
    DevGeom g, NllConst k, int32_t n, const float4* __restrict__ ev_geom,
    const short4* __restrict__ ev_box, const float* __restrict__ rho, float* __restrict__ grad,
    double* __restrict__ acc, unsigned long long* skipped) {
  __shared__ double s_acc[3];
  if (threadIdx.x < 3) s_acc[threadIdx.x] = 0.0;
  __syncthreads();
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  NllWindow wv{rho, grad, 0, 0, g.n_z};
  double loss = 0.0, gz = 0.0, gdl = 0.0;
  unsigned long long sk = 0;
  for (int e = warp; e < n; e += n_warps) nll_event(g, k, ev_geom[e], ev_box[e], wv, loss, gz, gdl, sk);
  nll_block_reduce(loss, gz, gdl, sk, s_acc, acc, skipped);
}

// grad += s; acc[0] += sum s * rho
__global__ void nll_finish_kernel(const float* __restrict__ s, const float* __restrict__ rho,
                                  float* __restrict__ grad, double* acc, int64_t n) {
  __shared__ double part[8];
  double v = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    v += static_cast<double>(s[i]) * rho[i];
    if (grad) grad[i] += s[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) t += part[w];
    atomicAdd(&acc[0], t);
  }
}

}  // namespace

NllConst make_nll_const(double sigma_z, double sigma_dl) {
  NllConst k;
  const double ipz = 1.0 / (sigma_z * sigma_z), ipd = 1.0 / (sigma_dl * sigma_dl);
  k.ipz = static_cast<float>(ipz);
  k.ipd = static_cast<float>(ipd);
  k.kz = static_cast<float>(-kNllLog2e * ipz);
  k.kz_lo = static_cast<float>(-kNllLog2e * ipz - static_cast<double>(k.kz));
  k.ipz_d = ipz;
  k.ipd_d = ipd;
  k.kdl_d = -2.0 * kNllLog2e * ipd;
  k.inv_ipz = static_cast<float>(1.0 / ipz);
  k.half_inv_ipd = static_cast<float>(0.5 / ipd);
  k.dipz_dsz = static_cast<float>(-2.0 / (sigma_z * sigma_z * sigma_z));
  k.dipd_dsdl = static_cast<float>(-2.0 / (sigma_dl * sigma_dl * sigma_dl));
  k.log_c0 = std::log(1.0 / (2.0 * 3.14159265358979323846 * 3.14159265358979323846) * ipz *
                      std::sqrt(ipd));
  return k;
}

cudaError_t launch_nll_grad(const DevGeom& g, const NllConst& k, const Tiling& t,
                            const Chunk* chunks, int32_t n_chunks, const float4* ev_geom,
                            const short4* ev_box, int32_t n_over, const float4* over_geom,
                            const short4* over_box, const float* rho, float* grad, double* acc,
                            unsigned long long* skipped, cudaStream_t s) {
  if (n_chunks > 0) {
    const size_t smem = 2ull * t.win_w * t.win_h * sizeof(float);
    cudaError_t err = cudaFuncSetAttribute(nll_grad_tiles_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem));
    if (err != cudaSuccess) return err;
    nll_grad_tiles_kernel<<<n_chunks, 256, smem, s>>>(g, k, t, chunks, ev_geom, ev_box, rho, grad,
                                                      acc, skipped);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
  }
  if (n_over > 0) {
    int blocks = (n_over + 7) / 8;
    if (blocks > 4096) blocks = 4096;
    nll_grad_global_kernel<<<blocks, 256, 0, s>>>(g, k, n_over, over_geom, over_box, rho, grad,
                                                   acc, skipped);
  }
  return cudaGetLastError();
}

cudaError_t launch_nll_finish(const float* sens, const float* rho, float* grad, double* acc,
                              int64_t n, cudaStream_t s) {
  nll_finish_kernel<<<152 * 4, 256, 0, s>>>(sens, rho, grad, acc, n);
  return cudaGetLastError();
}

}  // namespace jpet
