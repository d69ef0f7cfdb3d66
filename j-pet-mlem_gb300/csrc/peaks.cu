// Throughput microbenchmarks for the roofline of the strip MLEM kernel.
//
// The MLEM iteration is bound by the special-function unit (one exp per
// kernel-pixel evaluation), FP32 issue and shared-memory atomics; a copy
// bandwidth or a GEMM rate says nothing about those units.  These kernels
// measure them on the device the bench runs on:
//   ex2     ex2.approx.ftz.f32 results per second (MUFU; the form the kernels use)
//   ffma    fused multiply-adds per second (FP32 pipe)
//   atoms   shared-memory float atomicAdd per second (distinct lanes' addresses)
//   red     global float atomicAdd per second to an L2-resident buffer
// Each is the best of several launches of a grid of 8 CTAs per SM.
// Built as its own library (lib/libjpet_peaks.so); used by bench.py only.
#include <cuda_runtime.h>

#include <cstdio>

namespace {

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void ex2_kernel(float* out, int iters) {
  float a0 = 0.1f + threadIdx.x * 1e-6f, a1 = a0 + 0.01f, a2 = a0 + 0.02f, a3 = a0 + 0.03f;
  float a4 = a0 + 0.04f, a5 = a0 + 0.05f, a6 = a0 + 0.06f, a7 = a0 + 0.07f;
  for (int i = 0; i < iters; ++i) {
    a0 = ex2_approx(-a0);
    a1 = ex2_approx(-a1);
    a2 = ex2_approx(-a2);
    a3 = ex2_approx(-a3);
    a4 = ex2_approx(-a4);
    a5 = ex2_approx(-a5);
    a6 = ex2_approx(-a6);
    a7 = ex2_approx(-a7);
  }
  float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.0f) out[threadIdx.x] = s;
}

__global__ void ffma_kernel(float* out, int iters, float b, float c) {
  float a0 = threadIdx.x * 1e-6f, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  float a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a0 = fmaf(a0, b, c);
      a1 = fmaf(a1, b, c);
      a2 = fmaf(a2, b, c);
      a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c);
      a5 = fmaf(a5, b, c);
      a6 = fmaf(a6, b, c);
      a7 = fmaf(a7, b, c);
    }
  }
  float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.0f) out[threadIdx.x] = s;
}

__global__ void atoms_kernel(float* out, int iters) {
  __shared__ float sm[1024];
  sm[threadIdx.x] = 0.0f;
  __syncthreads();
  // four independent words per thread, each warp instruction conflict-free
  float* p = &sm[threadIdx.x & 255];
  for (int i = 0; i < iters; ++i) {
    atomicAdd(p, 1.0f);
    atomicAdd(p + 256, 1.0f);
    atomicAdd(p + 512, 1.0f);
    atomicAdd(p + 768, 1.0f);
  }
  __syncthreads();
  if (sm[threadIdx.x] == -1.0f) out[threadIdx.x] = sm[threadIdx.x];
}

__global__ void atoms_u32_kernel(unsigned* out, int iters) {
  __shared__ unsigned sm[1024];
  sm[threadIdx.x] = 0u;
  __syncthreads();
  unsigned* p = &sm[threadIdx.x & 255];
  for (int i = 0; i < iters; ++i) {
    atomicAdd(p, 3u);
    atomicAdd(p + 256, 3u);
    atomicAdd(p + 512, 3u);
    atomicAdd(p + 768, 3u);
  }
  __syncthreads();
  if (sm[threadIdx.x] == 1u) out[threadIdx.x] = sm[threadIdx.x];
}

__global__ void atoms_u64_kernel(unsigned long long* out, int iters) {
  __shared__ unsigned long long sm[512];
  if (threadIdx.x < 512) sm[threadIdx.x] = 0ull;
  __syncthreads();
  unsigned long long* p = &sm[threadIdx.x & 127];
  for (int i = 0; i < iters; ++i) {
    atomicAdd(p, 3ull);
    atomicAdd(p + 128, 3ull);
    atomicAdd(p + 256, 3ull);
    atomicAdd(p + 384, 3ull);
  }
  __syncthreads();
  if (threadIdx.x < 512 && sm[threadIdx.x] == 1ull) out[threadIdx.x] = sm[threadIdx.x];
}

// plain read-modify-write of a private shared word (LDS + FADD + STS)
__global__ void rmw_kernel(float* out, int iters) {
  __shared__ float sm[1024];
  sm[threadIdx.x] = 0.0f;
  __syncthreads();
  volatile float* p = &sm[threadIdx.x & 255];
  for (int i = 0; i < iters; ++i) {
    p[0] = p[0] + 1.0f;
    p[256] = p[256] + 1.0f;
    p[512] = p[512] + 1.0f;
    p[768] = p[768] + 1.0f;
  }
  __syncthreads();
  if (sm[threadIdx.x] == -1.0f) out[threadIdx.x] = sm[threadIdx.x];
}

__global__ void red_kernel(float* buf, int iters, int mask) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x);
  for (int i = 0; i < iters; ++i) {
    atomicAdd(&buf[(t + i * 4096) & mask], 1.0f);
  }
}

// global vector atomics (sm_90+): red.global.add.v4.f32 / v2.f32
__global__ void red_v4_kernel(float4* buf, int iters, int mask4) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x);
  const float4 one = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
  for (int i = 0; i < iters; ++i) atomicAdd(&buf[(t + i * 4096) & mask4], one);
}

__global__ void red_v2_kernel(float2* buf, int iters, int mask2) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x);
  const float2 one = make_float2(1.0f, 1.0f);
  for (int i = 0; i < iters; ++i) atomicAdd(&buf[(t + i * 4096) & mask2], one);
}

// conflict-free ld.shared.v2 throughput (elements per second)
__global__ void lds64_kernel(float* out, int iters) {
  __shared__ float2 sm[1024];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) sm[i] = make_float2(i, i);
  __syncthreads();
  float2 acc = make_float2(0.f, 0.f);
  int k = threadIdx.x;
  for (int i = 0; i < iters; ++i) {
    const float2 a = sm[(k + 0) & 1023], b = sm[(k + 256) & 1023], c = sm[(k + 512) & 1023],
                 d = sm[(k + 768) & 1023];
    acc.x += a.x + b.x + c.x + d.x;
    acc.y += a.y + b.y + c.y + d.y;
    k += 32;
  }
  if (acc.x == -1.0f) out[threadIdx.x] = acc.y;
}

template <class F>
double best_rate(F launch, double ops, int reps) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 0;
  launch();  // warm-up
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(a);
    launch();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (ms > 0) best = ops / (ms * 1e-3) > best ? ops / (ms * 1e-3) : best;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

}  // namespace

extern "C" {

// out[0] ex2/s, out[1] ffma/s, out[2] shared float atomics/s, out[3] global
// float atomics/s, out[4] number of SMs, out[5] SM clock (kHz, device
// attribute), out[6] shared u32 atomics/s, out[7] shared u64 atomics/s,
// out[8] plain shared read-modify-writes/s, out[9] global float4 atomics
// (floats/s), out[10] global float2 atomics (floats/s), out[11] conflict-free
// ld.shared.v2 (floats/s).  Returns 0 or a CUDA error code.
int jpet_peaks_measure(int device, double* out) {
  if (cudaSetDevice(device) != cudaSuccess) return 1;
  int sms = 0, clk = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, device);
  float* buf = nullptr;
  const int mask = (1 << 22) - 1;  // 16 MiB: resident in L2
  if (cudaMalloc(&buf, (mask + 1) * sizeof(float)) != cudaSuccess) return 2;
  cudaMemset(buf, 0, (mask + 1) * sizeof(float));
  const int blocks = sms * 8, threads = 256;
  const int it_ex2 = 4096, it_fma = 4096, it_ats = 2048, it_red = 512;
  out[0] = best_rate([&] { ex2_kernel<<<blocks, threads>>>(buf, it_ex2); },
                     double(blocks) * threads * it_ex2 * 8, 5);
  out[1] = best_rate([&] { ffma_kernel<<<blocks, threads>>>(buf, it_fma, 0.999f, 1e-3f); },
                     double(blocks) * threads * it_fma * 32, 5);
  out[2] = best_rate([&] { atoms_kernel<<<blocks, threads>>>(buf, it_ats); },
                     double(blocks) * threads * it_ats * 4, 5);
  out[3] = best_rate([&] { red_kernel<<<blocks, threads>>>(buf, it_red, mask); },
                     double(blocks) * threads * it_red, 5);
  out[4] = sms;
  out[5] = clk;
  out[6] = best_rate([&] { atoms_u32_kernel<<<blocks, threads>>>(reinterpret_cast<unsigned*>(buf),
                                                                 it_ats); },
                     double(blocks) * threads * it_ats * 4, 5);
  out[7] = best_rate([&] { atoms_u64_kernel<<<blocks, threads>>>(
                               reinterpret_cast<unsigned long long*>(buf), it_ats); },
                     double(blocks) * threads * it_ats * 4, 5);
  out[8] = best_rate([&] { rmw_kernel<<<blocks, threads>>>(buf, it_ats); },
                     double(blocks) * threads * it_ats * 4, 5);
  out[9] = best_rate([&] { red_v4_kernel<<<blocks, threads>>>(reinterpret_cast<float4*>(buf),
                                                              it_red, (mask + 1) / 4 - 1); },
                     double(blocks) * threads * it_red * 4, 5);
  out[10] = best_rate([&] { red_v2_kernel<<<blocks, threads>>>(reinterpret_cast<float2*>(buf),
                                                               it_red, (mask + 1) / 2 - 1); },
                      double(blocks) * threads * it_red * 2, 5);
  out[11] = best_rate([&] { lds64_kernel<<<blocks, threads>>>(buf, it_ats); },
                      double(blocks) * threads * it_ats * 8, 5);
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(buf);
  return e == cudaSuccess ? 0 : static_cast<int>(e);
}

}  // extern "C"
