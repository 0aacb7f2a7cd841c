// peaks.cu -- microbenchmarks of the non-tensor FP32/FP64 FMA rates and the
// HBM copy bandwidth, the denominators of the pair kernels' rooflines.
#include "launch.h"
#include <cstdio>

namespace coordgpu {

template <typename T>
__global__ void k_fma_chain(T *out, int iters, T a, T b) {
  // 8 independent chains per thread hide the FMA latency
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      x0 = x0 * a + b;
      x1 = x1 * a + b;
      x2 = x2 * a + b;
      x3 = x3 * a + b;
      x4 = x4 * a + b;
      x5 = x5 * a + b;
      x6 = x6 * a + b;
      x7 = x7 * a + b;
    }
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-1.2345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains alive
}

__global__ void k_copy(const float4 *__restrict__ src, float4 *__restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

template <typename T> static double fma_rate(int nsm, cudaStream_t s, T *out) {
  const int blocks = nsm * 8, threads = 256, iters = (sizeof(T) == 8) ? 64 : 2048;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chain<T><<<blocks, threads, 0, s>>>(out, iters / 8, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0, s);
  k_fma_chain<T><<<blocks, threads, 0, s>>>(out, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g_launches += 2;
  const double flops = 2.0 * blocks * threads * (double)iters * 16 * 8;
  return flops / (ms * 1e-3) / 1e12;
}

int measure_peaks(int device, double *fp32, double *fp64, double *hbm) {
  if (cudaSetDevice(device) != cudaSuccess) return 2;
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  void *out = nullptr;
  if (cudaMalloc(&out, (size_t)prop.multiProcessorCount * 8 * 256 * sizeof(double)) != cudaSuccess) return 5;
  if (fp32) *fp32 = fma_rate<float>(prop.multiProcessorCount, s, (float *)out);
  if (fp64) *fp64 = fma_rate<double>(prop.multiProcessorCount, s, (double *)out);
  cudaFree(out);
  if (hbm) {
    const size_t bytes = (size_t)1 << 31;  // 2 GiB each way, far above L2
    void *a = nullptr, *b = nullptr;
    if (cudaMalloc(&a, bytes) != cudaSuccess) return 5;
    if (cudaMalloc(&b, bytes) != cudaSuccess) {
      cudaFree(a);
      return 5;
    }
    cudaMemsetAsync(a, 0, bytes, s);
    const size_t n = bytes / sizeof(float4);
    const int blocks = prop.multiProcessorCount * 8;
    k_copy<<<blocks, 256, 0, s>>>((const float4 *)a, (float4 *)b, n);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
      cudaEventRecord(e0, s);
      k_copy<<<blocks, 256, 0, s>>>((const float4 *)a, (float4 *)b, n);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = ms < best ? ms : best;
    }
    g_launches += 6;
    *hbm = 2.0 * bytes / (best * 1e-3) / 1e9;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
  }
  cudaStreamDestroy(s);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

} // namespace coordgpu
