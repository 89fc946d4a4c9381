// peak.cu -- FP64 / FP32 fused-multiply-add throughput of this GPU.
//
// The energetic-particle kernels are bound by floating-point issue, not by
// HBM, so their roofline denominator is the ALU peak.  This measures it the
// plain way: every thread runs eight independent FMA chains; the result is
// 2 flops per FMA over the CUDA-event time of the launch.
#include <cuda_runtime.h>

#include "../../include/eprem_gpu.h"

namespace {
template <typename T>
__global__ void k_fma_chains(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)12345.678) out[0] = s;  // keeps the chains live; never true
}

template <typename T>
int measure(int iters, double *tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return EPREM_GPU_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return EPREM_GPU_ERR_CUDA;
  T *d = nullptr;
  if (cudaMalloc(&d, 64) != cudaSuccess) return EPREM_GPU_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 4, threads = 256;
  k_fma_chains<T><<<blocks, threads>>>(d, iters / 10 + 1, (T)0.999, (T)0.001);
  cudaEventRecord(e0);
  k_fma_chains<T><<<blocks, threads>>>(d, iters, (T)0.999, (T)0.001);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess || ms <= 0.f) return EPREM_GPU_ERR_CUDA;
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return EPREM_GPU_OK;
}
}  // namespace

extern "C" int eprem_gpu_alu_peak(int precision, double *tflops) {
  if (!tflops) return EPREM_GPU_ERR_ARG;
  return precision == EPREM_FP64 ? measure<double>(2000, tflops) : measure<float>(20000, tflops);
}
