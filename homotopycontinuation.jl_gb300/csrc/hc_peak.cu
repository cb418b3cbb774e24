// hc_peak.cu — FP64 / FP32 CUDA-core FMA throughput microbenchmark. The path tracker is
// bound by these pipes (no tensor cores on this path), so its roofline denominator is
// measured here on the running GPU. No counterpart in the reference.
#include <cuda_runtime.h>

#include "../../include/hcgpu.h"

namespace {

template <class T>
__global__ void __launch_bounds__(256) fma_chain(T* out, int iters, T b, T c) {
  T a0 = (T)threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a0 = fma(a0, b, c);
      a1 = fma(a1, b, c);
      a2 = fma(a2, b, c);
      a3 = fma(a3, b, c);
      a4 = fma(a4, b, c);
      a5 = fma(a5, b, c);
      a6 = fma(a6, b, c);
      a7 = fma(a7, b, c);
    }
  }
  T s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == (T)-1.2345) out[blockIdx.x] = s;  // keeps the chains alive
}

template <class T>
double run(int iters, int reps) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * sms * 8) != cudaSuccess) return -1;
  int blocks = sms * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chain<T><<<blocks, threads>>>(out, iters / 10 + 1, (T)0.9999999, (T)1e-7);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0);
    fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.9999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  double flops = 2.0 * 32.0 * (double)iters * blocks * threads;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace

extern "C" int hc_fma_peak(double* fp64_tflops, double* fp32_tflops) {
  if (!fp64_tflops || !fp32_tflops) return HC_ERR_INVALID_ARG;
  *fp64_tflops = run<double>(2000, 5);
  *fp32_tflops = run<float>(40000, 5);
  cudaError_t e = cudaGetLastError();
  return (e == cudaSuccess && *fp64_tflops > 0 && *fp32_tflops > 0) ? HC_OK : HC_ERR_CUDA;
}
