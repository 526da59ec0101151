// bench_fp_peak: measures the FP64 and FP32 fused multiply-add throughput of the current
// GPU (the ALU roof of the FP64 solver kernels).  Eight independent FMA chains per thread,
// 8 blocks of 256 threads per SM, timed with CUDA events after a warm-up launch.
// Prints one JSON object: {"fp64_tflops": ..., "fp32_tflops": ..., "sms": ..., "name": ...}.
#include <cstdio>
#include <cuda_runtime.h>

template <typename T>
__global__ void fma_chains(T *out, T a, T b, int iters) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
static double tflops(int blocks, int iters) {
  T *o = nullptr;
  if (cudaMalloc(&o, (size_t)blocks * 256 * sizeof(T)) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<blocks, 256>>>(o, (T)0.999, (T)1e-4, iters);
  cudaEventRecord(e0);
  fma_chains<T><<<blocks, 256>>>(o, (T)0.999, (T)1e-4, iters);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(o);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  return 2.0 * 8 * (double)iters * blocks * 256 / (ms * 1e-3) / 1e12;
}

int main() {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
    std::printf("{\"error\": \"no CUDA device\"}\n");
    return 1;
  }
  const int blocks = p.multiProcessorCount * 8;
  const double f64 = tflops<double>(blocks, 1 << 14);
  const double f32 = tflops<float>(blocks, 1 << 16);
  std::printf("{\"fp64_tflops\": %.4f, \"fp32_tflops\": %.4f, \"sms\": %d, \"name\": \"%s\"}\n", f64, f32,
              p.multiProcessorCount, p.name);
  return (f64 > 0 && f32 > 0) ? 0 : 1;
}
