// ati_probe.cu — FMA throughput probe: the FP64 (and FP32) compute roofline
// denominator of this GPU, measured with independent FMA chains and no memory
// traffic.  Instrumentation only.
#include <cuda_runtime.h>

#include "../../include/ati.h"

namespace {
template <typename T>
__global__ void k_fma_chains(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int run(double *tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ATI_ECUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, tpb = 256, iters = sizeof(T) == 8 ? 2048 : 16384, reps = 5;
  T *d = nullptr;
  if (cudaMalloc(&d, sizeof(T) * blocks * tpb) != cudaSuccess) return ATI_ENOMEM;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fma_chains<T><<<blocks, tpb>>>(d, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(a);
  for (int r = 0; r < reps; r++) k_fma_chains<T><<<blocks, tpb>>>(d, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(b);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  if (e != cudaSuccess) return ATI_ECUDA;
  *tflops = (double)reps * blocks * tpb * (double)iters * 8.0 * 2.0 / (ms * 1e-3) / 1e12;
  return ATI_OK;
}
}  // namespace

extern "C" int ati_probe_fma_tflops(int fp64, double *tflops) {
  if (!tflops) return ATI_EINVAL;
  return fp64 ? run<double>(tflops) : run<float>(tflops);
}
