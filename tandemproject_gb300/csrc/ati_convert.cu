// ati_convert.cu — device check of the integer-pipe FP32 -> FP64 conversion
// against the conversion instruction, over bit patterns that cover every
// exponent (normal, subnormal, zero, infinity, NaN).
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/ati.h"
#include "ati_convert.h"

void ati_set_thread_error(const char *msg);

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_check_conv(int64_t n, unsigned long long *bad) {
  unsigned long long nb = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r = mix64((uint64_t)i * 0x9E3779B97F4A7C15ull + 1);
    // any pattern, or a zero / subnormal / infinity / NaN exponent with random sign and significand
    unsigned fb = (unsigned)(r >> 17);
    if ((i & 3) == 3) fb = (fb & 0x807FFFFFu) | ((r & 1) ? 0x7F800000u : 0u);
    if ((i & 15) == 15) fb &= 0x80000000u;  // signed zeros
    const float f = __uint_as_float(fb);
    const double wa = ati::widen(f), wb = (double)f;
    if (!((wa != wa && wb != wb) || __double_as_longlong(wa) == __double_as_longlong(wb))) nb++;
  }
  if (nb) atomicAdd(bad, nb);
}

}  // namespace

extern "C" int ati_check_conversions(int64_t n, int64_t *mismatches) {
  if (n < 0 || !mismatches) {
    ati_set_thread_error("ati_check_conversions: bad argument");
    return ATI_EINVAL;
  }
  unsigned long long *d = nullptr, h = 0;
  cudaError_t e = cudaMalloc(&d, sizeof(*d));
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(*d));
  if (e == cudaSuccess && n > 0) {
    k_check_conv<<<1024, 256>>>(n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    ati_set_thread_error((std::string("ati_check_conversions: ") + cudaGetErrorString(e)).c_str());
    return ATI_ECUDA;
  }
  *mismatches = (int64_t)h;
  return ATI_OK;
}
