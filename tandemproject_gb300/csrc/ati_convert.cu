// ati_convert.cu — device check of the integer-pipe conversions (FP32 -> FP64
// widening, FP64 -> FP32 rounding) against the conversion instruction, over bit
// patterns that cover every exponent (normal, subnormal, zero, infinity, NaN) and
// the rounding ties; and of the Newton-refined reciprocal and inverse square root
// of the FP64 fast build against the IEEE division and square root.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
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
    // narrowing: random doubles over the whole exponent range, exact ties and near-ties of the dropped 29 bits,
    // the edges of the normal float range, zeros, infinities and NaNs
    const uint64_t r2 = mix64(r ^ 0xD1B54A32D192ED03ull);
    uint64_t db = r2;
    switch (i & 7) {
      case 1: db = (db & ~0x1fffffffull) | 0x10000000ull; break;                  // exact tie
      case 2: db = (db & ~0x1fffffffull) | (0x10000000ull + ((r >> 3) & 1 ? 1 : -1)); break;  // near tie
      case 3: db = (db & 0x800fffffffffffffull) | ((uint64_t)(896 + (r & 3)) << 52); break;    // below / at min normal
      case 4: db = (db & 0x800fffffffffffffull) | ((uint64_t)(1149 + (r & 3)) << 52); break;   // near max / overflow
      case 5: db = (db & 0x800fffffffffffffull) | ((uint64_t)(1023 + (int)(r % 41) - 20) << 52); break;  // O(1)
      case 6: db = (r & 1) ? (db & 0x8000000000000000ull) : ((db & 0x800fffffffffffffull) | 0x7ff0000000000000ull);
              break;                                                                  // zeros, inf, NaN
      default: break;
    }
    const double d = __longlong_as_double((long long)db);
    const float na = ati::narrow(d), nb2 = (float)d;
    if (!((na != na && nb2 != nb2) || __float_as_uint(na) == __float_as_uint(nb2))) nb++;
  }
  if (nb) atomicAdd(bad, nb);
}

// recip_nr / rsqrt_nr against the IEEE division and square root, positive normal arguments over 2^-200..2^200:
// the largest relative differences, as bit patterns of non-negative doubles (ordered like the values)
__global__ void k_check_recip(int64_t n, unsigned long long *worst) {
  double w0 = 0, w1 = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t r = mix64((uint64_t)i * 0x9E3779B97F4A7C15ull + 7);
    const uint64_t ex = 1023 - 200 + (r >> 52) % 401;
    const double a = __longlong_as_double((long long)((ex << 52) | (r & 0xfffffffffffffull)));
    const double x = ati::recip_nr(a), xr = 1.0 / a;
    const double y = ati::rsqrt_nr(a), yr = 1.0 / sqrt(a);
    w0 = fmax(w0, fabs(x - xr) / xr);
    w1 = fmax(w1, fabs(y - yr) / yr);
  }
  atomicMax(&worst[0], (unsigned long long)__double_as_longlong(w0));
  atomicMax(&worst[1], (unsigned long long)__double_as_longlong(w1));
}

}  // namespace

extern "C" int ati_check_recip(int64_t n, double worst[2]) {
  if (n < 0 || !worst) {
    ati_set_thread_error("ati_check_recip: bad argument");
    return ATI_EINVAL;
  }
  unsigned long long *d = nullptr, h[2] = {0, 0};
  cudaError_t e = cudaMalloc(&d, sizeof(h));
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(h));
  if (e == cudaSuccess && n > 0) {
    k_check_recip<<<1024, 256>>>(n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    ati_set_thread_error((std::string("ati_check_recip: ") + cudaGetErrorString(e)).c_str());
    return ATI_ECUDA;
  }
  for (int k = 0; k < 2; k++) {
    const long long b = (long long)h[k];
    double v;
    memcpy(&v, &b, sizeof v);
    worst[k] = v;
  }
  return ATI_OK;
}

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
