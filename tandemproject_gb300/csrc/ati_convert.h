// ati_convert.h — FP32 -> FP64 conversion on the integer pipes.
//
// On GB300 the FP64 pipe does 1/55 of the FP32 work per clock and also executes
// the F2F conversion instructions, so the mixed path's RK update and filter,
// which add FP32 increments to the FP64 state, spend much of their time there.
// widen() does the exact conversion with integer and bit operations, straight
// from the IEEE-754 binary32/binary64 layouts; zero is handled, and subnormals,
// infinities and NaNs fall back to the instruction.  It gives the instruction's
// result bit for bit (checked on the device by ati_check_conversions).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

namespace ati {

// float -> double, exact: re-bias the exponent (127 -> 1023) and pad the significand
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu, s = u & 0x80000000u;
  if (e - 1u < 254u) return __hiloint2double((int)(s | ((e + 896u) << 20) | (m >> 3)), (int)(m << 29));
  if ((u << 1) == 0u) return __hiloint2double((int)s, 0);  // signed zero
  return (double)f;  // subnormal, infinity, NaN
}

// double -> float, rounded to nearest even, for results in the normal float range:
// the significand's top 23 bits plus a rounding increment decided by the 29 bits
// dropped (above half, or exactly half with an odd result); a carry out of the
// significand moves into the exponent, as the rounding requires (up to infinity).
// Zero, results below the normal range, overflow, infinities and NaNs fall back
// to the instruction.  Bit for bit the instruction's result (checked on the device
// by ati_check_conversions).
__device__ __forceinline__ float narrow(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 254u) {  // float exponent e - 896 in 1..254
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29), r = lo & 0x1fffffffu;
    const unsigned f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
    return __uint_as_float(f + (unsigned)((r > 0x10000000u) | ((r == 0x10000000u) & (m & 1u))));
  }
  return (float)d;
}

// 1/a and 1/sqrt(a) for the FP64 fast build, for positive normal a: the
// hardware approximations (PTX rcp.approx.ftz.f64, rsqrt.approx.ftz.f64) refined
// by two Newton-Raphson steps each, x' = x + x (1 - a x) and
// y' = y + y (1 - a y^2) / 2, each of which squares the relative error.  The
// results are within a few ulp of the correctly rounded ones (the bound is
// checked against the division and the square root on the device by
// ati_check_recip); they take about half the FP64 operations of the IEEE
// division and square root.
__device__ __forceinline__ double recip_nr(double a) {
  double x;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(x) : "d"(a));
  double e = fma(-a, x, 1.0);
  x = fma(x, e, x);
  e = fma(-a, x, 1.0);
  return fma(x, e, x);
}
__device__ __forceinline__ double rsqrt_nr(double a) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
#pragma unroll
  for (int it = 0; it < 2; it++) {
    const double e = fma(-(a * y), y, 1.0);
    y = fma(y, 0.5 * e, y);
  }
  return y;
}

// conversion between the engine types: FP32 -> FP64 on the integer pipes.  The
// other direction stays with the conversion instruction here: rounding takes some
// 15 integer operations and branches, slower in the line sweeps' load loops than
// the FP64 pipe it would spare (measured on the mixed filter sweeps), and in the
// register-bounded flux kernel (297 -> 346 us); the primitives kernel, bound by
// the FP64 pipe, calls narrow() itself (142 -> 133 us)
template <typename TO, typename TI>
__device__ __forceinline__ TO cvt(TI v) {
  if constexpr (std::is_same<TO, TI>::value) return v;
  else if constexpr (std::is_same<TO, double>::value && std::is_same<TI, float>::value) return widen(v);
  else return (TO)v;
}

}  // namespace ati
