// Conversions and the SSP-RK3 stage for the mixed-precision kernels (float reconstruction and
// fluxes, double state).  On GB300 the FP64 pipe, which also executes the hardware float <->
// double conversions, runs at 1/64 of the FP32 rate; these conversions run on the integer pipes.
#pragma once

namespace hteno {
namespace mix {

// Double -> float and float -> double on the integer pipes: the same results as the hardware
// conversions (round to nearest even) for normal numbers, infinities and NaN; subnormal results
// are flushed to signed zero.
__device__ __forceinline__ float d2f(double d) {
  const unsigned hi = unsigned(__double2hiint(d)), lo = unsigned(__double2loint(d));
  const unsigned s = hi & 0x80000000u;
  const unsigned eb = (hi >> 20) & 0x7ffu;
  const int e = int(eb) - 896;  // float biased exponent
  unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;
  m += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
  if (eb == 0x7ffu) return __uint_as_float(s | 0x7f800000u | (((hi & 0xfffffu) | lo) ? 0x400000u : 0u));
  if (e <= 0) return __uint_as_float(s);
  if (e >= 255) return __uint_as_float(s | 0x7f800000u);
  return __uint_as_float(s | ((unsigned(e) << 23) + m));  // a mantissa carry bumps the exponent
}
__device__ __forceinline__ double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e == 0) return __hiloint2double(int(s), 0);
  const unsigned e2 = e == 255u ? 2047u : e + 896u;
  return __hiloint2double(int(s | (e2 << 20) | (m >> 3)), int(m << 29));
}

// SSP-RK3 stage (Schemes_SSPRK.cpp:3-15) in double with fused multiply-adds (the mixed path does
// not need the reference's rounding sequence, only FP64 accumulation).
__device__ __forceinline__ double rk_stage(double q0, double qn, double rhs, double dt, int stage) {
  if (stage == 1) return fma(dt, rhs, q0);
  const double t = fma(dt, rhs, qn);
  if (stage == 2) return fma(0.25, t, 0.75 * q0);
  return fma(2.0 / 3.0, t, q0 * (1.0 / 3.0));
}

}  // namespace mix
}  // namespace hteno
