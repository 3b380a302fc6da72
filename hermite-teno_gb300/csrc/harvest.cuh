// Training data for the learned stencil classifier, recorded by the plain FP64 solver: for a
// sampled subset of (face, characteristic field, side) the 6-cell characteristic stencil the
// reconstruction sees, normalised to (u - mean) / (max - min + 1e-30), and the three TENO
// cut-off bits the plain solver decides on it (cutOff, Schemes_Lagrange.cpp:1141-1149, through
// the bit-reproducible decision of parity_math.cuh).  The right-biased side is recorded as the
// mirrored stencil, whose left-biased decision is the right side's (bits mirrored).
// Included by FP64 translation units compiled with --fmad=false, after parity_math.cuh.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace hteno {
namespace harvest {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// Deterministic Bernoulli(p) draw for item `id` of a harvest with seed `seed`.
__device__ __forceinline__ bool keep(uint64_t seed, uint64_t id, double p) {
  return double(mix64(seed ^ mix64(id)) >> 11) * 0x1.0p-53 < p;
}

// Cut-off bits of the left-biased side of stencil w[0..5] (teno5, or teno5i when improved).
__device__ __forceinline__ int label(const double* w, bool improved) {
  double SI[3];
  par::lagrange_si(w, SI);
  double tau;
  if (!improved) {
    tau = fabs(par::lagrange_b35(w) - (SI[0] + SI[2] + 4.0 * SI[1]) / 6.0);
  } else {
    tau = SI[0];
    tau = (tau < SI[1]) ? SI[1] : tau;
    tau = (tau < SI[2]) ? SI[2] : tau;
  }
  return par::cutoff_pattern(SI, tau, HTENO_LAG_EPSZ, HTENO_LAG_CT);
}

// A stencil whose six values are equal once rounded to float is "flat": the float
// reconstruction of the mixed path sees a constant, for which plain TENO keeps all three
// candidates, so it takes the linear weights without asking the network (losslessly).  The
// plain FP64 solver's cut-off bits on such stencils are set by rounding noise (~1e-16 relative
// differences left by the flux evaluation in constant regions), so they are not recorded.
__device__ __forceinline__ bool flat_in_float(const double* w) {
  const float f0 = __double2float_rn(w[0]);
#pragma unroll
  for (int k = 1; k < 6; ++k)
    if (__double2float_rn(w[k]) != f0) return false;
  return true;
}

// Appends (normalised stencil as BF16 [8], label) unless the buffer is full; `count` keeps
// counting past the capacity so the caller sees how many were offered.  Normalised values are
// clamped to [-1, 1] (the bound in exact arithmetic).
__device__ __forceinline__ void emit(const double* w, int lab, uint16_t* X, uint8_t* Y, long cap,
                                     unsigned long long* count) {
  double mean = 0.0, mx = w[0], mn = w[0];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    mean += w[k];
    mx = fmax(mx, w[k]);
    mn = fmin(mn, w[k]);
  }
  mean /= 6.0;
  if (flat_in_float(w) || !(mx - mn >= 0.0)) return;  // flat, or NaN
  const double inv = 1.0 / (mx - mn + 1e-30);
  const unsigned long long slot = atomicAdd(count, 1ull);
  if (slot >= (unsigned long long)cap) return;
  uint16_t bits[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const __nv_bfloat16 b =
        __float2bfloat16_rn(k < 6 ? float(fmin(1.0, fmax(-1.0, (w[k] - mean) * inv))) : 0.0f);
    bits[k] = *reinterpret_cast<const uint16_t*>(&b);
  }
  uint4 packed;
  packed.x = bits[0] | (uint32_t(bits[1]) << 16);
  packed.y = bits[2] | (uint32_t(bits[3]) << 16);
  packed.z = bits[4] | (uint32_t(bits[5]) << 16);
  packed.w = 0u;
  *reinterpret_cast<uint4*>(X + slot * 8) = packed;
  Y[slot] = uint8_t(lab);
}

// Both sides of one characteristic stencil u[0..5] (left: u itself; right: reversed).
__device__ __forceinline__ void emit_both(const double* u, bool improved, uint64_t seed, uint64_t id,
                                          double p, uint16_t* X, uint8_t* Y, long cap,
                                          unsigned long long* count) {
  if (keep(seed, 2 * id, p)) emit(u, label(u, improved), X, Y, cap, count);
  if (keep(seed, 2 * id + 1, p)) {
    const double r[6] = {u[5], u[4], u[3], u[2], u[1], u[0]};
    emit(r, label(r, improved), X, Y, cap, count);
  }
}

}  // namespace harvest
}  // namespace hteno
