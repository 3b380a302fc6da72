// Bit-reproducible FP64 numerics of the plain path.
//
// Why: TENO's cut-off is a discontinuous decision.  In the tails of waves the data vary by
// ~1e-10 relative to their magnitude, so a rounding difference in the characteristic values
// (1e-16 absolute) can move a weight across the cut-off; the flip then changes the solution by
// ~1e-10.  Agreement with the reference to 1e-12 over hundreds of steps therefore needs the same
// rounding, not just the same formulas.  Every function here performs exactly the IEEE
// operations, in exactly the order, of the reference's expressions (reductions left to right),
// and this header is only compiled in translation units built with --fmad=false so that no
// multiply-add is fused.  Divisions and square roots are IEEE correctly rounded, as on the CPU.
//
// The one deliberate difference: the TENO cut-off weights (1 + tau/(SI+eps))^6 / sum only select
// one of 8 cut-off patterns, so they are compared in float (the ratios of the weights' bases to
// the largest, from SI + eps and tau scaled into float range, and their sixth powers); when a
// weight lies within a guard band of the threshold (several times the float evaluation's error
// bound), the decision is recomputed with the reference's divisions and pow.  The indicators and
// tau themselves are the reference's bits.  The reconstructed values use the pattern's weights
// from a table built with the reference's own normalisation, so they are bit-identical.
#pragma once

#include "device_math.cuh"
#include "mixed_conv.cuh"
#include "hermite_math.cuh"

namespace hteno {
namespace par {

// Tests on a double's bits, on the integer pipes: the FP64 pipe (1/64 of the FP32 rate on GB300)
// is left to the arithmetic.  Exactly the IEEE predicates: x == 0.0 (either sign), isnan(x).
__device__ __forceinline__ bool zero_bits(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) << 1) == 0ull;
}
__device__ __forceinline__ bool nan_bits(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffull) >
         0x7ff0000000000000ull;
}
__device__ __forceinline__ double catchnan(double x) { return nan_bits(x) ? 1e-15 : x; }

// dot of a 3-vector of coefficients with u[0..2], left to right (Eigen .dot in the reference)
__device__ __forceinline__ double dot3(double c0, double c1, double c2, const double* u) {
  double s = c0 * u[0];
  s = s + c1 * u[1];
  s = s + c2 * u[2];
  return s;
}
__device__ __forceinline__ double dot3v(const double* p, const double* w) {
  double s = p[0] * w[0];
  s = s + p[1] * w[1];
  s = s + p[2] * w[2];
  return s;
}

// Correctly rounded a / b for several numerators over one denominator: y = RN(1/b) once, then per
// numerator q0 = RN(a y), r = a - b q0 (exact, one FMA), q = RN(q0 + r y).  By Markstein's theorem
// (Markstein, IBM J. Res. Dev. 34(1), 1990; Muller et al., Handbook of Floating-Point Arithmetic,
// 2018, Sec. 4.7) q is a / b correctly rounded when y is within half an ulp of 1/b and q0 within
// one ulp of a / b, barring underflow and overflow: 3 FP64 operations per quotient instead of a
// division's ~10.  Operands outside [2^-500, 2^501) in magnitude (zeros, subnormals, infinities,
// NaN) take the division itself, so the theorem's conditions hold wherever the short form is used.
struct Den {
  double b, y;
  bool ok;
};
__device__ __forceinline__ bool mid_range(double x) {
  const unsigned e = (unsigned(__double2hiint(x)) >> 20) & 0x7ffu;
  return e - 523u <= 1000u;  // biased exponent in [523, 1523]
}
__device__ __forceinline__ Den den_of(double b) { return Den{b, __drcp_rn(b), mid_range(b)}; }
__device__ __forceinline__ double quot(double a, const Den& d) {
  if (d.ok && mid_range(a)) {
    const double q0 = a * d.y;
    const double r = fma(-d.b, q0, a);
    return fma(r, d.y, q0);
  }
  return a / d.b;
}
constexpr double kRcp24 = 1.0 / 24.0;  // RN(1/24), RN(1/6), RN(1/5040), folded at compile time
constexpr double kRcp6 = 1.0 / 6.0;
constexpr double kRcp5040 = 1.0 / 5040.0;

// ---- Schemes::Lagrange ----------------------------------------------------------------------

// smoothnessMeasure (Schemes_Lagrange.cpp:1013-1026)
__device__ __forceinline__ void lagrange_si(const double* v, double* SI) {
  double c[3], b[3];
  c[0] = v[2] - 2.0 * v[3] + v[4];
  b[0] = 3.0 * v[2] - 4.0 * v[3] + v[4];
  c[1] = v[1] - 2.0 * v[2] + v[3];
  b[1] = v[1] - v[3];
  c[2] = v[0] - 2.0 * v[1] + v[2];
  b[2] = v[0] - 4.0 * v[1] + 3.0 * v[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) b[k] = b[k] / 2.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) SI[k] = b[k] * b[k] + (13.0 / 12.0) * c[k] * c[k];
}
// fullpointsSmootness (:1029-1034)
__device__ __forceinline__ double lagrange_b35(const double* v) {
  double r = v[4] * (6908.0 * v[4] - 51001.0 * v[3] + 67923.0 * v[2] - 38947.0 * v[1] +
                     8209.0 * v[0]) +
             v[3] * (104963.0 * v[3] - 299076.0 * v[2] + 179098.0 * v[1] - 38947.0 * v[0]) +
             v[2] * (231153.0 * v[2] - 299076.0 * v[1] + 67923.0 * v[0]) +
             v[1] * (104963.0 * v[1] - 51001.0 * v[0]) + 6908.0 * v[0] * v[0];
  return quot(r, Den{5040.0, kRcp5040, true});  // r / 5040
}

// 1/x to a relative 2^-45 for the cut-off decision only (never for a value that is kept): a
// float reciprocal of x's significand (rcp.approx.ftz.f32, on the MUFU pipe), rescaled by x's
// exponent on the integer pipes, and one Newton step in double (2 FMAs instead of the ~10 FP64
// operations of a correctly rounded reciprocal).  Exponents near the ends of the range, zeros,
// infinities and NaN take the correctly rounded reciprocal.
__device__ __forceinline__ double decision_rcp(double x) {
  const unsigned hx = unsigned(__double2hiint(x)), lx = unsigned(__double2loint(x));
  const unsigned ex = (hx >> 20) & 0x7ffu;
  if (ex - 64u > 1916u) return __drcp_rn(x);
  const float m = __uint_as_float(0x3f800000u | ((hx & 0xfffffu) << 3) | (lx >> 29));
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(m));
  const unsigned r = __float_as_uint(rf), er = (r >> 23) & 0xffu, mr = r & 0x7fffffu;
  const unsigned hy = (hx & 0x80000000u) | ((er + 2046u - 127u - ex) << 20) | (mr >> 3);
  const double y = __hiloint2double(int(hy), int(mr << 29));
  return fma(y, fma(-x, y, 1.0), y);
}

// Largest r whose sixth power is finite with margin (pow(2e51, 6) = 6.4e306): beyond it the
// reference's weights overflow to inf and its normalised weights are NaN.
constexpr double kPow6Max = 2e51;

// The fast part of a cut-off decision, in float, from the ratios x_k = r_k / r_max (in (0, 1],
// or NaN): a_k = x_k^6, kept where a_k >= ct * (a_0 + a_1 + a_2).  Any a_k farther than `band` of
// the limit from it is decided as exact arithmetic decides it (the callers' error bounds are a
// fraction of the band); nearer ones set *near and the caller takes the reference's own
// arithmetic.  NaN ratios compare false, as in double.  (The FP64 pipe runs at 1/64 of the float
// rate on GB300.)
__device__ __forceinline__ int cutoff_core(const float* x, float ct, float band, bool* near) {
  float a[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float x2 = x[k] * x[k];
    a[k] = (x2 * x2) * x2;
  }
  const float lim = ct * ((a[0] + a[1]) + a[2]);
  int pat = 0;
  bool nr = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    pat |= (a[k] < lim ? 0 : 1) << k;
    nr |= fabsf(a[k] - lim) <= band * lim;
  }
  *near = nr;
  return pat;
}
// ... from double ratios (converted on the integer pipes): the float chain's relative error is
// below 1e-6 (x_k to 2^-24, six roundings in a_k, two in the sum), well inside a band of 1e-5.
__device__ __forceinline__ int cutoff_fast(const double* x, double ct, bool* near) {
  const float xf[3] = {mix::d2f(x[0]), mix::d2f(x[1]), mix::d2f(x[2])};
  return cutoff_core(xf, float(ct), 1e-5f, near);
}

// The ratios x_k = r_k / r_max of r_k = 1 + tau / d_k in float, without reciprocals or r_k's
// range: with d_min = min d_k, x_k = (d_min / d_k) (d_k + tau) / (d_min + tau).  The four doubles
// are first scaled by one power of two (exponent bits, on the integer pipes) so that the largest
// lies in [1, 2).  Relative error of x_k below 2^-19.7 (four inputs rounded to float, two
// __fdividef quotients of 2 ulp and three roundings), so of a_k below 7.4e-6.  False when a value
// is NaN, infinite, subnormal or more than 2^125 below the largest (the caller takes the double
// path).  d_k > 0 and tau >= 0 here; within 2^125 every r_k <= 1 + 2^126 < kPow6Max, so the
// reference's weights are finite.
__device__ __forceinline__ bool scaled_ratios(const double* d, double tau, float* x) {
  const double v[4] = {d[0], d[1], d[2], tau};
  int hi[4];
  unsigned lo[4], e[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    hi[i] = __double2hiint(v[i]);
    lo[i] = unsigned(__double2loint(v[i]));
    e[i] = (unsigned(hi[i]) >> 20) & 0x7ffu;
  }
  const unsigned em = max(max(e[0], e[1]), max(e[2], e[3]));
  // (the callers' indicators are sums of squares and tau an absolute value or a maximum of them;
  // a sign bit, even of -0, sends the decision to the double path all the same)
  if (em == 0x7ffu || (hi[0] | hi[1] | hi[2] | hi[3]) < 0) return false;
  float f[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i == 3 && ((unsigned(hi[3]) << 1) | lo[3]) == 0u) {
      f[3] = 0.0f;  // tau = 0: every r_k is 1
    } else {
      if (e[i] == 0u || e[i] + 125u < em) return false;
      // scaled exponent e - em + 1023 in [898, 1023]: a normal float in [2^-125, 2)
      f[i] = mix::d2f(__hiloint2double(hi[i] - (int(em) - 1023) * (1 << 20), int(lo[i])));
    }
  }
  const float dmin = fminf(fminf(f[0], f[1]), f[2]);
#pragma unroll
  for (int k = 0; k < 3; ++k)
    x[k] = __fdividef(dmin, f[k]) * __fdividef(f[k] + f[3], dmin + f[3]);
  return true;
}

// Cut-off pattern of the reference's cutOff() (:1141-1149) given SI and tau.  Fast path: the
// ratios in float from d_k = SI_k + epsz and tau (scaled_ratios, guard band 2^-13 relative, eight
// times its error bound), or in double where the scaling cannot reach (guard band 1e-5); inside
// the band the reference's arithmetic decides.
__device__ __forceinline__ int cutoff_pattern(const double* SI, double tau, double epsz, double ct) {
  const double d[3] = {SI[0] + epsz, SI[1] + epsz, SI[2] + epsz};
  float xf[3];
  bool near;
  int pat;
  if (scaled_ratios(d, tau, xf)) {
    pat = cutoff_core(xf, float(ct), 0x1p-13f, &near);
  } else {
    double r[3], x[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = 1.0 + tau * decision_rcp(d[k]);
    const double rm = fmax(fmax(r[0], r[1]), r[2]);
    const double inv = decision_rcp(rm);
#pragma unroll
    for (int k = 0; k < 3; ++k) x[k] = r[k] * inv;
    pat = cutoff_fast(x, ct, &near);
    // where pow(r, 6) overflows the reference's weights are inf / inf = NaN (a kept candidate):
    // its own arithmetic decides
    near = near || !(rm < kPow6Max);
  }
  if (near) {  // reference arithmetic: w_k = pow(1 + tau/(SI_k + epsz), 6) / sum
    double w[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) w[k] = pow(1.0 + tau / (SI[k] + epsz), 6.0);
    const double s = (w[0] + w[1]) + w[2];
    pat = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) pat |= ((w[k] / s) < ct ? 0 : 1) << k;
  }
  return pat;
}

// The cut-off pattern of one side of teno5 (:481-511) / teno5i (:1235-1263) for the window v with
// indicators SI (bit k set: candidate k kept).
__device__ __forceinline__ int teno_decide(const double* v, const double* SI, bool improved) {
  // All three indicators exactly zero (constant data): the three ratios 1 + tau/(0 + epsz) are
  // equal whatever tau is, and the cut-off keeps all candidates (pattern 7) -- decided without
  // tau, same bits.  (Equal values alone do not suffice: 3u - 4u + u can leave a rounding
  // residue in one indicator.)
  // The full arithmetic below gives pattern 7 on such a window too (three equal ratios), so the
  // shortcut is taken only when every active lane of the warp can take it: a warp never runs both.
  if (zero_bits(SI[0]) && zero_bits(SI[1]) && zero_bits(SI[2])) return 7;
  double tau;
  if (!improved) {
    const double b35 = lagrange_b35(v);
    tau = fabs(b35 - quot(SI[0] + SI[2] + 4.0 * SI[1], Den{6.0, kRcp6, true}));  // ... / 6.0
  } else {
    tau = SI[0];
    tau = (tau < SI[1]) ? SI[1] : tau;
    tau = (tau < SI[2]) ? SI[2] : tau;
  }
  return cutoff_pattern(SI, tau, HTENO_LAG_EPSZ, HTENO_LAG_CT);
}

// One side of teno5 / teno5i given the candidates p and stencil v.
__device__ __forceinline__ double teno_side_si(const DevConst& C, const double* p, const double* v,
                                               const double* SI, int side, bool improved) {
  const int pat = teno_decide(v, SI, improved);
  const double* w = side ? C.wtab_p[pat] : C.wtab_m[pat];
  return catchnan(dot3v(p, w));
}
__device__ __forceinline__ double teno_side(const DevConst& C, const double* p, const double* v,
                                            int side, bool improved) {
  double SI[3];
  lagrange_si(v, SI);
  return teno_side_si(C, p, v, SI, side, improved);
}

// ---- the selectable alternatives (Schemes_Lagrange.cpp:358-594, 1265-1294), one side each ----

// Cut-off pattern from the exact ratios r_k, whose sixth powers are the reference's raw weights:
// fast path on (r_k / r_max)^6 with a guard band, the reference's pow-and-divide inside it.
__device__ __forceinline__ int cutoff_from_r(const double* r, double ct) {
  const double rm = fmax(fmax(r[0], r[1]), r[2]);
  const double inv = __drcp_rn(rm);
  double x[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) x[k] = r[k] * inv;
  bool near;
  int pat = cutoff_fast(x, ct, &near);
  if (near || !(rm < kPow6Max)) {  // the reference's arithmetic (also where pow(r, 6) overflows)
    double w[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) w[k] = pow(r[k], 6.0);
    const double s = (w[0] + w[1]) + w[2];
    pat = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) pat |= ((w[k] / s) < ct ? 0 : 1) << k;
  }
  return pat;
}

__device__ __forceinline__ double normalised(const double* p, double* w) {
  const double s = (w[0] + w[1]) + w[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  return catchnan(dot3v(p, w));
}

// weno5N / teno5N indicators (:445-450) on the side's window v[0..4]; returns the 5-point
// difference |v0 - 4v1 + 6v2 - 4v3 + v4|
__device__ __forceinline__ double n_indicators(const double* v, double* SI) {
  SI[2] = 0.1 * fabs(v[0] - 3.0 * v[1] + 2.0 * v[2]) + fabs(v[0] - 2.0 * v[1] + v[2]);
  SI[1] = 0.1 * fabs(v[3] - v[2]) + fabs(v[1] - 2.0 * v[2] + v[3]);
  SI[0] = 0.1 * fabs(v[3] - v[2]) + fabs(v[2] - 2.0 * v[3] + v[4]);
  return fabs(v[0] - 4.0 * v[1] + 6.0 * v[2] - 4.0 * v[3] + v[4]);
}

// kind 3 weno5JS, 4 weno5Z, 5 weno5N, 6 teno5N, 7 teno5a
__device__ __forceinline__ double alt_side(const DevConst& C, int kind, const double* p,
                                           const double* v, int side) {
  const double* d = side ? C.dkp : C.dkm;
  double SI[3], w[3];
  if (kind == 3 || kind == 4 || kind == 7) lagrange_si(v, SI);
  if (kind == 3) {  // w_k = d_k / (eps + SI_k)^2
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double e = HTENO_LAG_EPS + SI[k];
      w[k] = d[k] / (e * e);
    }
    return normalised(p, w);
  }
  if (kind == 4) {  // tau = |SI_2 - SI_0|, w_k = d_k (1 + tau / (SI_k + epsz))
    const double tau = fabs(SI[2] - SI[0]);
#pragma unroll
    for (int k = 0; k < 3; ++k) w[k] = d[k] * (1.0 + (tau / (SI[k] + HTENO_LAG_EPSZ)));
    return normalised(p, w);
  }
  if (kind == 5) {  // tau = |5-point difference|^2.5, w_k = d_k (1 + tau / (SI_k + eps)^2)
    const double tau = pow(n_indicators(v, SI), 2.5);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double e = SI[k] + HTENO_LAG_EPS;
      w[k] = d[k] * (1.0 + (tau / (e * e)));
    }
    return normalised(p, w);
  }
  double r[3];
  if (kind == 6) {  // r_k = 1 + tau / (SI_k + eps)^2, tau = |5-point difference|^2
    const double x = n_indicators(v, SI);
    const double tau = x * x;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double e = SI[k] + HTENO_LAG_EPS;
      r[k] = 1.0 + tau / (e * e);
    }
  } else {  // teno5a: r_k = 1 / (SI_k + epsz)
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = 1.0 / (SI[k] + HTENO_LAG_EPSZ);
  }
  const int pat = cutoff_from_r(r, HTENO_LAG_CT);
  const double* tw = side ? C.wtab_p[pat] : C.wtab_m[pat];
  return catchnan(dot3v(p, tw));
}

// kind 0 teno5, 1 teno5i, 2 linear (:1219-1233), 3..7 the alternatives above
__device__ __forceinline__ void lagrange_recon(const DevConst& C, int kind, const double* u,
                                               double& outm, double& outp) {
  double p[3];
  p[0] = dot3(C.crj[0][1], C.crj[1][1], C.crj[2][1], u + 2);
  p[1] = dot3(C.crj[0][2], C.crj[1][2], C.crj[2][2], u + 1);
  p[2] = dot3(C.crj[0][3], C.crj[1][3], C.crj[2][3], u + 0);
  if (kind <= 1) {
    // teno5 / teno5i: the two sides' windows overlap in 5 cells, so the + side reuses two of the
    // - side's candidates (p1+ = p0-, p2+ = p1-) and two of its indicator terms: the same
    // expressions on the same operands, the same bits
    double c[4], SIm[3], SIp[3];
    c[0] = u[2] - 2.0 * u[3] + u[4];
    c[1] = u[1] - 2.0 * u[2] + u[3];
    c[2] = u[0] - 2.0 * u[1] + u[2];
    c[3] = u[3] - 2.0 * u[4] + u[5];  // c0 of the + side
    double t[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) t[k] = (13.0 / 12.0) * c[k] * c[k];
    double bm[3], bp[3];
    bm[0] = (3.0 * u[2] - 4.0 * u[3] + u[4]) / 2.0;
    bm[1] = (u[1] - u[3]) / 2.0;
    bm[2] = (u[0] - 4.0 * u[1] + 3.0 * u[2]) / 2.0;
    bp[0] = (3.0 * u[3] - 4.0 * u[4] + u[5]) / 2.0;
    bp[1] = (u[2] - u[4]) / 2.0;
    bp[2] = (u[1] - 4.0 * u[2] + 3.0 * u[3]) / 2.0;
    SIm[0] = bm[0] * bm[0] + t[0];
    SIm[1] = bm[1] * bm[1] + t[1];
    SIm[2] = bm[2] * bm[2] + t[2];
    SIp[0] = bp[0] * bp[0] + t[3];
    SIp[1] = bp[1] * bp[1] + t[0];
    SIp[2] = bp[2] * bp[2] + t[1];
    outm = teno_side_si(C, p, u, SIm, 0, kind == 1);
    double pp[3];
    pp[0] = dot3(C.crj[0][0], C.crj[1][0], C.crj[2][0], u + 3);
    pp[1] = p[0];
    pp[2] = p[1];
    outp = teno_side_si(C, pp, u + 1, SIp, 1, kind == 1);
    return;
  }
  outm = kind == 2 ? dot3v(p, C.dkm) : alt_side(C, kind, p, u, 0);
  p[0] = dot3(C.crj[0][0], C.crj[1][0], C.crj[2][0], u + 3);
  p[1] = dot3(C.crj[0][1], C.crj[1][1], C.crj[2][1], u + 2);
  p[2] = dot3(C.crj[0][2], C.crj[1][2], C.crj[2][2], u + 1);
  outp = kind == 2 ? dot3v(p, C.dkp) : alt_side(C, kind, p, u + 1, 1);
}

// One side of lagrange_recon (side 0: u^-, side 1: u^+), the same arithmetic.
__device__ __forceinline__ double lagrange_side(const DevConst& C, int kind, const double* u, int side) {
  double p[3];
  if (side == 0) {
    p[0] = dot3(C.crj[0][1], C.crj[1][1], C.crj[2][1], u + 2);
    p[1] = dot3(C.crj[0][2], C.crj[1][2], C.crj[2][2], u + 1);
    p[2] = dot3(C.crj[0][3], C.crj[1][3], C.crj[2][3], u + 0);
    return kind == 2 ? dot3v(p, C.dkm) : kind >= 3 ? alt_side(C, kind, p, u, 0)
                                                   : teno_side(C, p, u, 0, kind == 1);
  }
  p[0] = dot3(C.crj[0][0], C.crj[1][0], C.crj[2][0], u + 3);
  p[1] = dot3(C.crj[0][1], C.crj[1][1], C.crj[2][1], u + 2);
  p[2] = dot3(C.crj[0][2], C.crj[1][2], C.crj[2][2], u + 1);
  return kind == 2 ? dot3v(p, C.dkp) : kind >= 3 ? alt_side(C, kind, p, u + 1, 1)
                                                 : teno_side(C, p, u + 1, 1, kind == 1);
}


// weno5JS3PointsQuadrature (Schemes_Lagrange.cpp:1155-1217).  Not inlined: the flux kernels call
// it 8 times per face, and eight inlined copies overflow the instruction cache.
static __device__ __noinline__ void gl3(const DevConst& C, const double* u, double* out) {
  double bg[3], cg[3], s2[3];
  bg[0] = u[0] - 4.0 * u[1] + 3.0 * u[2];
  cg[0] = u[0] - 2.0 * u[1] + u[2];
  bg[1] = u[1] - u[3];
  cg[1] = u[1] - 2.0 * u[2] + u[3];
  bg[2] = 3.0 * u[2] - 4.0 * u[3] + u[4];
  cg[2] = u[2] - 2.0 * u[3] + u[4];
  // (taken only when every active lane of the warp can take it: the full arithmetic gives the same
  // bits on constant data, and a warp then never runs both)
  if (__all_sync(__activemask(), zero_bits(bg[0]) && zero_bits(bg[1]) && zero_bits(bg[2]) &&
                                     zero_bits(cg[0]) && zero_bits(cg[1]) && zero_bits(cg[2]))) {
    // every indicator is zero: the normalised weights are the constants gl3flat, which the host
    // computed with these same operations -- the same bits without the 24 divisions
    double p[3];
    p[0] = dot3(C.gp[0][0], C.gp[1][0], C.gp[2][0], u + 0);
    p[1] = dot3(C.gp[0][1], C.gp[1][1], C.gp[2][1], u + 1);
    p[2] = dot3(C.gp[0][2], C.gp[1][2], C.gp[2][2], u + 2);
    out[0] = dot3v(p, C.gl3flat[0]);
    const Den d24{24.0, kRcp24, true};
    p[0] = quot(-u[0] + 2.0 * u[1] + 23.0 * u[2], d24);
    p[1] = quot(-u[1] + 26.0 * u[2] - u[3], d24);
    p[2] = quot(23.0 * u[2] + 2.0 * u[3] - u[4], d24);
    double c = C.sumw0p * dot3v(p, C.gl3flat[1]);
    c = c - C.sumw0m * dot3v(p, C.gl3flat[2]);
    out[1] = c;
    p[0] = dot3(C.gm[0][0], C.gm[1][0], C.gm[2][0], u + 0);
    p[1] = dot3(C.gm[0][1], C.gm[1][1], C.gm[2][1], u + 1);
    p[2] = dot3(C.gm[0][2], C.gm[1][2], C.gm[2][2], u + 2);
    out[2] = dot3v(p, C.gl3flat[3]);
#pragma unroll
    for (int k = 0; k < 3; ++k) out[k] = catchnan(out[k]);
    return;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double si = 0.25 * (bg[k] * bg[k]) + (13.0 / 12.0) * (cg[k] * cg[k]);
    const double e = 1e-6 + si;
    s2[k] = e * e;  // pow(eps + SI, 2)
  }
  double p[3], w[3];
  const Den ds[3] = {den_of(s2[0]), den_of(s2[1]), den_of(s2[2])};  // each serves 4 weight sets
  auto weighted = [&](const double* lw) {
#pragma unroll
    for (int k = 0; k < 3; ++k) w[k] = quot(lw[k], ds[k]);
    const double s = (w[0] + w[1]) + w[2];
    const Den dn = den_of(s);
#pragma unroll
    for (int k = 0; k < 3; ++k) w[k] = quot(w[k], dn);
    return dot3v(p, w);
  };
  p[0] = dot3(C.gp[0][0], C.gp[1][0], C.gp[2][0], u + 0);
  p[1] = dot3(C.gp[0][1], C.gp[1][1], C.gp[2][1], u + 1);
  p[2] = dot3(C.gp[0][2], C.gp[1][2], C.gp[2][2], u + 2);
  out[0] = weighted(C.linwp);
  const Den d24{24.0, kRcp24, true};
  p[0] = quot(-u[0] + 2.0 * u[1] + 23.0 * u[2], d24);
  p[1] = quot(-u[1] + 26.0 * u[2] - u[3], d24);
  p[2] = quot(23.0 * u[2] + 2.0 * u[3] - u[4], d24);
  double c = C.sumw0p * weighted(C.linw0p);
  c = c - C.sumw0m * weighted(C.linw0m);
  out[1] = c;
  p[0] = dot3(C.gm[0][0], C.gm[1][0], C.gm[2][0], u + 0);
  p[1] = dot3(C.gm[0][1], C.gm[1][1], C.gm[2][1], u + 1);
  p[2] = dot3(C.gm[0][2], C.gm[1][2], C.gm[2][2], u + 2);
  out[2] = weighted(C.linwm);
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = catchnan(out[k]);
}

// ---- Equations::Euler2D ---------------------------------------------------------------------

__device__ __forceinline__ void primitive(double g1, const double* q, double* w) {  // :20-26
  w[0] = q[0];
  w[1] = q[1] / q[0];
  w[2] = q[2] / q[0];
  w[3] = (q[3] - 0.5 * (q[1] * w[1] + q[2] * w[2])) * g1;
}

__device__ __forceinline__ void flux(int dir, const double* q, const double* w, double* f) {
  if (dir == 1) {
    f[0] = q[1];
    f[1] = q[1] * w[1] + w[3];
    f[2] = q[1] * w[2];
    f[3] = w[1] * (q[3] + w[3]);
  } else {
    f[0] = q[2];
    f[1] = q[2] * w[1];
    f[2] = q[2] * w[2] + w[3];
    f[3] = w[2] * (q[3] + w[3]);
  }
}

// Face eigensystem (eigen2DEuler, FV_System2D.cpp:265-361): the entries of R and L are kept as
// the scalars the reference's matrices are built from.
struct Eig {
  double vxm, vym, hm, qm, cm, t0r;  // t0r = vn * cm (right eigenvectors)
  double rcm, b1, b2, s0, s1, t2;    // left eigenvectors
};

__device__ __forceinline__ Eig eig(double g1, int dir, double sra, double ua, double va, double ha,
                                   double srb, double ub, double vb, double hb) {
  Eig e;
  double t0 = sra / (sra + srb);
  const double t1 = 1.0 - t0;
  e.vxm = t0 * ua + t1 * ub;
  e.vym = t0 * va + t1 * vb;
  e.hm = t0 * ha + t1 * hb;
  e.qm = 0.5 * (e.vxm * e.vxm + e.vym * e.vym);
  e.cm = sqrt(fabs(g1 * (e.hm - e.qm)));
  const double vn = dir == 1 ? e.vxm : e.vym;
  e.t0r = vn * e.cm;
  e.rcm = 1.0 / e.cm;
  e.b1 = g1 * e.rcm * e.rcm;
  e.b2 = e.qm * e.b1;
  e.s0 = vn * e.rcm;
  e.s1 = e.b1 * vn;
  e.t2 = 0.5 * e.b1;
  return e;
}

// L * q with the reference's left-to-right row sums (leftEigenVectorx/y, :133-205).  Zero entries
// of L add exact zeros in the reference and are skipped; unit entries multiply exactly.
__device__ __forceinline__ void left(const Eig& e, int dir, const double* q, double* c) {
  const double l00 = 0.5 * (e.b2 + e.s0), l0n = -0.5 * (e.s1 + e.rcm);
  const double l30 = 0.5 * (e.b2 - e.s0), l3n = -0.5 * (e.s1 - e.rcm);
  const double l20 = 1.0 - e.b2;
  if (dir == 1) {
    const double lt = -e.t2 * e.vym, l2t = e.b1 * e.vym;
    double s = l00 * q[0]; s = s + l0n * q[1]; s = s + lt * q[2]; s = s + e.t2 * q[3]; c[0] = s;
    s = -e.vym * q[0]; s = s + q[2]; c[1] = s;
    s = l20 * q[0]; s = s + e.s1 * q[1]; s = s + l2t * q[2]; s = s + (-e.b1) * q[3]; c[2] = s;
    s = l30 * q[0]; s = s + l3n * q[1]; s = s + lt * q[2]; s = s + e.t2 * q[3]; c[3] = s;
  } else {
    const double lt = -e.t2 * e.vxm, l2t = e.b1 * e.vxm;
    double s = l00 * q[0]; s = s + lt * q[1]; s = s + l0n * q[2]; s = s + e.t2 * q[3]; c[0] = s;
    s = -e.vxm * q[0]; s = s + q[1]; c[1] = s;
    s = l20 * q[0]; s = s + l2t * q[1]; s = s + e.s1 * q[2]; s = s + (-e.b1) * q[3]; c[2] = s;
    s = l30 * q[0]; s = s + lt * q[1]; s = s + l3n * q[2]; s = s + e.t2 * q[3]; c[3] = s;
  }
}

// R * c (rightEigenVectorx/y, :100-131, 169-180)
__device__ __forceinline__ void right(const Eig& e, int dir, const double* c, double* q) {
  double s = c[0]; s = s + c[2]; s = s + c[3]; q[0] = s;
  if (dir == 1) {
    s = (e.vxm - e.cm) * c[0]; s = s + e.vxm * c[2]; s = s + (e.vxm + e.cm) * c[3]; q[1] = s;
    s = e.vym * c[0]; s = s + c[1]; s = s + e.vym * c[2]; s = s + e.vym * c[3]; q[2] = s;
    s = (e.hm - e.t0r) * c[0]; s = s + e.vym * c[1]; s = s + e.qm * c[2]; s = s + (e.hm + e.t0r) * c[3]; q[3] = s;
  } else {
    s = e.vxm * c[0]; s = s + c[1]; s = s + e.vxm * c[2]; s = s + e.vxm * c[3]; q[1] = s;
    s = (e.vym - e.cm) * c[0]; s = s + e.vym * c[2]; s = s + (e.vym + e.cm) * c[3]; q[2] = s;
    s = (e.hm - e.t0r) * c[0]; s = s + e.vxm * c[1]; s = s + e.qm * c[2]; s = s + (e.hm + e.t0r) * c[3]; q[3] = s;
  }
}

// HLLC (Equations_Euler2D.cpp:372-428)
__device__ __forceinline__ void hllc(double g1, int dir, const double* ql, const double* qr,
                                     double* F) {
  const int d1 = dir - 1;
  double wl[4], wr[4], fl[4], qs[4];
  primitive(g1, ql, wl);
  primitive(g1, qr, wr);
  const double hl = (ql[3] + wl[3]) / wl[0];
  const double hr = (qr[3] + wr[3]) / wr[0];
  const double rr = sqrt(fabs(wr[0] / wl[0]));
  const double rrr = 1.0 / (1.0 + rr);
  double vm[2];
  vm[0] = (wl[1] + wr[1] * rr) * rrr;
  vm[1] = (wl[2] + wr[2] * rr) * rrr;
  const double qm = 0.5 * (vm[0] * vm[0] + vm[1] * vm[1]);
  const double hm = (hl + hr * rr) * rrr;
  const double cm = sqrt(fabs(g1 * (hm - qm)));
  const double cl = sqrt(fabs(wl[3] / wl[0]));
  const double cr = sqrt(fabs(wr[3] / wr[0]));
  const double sl = fmin(wl[dir] - cl, vm[d1] - cm);
  const double sr = fmax(wr[dir] + cr, vm[d1] + cm);
  const double sm = (qr[dir] * (sr - wr[dir]) - ql[dir] * (sl - wl[dir]) + wl[3] - wr[3]) /
                    (wr[0] * (sr - wr[dir]) - wl[0] * (sl - wl[dir]));
  const double ps = wl[3] + wl[0] * (wl[dir] - sl) * (wl[dir] - sm);
  // The reference's four regions (:408-427).  The two star regions run the same expressions on
  // the left or the right operands (the energy term keeps the left pressure in both, as the
  // reference does), and so do the two outer regions, so the operands are selected first and
  // one copy of the arithmetic runs: a warp whose faces fall in different regions does not pay
  // for both.  Same operations in the same order on the same values: the same bits.
  const bool outer_l = sl > 0.0;
  const bool star_l = !outer_l && sl <= 0.0 && sm > 0.0;
  const bool star_r = !outer_l && !star_l && sm <= 0.0 && sr >= 0.0;
  const bool use_l = outer_l || star_l;
  double q[4], w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    q[k] = use_l ? ql[k] : qr[k];
    w[k] = use_l ? wl[k] : wr[k];
  }
  flux(dir, q, w, fl);
  if (star_l || star_r) {
    const double s = use_l ? sl : sr;
    const double nom = s - w[dir], den = s - sm;
    qs[0] = w[0] * nom / den;
    qs[1] = dir == 1 ? (nom * q[1] + ps - w[3]) / den : nom * q[1] / den;
    qs[2] = dir == 2 ? (nom * q[2] + ps - w[3]) / den : nom * q[2] / den;
    qs[3] = (nom * q[3] - wl[3] * w[dir] + ps * sm) / den;
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = fl[k] + s * (qs[k] - q[k]);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = fl[k];
  }
}

// characteristic Rusanov (:310-330) with maxLocalWaveSpeed (:221-246)
__device__ __forceinline__ void rusanov(double g, double g1, int dir, const Eig& e,
                                        const double* ql, const double* qr, double* F) {
  double wl[4], wr[4], a[4], fl[4], fr[4], d[4], m[4], rm[4];
  primitive(g1, ql, wl);
  primitive(g1, qr, wr);
  const double cl = sqrt(fabs(g * wl[3] / wl[0]));
  const double cr = sqrt(fabs(g * wr[3] / wr[0]));
  const double vl = wl[dir], vr = wr[dir];
  a[0] = fmax(fabs(vl - cl), fabs(vr - cr));
  a[1] = fmax(fabs(vl), fabs(vr));
  a[2] = a[1];
  a[3] = fmax(fabs(vl + cl), fabs(vr + cr));
  flux(dir, ql, wl, fl);
  flux(dir, qr, wr, fr);
#pragma unroll
  for (int k = 0; k < 4; ++k) d[k] = qr[k] - ql[k];
  left(e, dir, d, m);
#pragma unroll
  for (int k = 0; k < 4; ++k) m[k] = a[k] * m[k];
  right(e, dir, m, rm);
#pragma unroll
  for (int k = 0; k < 4; ++k) F[k] = 0.5 * (fl[k] + fr[k] - rm[k]);
}

// maxSpeed over both directions (Equations_Euler2D.cpp:207-219)
__device__ __forceinline__ double max_speed2(double g, const double* w) {
  const double c = sqrt(fabs(g * w[3] / w[0]));
  return fmax(fmax(w[1] - c, fabs(w[1] + c)), fmax(w[2] - c, fabs(w[2] + c)));
}

// ---- Equations::Euler1D (Equations_Euler1D.cpp) --------------------------------------------

__device__ __forceinline__ void primitive1(double g1, const double* q, double* w) {  // :18-23
  w[0] = q[0];
  w[1] = q[1] / q[0];
  w[2] = (q[2] - 0.5 * q[1] * w[1]) * g1;
}

// eigen1DEuler (FV_System1D.cpp:121-156), eigenvectors :55-89 as full row-major 3x3 matrices
__device__ __forceinline__ void eig1(double g1, double sra, double ua, double ha, double srb,
                                     double ub, double hb, double* R, double* L) {
  double t0 = sra / (sra + srb);
  const double t1 = 1.0 - t0;
  const double vxm = t0 * ua + t1 * ub;
  const double hm = t0 * ha + t1 * hb;
  const double qm = 0.5 * vxm * vxm;
  const double cm = sqrt(fabs(g1 * (hm - qm)));
  t0 = vxm * cm;
  R[0] = 1.0; R[1] = 1.0; R[2] = 1.0;
  R[3] = vxm - cm; R[4] = vxm; R[5] = vxm + cm;
  R[6] = hm - t0; R[7] = qm; R[8] = hm + t0;
  const double rcm = 1.0 / cm;
  const double b1 = g1 * rcm * rcm;
  const double b2 = qm * b1;
  const double s0 = vxm * rcm;
  const double s1 = b1 * vxm;
  const double t2 = 0.5 * b1;
  L[0] = 0.5 * (b2 + s0); L[1] = -0.5 * (s1 + rcm); L[2] = t2;
  L[3] = 1.0 - b2; L[4] = s1; L[5] = -b1;
  L[6] = 0.5 * (b2 - s0); L[7] = -0.5 * (s1 - rcm); L[8] = t2;
}

__device__ __forceinline__ void mv3(const double* M, const double* x, double* y) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double s = M[3 * i] * x[0];
    s = s + M[3 * i + 1] * x[1];
    s = s + M[3 * i + 2] * x[2];
    y[i] = s;
  }
}

__device__ __forceinline__ void flux1(const double* q, const double* w, double* f) {
  f[0] = q[1];
  f[1] = q[1] * w[1] + w[2];
  f[2] = w[1] * (q[2] + w[2]);
}

// Rusanov (Equations_Euler1D.cpp:129-135) with maxLocalWaveSpeed (:96-107)
__device__ __forceinline__ void rusanov1(double g, double g1, const double* L, const double* R,
                                         const double* ql, const double* qr, double* F) {
  double wl[3], wr[3], a[3], fl[3], fr[3], d[3], m[3], rm[3];
  primitive1(g1, ql, wl);
  primitive1(g1, qr, wr);
  const double cl = sqrt(fabs(g * wl[2] / wl[0]));
  const double cr = sqrt(fabs(g * wr[2] / wr[0]));
  a[0] = fmax(fabs(wl[1] - cl), fabs(wr[1] - cr));
  a[1] = fmax(fabs(wl[1]), fabs(wr[1]));
  a[2] = fmax(fabs(wl[1] + cl), fabs(wr[1] + cr));
  flux1(ql, wl, fl);
  flux1(qr, wr, fr);
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = qr[k] - ql[k];
  mv3(L, d, m);
#pragma unroll
  for (int k = 0; k < 3; ++k) m[k] = a[k] * m[k];
  mv3(R, m, rm);
#pragma unroll
  for (int k = 0; k < 3; ++k) F[k] = 0.5 * (fl[k] + fr[k] - rm[k]);
}

// HLLC (Equations_Euler1D.cpp:156-210)
__device__ __forceinline__ void hllc1(double g1, const double* ql, const double* qr, double* F) {
  double wl[3], wr[3], fl[3], fr[3], qs[3];
  primitive1(g1, ql, wl);
  primitive1(g1, qr, wr);
  const double hl = (ql[2] + wl[2]) / wl[0];
  const double hr = (qr[2] + wr[2]) / wr[0];
  const double rr = sqrt(fabs(wr[0] / wl[0]));
  const double rrr = 1.0 / (1.0 + rr);
  const double vm = (wl[1] + wr[1] * rr) * rrr;
  const double qm = 0.5 * vm * vm;
  const double hm = (hl + hr * rr) * rrr;
  const double cm = sqrt(fabs(g1 * (hm - qm)));
  const double cl = sqrt(fabs(wl[2] / wl[0]));
  const double cr = sqrt(fabs(wr[2] / wr[0]));
  const double sl = fmin(wl[1] - cl, vm - cm);
  const double sr = fmax(wr[1] + cr, vm + cm);
  const double sm = (qr[1] * (sr - wr[1]) - ql[1] * (sl - wl[1]) + wl[2] - wr[2]) /
                    (wr[0] * (sr - wr[1]) - wl[0] * (sl - wl[1]));
  const double ps = wl[2] + wl[0] * (wl[1] - sl) * (wl[1] - sm);
  flux1(ql, wl, fl);
  flux1(qr, wr, fr);
  if (sl > 0.0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) F[k] = fl[k];
  } else if (sl <= 0.0 && sm > 0.0) {
    const double nom = sl - wl[1], den = sl - sm;
    qs[0] = wl[0] * nom / den;
    qs[1] = (nom * ql[1] + ps - wl[2]) / den;
    qs[2] = (nom * ql[2] - wl[2] * wl[1] + ps * sm) / den;
#pragma unroll
    for (int k = 0; k < 3; ++k) F[k] = fl[k] + sl * (qs[k] - ql[k]);
  } else if (sm <= 0.0 && sr >= 0.0) {
    const double nom = sr - wr[1], den = sr - sm;
    qs[0] = wr[0] * nom / den;
    qs[1] = (nom * qr[1] + ps - wr[2]) / den;
    qs[2] = (nom * qr[2] - wl[2] * wr[1] + ps * sm) / den;
#pragma unroll
    for (int k = 0; k < 3; ++k) F[k] = fr[k] + sr * (qs[k] - qr[k]);
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) F[k] = fr[k];
  }
}

__device__ __forceinline__ double max_speed1(double g, const double* w) {  // :91-94
  const double c = sqrt(fabs(g * w[2] / w[0]));
  return fmax(fabs(w[1] - c), fabs(w[1] + c));
}

// ---- Schemes::Hermite (Schemes_Hermite.cpp) -------------------------------------------------

// smoothnessMeasure (:515-526)
__device__ __forceinline__ void hermite_si(const double* u, const double* v, double* SI) {
  double b[3], c[3];
  b[0] = -2.0 * (u[0] - u[1]) - v[0];
  c[0] = -2.0 * (u[0] - u[1] + v[0]);
  b[1] = -2.0 * (u[1] - u[2]) - v[2];
  c[1] = 2.0 * (u[1] - u[2]) + 2.0 * v[2];
  b[2] = (-u[0] + u[2]) / 2.0;
  c[2] = u[0] - 2.0 * u[1] + u[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) SI[k] = (13.0 / 12.0) * (c[k] * c[k]) + b[k] * b[k];
}
// smoothnessMeasureDerivative (:528-541)
__device__ __forceinline__ void hermite_sid(const double* u, const double* d, double* SI) {
  double b[3], c[3];
  b[0] = 6.0 * (u[0] - u[1]) + (2.0 * d[0] + 4.0 * d[1]);
  c[0] = 12.0 * (u[0] - u[1]) + 6.0 * (d[0] + d[1]);
  b[1] = 6.0 * (u[2] - u[1]) - (4.0 * d[1] + 2.0 * d[2]);
  c[1] = 12.0 * (u[1] - u[2]) + 6.0 * (d[1] + d[2]);
  b[2] = u[0] - 2.0 * u[1] + u[2];
  c[2] = 3.0 * (u[2] - u[0]) - 6.0 * d[1];
#pragma unroll
  for (int k = 0; k < 3; ++k) SI[k] = (13.0 / 12.0) * (c[k] * c[k]) + b[k] * b[k];
}
// fullPointsSI (:597-603)
__device__ __forceinline__ double hermite_brk(const double* u, const double* d) {
  return fabs((1029270.0 * u[2] - 2129184.0 * u[1] + 1099914.0 * u[0] + 281121.0 * d[0] -
               494958.0 * d[2]) * d[0] +
              (-1029270.0 * u[0] + 2129184.0 * u[1] - 1099914.0 * u[2] + 281121.0 * d[2]) * d[2] +
              (1099445.0 * u[2] - 4317056.0 * u[1] + 2118166.0 * u[0]) * u[2] +
              4317056.0 * (u[1] - u[0]) * u[1] + 1099445.0 * u[0] * u[0]) /
         6720.0;
}
// fullPointsSId (:605-612)
__device__ __forceinline__ double hermite_brkd(const double* u, const double* d) {
  return fabs((3156862.0 * d[2] + 13189240.0 * d[1] + 1710479.0 * d[0] - 9617754.0 * u[2] -
               531552.0 * u[1] + 10149306.0 * u[0]) * d[0] +
              (13189240.0 * d[2] + 26511200.0 * d[1] - 39700440.0 * u[2] + 39700440.0 * u[0]) * d[1] +
              (1710479.0 * d[2] - 10149306.0 * u[2] + 531552.0 * u[1] + 9617754.0 * u[0]) * d[2] +
              (15136011.0 * u[2] - 1076544.0 * u[1] - 29195478.0 * u[0]) * u[2] +
              1076544.0 * (u[1] - u[0]) * u[1] + 15136011.0 * u[0] * u[0]) /
         1680.0;
}
__device__ __forceinline__ double maxof3(const double* s) {
  double t = s[0];
  t = (t < s[1]) ? s[1] : t;
  t = (t < s[2]) ? s[2] : t;
  return t;
}
// one hteno/htenoi output: cut-off (cutOff/cutOffd, :614-628) and the table weights
__device__ __forceinline__ double hermite_weighted(const DevConst& C, int which, const double* p,
                                                   const double* SI, double tau) {
  const int pat = cutoff_pattern(SI, tau, 1e-40, 1e-3);
  const double* w = which == 0 ? C.hwtab_m[pat] : which == 1 ? C.hwtab_p[pat]
                  : which == 2 ? C.hwtab_md[pat] : C.hwtab_pd[pat];
  return catchnan(dot3v(p, w));
}

// kind 0 hteno (:295-379), 1 htenoi (:670-758), 2 linear (:760-812);
// out = {u^-, u^+, d^-, d^+} at x_{i+1/2}
__device__ __forceinline__ void hermite_recon(const DevConst& C, const HermiteK<double>& K,
                                              int kind, const double* u, const double* d,
                                              double* out) {
  if (kind == 2) {
    out[0] = dot3(K.crjlin[0][0], K.crjlin[1][0], K.crjlin[2][0], u) + K.crjlin[3][0] * d[0] +
             K.crjlin[4][0] * d[2];
    out[1] = dot3(K.crjlin[0][1], K.crjlin[1][1], K.crjlin[2][1], u + 1) + K.crjlin[3][1] * d[1] +
             K.crjlin[4][1] * d[3];
    out[2] = dot3(K.crjlind[0][0], K.crjlind[1][0], K.crjlind[2][0], u) +
             dot3(K.crjlind[3][0], K.crjlind[4][0], K.crjlind[5][0], d);
    out[3] = dot3(K.crjlind[0][1], K.crjlind[1][1], K.crjlind[2][1], u + 1) +
             dot3(K.crjlind[3][1], K.crjlind[4][1], K.crjlind[5][1], d + 1);
    return;
  }
  const bool imp = kind == 1;
  double ud[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) ud[k] = d[k] * K.dif;
  double p[3], SI[3], tau;
  p[0] = K.crj[0][0] * u[0] + K.crj[1][0] * u[1] + K.crj[2][0] * d[0];
  p[1] = K.crj[0][1] * u[1] + K.crj[1][1] * u[2] + K.crj[2][1] * d[2];
  p[2] = K.crj[0][2] * u[0] + K.crj[1][2] * u[1] + K.crj[2][2] * u[2];
  hermite_si(u, ud, SI);
  tau = imp ? maxof3(SI) : fabs(hermite_brk(u, ud) - 0.25 * (SI[0] + SI[1] + 2.0 * SI[2]));
  out[0] = hermite_weighted(C, 0, p, SI, tau);

  p[0] = K.crjd[0][0] * u[0] + K.crjd[1][0] * u[1] + K.crjd[2][0] * d[0] + K.crjd[3][0] * d[1];
  p[1] = K.crjd[0][1] * u[1] + K.crjd[1][1] * u[2] + K.crjd[2][1] * d[1] + K.crjd[3][1] * d[2];
  p[2] = K.crjd[0][2] * u[0] + K.crjd[1][2] * u[1] + K.crjd[2][2] * u[2] + K.crjd[3][2] * d[1];
  hermite_sid(u, ud, SI);
  tau = imp ? maxof3(SI) : fabs(hermite_brkd(u, ud) - 0.25 * (SI[0] + SI[1] + 2.0 * SI[2]));
  out[2] = hermite_weighted(C, 2, p, SI, tau);

  p[0] = K.crj[1][1] * u[1] + K.crj[0][1] * u[2] - K.crj[2][1] * d[1];
  p[1] = K.crj[1][0] * u[2] + K.crj[0][0] * u[3] - K.crj[2][0] * d[3];
  p[2] = K.crj[2][2] * u[1] + K.crj[1][2] * u[2] + K.crj[0][2] * u[3];
  hermite_si(u + 1, ud + 1, SI);
  tau = imp ? maxof3(SI) : fabs(hermite_brk(u + 1, ud + 1) - 0.25 * (SI[0] + SI[1] + 2.0 * SI[2]));
  out[1] = hermite_weighted(C, 1, p, SI, tau);

  p[0] = K.crjd[0][1] * u[1] + K.crjd[1][1] * u[2] + K.crjd[3][1] * d[1] + K.crjd[2][1] * d[2];
  p[1] = K.crjd[0][0] * u[2] + K.crjd[1][0] * u[3] + K.crjd[3][0] * d[2] + K.crjd[2][0] * d[3];
  p[2] = -(K.crjd[2][2] * u[1] + K.crjd[1][2] * u[2] + K.crjd[0][2] * u[3]) + K.crjd[3][2] * d[2];
  hermite_sid(u + 1, ud + 1, SI);
  tau = imp ? maxof3(SI) : fabs(hermite_brkd(u + 1, ud + 1) - 0.25 * (SI[0] + SI[1] + 2.0 * SI[2]));
  out[3] = hermite_weighted(C, 3, p, SI, tau);
}

// hermiteLimiter (Schemes_Hermite.cpp:634-662)
__device__ __forceinline__ double hermite_limiter(const HermiteK<double>& K, const double* u,
                                                  const double* d) {
  double p[3];
  p[0] = 0.75 * (u[2] - u[0]) / K.dif - 0.25 * (d[0] + d[2]);
  p[1] = (u[1] - u[0]) / K.dif;
  p[2] = (u[2] - u[1]) / K.dif;
  const double lw[3] = {1.0 - 2E-5, 1E-5, 1E-5};
  const double ud[3] = {d[0] * K.dif, d[1] * K.dif, d[2] * K.dif};
  double sm[3];
  sm[0] = hermite_brk(u, ud);
  sm[1] = (u[0] - u[1]) * (u[0] - u[1]);
  sm[2] = (u[1] - u[2]) * (u[1] - u[2]);
  const double ta = fabs(sm[0] - sm[1]) + fabs(sm[0] - sm[2]);
  const double tau = ta * ta / 4.0;
  double w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = lw[k] * (1.0 + tau / (sm[k] + 1e-6));
  const double s = (w[0] + w[1]) + w[2];
#pragma unroll
  for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  const double r1 = lw[1] / lw[0], r2 = lw[2] / lw[0];
  double inner = r1 * p[1];
  inner = inner + r2 * p[2];
  double w12 = w[1] * p[1];
  w12 = w12 + w[2] * p[2];
  return w[0] * (p[0] / lw[0] - inner) + w12;
}

// A(q) * x with the Jacobians dfluxx / dfluxy (Equations_Euler2D.cpp:52-98), row sums left to
// right; zero and unit entries as in the reference's matrices.
__device__ __forceinline__ void dflux_apply(double g, double g1, double g3, int dir, const double* q,
                                            const double* w, const double* x, double* y) {
  if (dir == 1) {
    const double sv = w[1] * w[1];
    const double dv = 0.5 * g1 * (sv + w[2] * w[2]);
    const double h = (q[3] + w[3]) / w[0];
    y[0] = x[1];
    double s = (dv - sv) * x[0]; s = s + (-g3 * w[1]) * x[1]; s = s + (-g1 * w[2]) * x[2]; s = s + g1 * x[3]; y[1] = s;
    s = (-w[1] * w[2]) * x[0]; s = s + w[2] * x[1]; s = s + w[1] * x[2]; y[2] = s;
    s = ((dv - h) * w[1]) * x[0]; s = s + (h - g1 * sv) * x[1]; s = s + (-g1 * w[1] * w[2]) * x[2];
    s = s + (g * w[1]) * x[3]; y[3] = s;
  } else {
    const double sv = w[2] * w[2];
    const double dv = 0.5 * g1 * (sv + w[1] * w[1]);
    const double h = (q[3] + w[3]) / w[0];
    y[0] = x[2];
    double s = (-w[1] * w[2]) * x[0]; s = s + w[2] * x[1]; s = s + w[1] * x[2]; y[1] = s;
    s = (dv - sv) * x[0]; s = s + (-g1 * w[1]) * x[1]; s = s + (-g3 * w[2]) * x[2]; s = s + g1 * x[3]; y[2] = s;
    s = ((dv - h) * w[2]) * x[0]; s = s + (-g1 * w[1] * w[2]) * x[1]; s = s + (h - g1 * sv) * x[2];
    s = s + (g * w[2]) * x[3]; y[3] = s;
  }
}

// dRusanov (Equations_Euler2D.cpp:352-360) as called in FVHermite_System2D.cpp:553-589
__device__ __forceinline__ void drusanov(double g, double g1, double g3, int dir, const Eig& e,
                                         const double* ql, const double* qr, const double* dql,
                                         const double* dqr, double* F) {
  double wl[4], wr[4], a[4], d[4], m[4], al[4], ar[4], rm[4];
  primitive(g1, ql, wl);
  primitive(g1, qr, wr);
  dflux_apply(g, g1, g3, dir, ql, wl, dql, al);
  dflux_apply(g, g1, g3, dir, qr, wr, dqr, ar);
  const double cl = sqrt(fabs(g * wl[3] / wl[0]));
  const double cr = sqrt(fabs(g * wr[3] / wr[0]));
  const double vl = wl[dir], vr = wr[dir];
  a[0] = fmax(fabs(vl - cl), fabs(vr - cr));
  a[1] = fmax(fabs(vl), fabs(vr));
  a[2] = a[1];
  a[3] = fmax(fabs(vl + cl), fabs(vr + cr));
#pragma unroll
  for (int k = 0; k < 4; ++k) d[k] = dqr[k] - dql[k];
  left(e, dir, d, m);
#pragma unroll
  for (int k = 0; k < 4; ++k) m[k] = a[k] * m[k];
  right(e, dir, m, rm);
#pragma unroll
  for (int k = 0; k < 4; ++k) F[k] = 0.5 * (al[k] + ar[k] - rm[k]);
}

// dflux 1D (Equations_Euler1D.cpp:39-53) applied to x; dRusanov 1D (:212-220)
__device__ __forceinline__ void drusanov1(double g, double g1, double g3, const double* L,
                                          const double* R, const double* ql, const double* qr,
                                          const double* dql, const double* dqr, double* F) {
  double wl[3], wr[3], a[3], d[3], m[3], rm[3], al[3], ar[3];
  primitive1(g1, ql, wl);
  primitive1(g1, qr, wr);
  auto apply = [&](const double* q, const double* w, const double* x, double* y) {
    double A[9];
    A[0] = 0.0; A[1] = 1.0; A[2] = 0.0;
    A[3] = 0.5 * g3 * w[1] * w[1];
    A[4] = -g3 * w[1];
    A[5] = g1;
    A[6] = (g1 * (w[1] * w[1]) - g * q[2] / w[0]) * w[1];
    A[7] = g * q[2] / w[0] - 1.5 * g1 * w[1] * w[1];
    A[8] = g * w[1];
    y[0] = x[1];
    double s = A[3] * x[0]; s = s + A[4] * x[1]; s = s + A[5] * x[2]; y[1] = s;
    s = A[6] * x[0]; s = s + A[7] * x[1]; s = s + A[8] * x[2]; y[2] = s;
  };
  apply(ql, wl, dql, al);
  apply(qr, wr, dqr, ar);
  const double cl = sqrt(fabs(g * wl[2] / wl[0]));
  const double cr = sqrt(fabs(g * wr[2] / wr[0]));
  a[0] = fmax(fabs(wl[1] - cl), fabs(wr[1] - cr));
  a[1] = fmax(fabs(wl[1]), fabs(wr[1]));
  a[2] = fmax(fabs(wl[1] + cl), fabs(wr[1] + cr));
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = dqr[k] - dql[k];
  mv3(L, d, m);
#pragma unroll
  for (int k = 0; k < 3; ++k) m[k] = a[k] * m[k];
  mv3(R, m, rm);
#pragma unroll
  for (int k = 0; k < 3; ++k) F[k] = 0.5 * (al[k] + ar[k] - rm[k]);
}

}  // namespace par
}  // namespace hteno
