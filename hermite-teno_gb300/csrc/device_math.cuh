// Device-side numerics of the Hermite-TENO hot path, templated on the compute type T (double for
// the plain path, float for the mixed path).  Each function names the reference function it
// computes.  Reformulations relative to the reference, all exact up to rounding:
//   * pow(r, 6) is r^2 * r^2 * r^2; x/(y) in weight formulas uses reciprocals;
//   * the TENO cut-off test  a_k / sum(a) < C_T  is evaluated as  a_k < C_T * sum(a)  on
//     ratios normalised by the largest a (no overflow in float);
//   * the normalised optimal weights of every cut-off pattern come from a table that the host
//     fills with the reference's own normalisation (s_k d_k / sum(s d)), so reconstructions on
//     smooth data reproduce the reference's weights bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "dev_const.h"

namespace hteno {

#define HTENO_LAG_EPS 1e-6
#define HTENO_LAG_EPSZ 1e-40
#define HTENO_LAG_CT 5e-4
#define HTENO_C1 (13.0 / 12.0)
#define HTENO_MACHINE_EPS 1e-15
#define HTENO_HER_CT 1e-3
// Smallest normal-range offset used for the float path in place of 1e-40 (subnormal in float).
#define HTENO_F32_EPSZ 1e-30f

template <typename T> struct Cst;
template <> struct Cst<double> {
  __device__ static double crj(const DevConst& c, int r, int k) { return c.crj[r][k]; }
  __device__ static double gp(const DevConst& c, int r, int k) { return c.gp[r][k]; }
  __device__ static double gm(const DevConst& c, int r, int k) { return c.gm[r][k]; }
  __device__ static const double* linwp(const DevConst& c) { return c.linwp; }
  __device__ static const double* linwm(const DevConst& c) { return c.linwm; }
  __device__ static const double* linw0p(const DevConst& c) { return c.linw0p; }
  __device__ static const double* linw0m(const DevConst& c) { return c.linw0m; }
  __device__ static double sumw0p(const DevConst& c) { return c.sumw0p; }
  __device__ static double sumw0m(const DevConst& c) { return c.sumw0m; }
  __device__ static double gl3w(const DevConst& c, int m) { return c.gl3w[m]; }
  __device__ static const double* wtab(const DevConst& c, int side, int pat) {
    return side ? c.wtab_p[pat] : c.wtab_m[pat];
  }
  __device__ static const double* hwtab(const DevConst& c, int which, int pat) {
    return which == 0 ? c.hwtab_m[pat] : which == 1 ? c.hwtab_p[pat]
         : which == 2 ? c.hwtab_md[pat] : c.hwtab_pd[pat];
  }
  __device__ static double epsz() { return HTENO_LAG_EPSZ; }
  __device__ static double rcp(double x) { return __drcp_rn(x); }
  __device__ static double sqrt_(double x) { return sqrt(x); }
};
template <> struct Cst<float> {
  __device__ static float crj(const DevConst& c, int r, int k) { return c.f_crj[r][k]; }
  __device__ static float gp(const DevConst& c, int r, int k) { return c.f_gp[r][k]; }
  __device__ static float gm(const DevConst& c, int r, int k) { return c.f_gm[r][k]; }
  __device__ static const float* linwp(const DevConst& c) { return c.f_linwp; }
  __device__ static const float* linwm(const DevConst& c) { return c.f_linwm; }
  __device__ static const float* linw0p(const DevConst& c) { return c.f_linw0p; }
  __device__ static const float* linw0m(const DevConst& c) { return c.f_linw0m; }
  __device__ static float sumw0p(const DevConst& c) { return c.f_sumw0p; }
  __device__ static float sumw0m(const DevConst& c) { return c.f_sumw0m; }
  __device__ static float gl3w(const DevConst& c, int m) { return c.f_gl3w[m]; }
  __device__ static const float* wtab(const DevConst& c, int side, int pat) {
    return side ? c.f_wtab_p[pat] : c.f_wtab_m[pat];
  }
  __device__ static const float* hwtab(const DevConst& c, int which, int pat) {
    return which == 0 ? c.f_hwtab_m[pat] : which == 1 ? c.f_hwtab_p[pat]
         : which == 2 ? c.f_hwtab_md[pat] : c.f_hwtab_pd[pat];
  }
  __device__ static float epsz() { return HTENO_F32_EPSZ; }
  // The MUFU reciprocal (rcp.approx.ftz.f32, relative error below 2^-23): one instruction
  // instead of a correctly rounded reciprocal's refinement and range checks.  Every float
  // reciprocal of the mixed path goes through here: weights, cut-off ratios, 1/rho, the HLLC
  // star-state denominators -- none takes a subnormal argument (their floors: eps^2 = 1e-12,
  // epsz = 1e-30, densities of the state).
  __device__ static float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  // Likewise the MUFU-based square root (sqrt.approx.ftz.f32) for sound speeds and sqrt|rho|.
  __device__ static float sqrt_(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
};

// a / b: in float through the MUFU reciprocal, in double the correctly rounded division (the
// double instantiations serve the bit-reproducible paths).
template <typename T>
__device__ __forceinline__ T fdiv(T a, T b) {
  if constexpr (sizeof(T) == 4) return a * Cst<T>::rcp(b);
  else return a / b;
}

// a * b + c: an explicit fused multiply-add in float (so every instantiation rounds alike even
// where the compiler is not allowed to contract); for double the unfused expression, which
// rounds as written where contraction is off.
template <typename T>
__device__ __forceinline__ T mad(T a, T b, T c) {
  if constexpr (sizeof(T) == 4) return fmaf(a, b, c);
  else return a * b + c;
}
// x0 y0 + x1 y1 + x2 y2, summed left to right
template <typename T>
__device__ __forceinline__ T dot3m(T x0, T y0, T x1, T y1, T x2, T y2) {
  return mad(x2, y2, mad(x1, y1, x0 * y0));
}

template <typename T>
__device__ __forceinline__ T catchnan(T x) {  // Schemes_Lagrange.cpp:1151-1153
  return isnan(x) ? T(HTENO_MACHINE_EPS) : x;
}

// ---------------------------------------------------------------------------------------------
// Schemes::Lagrange
// ---------------------------------------------------------------------------------------------

// TENO cut-off (cutOff(), Schemes_Lagrange.cpp:1141-1149) on r_k = 1 + tau/(SI_k + epsz).
// Returns the pattern bits sigma_0 | sigma_1 << 1 | sigma_2 << 2.
template <typename T>
__device__ __forceinline__ int teno_pattern(T r0, T r1, T r2, T ct) {
  // normalise by the largest ratio so that r^6 cannot overflow (float path)
  T rm = fmax(fmax(r0, r1), r2);
  T inv = Cst<T>::rcp(rm);
  T a0 = r0 * inv, a1 = r1 * inv, a2 = r2 * inv;
  a0 = a0 * a0; a0 = a0 * a0 * a0;
  a1 = a1 * a1; a1 = a1 * a1 * a1;
  a2 = a2 * a2; a2 = a2 * a2 * a2;
  T lim = ct * ((a0 + a1) + a2);
  // NaN anywhere makes every comparison false -> sigma = 1, as in the reference
  return (a0 < lim ? 0 : 1) | (a1 < lim ? 0 : 2) | (a2 < lim ? 0 : 4);
}

// smoothnessMeasure (:1013-1026) + optional fullpointsSmootness (:1029-1034)
template <typename T>
__device__ __forceinline__ void lagrange_si(const T* v, T& SI0, T& SI1, T& SI2) {
  T c0 = mad(T(-2.0), v[3], v[2]) + v[4];
  T b0 = (mad(T(-4.0), v[3], T(3.0) * v[2]) + v[4]) * T(0.5);
  T c1 = mad(T(-2.0), v[2], v[1]) + v[3];
  T b1 = (v[1] - v[3]) * T(0.5);
  T c2 = mad(T(-2.0), v[1], v[0]) + v[2];
  T b2 = mad(T(3.0), v[2], mad(T(-4.0), v[1], v[0])) * T(0.5);
  SI0 = mad(T(HTENO_C1) * c0, c0, b0 * b0);
  SI1 = mad(T(HTENO_C1) * c1, c1, b1 * b1);
  SI2 = mad(T(HTENO_C1) * c2, c2, b2 * b2);
}
template <typename T>
__device__ __forceinline__ T lagrange_b35(const T* v) {
  const T a4 = mad(T(8209.0), v[0], mad(T(-38947.0), v[1], mad(T(67923.0), v[2],
                  mad(T(-51001.0), v[3], T(6908.0) * v[4]))));
  const T a3 = mad(T(-38947.0), v[0], mad(T(179098.0), v[1], mad(T(-299076.0), v[2], T(104963.0) * v[3])));
  const T a2 = mad(T(67923.0), v[0], mad(T(-299076.0), v[1], T(231153.0) * v[2]));
  const T a1 = mad(T(-51001.0), v[0], T(104963.0) * v[1]);
  const T r = mad(T(6908.0) * v[0], v[0], mad(v[1], a1, mad(v[2], a2, mad(v[3], a3, v[4] * a4))));
  return r * T(1.0 / 5040.0);
}

// One side of teno5 (improved = false, :481-511) or teno5i (improved = true, :1235-1263).
template <typename T>
__device__ __forceinline__ T teno_side(const DevConst& C, T p0, T p1, T p2, const T* v, int side,
                                       bool improved) {
  T SI0, SI1, SI2;
  lagrange_si(v, SI0, SI1, SI2);
  T tau;
  if (!improved) {
    tau = fabs(lagrange_b35(v) - (SI0 + SI2 + T(4.0) * SI1) * T(1.0 / 6.0));
  } else {
    tau = fmax(fmax(SI0, SI1), SI2);
  }
  const T ez = Cst<T>::epsz();
  T r0 = mad(tau, Cst<T>::rcp(SI0 + ez), T(1.0));
  T r1 = mad(tau, Cst<T>::rcp(SI1 + ez), T(1.0));
  T r2 = mad(tau, Cst<T>::rcp(SI2 + ez), T(1.0));
  int pat = teno_pattern(r0, r1, r2, T(HTENO_LAG_CT));
  const T* w = Cst<T>::wtab(C, side, pat);
  return catchnan(dot3m(p0, w[0], p1, w[1], p2, w[2]));
}

// The selectable alternatives (Schemes_Lagrange.cpp:358-594, 1265-1294), one side, compute type
// T: kind 3 weno5JS, 4 weno5Z, 5 weno5N, 6 teno5N, 7 teno5a.  tab: this side's TENO weights per
// cut-off pattern [8][3]; d: its optimal weights.  The WENO weights are scaled by the smallest
// denominator so float stays in range.
template <typename T>
__device__ __forceinline__ T alt_side(int kind, T p0, T p1, T p2, const T* v, const T (*tab)[3],
                                      const T* d) {
  T SI0, SI1, SI2, w0, w1, w2;
  if (kind == 5 || kind == 6) {
    SI2 = T(0.1) * fabs(v[0] - T(3.0) * v[1] + T(2.0) * v[2]) + fabs(v[0] - T(2.0) * v[1] + v[2]);
    SI1 = T(0.1) * fabs(v[3] - v[2]) + fabs(v[1] - T(2.0) * v[2] + v[3]);
    SI0 = T(0.1) * fabs(v[3] - v[2]) + fabs(v[2] - T(2.0) * v[3] + v[4]);
    const T x = fabs(v[0] - T(4.0) * v[1] + T(6.0) * v[2] - T(4.0) * v[3] + v[4]);
    const T e0 = SI0 + T(HTENO_LAG_EPS), e1 = SI1 + T(HTENO_LAG_EPS), e2 = SI2 + T(HTENO_LAG_EPS);
    if (kind == 5) {
      const T tau = x * x * sqrt(x);  // |.|^2.5
      w0 = d[0] * (T(1.0) + tau * Cst<T>::rcp(e0 * e0));
      w1 = d[1] * (T(1.0) + tau * Cst<T>::rcp(e1 * e1));
      w2 = d[2] * (T(1.0) + tau * Cst<T>::rcp(e2 * e2));
    } else {
      const T tau = x * x;
      const int pat = teno_pattern(T(1.0) + tau * Cst<T>::rcp(e0 * e0), T(1.0) + tau * Cst<T>::rcp(e1 * e1),
                                   T(1.0) + tau * Cst<T>::rcp(e2 * e2), T(HTENO_LAG_CT));
      return catchnan(p0 * tab[pat][0] + p1 * tab[pat][1] + p2 * tab[pat][2]);
    }
  } else {
    lagrange_si(v, SI0, SI1, SI2);
    if (kind == 3) {
      const T e0 = T(HTENO_LAG_EPS) + SI0, e1 = T(HTENO_LAG_EPS) + SI1, e2 = T(HTENO_LAG_EPS) + SI2;
      const T em = fmin(fmin(e0, e1), e2);
      const T a0 = em * Cst<T>::rcp(e0), a1 = em * Cst<T>::rcp(e1), a2 = em * Cst<T>::rcp(e2);
      w0 = d[0] * a0 * a0;
      w1 = d[1] * a1 * a1;
      w2 = d[2] * a2 * a2;
    } else if (kind == 4) {
      const T tau = fabs(SI2 - SI0), ez = Cst<T>::epsz();
      w0 = d[0] * (T(1.0) + tau * Cst<T>::rcp(SI0 + ez));
      w1 = d[1] * (T(1.0) + tau * Cst<T>::rcp(SI1 + ez));
      w2 = d[2] * (T(1.0) + tau * Cst<T>::rcp(SI2 + ez));
    } else {  // teno5a
      const T ez = Cst<T>::epsz();
      const int pat = teno_pattern(Cst<T>::rcp(SI0 + ez), Cst<T>::rcp(SI1 + ez), Cst<T>::rcp(SI2 + ez),
                                   T(HTENO_LAG_CT));
      return catchnan(p0 * tab[pat][0] + p1 * tab[pat][1] + p2 * tab[pat][2]);
    }
  }
  return catchnan((p0 * w0 + p1 * w1 + p2 * w2) * Cst<T>::rcp(w0 + w1 + w2));
}

// kind: 0 teno5, 1 teno5i, 2 linear, 3..7 the alternatives.  u[0..5] -> (u^-, u^+) at i+1/2.
template <typename T>
__device__ __forceinline__ void lagrange_recon(const DevConst& C, int kind, const T* u, T& outm,
                                               T& outp) {
  typedef Cst<T> K;
  T p0 = dot3m(K::crj(C, 0, 1), u[2], K::crj(C, 1, 1), u[3], K::crj(C, 2, 1), u[4]);
  T p1 = dot3m(K::crj(C, 0, 2), u[1], K::crj(C, 1, 2), u[2], K::crj(C, 2, 2), u[3]);
  T p2 = dot3m(K::crj(C, 0, 3), u[0], K::crj(C, 1, 3), u[1], K::crj(C, 2, 3), u[2]);
  if (kind == 2) {
    const T* w = K::wtab(C, 0, 7);
    outm = dot3m(p0, w[0], p1, w[1], p2, w[2]);
  } else if (kind >= 3) {
    outm = alt_side(kind, p0, p1, p2, u, reinterpret_cast<const T(*)[3]>(K::wtab(C, 0, 0)), K::wtab(C, 0, 7));
  } else {
    outm = teno_side(C, p0, p1, p2, u, 0, kind == 1);
  }
  p0 = dot3m(K::crj(C, 0, 0), u[3], K::crj(C, 1, 0), u[4], K::crj(C, 2, 0), u[5]);
  p1 = dot3m(K::crj(C, 0, 1), u[2], K::crj(C, 1, 1), u[3], K::crj(C, 2, 1), u[4]);
  p2 = dot3m(K::crj(C, 0, 2), u[1], K::crj(C, 1, 2), u[2], K::crj(C, 2, 2), u[3]);
  if (kind == 2) {
    const T* w = K::wtab(C, 1, 7);
    outp = dot3m(p0, w[0], p1, w[1], p2, w[2]);
  } else if (kind >= 3) {
    outp = alt_side(kind, p0, p1, p2, u + 1, reinterpret_cast<const T(*)[3]>(K::wtab(C, 1, 0)),
                    K::wtab(C, 1, 7));
  } else {
    outp = teno_side(C, p0, p1, p2, u + 1, 1, kind == 1);
  }
}

// weno5JS3PointsQuadrature (Schemes_Lagrange.cpp:1155-1217): face values at j-2..j+2 -> the
// three Gauss-Legendre points of face j.  Each output is sum(p_k lw_k / s_k) / sum(lw_k / s_k)
// with s_k = (eps + SI_k)^2, computed with one reciprocal per weight set.
template <typename T>
__device__ __forceinline__ void gl3(const DevConst& C, const T* u, T& o0, T& o1, T& o2) {
  typedef Cst<T> K;
  T bg0 = mad(T(3.0), u[2], mad(T(-4.0), u[1], u[0]));
  T cg0 = mad(T(-2.0), u[1], u[0]) + u[2];
  T bg1 = u[1] - u[3];
  T cg1 = mad(T(-2.0), u[2], u[1]) + u[3];
  T bg2 = mad(T(-4.0), u[3], T(3.0) * u[2]) + u[4];
  T cg2 = mad(T(-2.0), u[3], u[2]) + u[4];
  T s0 = T(HTENO_LAG_EPS) + mad(T(HTENO_C1) * cg0, cg0, T(0.25) * bg0 * bg0);
  T s1 = T(HTENO_LAG_EPS) + mad(T(HTENO_C1) * cg1, cg1, T(0.25) * bg1 * bg1);
  T s2 = T(HTENO_LAG_EPS) + mad(T(HTENO_C1) * cg2, cg2, T(0.25) * bg2 * bg2);
  s0 = s0 * s0; s1 = s1 * s1; s2 = s2 * s2;
  // alpha_k = 1 / s_k, scaled by the smallest s to keep float in range
  T smin = fmin(fmin(s0, s1), s2);
  T a0 = smin * K::rcp(s0), a1 = smin * K::rcp(s1), a2 = smin * K::rcp(s2);

  const T* lw = K::linwp(C);
  T g0 = lw[0] * a0, g1 = lw[1] * a1, g2 = lw[2] * a2;
  T q0 = dot3m(K::gp(C, 0, 0), u[0], K::gp(C, 1, 0), u[1], K::gp(C, 2, 0), u[2]);
  T q1 = dot3m(K::gp(C, 0, 1), u[1], K::gp(C, 1, 1), u[2], K::gp(C, 2, 1), u[3]);
  T q2 = dot3m(K::gp(C, 0, 2), u[2], K::gp(C, 1, 2), u[3], K::gp(C, 2, 2), u[4]);
  o0 = catchnan(dot3m(q0, g0, q1, g1, q2, g2) * K::rcp(g0 + g1 + g2));

  q0 = mad(T(23.0), u[2], mad(T(2.0), u[1], -u[0])) * T(1.0 / 24.0);
  q1 = (mad(T(26.0), u[2], -u[1]) - u[3]) * T(1.0 / 24.0);
  q2 = (mad(T(2.0), u[3], T(23.0) * u[2]) - u[4]) * T(1.0 / 24.0);
  lw = K::linw0p(C);
  g0 = lw[0] * a0; g1 = lw[1] * a1; g2 = lw[2] * a2;
  T c = K::sumw0p(C) * (dot3m(q0, g0, q1, g1, q2, g2) * K::rcp(g0 + g1 + g2));
  lw = K::linw0m(C);
  g0 = lw[0] * a0; g1 = lw[1] * a1; g2 = lw[2] * a2;
  o1 = catchnan(c - K::sumw0m(C) * (dot3m(q0, g0, q1, g1, q2, g2) * K::rcp(g0 + g1 + g2)));

  lw = K::linwm(C);
  g0 = lw[0] * a0; g1 = lw[1] * a1; g2 = lw[2] * a2;
  q0 = dot3m(K::gm(C, 0, 0), u[0], K::gm(C, 1, 0), u[1], K::gm(C, 2, 0), u[2]);
  q1 = dot3m(K::gm(C, 0, 1), u[1], K::gm(C, 1, 1), u[2], K::gm(C, 2, 1), u[3]);
  q2 = dot3m(K::gm(C, 0, 2), u[2], K::gm(C, 1, 2), u[3], K::gm(C, 2, 2), u[4]);
  o2 = catchnan(dot3m(q0, g0, q1, g1, q2, g2) * K::rcp(g0 + g1 + g2));
}

// ---------------------------------------------------------------------------------------------
// Equations::Euler2D
// ---------------------------------------------------------------------------------------------

// Roe-averaged face state (eigen2DEuler, FV_System2D.cpp:265-361).  The eigenvector matrices
// (right/leftEigenVectorx/y, Equations_Euler2D.cpp:100-205) are rebuilt from these scalars.
template <typename T>
struct Roe2 {
  T vxm, vym, hm, qm, cm, rcm, b1;  // b1 = gamma_1 / cm^2
};

template <typename T>
__device__ __forceinline__ Roe2<T> roe2(T g1, T ra, T ua, T va, T ha, T rb, T ub, T vb, T hb) {
  // ra, rb: sqrt(|rho|) of the two cells; u, v velocities; h total enthalpy
  Roe2<T> s;
  T t0 = ra * Cst<T>::rcp(ra + rb);
  T t1 = T(1.0) - t0;
  s.vxm = mad(t1, ub, t0 * ua);
  s.vym = mad(t1, vb, t0 * va);
  s.hm = mad(t1, hb, t0 * ha);
  s.qm = T(0.5) * mad(s.vym, s.vym, s.vxm * s.vxm);
  s.cm = Cst<T>::sqrt_(fabs(g1 * (s.hm - s.qm)));
  s.rcm = Cst<T>::rcp(s.cm);
  s.b1 = g1 * s.rcm * s.rcm;
  return s;
}

// L * q for the x (dir 1) or y (dir 2) face (leftEigenVectorx/y).
template <typename T>
__device__ __forceinline__ void roe_left(const Roe2<T>& s, int dir, const T* q, T* c) {
  const T vn = dir == 1 ? s.vxm : s.vym, vt = dir == 1 ? s.vym : s.vxm;
  const T b2 = s.qm * s.b1, s0 = vn * s.rcm, s1 = s.b1 * vn, t2 = T(0.5) * s.b1;
  const T qn = dir == 1 ? q[1] : q[2], qt = dir == 1 ? q[2] : q[1];
  // row 0: 0.5(b2 + s0), -0.5(s1 + rcm) [normal], -t2 vt [tangential], t2
  c[0] = mad(t2, q[3], mad(-t2 * vt, qt, mad(T(-0.5) * (s1 + s.rcm), qn, T(0.5) * (b2 + s0) * q[0])));
  c[1] = mad(-vt, q[0], qt);
  c[2] = mad(-s.b1, q[3], mad(s.b1 * vt, qt, mad(s1, qn, (T(1.0) - b2) * q[0])));
  c[3] = mad(t2, q[3], mad(-t2 * vt, qt, mad(T(-0.5) * (s1 - s.rcm), qn, T(0.5) * (b2 - s0) * q[0])));
}
// R * c (rightEigenVectorx/y)
template <typename T>
__device__ __forceinline__ void roe_right(const Roe2<T>& s, int dir, const T* c, T* q) {
  const T vn = dir == 1 ? s.vxm : s.vym, vt = dir == 1 ? s.vym : s.vxm;
  const T t0 = vn * s.cm;
  q[0] = c[0] + c[2] + c[3];
  const T qn = mad(vn + s.cm, c[3], mad(vn, c[2], (vn - s.cm) * c[0]));
  const T qt = mad(vt, c[3], mad(vt, c[2], mad(vt, c[0], c[1])));
  q[dir == 1 ? 1 : 2] = qn;
  q[dir == 1 ? 2 : 1] = qt;
  q[3] = mad(s.hm + t0, c[3], mad(s.qm, c[2], mad(vt, c[1], (s.hm - t0) * c[0])));
}

template <typename T>
__device__ __forceinline__ void primitive2(T g1, const T* q, T* w) {  // Euler2D::primitive :20-26
  T ir = fdiv(T(1.0), q[0]);
  w[0] = q[0];
  w[1] = q[1] * ir;
  w[2] = q[2] * ir;
  w[3] = (q[3] - T(0.5) * mad(q[2], w[2], q[1] * w[1])) * g1;
}

template <typename T>
__device__ __forceinline__ void flux2(int dir, const T* q, const T* w, T* f) {  // fluxx/fluxy
  if (dir == 1) {
    f[0] = q[1];
    f[1] = mad(q[1], w[1], w[3]);
    f[2] = q[1] * w[2];
    f[3] = w[1] * (q[3] + w[3]);
  } else {
    f[0] = q[2];
    f[1] = q[2] * w[1];
    f[2] = mad(q[2], w[2], w[3]);
    f[3] = w[2] * (q[3] + w[3]);
  }
}

// HLLC (Equations_Euler2D.cpp:372-428), with the reference's sound speeds sqrt(|p/rho|) and
// the left pressure in the right star energy.
template <typename T>
__device__ __forceinline__ void hllc2(T g1, int dir, const T* ql, const T* qr, T* F) {
  T wl[4], wr[4];
  const T il = Cst<T>::rcp(ql[0]), ir = Cst<T>::rcp(qr[0]);
  wl[0] = ql[0]; wl[1] = ql[1] * il; wl[2] = ql[2] * il;
  wl[3] = (ql[3] - T(0.5) * mad(ql[2], wl[2], ql[1] * wl[1])) * g1;
  wr[0] = qr[0]; wr[1] = qr[1] * ir; wr[2] = qr[2] * ir;
  wr[3] = (qr[3] - T(0.5) * mad(qr[2], wr[2], qr[1] * wr[1])) * g1;
  const T hl = (ql[3] + wl[3]) * il;
  const T hr = (qr[3] + wr[3]) * ir;
  const T rr = Cst<T>::sqrt_(fabs(wr[0] * il));
  const T rrr = Cst<T>::rcp(T(1.0) + rr);
  const T vm0 = mad(wr[1], rr, wl[1]) * rrr;
  const T vm1 = mad(wr[2], rr, wl[2]) * rrr;
  const T qm = T(0.5) * mad(vm1, vm1, vm0 * vm0);
  const T hm = mad(hr, rr, hl) * rrr;
  const T cm = Cst<T>::sqrt_(fabs(g1 * (hm - qm)));
  const T cl = Cst<T>::sqrt_(fabs(wl[3] * il));
  const T cr = Cst<T>::sqrt_(fabs(wr[3] * ir));
  const T vmd = dir == 1 ? vm0 : vm1;
  const T ul = wl[dir], ur = wr[dir];
  const T sl = fmin(ul - cl, vmd - cm);
  const T sr = fmax(ur + cr, vmd + cm);
  const T sm = (mad(-ql[dir], sl - ul, qr[dir] * (sr - ur)) + wl[3] - wr[3]) *
               Cst<T>::rcp(mad(-wl[0], sl - ul, wr[0] * (sr - ur)));
  const T ps = mad(wl[0] * (ul - sl), ul - sm, wl[3]);
  if (sl > T(0.0)) {
    flux2(dir, ql, wl, F);
  } else if (sl <= T(0.0) && sm > T(0.0)) {
    T fl[4];
    flux2(dir, ql, wl, fl);
    const T nom = sl - ul, iden = Cst<T>::rcp(sl - sm);
    T qs[4];
    qs[0] = wl[0] * nom * iden;
    qs[1] = dir == 1 ? (mad(nom, ql[1], ps) - wl[3]) * iden : nom * ql[1] * iden;
    qs[2] = dir == 2 ? (mad(nom, ql[2], ps) - wl[3]) * iden : nom * ql[2] * iden;
    qs[3] = mad(ps, sm, mad(-wl[3], ul, nom * ql[3])) * iden;
    for (int k = 0; k < 4; ++k) F[k] = mad(sl, qs[k] - ql[k], fl[k]);
  } else if (sm <= T(0.0) && sr >= T(0.0)) {
    T fr[4];
    flux2(dir, qr, wr, fr);
    const T nom = sr - ur, iden = Cst<T>::rcp(sr - sm);
    T qs[4];
    qs[0] = wr[0] * nom * iden;
    qs[1] = dir == 1 ? (mad(nom, qr[1], ps) - wr[3]) * iden : nom * qr[1] * iden;
    qs[2] = dir == 2 ? (mad(nom, qr[2], ps) - wr[3]) * iden : nom * qr[2] * iden;
    qs[3] = mad(ps, sm, mad(-wl[3], ur, nom * qr[3])) * iden;
    for (int k = 0; k < 4; ++k) F[k] = mad(sr, qs[k] - qr[k], fr[k]);
  } else {
    flux2(dir, qr, wr, F);
  }
}

// Characteristic Rusanov (Equations_Euler2D.cpp:310-330) with aM = maxLocalWaveSpeed (:221-246)
// as called in FV_System2D.cpp:460-464.
template <typename T>
__device__ __forceinline__ void rusanov2(T g, T g1, int dir, const Roe2<T>& s, const T* ql,
                                         const T* qr, T* F) {
  T wl[4], wr[4], fl[4], fr[4], d[4], m[4], a[4];
  primitive2(g1, ql, wl);
  primitive2(g1, qr, wr);
  const T cl = Cst<T>::sqrt_(fabs(fdiv(g * wl[3], wl[0])));
  const T cr = Cst<T>::sqrt_(fabs(fdiv(g * wr[3], wr[0])));
  const T vl = wl[dir], vr = wr[dir];
  a[0] = fmax(fabs(vl - cl), fabs(vr - cr));
  a[1] = fmax(fabs(vl), fabs(vr));
  a[2] = a[1];
  a[3] = fmax(fabs(vl + cl), fabs(vr + cr));
  flux2(dir, ql, wl, fl);
  flux2(dir, qr, wr, fr);
  for (int k = 0; k < 4; ++k) d[k] = qr[k] - ql[k];
  roe_left(s, dir, d, m);
  for (int k = 0; k < 4; ++k) m[k] = a[k] * m[k];
  T rm[4];
  roe_right(s, dir, m, rm);
  for (int k = 0; k < 4; ++k) F[k] = T(0.5) * (fl[k] + fr[k] - rm[k]);
}

// maxSpeed (Equations_Euler2D.cpp:207-219)
template <typename T>
__device__ __forceinline__ T max_speed2(T g, const T* w, int dir) {
  T c = Cst<T>::sqrt_(fabs(fdiv(g * w[3], w[0])));
  return fmax(w[dir] - c, fabs(w[dir] + c));
}

// Schemes::SSPRK::RungeKuttaIII (Schemes_SSPRK.cpp:3-15), always in double and without
// contraction, so the stage combination rounds exactly like the reference.
__device__ __forceinline__ double ssprk3(double q0, double qn, double rhs, double dt, int stage) {
  if (stage == 1) return __dadd_rn(q0, __dmul_rn(dt, rhs));
  if (stage == 2)
    return __dadd_rn(__dmul_rn(0.75, q0), __dmul_rn(0.25, __dadd_rn(qn, __dmul_rn(rhs, dt))));
  return __ddiv_rn(__dadd_rn(q0, __dmul_rn(2.0, __dadd_rn(qn, __dmul_rn(dt, rhs)))), 3.0);
}

// ---------------------------------------------------------------------------------------------
// Equations::Euler1D (3 conserved variables)
// ---------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void hllc1(T g1, const T* ql, const T* qr, T* F) {  // :156-210
  T wl[3], wr[3];
  const T il = T(1.0) / ql[0], ir = T(1.0) / qr[0];
  wl[0] = ql[0]; wl[1] = ql[1] * il; wl[2] = (ql[2] - T(0.5) * ql[1] * wl[1]) * g1;
  wr[0] = qr[0]; wr[1] = qr[1] * ir; wr[2] = (qr[2] - T(0.5) * qr[1] * wr[1]) * g1;
  const T hl = (ql[2] + wl[2]) * il, hr = (qr[2] + wr[2]) * ir;
  const T rr = Cst<T>::sqrt_(fabs(wr[0] * il));
  const T rrr = T(1.0) / (T(1.0) + rr);
  const T vm = (wl[1] + wr[1] * rr) * rrr;
  const T qm = T(0.5) * vm * vm;
  const T hm = (hl + hr * rr) * rrr;
  const T cm = Cst<T>::sqrt_(fabs(g1 * (hm - qm)));
  const T cl = Cst<T>::sqrt_(fabs(wl[2] * il));
  const T cr = Cst<T>::sqrt_(fabs(wr[2] * ir));
  const T sl = fmin(wl[1] - cl, vm - cm);
  const T sr = fmax(wr[1] + cr, vm + cm);
  const T sm = (qr[1] * (sr - wr[1]) - ql[1] * (sl - wl[1]) + wl[2] - wr[2]) /
               (wr[0] * (sr - wr[1]) - wl[0] * (sl - wl[1]));
  const T ps = wl[2] + wl[0] * (wl[1] - sl) * (wl[1] - sm);
  if (sl > T(0.0)) {
    F[0] = ql[1]; F[1] = ql[1] * wl[1] + wl[2]; F[2] = wl[1] * (ql[2] + wl[2]);
  } else if (sl <= T(0.0) && sm > T(0.0)) {
    const T fl[3] = {ql[1], ql[1] * wl[1] + wl[2], wl[1] * (ql[2] + wl[2])};
    const T nom = sl - wl[1], iden = T(1.0) / (sl - sm);
    const T qs[3] = {wl[0] * nom * iden, (nom * ql[1] + ps - wl[2]) * iden,
                     (nom * ql[2] - wl[2] * wl[1] + ps * sm) * iden};
    for (int k = 0; k < 3; ++k) F[k] = fl[k] + sl * (qs[k] - ql[k]);
  } else if (sm <= T(0.0) && sr >= T(0.0)) {
    const T fr[3] = {qr[1], qr[1] * wr[1] + wr[2], wr[1] * (qr[2] + wr[2])};
    const T nom = sr - wr[1], iden = T(1.0) / (sr - sm);
    const T qs[3] = {wr[0] * nom * iden, (nom * qr[1] + ps - wr[2]) * iden,
                     (nom * qr[2] - wl[2] * wr[1] + ps * sm) * iden};
    for (int k = 0; k < 3; ++k) F[k] = fr[k] + sr * (qs[k] - qr[k]);
  } else {
    F[0] = qr[1]; F[1] = qr[1] * wr[1] + wr[2]; F[2] = wr[1] * (qr[2] + wr[2]);
  }
}

// Roe-averaged face state in 1D (eigen1DEuler, FV_System1D.cpp:121-156); eigenvector matrices
// rightEigenVector / leftEigenVector (Equations_Euler1D.cpp:55-89) are applied from these.
template <typename T>
struct Roe1 {
  T vxm, hm, qm, cm, rcm, b1;
};
template <typename T>
__device__ __forceinline__ Roe1<T> roe1(T g1, T ra, T ua, T ha, T rb, T ub, T hb) {
  Roe1<T> s;
  T t0 = ra / (ra + rb);
  T t1 = T(1.0) - t0;
  s.vxm = t0 * ua + t1 * ub;
  s.hm = t0 * ha + t1 * hb;
  s.qm = T(0.5) * s.vxm * s.vxm;
  s.cm = Cst<T>::sqrt_(fabs(g1 * (s.hm - s.qm)));
  s.rcm = T(1.0) / s.cm;
  s.b1 = g1 * s.rcm * s.rcm;
  return s;
}
template <typename T>
__device__ __forceinline__ void roe1_left(const Roe1<T>& s, const T* q, T* c) {
  const T b2 = s.qm * s.b1, s0 = s.vxm * s.rcm, s1 = s.b1 * s.vxm, t2 = T(0.5) * s.b1;
  c[0] = T(0.5) * (b2 + s0) * q[0] + T(-0.5) * (s1 + s.rcm) * q[1] + t2 * q[2];
  c[1] = (T(1.0) - b2) * q[0] + s1 * q[1] + (-s.b1) * q[2];
  c[2] = T(0.5) * (b2 - s0) * q[0] + T(-0.5) * (s1 - s.rcm) * q[1] + t2 * q[2];
}
template <typename T>
__device__ __forceinline__ void roe1_right(const Roe1<T>& s, const T* c, T* q) {
  const T t0 = s.vxm * s.cm;
  q[0] = c[0] + c[1] + c[2];
  q[1] = (s.vxm - s.cm) * c[0] + s.vxm * c[1] + (s.vxm + s.cm) * c[2];
  q[2] = (s.hm - t0) * c[0] + s.qm * c[1] + (s.hm + t0) * c[2];
}
template <typename T>
__device__ __forceinline__ void primitive1(T g1, const T* q, T* w) {  // Euler1D::primitive
  w[0] = q[0];
  w[1] = q[1] / q[0];
  w[2] = (q[2] - T(0.5) * q[1] * w[1]) * g1;
}
// maxLocalWaveSpeed (Equations_Euler1D.cpp:96-107)
template <typename T>
__device__ __forceinline__ void local_speed1(T g, const T* wl, const T* wr, T* a) {
  const T cl = Cst<T>::sqrt_(fabs(g * wl[2] / wl[0]));
  const T cr = Cst<T>::sqrt_(fabs(g * wr[2] / wr[0]));
  a[0] = fmax(fabs(wl[1] - cl), fabs(wr[1] - cr));
  a[1] = fmax(fabs(wl[1]), fabs(wr[1]));
  a[2] = fmax(fabs(wl[1] + cl), fabs(wr[1] + cr));
}
// characteristic Rusanov (Equations_Euler1D.cpp:129-135)
template <typename T>
__device__ __forceinline__ void rusanov1(T g, T g1, const Roe1<T>& s, const T* ql, const T* qr,
                                         T* F) {
  T wl[3], wr[3], a[3], d[3], m[3], rm[3];
  primitive1(g1, ql, wl);
  primitive1(g1, qr, wr);
  local_speed1(g, wl, wr, a);
  for (int k = 0; k < 3; ++k) d[k] = qr[k] - ql[k];
  roe1_left(s, d, m);
  for (int k = 0; k < 3; ++k) m[k] = a[k] * m[k];
  roe1_right(s, m, rm);
  const T fl[3] = {ql[1], ql[1] * wl[1] + wl[2], wl[1] * (ql[2] + wl[2])};
  const T fr[3] = {qr[1], qr[1] * wr[1] + wr[2], wr[1] * (qr[2] + wr[2])};
  for (int k = 0; k < 3; ++k) F[k] = T(0.5) * (fl[k] + fr[k] - rm[k]);
}
// dflux (Equations_Euler1D.cpp:39-53) applied to x
template <typename T>
__device__ __forceinline__ void dflux1_apply(T g, T g1, const T* q, const T* w, const T* x, T* y) {
  const T g3 = g1 - T(2.0);
  const T u = w[1];
  y[0] = x[1];
  y[1] = T(0.5) * g3 * u * u * x[0] + (-g3 * u) * x[1] + g1 * x[2];
  const T e = g * q[2] / w[0];
  y[2] = (g1 * u * u - e) * u * x[0] + (e - T(1.5) * g1 * u * u) * x[1] + g * u * x[2];
}
// dRusanov (Equations_Euler1D.cpp:212-220)
template <typename T>
__device__ __forceinline__ void drusanov1(T g, T g1, const Roe1<T>& s, const T* ql, const T* qr,
                                          const T* dql, const T* dqr, T* F) {
  T wl[3], wr[3], a[3], d[3], m[3], rm[3], al[3], ar[3];
  primitive1(g1, ql, wl);
  primitive1(g1, qr, wr);
  local_speed1(g, wl, wr, a);
  dflux1_apply(g, g1, ql, wl, dql, al);
  dflux1_apply(g, g1, qr, wr, dqr, ar);
  for (int k = 0; k < 3; ++k) d[k] = dqr[k] - dql[k];
  roe1_left(s, d, m);
  for (int k = 0; k < 3; ++k) m[k] = a[k] * m[k];
  roe1_right(s, m, rm);
  for (int k = 0; k < 3; ++k) F[k] = T(0.5) * (al[k] + ar[k] - rm[k]);
}
// maxSpeed (Equations_Euler1D.cpp:91-94)
__device__ __forceinline__ double max_speed1(double g, const double* w) {
  const double c = sqrt(fabs(g * w[2] / w[0]));
  return fmax(fabs(w[1] - c), fabs(w[1] + c));
}

}  // namespace hteno
