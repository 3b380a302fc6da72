// Device numerics of the Hermite schemes (Schemes_Hermite.cpp) and the derivative-moment flux
// (Equations_Euler2D.cpp:52-98, 352-360).  Same conventions as device_math.cuh.
#pragma once

#include "device_math.cuh"

namespace hteno {

// Grid-size dependent coefficients of Schemes::Hermite::setGridSize (Schemes_Hermite.cpp:15-92).
template <typename T>
struct HermiteK {
  T dif, rdif;
  T crj[3][3], crjd[4][3], crjlin[5][2], crjlind[6][2];
};

template <typename T>
inline HermiteK<T> make_hermite_k(double dif) {
  double crj[3][3], crjd[4][3], lin[5][2], lind[6][2];
  crj[0][0] = -7.0 / 6.0;
  crj[1][0] = 13.0 / 6.0;
  crj[2][0] = -2.0 / 3.0 * dif;
  crj[0][1] = 1.0 / 6.0;
  crj[1][1] = 5.0 / 6.0;
  crj[2][1] = -1.0 / 3.0 * dif;
  crj[0][2] = -1.0 / 6.0;
  crj[1][2] = 5.0 / 6.0;
  crj[2][2] = 1.0 / 3.0;
  crjd[0][0] = 4.0 / dif;
  crjd[1][0] = -4.0 / dif;
  crjd[2][0] = 1.5;
  crjd[3][0] = 3.5;
  crjd[0][1] = -2.0 / dif;
  crjd[1][1] = 2.0 / dif;
  crjd[2][1] = -0.5;
  crjd[3][1] = -0.5;
  crjd[0][2] = 0.25 / dif;
  crjd[1][2] = -1.0 / dif;
  crjd[2][2] = 0.75 / dif;
  crjd[3][2] = 0.5;
  lin[0][0] = -23.0 / 120.0;
  lin[1][0] = 19.0 / 30.0;
  lin[2][0] = 67.0 / 120.0;
  lin[3][0] = -3.0 / 40.0 * dif;
  lin[4][0] = -7.0 / 40.0 * dif;
  lin[0][1] = 67.0 / 120.0;
  lin[1][1] = 19.0 / 30.0;
  lin[2][1] = -23.0 / 120.0;
  lin[3][1] = 7.0 / 40.0 * dif;
  lin[4][1] = 3.0 / 40.0 * dif;
  lind[0][0] = 0.25 / dif;
  lind[1][0] = -2.0 / dif;
  lind[2][0] = 1.75 / dif;
  lind[3][0] = 1.0 / 12.0;
  lind[4][0] = -1.0 / 6.0;
  lind[5][0] = -5.0 / 12.0;
  lind[0][1] = -7.0 / 4.0 / dif;
  lind[1][1] = 2.0 / dif;
  lind[2][1] = -0.25 / dif;
  lind[3][1] = -5.0 / 12.0;
  lind[4][1] = -1.0 / 6.0;
  lind[5][1] = 1.0 / 12.0;
  HermiteK<T> k;
  k.dif = T(dif);
  k.rdif = T(1.0 / dif);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) k.crj[i][j] = T(crj[i][j]);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) k.crjd[i][j] = T(crjd[i][j]);
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 2; ++j) k.crjlin[i][j] = T(lin[i][j]);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 2; ++j) k.crjlind[i][j] = T(lind[i][j]);
  return k;
}

// smoothnessMeasure (Schemes_Hermite.cpp:515-526)
template <typename T>
__device__ __forceinline__ void hermite_si(const T* u, const T* v, T& S0, T& S1, T& S2) {
  T b0 = T(-2.0) * (u[0] - u[1]) - v[0];
  T c0 = T(-2.0) * (u[0] - u[1] + v[0]);
  T b1 = T(-2.0) * (u[1] - u[2]) - v[2];
  T c1 = T(2.0) * (u[1] - u[2]) + T(2.0) * v[2];
  T b2 = (u[2] - u[0]) * T(0.5);
  T c2 = u[0] - T(2.0) * u[1] + u[2];
  S0 = T(HTENO_C1) * c0 * c0 + b0 * b0;
  S1 = T(HTENO_C1) * c1 * c1 + b1 * b1;
  S2 = T(HTENO_C1) * c2 * c2 + b2 * b2;
}
// smoothnessMeasureDerivative (:528-541)
template <typename T>
__device__ __forceinline__ void hermite_sid(const T* u, const T* d, T& S0, T& S1, T& S2) {
  T b0 = T(6.0) * (u[0] - u[1]) + (T(2.0) * d[0] + T(4.0) * d[1]);
  T c0 = T(12.0) * (u[0] - u[1]) + T(6.0) * (d[0] + d[1]);
  T b1 = T(6.0) * (u[2] - u[1]) - (T(4.0) * d[1] + T(2.0) * d[2]);
  T c1 = T(12.0) * (u[1] - u[2]) + T(6.0) * (d[1] + d[2]);
  T b2 = u[0] - T(2.0) * u[1] + u[2];
  T c2 = T(3.0) * (u[2] - u[0]) - T(6.0) * d[1];
  S0 = T(HTENO_C1) * c0 * c0 + b0 * b0;
  S1 = T(HTENO_C1) * c1 * c1 + b1 * b1;
  S2 = T(HTENO_C1) * c2 * c2 + b2 * b2;
}
// fullPointsSI (:597-603)
template <typename T>
__device__ __forceinline__ T hermite_brk(const T* u, const T* d) {
  return fabs((T(1029270.0) * u[2] - T(2129184.0) * u[1] + T(1099914.0) * u[0] +
               T(281121.0) * d[0] - T(494958.0) * d[2]) * d[0] +
              (T(-1029270.0) * u[0] + T(2129184.0) * u[1] - T(1099914.0) * u[2] +
               T(281121.0) * d[2]) * d[2] +
              (T(1099445.0) * u[2] - T(4317056.0) * u[1] + T(2118166.0) * u[0]) * u[2] +
              T(4317056.0) * (u[1] - u[0]) * u[1] + T(1099445.0) * u[0] * u[0]) *
         T(1.0 / 6720.0);
}
// fullPointsSId (:605-612)
template <typename T>
__device__ __forceinline__ T hermite_brkd(const T* u, const T* d) {
  return fabs((T(3156862.0) * d[2] + T(13189240.0) * d[1] + T(1710479.0) * d[0] -
               T(9617754.0) * u[2] - T(531552.0) * u[1] + T(10149306.0) * u[0]) * d[0] +
              (T(13189240.0) * d[2] + T(26511200.0) * d[1] - T(39700440.0) * u[2] +
               T(39700440.0) * u[0]) * d[1] +
              (T(1710479.0) * d[2] - T(10149306.0) * u[2] + T(531552.0) * u[1] +
               T(9617754.0) * u[0]) * d[2] +
              (T(15136011.0) * u[2] - T(1076544.0) * u[1] - T(29195478.0) * u[0]) * u[2] +
              T(1076544.0) * (u[1] - u[0]) * u[1] + T(15136011.0) * u[0] * u[0]) *
         T(1.0 / 1680.0);
}

// Weighted value of one hteno/htenoi output (cutOff/cutOffd, :614-628, ct = ctd = 1e-3).
template <typename T>
__device__ __forceinline__ T hermite_weighted(const DevConst& C, int which, T p0, T p1, T p2, T S0,
                                              T S1, T S2, T tau) {
  const T ez = Cst<T>::epsz();
  T r0 = T(1.0) + tau * Cst<T>::rcp(S0 + ez);
  T r1 = T(1.0) + tau * Cst<T>::rcp(S1 + ez);
  T r2 = T(1.0) + tau * Cst<T>::rcp(S2 + ez);
  int pat = teno_pattern(r0, r1, r2, T(HTENO_HER_CT));
  const T* w = Cst<T>::hwtab(C, which, pat);
  return catchnan(p0 * w[0] + p1 * w[1] + p2 * w[2]);
}

// kind: 0 hteno (:295-379), 1 htenoi (:670-758), 2 linear (:760-812).
// out = {u^-_{i+1/2}, u^+_{i+1/2}, d^-_{i+1/2}, d^+_{i+1/2}}
template <typename T>
__device__ __forceinline__ void hermite_recon(const DevConst& C, const HermiteK<T>& K, int kind,
                                              const T* u, const T* d, T* out) {
  if (kind == 2) {
    out[0] = K.crjlin[0][0] * u[0] + K.crjlin[1][0] * u[1] + K.crjlin[2][0] * u[2] +
             K.crjlin[3][0] * d[0] + K.crjlin[4][0] * d[2];
    out[1] = K.crjlin[0][1] * u[1] + K.crjlin[1][1] * u[2] + K.crjlin[2][1] * u[3] +
             K.crjlin[3][1] * d[1] + K.crjlin[4][1] * d[3];
    out[2] = K.crjlind[0][0] * u[0] + K.crjlind[1][0] * u[1] + K.crjlind[2][0] * u[2] +
             (K.crjlind[3][0] * d[0] + K.crjlind[4][0] * d[1] + K.crjlind[5][0] * d[2]);
    out[3] = K.crjlind[0][1] * u[1] + K.crjlind[1][1] * u[2] + K.crjlind[2][1] * u[3] +
             (K.crjlind[3][1] * d[1] + K.crjlind[4][1] * d[2] + K.crjlind[5][1] * d[3]);
    return;
  }
  const bool imp = kind == 1;
  T ud[4];
  for (int k = 0; k < 4; ++k) ud[k] = d[k] * K.dif;
  T p0, p1, p2, S0, S1, S2, tau;

  // u^-_{i+1/2}
  p0 = K.crj[0][0] * u[0] + K.crj[1][0] * u[1] + K.crj[2][0] * d[0];
  p1 = K.crj[0][1] * u[1] + K.crj[1][1] * u[2] + K.crj[2][1] * d[2];
  p2 = K.crj[0][2] * u[0] + K.crj[1][2] * u[1] + K.crj[2][2] * u[2];
  hermite_si(u, ud, S0, S1, S2);
  tau = imp ? fmax(fmax(S0, S1), S2)
            : fabs(hermite_brk(u, ud) - T(0.25) * (S0 + S1 + T(2.0) * S2));
  out[0] = hermite_weighted(C, 0, p0, p1, p2, S0, S1, S2, tau);

  // d^-_{i+1/2}
  p0 = K.crjd[0][0] * u[0] + K.crjd[1][0] * u[1] + K.crjd[2][0] * d[0] + K.crjd[3][0] * d[1];
  p1 = K.crjd[0][1] * u[1] + K.crjd[1][1] * u[2] + K.crjd[2][1] * d[1] + K.crjd[3][1] * d[2];
  p2 = K.crjd[0][2] * u[0] + K.crjd[1][2] * u[1] + K.crjd[2][2] * u[2] + K.crjd[3][2] * d[1];
  hermite_sid(u, ud, S0, S1, S2);
  tau = imp ? fmax(fmax(S0, S1), S2)
            : fabs(hermite_brkd(u, ud) - T(0.25) * (S0 + S1 + T(2.0) * S2));
  out[2] = hermite_weighted(C, 2, p0, p1, p2, S0, S1, S2, tau);

  // u^+_{i+1/2}
  p0 = K.crj[1][1] * u[1] + K.crj[0][1] * u[2] - K.crj[2][1] * d[1];
  p1 = K.crj[1][0] * u[2] + K.crj[0][0] * u[3] - K.crj[2][0] * d[3];
  p2 = K.crj[2][2] * u[1] + K.crj[1][2] * u[2] + K.crj[0][2] * u[3];
  hermite_si(u + 1, ud + 1, S0, S1, S2);
  tau = imp ? fmax(fmax(S0, S1), S2)
            : fabs(hermite_brk(u + 1, ud + 1) - T(0.25) * (S0 + S1 + T(2.0) * S2));
  out[1] = hermite_weighted(C, 1, p0, p1, p2, S0, S1, S2, tau);

  // d^+_{i+1/2}
  p0 = K.crjd[0][1] * u[1] + K.crjd[1][1] * u[2] + K.crjd[3][1] * d[1] + K.crjd[2][1] * d[2];
  p1 = K.crjd[0][0] * u[2] + K.crjd[1][0] * u[3] + K.crjd[3][0] * d[2] + K.crjd[2][0] * d[3];
  p2 = -(K.crjd[2][2] * u[1] + K.crjd[1][2] * u[2] + K.crjd[0][2] * u[3]) + K.crjd[3][2] * d[2];
  hermite_sid(u + 1, ud + 1, S0, S1, S2);
  tau = imp ? fmax(fmax(S0, S1), S2)
            : fabs(hermite_brkd(u + 1, ud + 1) - T(0.25) * (S0 + S1 + T(2.0) * S2));
  out[3] = hermite_weighted(C, 3, p0, p1, p2, S0, S1, S2, tau);
}

// hermiteLimiter (Schemes_Hermite.cpp:634-662)
template <typename T>
__device__ __forceinline__ T hermite_limiter(const HermiteK<T>& K, const T* u, const T* d) {
  const T p0 = T(0.75) * (u[2] - u[0]) * K.rdif - T(0.25) * (d[0] + d[2]);
  const T p1 = (u[1] - u[0]) * K.rdif;
  const T p2 = (u[2] - u[1]) * K.rdif;
  const T lw0 = T(1.0 - 2E-5), lw1 = T(1E-5), lw2 = T(1E-5);
  T ud[3] = {d[0] * K.dif, d[1] * K.dif, d[2] * K.dif};
  const T s0 = hermite_brk(u, ud);
  const T s1 = (u[0] - u[1]) * (u[0] - u[1]);
  const T s2 = (u[1] - u[2]) * (u[1] - u[2]);
  T tau = fabs(s0 - s1) + fabs(s0 - s2);
  tau = tau * tau * T(0.25);
  const T w0 = lw0 * (T(1.0) + tau / (s0 + T(HTENO_LAG_EPS)));
  const T w1 = lw1 * (T(1.0) + tau / (s1 + T(HTENO_LAG_EPS)));
  const T w2 = lw2 * (T(1.0) + tau / (s2 + T(HTENO_LAG_EPS)));
  const T is = T(1.0) / (w0 + w1 + w2);
  const T r1 = lw1 / lw0, r2 = lw2 / lw0;
  return (w0 * is) * (p0 / lw0 - (r1 * p1 + r2 * p2)) + ((w1 * is) * p1 + (w2 * is) * p2);
}

// dfluxx / dfluxy (Equations_Euler2D.cpp:52-98) applied to a vector: A(q) * x
template <typename T>
__device__ __forceinline__ void dflux2_apply(T g, T g1, int dir, const T* q, const T* w,
                                             const T* x, T* y) {
  const T g3 = g1 - T(2.0);
  const T un = dir == 1 ? w[1] : w[2], ut = dir == 1 ? w[2] : w[1];
  const T xn = dir == 1 ? x[1] : x[2], xt = dir == 1 ? x[2] : x[1];
  const T sv = un * un;
  const T dv = T(0.5) * g1 * (sv + ut * ut);
  const T h = fdiv(q[3] + w[3], w[0]);
  y[0] = xn;
  // normal momentum row: (dv - sv, -g3 un, -g1 ut, g1)
  const T yn = (dv - sv) * x[0] + (-g3 * un) * xn + (-g1 * ut) * xt + g1 * x[3];
  // tangential momentum row: (-un ut, ut, un, 0)  [x: (-w1 w2, w2, w1, 0) on (q0, q1, q2, q3)]
  const T yt = (-un * ut) * x[0] + ut * xn + un * xt;
  y[dir == 1 ? 1 : 2] = yn;
  y[dir == 1 ? 2 : 1] = yt;
  y[3] = (dv - h) * un * x[0] + (h - g1 * sv) * xn + (-g1 * un * ut) * xt + g * un * x[3];
}

// dRusanov (:352-360) with aM = maxLocalWaveSpeed(w(ql), w(qr)) as in
// FVHermite_System2D.cpp:553-589.
template <typename T>
__device__ __forceinline__ void drusanov2(T g, T g1, int dir, const Roe2<T>& s, const T* ql,
                                          const T* qr, const T* dql, const T* dqr, T* F) {
  T wl[4], wr[4], a[4], d[4], m[4], al[4], ar[4], rm[4];
  primitive2(g1, ql, wl);
  primitive2(g1, qr, wr);
  const T cl = Cst<T>::sqrt_(fabs(fdiv(g * wl[3], wl[0])));
  const T cr = Cst<T>::sqrt_(fabs(fdiv(g * wr[3], wr[0])));
  const T vl = wl[dir], vr = wr[dir];
  a[0] = fmax(fabs(vl - cl), fabs(vr - cr));
  a[1] = fmax(fabs(vl), fabs(vr));
  a[2] = a[1];
  a[3] = fmax(fabs(vl + cl), fabs(vr + cr));
  dflux2_apply(g, g1, dir, ql, wl, dql, al);
  dflux2_apply(g, g1, dir, qr, wr, dqr, ar);
  for (int k = 0; k < 4; ++k) d[k] = dqr[k] - dql[k];
  roe_left(s, dir, d, m);
  for (int k = 0; k < 4; ++k) m[k] = a[k] * m[k];
  roe_right(s, dir, m, rm);
  for (int k = 0; k < 4; ++k) F[k] = T(0.5) * (al[k] + ar[k] - rm[k]);
}

}  // namespace hteno
