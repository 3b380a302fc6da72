// CPU oracle: a restatement of the reference solver's hot path (indrow/Hermite-TENO), written
// for this project as test infrastructure.  It is the checker for the CUDA library, never
// part of it: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
//
// Parity pinning: every scheme, flux and solver here is validated against the reference's own
// sources compiled unmodified against oracle/eigen_compat (oracle/ref_driver.cpp, built by
// oracle/Makefile into oracle/_ref/).  With -ffp-contract=off the two agree bitwise.
//
// Arithmetic order: each expression keeps the reference's per-coefficient expression tree;
// reductions (dot products, sums, matrix-vector rows, rowwise sums) run left to right.
//
// Layout: SoA planes q[var][j][i], interior cells only.  Ghost cells are never stored: the
// reference's ghost fills (zeroGradBc, periodicBc) copy interior cells, so a ghost read equals
// an interior read at a clamped (zero-gradient) or wrapped (periodic) index.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace orc {

using std::fabs;
using std::fmax;
using std::fmin;
using std::pow;
using std::sqrt;

template <typename T>
inline T catchnan(T x, T machine_eps) {  // Schemes_Lagrange.cpp:1151-1153
  using std::isnan;
  return isnan(x) ? machine_eps : x;
}

// =============================================================================================
// Schemes::Lagrange coefficients (Schemes_Lagrange.cpp:6-304, only the live entries)
// =============================================================================================
struct LagrangeCoef {
  double eps = 1e-6, machine_eps = 1e-15, epsz = 1e-40, ct = 5e-4, c1 = 13.0 / 12.0;
  double crj[3][4];     // crj(r, c)  (Schemes_Lagrange.cpp:125-136)
  double dkm[3], dkp[3];  // :140-142
  double gp[3][3], gm[3][3];  // crjgp3L / crjgm3L (r, c)  :65-83
  double linwp[3], linwm[3], linw0p[3], linw0m[3], sumw0p, sumw0m;  // :86-104
  double gl3w[3];  // three-point Gauss-Legendre weights / 2 (FV_System2D.cpp:28, :61-62)

  LagrangeCoef() {
    const double sq15 = sqrt(15.0);
    gp[0][0] = 1.0 / 30.0 + sq15 / 20.0;
    gp[1][0] = -1.0 / 15.0 - sq15 / 5.0;
    gp[2][0] = 31.0 / 30.0 + 3.0 * sq15 / 20.0;
    gp[0][1] = 1.0 / 30.0 - sq15 / 20.0;
    gp[1][1] = 14.0 / 15.0;
    gp[2][1] = 1.0 / 30.0 + sq15 / 20.0;
    gp[0][2] = 31.0 / 30.0 - 3.0 * sq15 / 20.0;
    gp[1][2] = -1.0 / 15.0 + sq15 / 5.0;
    gp[2][2] = 1.0 / 30.0 - sq15 / 20.0;

    gm[0][0] = 1.0 / 30.0 - sq15 / 20.0;
    gm[1][0] = -1.0 / 15.0 + sq15 / 5.0;
    gm[2][0] = 31.0 / 30.0 - 3.0 * sq15 / 20.0;
    gm[0][1] = 1.0 / 30.0 + sq15 / 20.0;
    gm[1][1] = 14.0 / 15.0;
    gm[2][1] = 1.0 / 30.0 - sq15 / 20.0;
    gm[0][2] = 31.0 / 30.0 + 3.0 * sq15 / 20.0;
    gm[1][2] = -1.0 / 15.0 - sq15 / 5.0;
    gm[2][2] = 1.0 / 30.0 + sq15 / 20.0;

    double lin0[3] = {-9.0 / 80.0, 49.0 / 40.0, -9.0 / 80.0};
    for (int i = 0; i < 3; ++i) {
      linw0p[i] = 0.5 * (lin0[i] + 3.0 * fabs(lin0[i]));
      linw0m[i] = linw0p[i] - lin0[i];
    }
    sumw0p = (linw0p[0] + linw0p[1]) + linw0p[2];
    sumw0m = (linw0m[0] + linw0m[1]) + linw0m[2];
    for (int i = 0; i < 3; ++i) {
      linw0p[i] = linw0p[i] / sumw0p;
      linw0m[i] = linw0m[i] / sumw0m;
    }
    double den = 15720.0 * sq15 + 10480.0;
    linwp[0] = (2882.0 * sq15 - 1179.0) / den;
    linwp[1] = (9672.0 * sq15 + 6448.0) / den;
    linwp[2] = (3166.0 * sq15 + 5211.0) / den;
    den = 15720.0 * sq15 - 10480;
    linwm[0] = (2882.0 * sq15 + 1179.0) / den;
    linwm[1] = (9672.0 * sq15 - 6448.0) / den;
    linwm[2] = (3166.0 * sq15 - 5211.0) / den;

    const double c[3][4] = {{11.0 / 6.0, 1.0 / 3.0, -1.0 / 6.0, 1.0 / 3.0},
                            {-7.0 / 6.0, 5.0 / 6.0, 5.0 / 6.0, -7.0 / 6.0},
                            {1.0 / 3.0, -1.0 / 6.0, 1.0 / 3.0, 11.0 / 6.0}};
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 4; ++k) crj[r][k] = c[r][k];
    dkm[0] = 0.3; dkm[1] = 0.6; dkm[2] = 0.1;
    dkp[0] = 0.1; dkp[1] = 0.6; dkp[2] = 0.3;
    gl3w[0] = 5.0 / 9.0 / 2.0;
    gl3w[1] = 8.0 / 9.0 / 2.0;
    gl3w[2] = 5.0 / 9.0 / 2.0;
  }
};

inline const LagrangeCoef& lag() {
  static const LagrangeCoef c;
  return c;
}

template <typename T>
inline T dot3c(const double* cc, int stride, const T* u) {  // column of a coefficient matrix . u
  T s = T(cc[0]) * u[0];
  s = s + T(cc[stride]) * u[1];
  s = s + T(cc[2 * stride]) * u[2];
  return s;
}
template <typename T>
inline T dot3(const T* a, const T* b) {
  T s = a[0] * b[0];
  s = s + a[1] * b[1];
  s = s + a[2] * b[2];
  return s;
}

// smoothnessMeasure (Schemes_Lagrange.cpp:1013-1026) on v[0..4]
template <typename T>
inline void lagrange_si(const T* v, T* SI) {
  const LagrangeCoef& K = lag();
  T c[3], b[3];
  c[0] = v[2] - T(2.0) * v[3] + v[4];
  b[0] = T(3.0) * v[2] - T(4.0) * v[3] + v[4];
  c[1] = v[1] - T(2.0) * v[2] + v[3];
  b[1] = v[1] - v[3];
  c[2] = v[0] - T(2.0) * v[1] + v[2];
  b[2] = v[0] - T(4.0) * v[1] + T(3.0) * v[2];
  for (int k = 0; k < 3; ++k) b[k] = b[k] / T(2.0);
  for (int k = 0; k < 3; ++k) SI[k] = b[k] * b[k] + T(K.c1) * c[k] * c[k];
}

// fullpointsSmootness (Schemes_Lagrange.cpp:1029-1034) on v[0..4]
template <typename T>
inline T lagrange_b35(const T* v) {
  T r = v[4] * (T(6908.0) * v[4] - T(51001.0) * v[3] + T(67923.0) * v[2] - T(38947.0) * v[1] +
                T(8209.0) * v[0]) +
        v[3] * (T(104963.0) * v[3] - T(299076.0) * v[2] + T(179098.0) * v[1] - T(38947.0) * v[0]) +
        v[2] * (T(231153.0) * v[2] - T(299076.0) * v[1] + T(67923.0) * v[0]) +
        v[1] * (T(104963.0) * v[1] - T(51001.0) * v[0]) + T(6908.0) * v[0] * v[0];
  return r / T(5040.0);
}

// One side of teno5 / teno5i given candidates p, stencil v[0..4], optimal weights d.
// improved = false: tau = |b35 - (SI0 + SI2 + 4 SI1)/6| (teno5, :481-511)
// improved = true : tau = max(SI)                         (teno5i, :1235-1263)
template <typename T>
inline T teno_side(const T* p, const T* v, const double* d, bool improved) {
  const LagrangeCoef& K = lag();
  T SI[3];
  lagrange_si(v, SI);
  T tau;
  if (!improved) {
    T b35 = lagrange_b35(v);
    tau = fabs(b35 - (SI[0] + SI[2] + T(4.0) * SI[1]) / T(6.0));
  } else {
    tau = SI[0];
    tau = (tau < SI[1]) ? SI[1] : tau;
    tau = (tau < SI[2]) ? SI[2] : tau;
  }
  T w[3];
  for (int k = 0; k < 3; ++k) w[k] = pow(T(1.0) + tau / (SI[k] + T(K.epsz)), T(6));
  // cutOff (:1141-1149)
  T s = (w[0] + w[1]) + w[2];
  T sig[3];
  for (int k = 0; k < 3; ++k) {
    w[k] = w[k] / s;
    sig[k] = w[k] < T(K.ct) ? T(0.0) : T(1.0);
  }
  for (int k = 0; k < 3; ++k) w[k] = sig[k] * T(d[k]);
  s = (w[0] + w[1]) + w[2];
  for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  return catchnan(dot3(p, w), T(K.machine_eps));
}

// The selectable alternatives of Schemes::Lagrange, one side each.  v[0..4] is the side's
// 5-cell window (the left side's u[0..4], the right side's u[1..5]), as smoothnessMeasure sees it.

// cutOff (:1141-1149) of raw weights w followed by the sigma-weighted optimal weights
template <typename T>
inline T cutoff_weighted(const T* p, T* w, const double* d) {
  const LagrangeCoef& K = lag();
  T s = (w[0] + w[1]) + w[2];
  T sig[3];
  for (int k = 0; k < 3; ++k) {
    w[k] = w[k] / s;
    sig[k] = w[k] < T(K.ct) ? T(0.0) : T(1.0);
  }
  for (int k = 0; k < 3; ++k) w[k] = sig[k] * T(d[k]);
  s = (w[0] + w[1]) + w[2];
  for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  return catchnan(dot3(p, w), T(K.machine_eps));
}

template <typename T>
inline T normalised(const T* p, T* w) {
  const LagrangeCoef& K = lag();
  const T s = (w[0] + w[1]) + w[2];
  for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  return catchnan(dot3(p, w), T(K.machine_eps));
}

// weno5JS (:358-381): w_k = d_k / (eps + SI_k)^2
template <typename T>
inline T weno5js_side(const T* p, const T* v, const double* d) {
  const LagrangeCoef& K = lag();
  T SI[3], w[3];
  lagrange_si(v, SI);
  for (int k = 0; k < 3; ++k) {
    const T e = T(K.eps) + SI[k];
    w[k] = T(d[k]) / (e * e);
  }
  return normalised(p, w);
}

// weno5Z (:383-408): tau = |SI_2 - SI_0|, w_k = d_k (1 + tau / (SI_k + epsz))
template <typename T>
inline T weno5z_side(const T* p, const T* v, const double* d) {
  const LagrangeCoef& K = lag();
  T SI[3], w[3];
  lagrange_si(v, SI);
  const T tau = fabs(SI[2] - SI[0]);
  for (int k = 0; k < 3; ++k) w[k] = T(d[k]) * (T(1.0) + (tau / (SI[k] + T(K.epsz))));
  return normalised(p, w);
}

// The indicators of weno5N / teno5N (:445-450 and :558-563) on the side's window v[0..4]:
// SI_2 = theta |v0 - 3v1 + 2v2| + |v0 - 2v1 + v2|, SI_1 = theta |v3 - v2| + |v1 - 2v2 + v3|,
// SI_0 = theta |v3 - v2| + |v2 - 2v3 + v4|; and the 5-point difference v0 - 4v1 + 6v2 - 4v3 + v4.
template <typename T>
inline T n_indicators(const T* v, T* SI) {
  const T theta = T(0.1);
  SI[2] = theta * fabs(v[0] - T(3.0) * v[1] + T(2.0) * v[2]) + fabs(v[0] - T(2.0) * v[1] + v[2]);
  SI[1] = theta * fabs(v[3] - v[2]) + fabs(v[1] - T(2.0) * v[2] + v[3]);
  SI[0] = theta * fabs(v[3] - v[2]) + fabs(v[2] - T(2.0) * v[3] + v[4]);
  return fabs(v[0] - T(4.0) * v[1] + T(6.0) * v[2] - T(4.0) * v[3] + v[4]);
}

// weno5N (:440-479): tau = |5-point difference|^2.5, w_k = d_k (1 + tau / (SI_k + eps)^2)
template <typename T>
inline T weno5n_side(const T* p, const T* v, const double* d) {
  const LagrangeCoef& K = lag();
  T SI[3], w[3];
  const T tau = pow(n_indicators(v, SI), T(2.5));
  for (int k = 0; k < 3; ++k) {
    const T e = SI[k] + T(K.eps);
    w[k] = T(d[k]) * (T(1.0) + (tau / (e * e)));
  }
  return normalised(p, w);
}

// teno5N (:553-594): tau = |5-point difference|^2, w_k = (1 + tau / (SI_k + eps)^2)^6, cut-off
template <typename T>
inline T teno5n_side(const T* p, const T* v, const double* d) {
  const LagrangeCoef& K = lag();
  T SI[3], w[3];
  const T x = n_indicators(v, SI);
  const T tau = x * x;
  for (int k = 0; k < 3; ++k) {
    const T e = SI[k] + T(K.eps);
    w[k] = pow(T(1.0) + tau / (e * e), T(6));
  }
  return cutoff_weighted(p, w, d);
}

// teno5a (:1265-1294): tau = 1, w_k = (1 / (SI_k + epsz))^6, cut-off
template <typename T>
inline T teno5a_side(const T* p, const T* v, const double* d) {
  const LagrangeCoef& K = lag();
  T SI[3], w[3];
  lagrange_si(v, SI);
  for (int k = 0; k < 3; ++k) w[k] = pow(T(1.0) / (SI[k] + T(K.epsz)), T(6));
  return cutoff_weighted(p, w, d);
}

template <typename T>
inline T lagrange_side(int kind, const T* p, const T* v, const double* d) {
  switch (kind) {
    case 3: return weno5js_side(p, v, d);
    case 4: return weno5z_side(p, v, d);
    case 5: return weno5n_side(p, v, d);
    case 6: return teno5n_side(p, v, d);
    case 7: return teno5a_side(p, v, d);
    default: return teno_side(p, v, d, kind == 1);
  }
}

// kind: 0 teno5, 1 teno5i, 2 linear, 3 weno5JS, 4 weno5Z, 5 weno5N, 6 teno5N, 7 teno5a.
// u[0..5] -> out[0] = u^-_{i+1/2}, out[1] = u^+_{i+1/2}
template <typename T>
inline void lagrange_recon(int kind, const T* u, T* out) {
  const LagrangeCoef& K = lag();
  const double* C = &K.crj[0][0];
  T p[3];
  p[0] = dot3c(C + 1, 4, u + 2);
  p[1] = dot3c(C + 2, 4, u + 1);
  p[2] = dot3c(C + 3, 4, u + 0);
  if (kind == 2) {
    T d[3] = {T(K.dkm[0]), T(K.dkm[1]), T(K.dkm[2])};
    out[0] = dot3(p, d);
  } else {
    out[0] = lagrange_side(kind, p, u + 0, K.dkm);
  }
  p[0] = dot3c(C + 0, 4, u + 3);
  p[1] = dot3c(C + 1, 4, u + 2);
  p[2] = dot3c(C + 2, 4, u + 1);
  if (kind == 2) {
    T d[3] = {T(K.dkp[0]), T(K.dkp[1]), T(K.dkp[2])};
    out[1] = dot3(p, d);
  } else {
    out[1] = lagrange_side(kind, p, u + 1, K.dkp);
  }
}

// weno5JS3PointsQuadrature (Schemes_Lagrange.cpp:1155-1217): face values u[0..4] at j-2..j+2
// -> values at the three Gauss-Legendre points of face j.
template <typename T>
inline void gl3(const T* u, T* out) {
  const LagrangeCoef& K = lag();
  T bg[3], cg[3], SI[3];
  bg[0] = u[0] - T(4.0) * u[1] + T(3.0) * u[2];
  cg[0] = u[0] - T(2.0) * u[1] + u[2];
  bg[1] = u[1] - u[3];
  cg[1] = u[1] - T(2.0) * u[2] + u[3];
  bg[2] = T(3.0) * u[2] - T(4.0) * u[3] + u[4];
  cg[2] = u[2] - T(2.0) * u[3] + u[4];
  for (int k = 0; k < 3; ++k) {
    bg[k] = T(0.25) * pow(bg[k], T(2));
    cg[k] = T(K.c1) * pow(cg[k], T(2));
    SI[k] = bg[k] + cg[k];
  }
  T p[3], w[3], s;
  auto weights = [&](const double* lw) {
    for (int k = 0; k < 3; ++k) w[k] = T(lw[k]) / pow(T(K.eps) + SI[k], T(2));
    s = (w[0] + w[1]) + w[2];
    for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  };
  p[0] = dot3c(&K.gp[0][0], 3, u + 0);
  p[1] = dot3c(&K.gp[0][1], 3, u + 1);
  p[2] = dot3c(&K.gp[0][2], 3, u + 2);
  weights(K.linwp);
  out[0] = dot3(p, w);

  p[0] = (-u[0] + T(2) * u[1] + T(23.0) * u[2]) / T(24.0);
  p[1] = (-u[1] + T(26.0) * u[2] - u[3]) / T(24.0);
  p[2] = (T(23.0) * u[2] + T(2.0) * u[3] - u[4]) / T(24.0);
  weights(K.linw0p);
  out[1] = T(K.sumw0p) * dot3(p, w);
  weights(K.linw0m);
  out[1] = out[1] - T(K.sumw0m) * dot3(p, w);

  p[0] = dot3c(&K.gm[0][0], 3, u + 0);
  p[1] = dot3c(&K.gm[0][1], 3, u + 1);
  p[2] = dot3c(&K.gm[0][2], 3, u + 2);
  weights(K.linwm);
  out[2] = dot3(p, w);
  for (int k = 0; k < 3; ++k) out[k] = catchnan(out[k], T(K.machine_eps));
}

// =============================================================================================
// Schemes::Hermite (Schemes_Hermite.cpp); coefficients depend on the grid size (setGridSize)
// =============================================================================================
struct HermiteCoef {
  double eps = 1e-6, machine_eps = 1e-15, epsz = 1e-40, epszd = 1e-40, ct = 1e-3, ctd = 1e-3;
  double c1 = 13.0 / 12.0, dif;
  double crj[3][3], crjd[4][3], crjlin[5][2], crjlind[6][2];
  double dkm[3], dkp[3], dkmd[3], dkpd[3];

  explicit HermiteCoef(double h) : dif(h) {  // setGridSize, Schemes_Hermite.cpp:15-92
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

    dkm[0] = 9.0 / 80.0; dkm[1] = 42.0 / 80.0; dkm[2] = 29.0 / 80.0;
    dkp[0] = dkm[1]; dkp[1] = dkm[0]; dkp[2] = dkm[2];
    dkmd[0] = 1.0 / 18.0; dkmd[1] = 5.0 / 6.0; dkmd[2] = 1.0 / 9.0;
    dkpd[0] = dkmd[1]; dkpd[1] = dkmd[0]; dkpd[2] = dkmd[2];

    crjlin[0][0] = -23.0 / 120.0;
    crjlin[1][0] = 19.0 / 30.0;
    crjlin[2][0] = 67.0 / 120.0;
    crjlin[3][0] = -3.0 / 40.0 * dif;
    crjlin[4][0] = -7.0 / 40.0 * dif;
    crjlin[0][1] = 67.0 / 120.0;
    crjlin[1][1] = 19.0 / 30.0;
    crjlin[2][1] = -23.0 / 120.0;
    crjlin[3][1] = 7.0 / 40.0 * dif;
    crjlin[4][1] = 3.0 / 40.0 * dif;

    crjlind[0][0] = 0.25 / dif;
    crjlind[1][0] = -2.0 / dif;
    crjlind[2][0] = 1.75 / dif;
    crjlind[3][0] = 1.0 / 12.0;
    crjlind[4][0] = -1.0 / 6.0;
    crjlind[5][0] = -5.0 / 12.0;
    crjlind[0][1] = -7.0 / 4.0 / dif;
    crjlind[1][1] = 2.0 / dif;
    crjlind[2][1] = -0.25 / dif;
    crjlind[3][1] = -5.0 / 12.0;
    crjlind[4][1] = -1.0 / 6.0;
    crjlind[5][1] = 1.0 / 12.0;
  }
};

// smoothnessMeasure (Schemes_Hermite.cpp:515-526)
template <typename T>
inline void hermite_si(const HermiteCoef& K, const T* u, const T* v, T* SI) {
  T b[3], c[3];
  b[0] = T(-2.0) * (u[0] - u[1]) - v[0];
  c[0] = T(-2.0) * (u[0] - u[1] + v[0]);
  b[1] = T(-2.0) * (u[1] - u[2]) - v[2];
  c[1] = T(2.0) * (u[1] - u[2]) + T(2.0) * v[2];
  b[2] = (-u[0] + u[2]) / T(2.0);
  c[2] = u[0] - T(2.0) * u[1] + u[2];
  for (int k = 0; k < 3; ++k) SI[k] = T(K.c1) * pow(c[k], T(2)) + pow(b[k], T(2));
}
// smoothnessMeasureDerivative (:528-541)
template <typename T>
inline void hermite_sid(const HermiteCoef& K, const T* u, const T* d, T* SI) {
  T b[3], c[3];
  b[0] = T(6.0) * (u[0] - u[1]) + (T(2.0) * d[0] + T(4.0) * d[1]);
  c[0] = T(12.0) * (u[0] - u[1]) + T(6.0) * (d[0] + d[1]);
  b[1] = T(6.0) * (u[2] - u[1]) - (T(4.0) * d[1] + T(2.0) * d[2]);
  c[1] = T(12.0) * (u[1] - u[2]) + T(6.0) * (d[1] + d[2]);
  b[2] = u[0] - T(2.0) * u[1] + u[2];
  c[2] = T(3.0) * (u[2] - u[0]) - T(6.0) * d[1];
  for (int k = 0; k < 3; ++k) SI[k] = T(K.c1) * pow(c[k], T(2)) + pow(b[k], T(2));
}
// fullPointsSI (:597-603)
template <typename T>
inline T hermite_brk(const T* u, const T* d) {
  return fabs((T(1029270.0) * u[2] - T(2129184.0) * u[1] + T(1099914.0) * u[0] +
               T(281121.0) * d[0] - T(494958.0) * d[2]) * d[0] +
              (T(-1029270.0) * u[0] + T(2129184.0) * u[1] - T(1099914.0) * u[2] +
               T(281121.0) * d[2]) * d[2] +
              (T(1099445.0) * u[2] - T(4317056.0) * u[1] + T(2118166.0) * u[0]) * u[2] +
              T(4317056.0) * (u[1] - u[0]) * u[1] + T(1099445.0) * u[0] * u[0]) /
         T(6720.0);
}
// fullPointsSId (:605-612)
template <typename T>
inline T hermite_brkd(const T* u, const T* d) {
  return fabs((T(3156862.0) * d[2] + T(13189240.0) * d[1] + T(1710479.0) * d[0] -
               T(9617754.0) * u[2] - T(531552.0) * u[1] + T(10149306.0) * u[0]) * d[0] +
              (T(13189240.0) * d[2] + T(26511200.0) * d[1] - T(39700440.0) * u[2] +
               T(39700440.0) * u[0]) * d[1] +
              (T(1710479.0) * d[2] - T(10149306.0) * u[2] + T(531552.0) * u[1] +
               T(9617754.0) * u[0]) * d[2] +
              (T(15136011.0) * u[2] - T(1076544.0) * u[1] - T(29195478.0) * u[0]) * u[2] +
              T(1076544.0) * (u[1] - u[0]) * u[1] + T(15136011.0) * u[0] * u[0]) /
         T(1680.0);
}

// nonlinear weights of one hteno/htenoi output; SI given, brk (or -1 for htenoi's max SI)
template <typename T>
inline T hermite_weighted(const T* p, const T* SI, T tau, double epsz, double ct, const double* d,
                          double machine_eps) {
  T w[3];
  for (int k = 0; k < 3; ++k) w[k] = pow(T(1.0) + tau / (SI[k] + T(epsz)), T(6));
  T s = (w[0] + w[1]) + w[2];
  T sig[3];
  for (int k = 0; k < 3; ++k) {
    w[k] = w[k] / s;
    sig[k] = w[k] < T(ct) ? T(0.0) : T(1.0);
  }
  for (int k = 0; k < 3; ++k) w[k] = sig[k] * T(d[k]);
  s = (w[0] + w[1]) + w[2];
  for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  return catchnan(dot3(p, w), T(machine_eps));
}

template <typename T>
inline T maxof3(const T* s) {
  T t = s[0];
  t = (t < s[1]) ? s[1] : t;
  t = (t < s[2]) ? s[2] : t;
  return t;
}

// kind: 0 hteno (:295-379), 1 htenoi (:670-758), 2 linear (:760-812).
// u[0..3], d[0..3] -> out = {u^-_{i+1/2}, u^+_{i+1/2}, d^-_{i+1/2}, d^+_{i+1/2}}
template <typename T>
inline void hermite_recon(const HermiteCoef& K, int kind, const T* u, const T* d, T* out) {
  if (kind == 2) {
    out[0] = dot3c(&K.crjlin[0][0], 2, u) + T(K.crjlin[3][0]) * d[0] + T(K.crjlin[4][0]) * d[2];
    out[1] = dot3c(&K.crjlin[0][1], 2, u + 1) + T(K.crjlin[3][1]) * d[1] + T(K.crjlin[4][1]) * d[3];
    out[2] = dot3c(&K.crjlind[0][0], 2, u) + dot3c(&K.crjlind[3][0], 2, d);
    out[3] = dot3c(&K.crjlind[0][1], 2, u + 1) + dot3c(&K.crjlind[3][1], 2, d + 1);
    return;
  }
  const bool imp = (kind == 1);
  T ud[4];
  for (int k = 0; k < 4; ++k) ud[k] = d[k] * T(K.dif);
  T p[3], SI[3], tau;

  // u^-_{i+1/2}
  p[0] = T(K.crj[0][0]) * u[0] + T(K.crj[1][0]) * u[1] + T(K.crj[2][0]) * d[0];
  p[1] = T(K.crj[0][1]) * u[1] + T(K.crj[1][1]) * u[2] + T(K.crj[2][1]) * d[2];
  p[2] = T(K.crj[0][2]) * u[0] + T(K.crj[1][2]) * u[1] + T(K.crj[2][2]) * u[2];
  hermite_si(K, u, ud, SI);
  tau = imp ? maxof3(SI)
            : fabs(hermite_brk(u, ud) - T(0.25) * (SI[0] + SI[1] + T(2.0) * SI[2]));
  out[0] = hermite_weighted(p, SI, tau, K.epsz, K.ct, K.dkm, K.machine_eps);

  // d^-_{i+1/2}
  p[0] = T(K.crjd[0][0]) * u[0] + T(K.crjd[1][0]) * u[1] + T(K.crjd[2][0]) * d[0] +
         T(K.crjd[3][0]) * d[1];
  p[1] = T(K.crjd[0][1]) * u[1] + T(K.crjd[1][1]) * u[2] + T(K.crjd[2][1]) * d[1] +
         T(K.crjd[3][1]) * d[2];
  p[2] = T(K.crjd[0][2]) * u[0] + T(K.crjd[1][2]) * u[1] + T(K.crjd[2][2]) * u[2] +
         T(K.crjd[3][2]) * d[1];
  hermite_sid(K, u, ud, SI);
  tau = imp ? maxof3(SI)
            : fabs(hermite_brkd(u, ud) - T(0.25) * (SI[0] + SI[1] + T(2.0) * SI[2]));
  out[2] = hermite_weighted(p, SI, tau, K.epszd, K.ctd, K.dkmd, K.machine_eps);

  // u^+_{i+1/2}
  p[0] = T(K.crj[1][1]) * u[1] + T(K.crj[0][1]) * u[2] - T(K.crj[2][1]) * d[1];
  p[1] = T(K.crj[1][0]) * u[2] + T(K.crj[0][0]) * u[3] - T(K.crj[2][0]) * d[3];
  p[2] = T(K.crj[2][2]) * u[1] + T(K.crj[1][2]) * u[2] + T(K.crj[0][2]) * u[3];
  hermite_si(K, u + 1, ud + 1, SI);
  tau = imp ? maxof3(SI)
            : fabs(hermite_brk(u + 1, ud + 1) - T(0.25) * (SI[0] + SI[1] + T(2.0) * SI[2]));
  out[1] = hermite_weighted(p, SI, tau, K.epsz, K.ct, K.dkp, K.machine_eps);

  // d^+_{i+1/2}
  p[0] = T(K.crjd[0][1]) * u[1] + T(K.crjd[1][1]) * u[2] + T(K.crjd[3][1]) * d[1] +
         T(K.crjd[2][1]) * d[2];
  p[1] = T(K.crjd[0][0]) * u[2] + T(K.crjd[1][0]) * u[3] + T(K.crjd[3][0]) * d[2] +
         T(K.crjd[2][0]) * d[3];
  p[2] = -(T(K.crjd[2][2]) * u[1] + T(K.crjd[1][2]) * u[2] + T(K.crjd[0][2]) * u[3]) +
         T(K.crjd[3][2]) * d[2];
  hermite_sid(K, u + 1, ud + 1, SI);
  tau = imp ? maxof3(SI)
            : fabs(hermite_brkd(u + 1, ud + 1) - T(0.25) * (SI[0] + SI[1] + T(2.0) * SI[2]));
  out[3] = hermite_weighted(p, SI, tau, K.epszd, K.ctd, K.dkpd, K.machine_eps);
}

// hermiteLimiter (Schemes_Hermite.cpp:634-662): u[0..2], d[0..2] -> limited derivative average
template <typename T>
inline T hermite_limiter(const HermiteCoef& K, const T* u, const T* d) {
  T p[3];
  p[0] = T(0.75) * (u[2] - u[0]) / T(K.dif) - T(0.25) * (d[0] + d[2]);
  p[1] = (u[1] - u[0]) / T(K.dif);
  p[2] = (u[2] - u[1]) / T(K.dif);
  const T lw[3] = {T(1.0 - 2E-5), T(1E-5), T(1E-5)};
  T ud[3];
  for (int k = 0; k < 3; ++k) ud[k] = d[k] * T(K.dif);
  T sm[3];
  sm[0] = hermite_brk(u, ud);
  sm[1] = pow(u[0] - u[1], T(2));
  sm[2] = pow(u[1] - u[2], T(2));
  T tau = pow(fabs(sm[0] - sm[1]) + fabs(sm[0] - sm[2]), T(2)) / T(4.0);
  T w[3];
  for (int k = 0; k < 3; ++k) w[k] = lw[k] * (T(1.0) + tau / (sm[k] + T(K.eps)));
  T s = (w[0] + w[1]) + w[2];
  for (int k = 0; k < 3; ++k) w[k] = w[k] / s;
  T r1 = lw[1] / lw[0], r2 = lw[2] / lw[0];
  T inner = r1 * p[1];
  inner = inner + r2 * p[2];
  T w12 = w[1] * p[1];
  w12 = w12 + w[2] * p[2];
  return w[0] * (p[0] / lw[0] - inner) + w12;
}

// =============================================================================================
// Equations::Euler2D (Equations_Euler2D.cpp); dir 1 = x, 2 = y
// =============================================================================================
template <typename T>
struct Euler2 {
  T g, g1, g3;
  explicit Euler2(double gamma) : g(gamma), g1(gamma - 1.0), g3(gamma - 3.0) {}

  void primitive(const T* q, T* w) const {  // :20-26
    w[0] = q[0];
    w[1] = q[1] / q[0];
    w[2] = q[2] / q[0];
    w[3] = (q[3] - T(0.5) * (q[1] * w[1] + q[2] * w[2])) * g1;
  }
  void conservative(const T* w, T* q) const {  // :28-34
    q[0] = w[0];
    q[1] = w[0] * w[1];
    q[2] = w[0] * w[2];
    q[3] = w[3] / g1 + T(0.5) * (q[1] * w[1] + q[2] * w[2]);
  }
  void flux(int dir, const T* q, const T* w, T* f) const {  // :36-50
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
  void dflux(int dir, const T* q, const T* w, T* A) const {  // :52-98, row-major
    if (dir == 1) {
      T sv = w[1] * w[1];
      T dv = T(0.5) * g1 * (sv + w[2] * w[2]);
      T h = (q[3] + w[3]) / w[0];
      T m[16] = {T(0.0), T(1.0), T(0.0), T(0.0),
                 dv - sv, -g3 * w[1], -g1 * w[2], g1,
                 -w[1] * w[2], w[2], w[1], T(0.0),
                 (dv - h) * w[1], h - g1 * sv, -g1 * w[1] * w[2], g * w[1]};
      for (int k = 0; k < 16; ++k) A[k] = m[k];
    } else {
      T sv = w[2] * w[2];
      T dv = T(0.5) * g1 * (sv + w[1] * w[1]);
      T h = (q[3] + w[3]) / w[0];
      T m[16] = {T(0.0), T(0.0), T(1.0), T(0.0),
                 -w[1] * w[2], w[2], w[1], T(0.0),
                 dv - sv, -g1 * w[1], -g3 * w[2], g1,
                 (dv - h) * w[2], -g1 * w[1] * w[2], h - g1 * sv, g * w[2]};
      for (int k = 0; k < 16; ++k) A[k] = m[k];
    }
  }
  T maxSpeed(const T* w, int dir) const {  // :207-219
    T c = sqrt(fabs(g * w[3] / w[0]));
    return fmax((w[dir] - c), fabs(w[dir] + c));
  }
  void maxLocalWaveSpeed(const T* wl, const T* wr, int dir, T* a) const {  // :221-246
    T cl = sqrt(fabs(g * wl[3] / wl[0]));
    T cr = sqrt(fabs(g * wr[3] / wr[0]));
    T vl = wl[dir], vr = wr[dir];
    a[0] = fmax(fabs(vl - cl), fabs(vr - cr));
    a[1] = fmax(fabs(vl), fabs(vr));
    a[2] = a[1];
    a[3] = fmax(fabs(vl + cl), fabs(vr + cr));
  }
  // Roe-averaged eigenvectors of a face (eigen2DEuler, FV_System2D.cpp:265-361; matrices from
  // right/leftEigenVectorx/y, Equations_Euler2D.cpp:100-205).  Row-major 4x4.
  void roe(int dir, const T* wa, T sra, T ha, const T* wb, T srb, T hb, T* R, T* L) const {
    T t0 = sra / (sra + srb);
    T t1 = T(1.0) - t0;
    T vxm = t0 * wa[1] + t1 * wb[1];
    T vym = t0 * wa[2] + t1 * wb[2];
    T hm = t0 * ha + t1 * hb;
    T qm = T(0.5) * (vxm * vxm + vym * vym);
    T cm = sqrt(fabs(g1 * (hm - qm)));
    T vn = dir == 1 ? vxm : vym;
    T vt = dir == 1 ? vym : vxm;
    t0 = vn * cm;
    T rcm = T(1.0) / cm;
    T b1 = g1 * rcm * rcm;
    T b2 = qm * b1;
    T s0 = vn * rcm;
    T s1 = b1 * vn;
    T t2 = T(0.5) * b1;
    if (dir == 1) {
      T r[16] = {T(1.0), T(0.0), T(1.0), T(1.0),
                 vxm - cm, T(0.0), vxm, vxm + cm,
                 vym, T(1.0), vym, vym,
                 hm - t0, vym, qm, hm + t0};
      T l[16] = {T(0.5) * (b2 + s0), T(-0.5) * (s1 + rcm), -t2 * vt, t2,
                 -vt, T(0.0), T(1.0), T(0.0),
                 T(1.0) - b2, s1, b1 * vt, -b1,
                 T(0.5) * (b2 - s0), T(-0.5) * (s1 - rcm), -t2 * vt, t2};
      for (int k = 0; k < 16; ++k) { R[k] = r[k]; L[k] = l[k]; }
    } else {
      T r[16] = {T(1.0), T(0.0), T(1.0), T(1.0),
                 vxm, T(1.0), vxm, vxm,
                 vym - cm, T(0.0), vym, vym + cm,
                 hm - t0, vxm, qm, hm + t0};
      T l[16] = {T(0.5) * (b2 + s0), -t2 * vt, T(-0.5) * (s1 + rcm), t2,
                 -vt, T(1.0), T(0.0), T(0.0),
                 T(1.0) - b2, b1 * vt, s1, -b1,
                 T(0.5) * (b2 - s0), -t2 * vt, T(-0.5) * (s1 - rcm), t2};
      for (int k = 0; k < 16; ++k) { R[k] = r[k]; L[k] = l[k]; }
    }
  }
  // characteristic Rusanov (:310-330) with aM = maxLocalWaveSpeed (FV_System2D.cpp:460-464)
  void rusanov(int dir, const T* ql, const T* qr, const T* L, const T* R, T* F) const {
    T wl[4], wr[4], a[4], fl[4], fr[4], d[4], m[4];
    primitive(ql, wl);
    primitive(qr, wr);
    maxLocalWaveSpeed(wl, wr, dir, a);
    flux(dir, ql, wl, fl);
    flux(dir, qr, wr, fr);
    for (int k = 0; k < 4; ++k) d[k] = qr[k] - ql[k];
    for (int i = 0; i < 4; ++i) {
      T s = L[4 * i] * d[0];
      for (int j = 1; j < 4; ++j) s = s + L[4 * i + j] * d[j];
      m[i] = a[i] * s;
    }
    for (int i = 0; i < 4; ++i) {
      T s = R[4 * i] * m[0];
      for (int j = 1; j < 4; ++j) s = s + R[4 * i + j] * m[j];
      F[i] = T(0.5) * (fl[i] + fr[i] - s);
    }
  }
  // dRusanov (:352-360) as called in FVHermite_System2D.cpp:553-589
  void drusanov(int dir, const T* ql, const T* qr, const T* dql, const T* dqr, const T* L,
                const T* R, T* F) const {
    T wl[4], wr[4], a[4], Al[16], Ar[16], d[4], m[4];
    primitive(ql, wl);
    primitive(qr, wr);
    dflux(dir, ql, wl, Al);
    dflux(dir, qr, wr, Ar);
    maxLocalWaveSpeed(wl, wr, dir, a);
    for (int k = 0; k < 4; ++k) d[k] = dqr[k] - dql[k];
    for (int i = 0; i < 4; ++i) {
      T s = L[4 * i] * d[0];
      for (int j = 1; j < 4; ++j) s = s + L[4 * i + j] * d[j];
      m[i] = a[i] * s;
    }
    for (int i = 0; i < 4; ++i) {
      T sl = Al[4 * i] * dql[0], sr = Ar[4 * i] * dqr[0], s = R[4 * i] * m[0];
      for (int j = 1; j < 4; ++j) {
        sl = sl + Al[4 * i + j] * dql[j];
        sr = sr + Ar[4 * i + j] * dqr[j];
        s = s + R[4 * i + j] * m[j];
      }
      F[i] = T(0.5) * (sl + sr - s);
    }
  }
  // HLLC (:372-428), including the reference's sound speeds without gamma and the left
  // pressure in the right star energy.
  void hllc(int dir, const T* ql, const T* qr, T* F) const {
    const int d1 = dir - 1;
    T wl[4], wr[4], fl[4], fr[4], qs[4];
    primitive(ql, wl);
    primitive(qr, wr);
    T hl = (ql[3] + wl[3]) / wl[0];
    T hr = (qr[3] + wr[3]) / wr[0];
    T rr = sqrt(fabs(wr[0] / wl[0]));
    T rrr = T(1.0) / (T(1.0) + rr);
    T vm[2];
    vm[0] = (wl[1] + wr[1] * rr) * rrr;
    vm[1] = (wl[2] + wr[2] * rr) * rrr;
    T qm = T(0.5) * (vm[0] * vm[0] + vm[1] * vm[1]);
    T hm = (hl + hr * rr) * rrr;
    T cm = sqrt(fabs(g1 * (hm - qm)));
    T cl = sqrt(fabs(wl[3] / wl[0]));
    T cr = sqrt(fabs(wr[3] / wr[0]));
    T sl = fmin(wl[dir] - cl, vm[d1] - cm);
    T sr = fmax(wr[dir] + cr, vm[d1] + cm);
    T sm = (qr[dir] * (sr - wr[dir]) - ql[dir] * (sl - wl[dir]) + wl[3] - wr[3]) /
           (wr[0] * (sr - wr[dir]) - wl[0] * (sl - wl[dir]));
    T ps = wl[3] + wl[0] * (wl[dir] - sl) * (wl[dir] - sm);
    flux(dir, ql, wl, fl);
    flux(dir, qr, wr, fr);
    if (sl > T(0.0)) {
      for (int k = 0; k < 4; ++k) F[k] = fl[k];
    } else if (sl <= T(0.0) && sm > T(0.0)) {
      T nom = sl - wl[dir], den = sl - sm;
      qs[0] = wl[0] * nom / den;
      qs[1] = dir == 1 ? (nom * ql[1] + ps - wl[3]) / den : nom * ql[1] / den;
      qs[2] = dir == 2 ? (nom * ql[2] + ps - wl[3]) / den : nom * ql[2] / den;
      qs[3] = (nom * ql[3] - wl[3] * wl[dir] + ps * sm) / den;
      for (int k = 0; k < 4; ++k) F[k] = fl[k] + sl * (qs[k] - ql[k]);
    } else if (sm <= T(0.0) && sr >= T(0.0)) {
      T nom = sr - wr[dir], den = sr - sm;
      qs[0] = wr[0] * nom / den;
      qs[1] = dir == 1 ? (nom * qr[1] + ps - wr[3]) / den : nom * qr[1] / den;
      qs[2] = dir == 2 ? (nom * qr[2] + ps - wr[3]) / den : nom * qr[2] / den;
      qs[3] = (nom * qr[3] - wl[3] * wr[dir] + ps * sm) / den;
      for (int k = 0; k < 4; ++k) F[k] = fr[k] + sr * (qs[k] - qr[k]);
    } else {
      for (int k = 0; k < 4; ++k) F[k] = fr[k];
    }
  }
};

// =============================================================================================
// Equations::Euler1D (Equations_Euler1D.cpp)
// =============================================================================================
template <typename T>
struct Euler1 {
  T g, g1, g3;
  explicit Euler1(double gamma) : g(gamma), g1(gamma - 1.0), g3(gamma - 3.0) {}
  void primitive(const T* q, T* w) const {  // :18-23
    w[0] = q[0];
    w[1] = q[1] / q[0];
    w[2] = (q[2] - T(0.5) * q[1] * w[1]) * g1;
  }
  void conservative(const T* w, T* q) const {  // :25-30
    q[0] = w[0];
    q[1] = w[0] * w[1];
    q[2] = w[2] / g1 + T(0.5) * q[1] * w[1];
  }
  void flux(const T* q, const T* w, T* f) const {  // :32-37
    f[0] = q[1];
    f[1] = q[1] * w[1] + w[2];
    f[2] = w[1] * (q[2] + w[2]);
  }
  void dflux(const T* q, const T* w, T* A) const {  // :39-53
    A[0] = T(0.0); A[1] = T(1.0); A[2] = T(0.0);
    A[3] = T(0.5) * g3 * w[1] * w[1];
    A[4] = -g3 * w[1];
    A[5] = g1;
    A[6] = (g1 * pow(w[1], T(2)) - g * q[2] / w[0]) * w[1];
    A[7] = g * q[2] / w[0] - T(1.5) * g1 * w[1] * w[1];
    A[8] = g * w[1];
  }
  T maxSpeed(const T* w) const {  // :91-94
    T c = sqrt(fabs(g * w[2] / w[0]));
    return fmax(fabs(w[1] - c), fabs(w[1] + c));
  }
  void maxLocalWaveSpeed(const T* wl, const T* wr, T* a) const {  // :96-107
    T cl = sqrt(fabs(g * wl[2] / wl[0]));
    T cr = sqrt(fabs(g * wr[2] / wr[0]));
    a[0] = fmax(fabs(wl[1] - cl), fabs(wr[1] - cr));
    a[1] = fmax(fabs(wl[1]), fabs(wr[1]));
    a[2] = fmax(fabs(wl[1] + cl), fabs(wr[1] + cr));
  }
  // eigen1DEuler (FV_System1D.cpp:121-156); eigenvectors :55-89.  Row-major 3x3.
  void roe(const T* wa, T sra, T ha, const T* wb, T srb, T hb, T* R, T* L) const {
    T t0 = sra / (sra + srb);
    T t1 = T(1.0) - t0;
    T vxm = t0 * wa[1] + t1 * wb[1];
    T hm = t0 * ha + t1 * hb;
    T qm = T(0.5) * vxm * vxm;
    T cm = sqrt(fabs(g1 * (hm - qm)));
    t0 = vxm * cm;
    T r[9] = {T(1.0), T(1.0), T(1.0), vxm - cm, vxm, vxm + cm, hm - t0, qm, hm + t0};
    T rcm = T(1.0) / cm;
    T b1 = g1 * rcm * rcm;
    T b2 = qm * b1;
    T s0 = vxm * rcm;
    T s1 = b1 * vxm;
    T t2 = T(0.5) * b1;
    T l[9] = {T(0.5) * (b2 + s0), T(-0.5) * (s1 + rcm), t2,
              T(1.0) - b2, s1, -b1,
              T(0.5) * (b2 - s0), T(-0.5) * (s1 - rcm), t2};
    for (int k = 0; k < 9; ++k) { R[k] = r[k]; L[k] = l[k]; }
  }
  void rusanov(const T* ql, const T* qr, const T* L, const T* R, T* F) const {  // :129-135
    T wl[3], wr[3], a[3], fl[3], fr[3], d[3], m[3];
    primitive(ql, wl);
    primitive(qr, wr);
    maxLocalWaveSpeed(wl, wr, a);
    flux(ql, wl, fl);
    flux(qr, wr, fr);
    for (int k = 0; k < 3; ++k) d[k] = qr[k] - ql[k];
    for (int i = 0; i < 3; ++i) {
      T s = L[3 * i] * d[0];
      for (int j = 1; j < 3; ++j) s = s + L[3 * i + j] * d[j];
      m[i] = a[i] * s;
    }
    for (int i = 0; i < 3; ++i) {
      T s = R[3 * i] * m[0];
      for (int j = 1; j < 3; ++j) s = s + R[3 * i + j] * m[j];
      F[i] = T(0.5) * (fl[i] + fr[i] - s);
    }
  }
  void drusanov(const T* ql, const T* qr, const T* dql, const T* dqr, const T* L, const T* R,
                T* F) const {  // :212-220, as called in FVHermite_System1D.cpp:306-337
    T wl[3], wr[3], a[3], Al[9], Ar[9], d[3], m[3];
    primitive(ql, wl);
    primitive(qr, wr);
    dflux(ql, wl, Al);
    dflux(qr, wr, Ar);
    maxLocalWaveSpeed(wl, wr, a);
    for (int k = 0; k < 3; ++k) d[k] = dqr[k] - dql[k];
    for (int i = 0; i < 3; ++i) {
      T s = L[3 * i] * d[0];
      for (int j = 1; j < 3; ++j) s = s + L[3 * i + j] * d[j];
      m[i] = a[i] * s;
    }
    for (int i = 0; i < 3; ++i) {
      T sl = Al[3 * i] * dql[0], sr = Ar[3 * i] * dqr[0], s = R[3 * i] * m[0];
      for (int j = 1; j < 3; ++j) {
        sl = sl + Al[3 * i + j] * dql[j];
        sr = sr + Ar[3 * i + j] * dqr[j];
        s = s + R[3 * i + j] * m[j];
      }
      F[i] = T(0.5) * (sl + sr - s);
    }
  }
  void hllc(const T* ql, const T* qr, T* F) const {  // :156-210
    T wl[3], wr[3], fl[3], fr[3], qs[3];
    primitive(ql, wl);
    primitive(qr, wr);
    T hl = (ql[2] + wl[2]) / wl[0];
    T hr = (qr[2] + wr[2]) / wr[0];
    T rr = sqrt(fabs(wr[0] / wl[0]));
    T rrr = T(1.0) / (T(1.0) + rr);
    T vm = (wl[1] + wr[1] * rr) * rrr;
    T qm = T(0.5) * vm * vm;
    T hm = (hl + hr * rr) * rrr;
    T cm = sqrt(fabs(g1 * (hm - qm)));
    T cl = sqrt(fabs(wl[2] / wl[0]));
    T cr = sqrt(fabs(wr[2] / wr[0]));
    T sl = fmin(wl[1] - cl, vm - cm);
    T sr = fmax(wr[1] + cr, vm + cm);
    T sm = (qr[1] * (sr - wr[1]) - ql[1] * (sl - wl[1]) + wl[2] - wr[2]) /
           (wr[0] * (sr - wr[1]) - wl[0] * (sl - wl[1]));
    T ps = wl[2] + wl[0] * (wl[1] - sl) * (wl[1] - sm);
    flux(ql, wl, fl);
    flux(qr, wr, fr);
    if (sl > T(0.0)) {
      for (int k = 0; k < 3; ++k) F[k] = fl[k];
    } else if (sl <= T(0.0) && sm > T(0.0)) {
      T nom = sl - wl[1], den = sl - sm;
      qs[0] = wl[0] * nom / den;
      qs[1] = (nom * ql[1] + ps - wl[2]) / den;
      qs[2] = (nom * ql[2] - wl[2] * wl[1] + ps * sm) / den;
      for (int k = 0; k < 3; ++k) F[k] = fl[k] + sl * (qs[k] - ql[k]);
    } else if (sm <= T(0.0) && sr >= T(0.0)) {
      T nom = sr - wr[1], den = sr - sm;
      qs[0] = wr[0] * nom / den;
      qs[1] = (nom * qr[1] + ps - wr[2]) / den;
      qs[2] = (nom * qr[2] - wl[2] * wr[1] + ps * sm) / den;
      for (int k = 0; k < 3; ++k) F[k] = fr[k] + sr * (qs[k] - qr[k]);
    } else {
      for (int k = 0; k < 3; ++k) F[k] = fr[k];
    }
  }
};

// Schemes::SSPRK::RungeKuttaIII (Schemes_SSPRK.cpp:3-15)
template <typename T>
inline T ssprk3(T q0, T qn, T rhs, T dt, int stage) {
  if (stage == 1) return q0 + dt * rhs;
  if (stage == 2) return T(0.75) * q0 + T(0.25) * (qn + rhs * dt);
  return (q0 + T(2.0) * (qn + dt * rhs)) / T(3.0);
}

// =============================================================================================
// Solvers
// =============================================================================================
enum Bc { BC_ZEROGRAD = 0, BC_PERIODIC = 1, BC_TAYLOR = 2, BC_DOUBLE_MACH = 3 };
enum Flux { FLUX_RUSANOV = 0, FLUX_HLLC = 1 };
enum Recon { RECON_TENO5 = 0, RECON_TENO5I = 1, RECON_LINEAR = 2 };

inline int bcmap(int i, int n, int bc) {
  if (bc == BC_PERIODIC) return ((i % n) + n) % n;
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// FV::System2D (FV_System2D.cpp): characteristic TENO5 per direction, GL3 transverse WENO5-JS
// along each face, flux at three Gauss points, SSP-RK3 (rhs :363-573, RungeKutta3 :575-612,
// timeStepping :614-651).
struct FV2D {
  int nx, ny, bc, flux, recon;
  double dx, dy, area, cfl, gamma, t = 0.0, dt = 0.0;
  double x0, y0;                                // xl, yb (cell centres for the ghost rules)
  double qb[4], qu[4], qpost[4], qpre[4];       // fixed ghost states (TaylorInstBc, doubleMachBc)
  double ctan, c16, s3;                         // tan(pi/6), 1/6, sqrt(3) as the reference computes them
  std::vector<double> gxl, gxr, gyl, gyr;       // face values of the 2 + 2 ghost face rows [4][4][...]
  std::vector<double> q, q0, q1, rhsu;          // [4][ny][nx]
  std::vector<double> w, sr, h;                 // primitives [4][ny][nx], sqrt(rho), enthalpy
  std::vector<double> xl, xr, yl, yr;           // characteristic face values [4][...]
  std::vector<double> xR, xL, yR, yL;           // face eigenvectors [16][...]
  std::vector<double> fx, fy;                   // face fluxes [4][...]

  FV2D(int nx_, int ny_, double xl0, double xr0, double yb, double yt, double cfl_, double g,
       int bc_ = BC_ZEROGRAD, int flux_ = FLUX_RUSANOV, int recon_ = RECON_TENO5)
      : nx(nx_), ny(ny_), bc(bc_), flux(flux_), recon(recon_), cfl(cfl_), gamma(g) {
    dx = (xr0 - xl0) / nx;
    dy = (yt - yb) / ny;
    area = dx * dy;
    x0 = xl0;
    y0 = yb;
    Euler2<double> E(gamma);
    const double wb[4] = {2.0, 0.0, 0.0, 1.0}, wu[4] = {1.0, 0.0, 0.0, 2.5};  // :169-172
    E.conservative(wb, qb);
    E.conservative(wu, qu);
    s3 = std::sqrt(3.0);
    c16 = 1.0 / 6.0;
    const double wpost[4] = {8.0, 8.25 * 0.5 * s3, -8.25 * 0.5, 116.5};  // Equations_Euler2D.cpp:637-655
    const double wpre[4] = {1.4, 0.0, 0.0, 1.0};
    E.conservative(wpost, qpost);
    E.conservative(wpre, qpre);
    const double pi = 4.0 * std::atan(1.0);  // doubleMachBc :189-190
    ctan = std::tan(pi / 6.0);
    const size_t n = size_t(nx) * ny;
    q.assign(4 * n, 0.0); q0 = q; q1 = q; rhsu = q; w = q;
    sr.assign(n, 0.0); h = sr;
    const size_t nxf = size_t(nx + 1) * ny, nyf = size_t(nx) * (ny + 1);
    xl.assign(4 * nxf, 0.0); xr = xl; fx = xl; xR.assign(16 * nxf, 0.0); xL = xR;
    yl.assign(4 * nyf, 0.0); yr = yl; fy = yl; yR.assign(16 * nyf, 0.0); yL = yR;
    gxl.assign(16 * size_t(nx + 1), 0.0); gxr = gxl;
    gyl.assign(16 * size_t(ny + 1), 0.0); gyr = gyl;
  }

  // State of cell (i, j), -6 <= i < nx + 6, -6 <= j < ny + 6, ghosts as the reference fills them.
  // Zero-gradient and periodic ghosts copy interior cells (an index map).  TaylorInstBc
  // (:154-182): x ghosts of interior rows mirror the row with the x momentum negated; the ghost
  // rows (all columns) hold the fixed bottom / top states.  doubleMachBc (:184-224): below the
  // first interior row, columns with x <= 1/6 hold conservativeOfDoubleMach2D at the ghost's
  // centre and the others mirror the column with the y momentum negated; above the last row,
  // the state of interior cell (0, 6) where x < 1/6 + tan(pi/6) (y + (1 + m) dy + 20 t) and of
  // cell (nx - 7, 6) elsewhere; the x ghosts of every row copy the row's first / last column.
  void ghost(int i, int j, double* out) const {
    auto cp = [&](const double* src) { for (int v = 0; v < 4; ++v) out[v] = src[v]; };
    auto ld = [&](int ii, int jj) { for (int v = 0; v < 4; ++v) out[v] = q[c(v, ii, jj)]; };
    if (bc == BC_TAYLOR) {
      if (j < 0) return cp(qb);
      if (j >= ny) return cp(qu);
      if (i < 0) { ld(-1 - i, j); out[1] = -out[1]; return; }
      if (i >= nx) { ld(2 * nx - 1 - i, j); out[1] = -out[1]; return; }
      return ld(i, j);
    }
    if (bc == BC_DOUBLE_MACH) {
      const int ic = i < 0 ? 0 : (i >= nx ? nx - 1 : i);
      if (j >= 0 && j < ny) return ld(ic, j);
      const double x = ((double) (ic + 6) - 6.0 + 0.5) * dx + x0;
      if (j < 0) {
        if (x <= c16) {
          const double y = ((double) (j + 6) - 6.0 + 0.5) * dy + y0;
          const double lim = c16 + y / s3;
          return cp(x < lim ? qpost : qpre);
        }
        ld(ic, -1 - j);
        out[2] = -out[2];
        return;
      }
      const int m = j - ny;
      const double ytop = ((double) (ny + 6 - 1) - 6.0 + 0.5) * dy + y0;
      const double hx = ctan * (ytop + (1.0 + (double) m) * dy + 20.0 * t) + c16;
      return x < hx ? ld(0, 6) : ld(nx - 7, 6);
    }
    ld(bcmap(i, nx, bc), bcmap(j, ny, bc));
  }
  bool ghost_rows() const { return bc >= BC_TAYLOR; }
  size_t c(int v, int i, int j) const { return (size_t(v) * ny + j) * nx + i; }
  size_t cm(int v, int i, int j) const { return c(v, bcmap(i, nx, bc), bcmap(j, ny, bc)); }
  // x-face f in [0, nx] lies between cells f-1 and f of row j
  size_t xf(int v, int f, int j) const { return (size_t(v) * ny + j) * (nx + 1) + f; }
  // y-face g in [0, ny] lies between rows g-1 and g of column i
  size_t yf(int v, int i, int g) const { return (size_t(v) * (ny + 1) + g) * nx + i; }

  void prim() {  // calcPrimitiveVariable (:226-263)
    Euler2<double> E(gamma);
#pragma omp parallel for
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double qq[4], ww[4];
        for (int v = 0; v < 4; ++v) qq[v] = q[c(v, i, j)];
        E.primitive(qq, ww);
        for (int v = 0; v < 4; ++v) w[c(v, i, j)] = ww[v];
        sr[c(0, i, j)] = std::sqrt(std::fabs(ww[0]));
        h[c(0, i, j)] = (qq[3] + ww[3]) / ww[0];
      }
  }

  void faces(int dir) {  // eigen2DEuler + the x/y characteristic sweeps (:265-400)
    if (ghost_rows()) return faces_ghost(dir);
    Euler2<double> E(gamma);
    const int nf = dir == 1 ? nx + 1 : ny + 1, nt = dir == 1 ? ny : nx;
#pragma omp parallel for
    for (int t_ = 0; t_ < nt; ++t_)
      for (int f = 0; f < nf; ++f) {
        auto at = [&](int v, int s) {  // cell s along the sweep (s = f - 1 is left of face)
          return dir == 1 ? cm(v, s, t_) : cm(v, t_, s);
        };
        double wa[4], wb[4], R[16], L[16];
        for (int v = 0; v < 4; ++v) { wa[v] = w[at(v, f - 1)]; wb[v] = w[at(v, f)]; }
        E.roe(dir, wa, sr[at(0, f - 1)], h[at(0, f - 1)], wb, sr[at(0, f)], h[at(0, f)], R, L);
        double ch[4][6];
        for (int m = 0; m < 6; ++m) {
          double qq[4];
          for (int v = 0; v < 4; ++v) qq[v] = q[at(v, f - 3 + m)];
          for (int r = 0; r < 4; ++r) {
            double s = L[4 * r] * qq[0];
            for (int k = 1; k < 4; ++k) s = s + L[4 * r + k] * qq[k];
            ch[r][m] = s;
          }
        }
        for (int r = 0; r < 4; ++r) {
          double o[2];
          lagrange_recon(recon, ch[r], o);
          const size_t idx = dir == 1 ? xf(r, f, t_) : yf(r, t_, f);
          (dir == 1 ? xl : yl)[idx] = o[0];
          (dir == 1 ? xr : yr)[idx] = o[1];
        }
        const size_t base = dir == 1 ? xf(0, f, t_) : yf(0, t_, f);
        const size_t stride = dir == 1 ? size_t(ny) * (nx + 1) : size_t(ny + 1) * nx;
        for (int k = 0; k < 16; ++k) {
          (dir == 1 ? xR : yR)[base + k * stride] = R[k];
          (dir == 1 ? xL : yL)[base + k * stride] = L[k];
        }
      }
  }

  // The same for boundaries whose ghosts are not copies of interior cells: every state comes
  // from ghost(), primitives of ghost cells are computed from their states (calcPrimitiveVariable
  // covers the ghosts), and the face rows -2, -1, nt, nt + 1 that the transverse GL3 reads are
  // computed too (the reference sweeps every row, :373-400), into gxl/gxr/gyl/gyr.
  void faces_ghost(int dir) {
    Euler2<double> E(gamma);
    const int nf = dir == 1 ? nx + 1 : ny + 1, nt = dir == 1 ? ny : nx;
#pragma omp parallel for
    for (int t_ = -2; t_ < nt + 2; ++t_)
      for (int f = 0; f < nf; ++f) {
        auto st = [&](int s_, double* qq) { dir == 1 ? ghost(s_, t_, qq) : ghost(t_, s_, qq); };
        auto pr = [&](int s_, double* ww, double& sr_, double& h_) {
          double qq[4];
          st(s_, qq);
          E.primitive(qq, ww);
          sr_ = std::sqrt(std::fabs(ww[0]));
          h_ = (qq[3] + ww[3]) / ww[0];
        };
        double wa[4], wb[4], sra, srb, ha, hb, R[16], L[16];
        pr(f - 1, wa, sra, ha);
        pr(f, wb, srb, hb);
        E.roe(dir, wa, sra, ha, wb, srb, hb, R, L);
        double ch[4][6];
        for (int m = 0; m < 6; ++m) {
          double qq[4];
          st(f - 3 + m, qq);
          for (int r = 0; r < 4; ++r) {
            double s = L[4 * r] * qq[0];
            for (int k = 1; k < 4; ++k) s = s + L[4 * r + k] * qq[k];
            ch[r][m] = s;
          }
        }
        const bool interior = t_ >= 0 && t_ < nt;
        const int gr = t_ < 0 ? t_ + 2 : t_ - nt + 2;  // ghost face row 0..3
        for (int r = 0; r < 4; ++r) {
          double o[2];
          lagrange_recon(recon, ch[r], o);
          if (interior) {
            const size_t idx = dir == 1 ? xf(r, f, t_) : yf(r, t_, f);
            (dir == 1 ? xl : yl)[idx] = o[0];
            (dir == 1 ? xr : yr)[idx] = o[1];
          } else {
            const size_t idx = (size_t(gr) * 4 + r) * nf + f;
            (dir == 1 ? gxl : gyl)[idx] = o[0];
            (dir == 1 ? gxr : gyr)[idx] = o[1];
          }
        }
        if (!interior) continue;
        const size_t base = dir == 1 ? xf(0, f, t_) : yf(0, t_, f);
        const size_t stride = dir == 1 ? size_t(ny) * (nx + 1) : size_t(ny + 1) * nx;
        for (int k = 0; k < 16; ++k) {
          (dir == 1 ? xR : yR)[base + k * stride] = R[k];
          (dir == 1 ? xL : yL)[base + k * stride] = L[k];
        }
      }
  }

  void fluxes(int dir) {  // transverse GL3 (:402-423), R back-projection (:425-430), flux (:432-497)
    Euler2<double> E(gamma);
    const int nf = dir == 1 ? nx + 1 : ny + 1, nt = dir == 1 ? ny : nx;
    const int ntr = nt;  // transverse extent
    const std::vector<double>& FL = dir == 1 ? xl : yl;
    const std::vector<double>& FR = dir == 1 ? xr : yr;
    const size_t stride = dir == 1 ? size_t(ny) * (nx + 1) : size_t(ny + 1) * nx;
    const LagrangeCoef& K = lag();
#pragma omp parallel for
    for (int t_ = 0; t_ < nt; ++t_)
      for (int f = 0; f < nf; ++f) {
        double gl[4][3], gr[4][3];
        for (int r = 0; r < 4; ++r) {
          double a[5], b[5];
          for (int m = 0; m < 5; ++m) {
            const int tr = t_ - 2 + m;
            if (ghost_rows() && (tr < 0 || tr >= ntr)) {
              const int gr = tr < 0 ? tr + 2 : tr - ntr + 2;
              const size_t idx = (size_t(gr) * 4 + r) * nf + f;
              a[m] = (dir == 1 ? gxl : gyl)[idx];
              b[m] = (dir == 1 ? gxr : gyr)[idx];
              continue;
            }
            const int tt = bcmap(tr, ntr, bc);
            const size_t idx = dir == 1 ? xf(r, f, tt) : yf(r, tt, f);
            a[m] = FL[idx];
            b[m] = FR[idx];
          }
          gl3(a, gl[r]);
          gl3(b, gr[r]);
        }
        const size_t base = dir == 1 ? xf(0, f, t_) : yf(0, t_, f);
        double R[16], L[16];
        for (int k = 0; k < 16; ++k) {
          R[k] = (dir == 1 ? xR : yR)[base + k * stride];
          L[k] = (dir == 1 ? xL : yL)[base + k * stride];
        }
        double Fm[3][4];
        for (int m = 0; m < 3; ++m) {
          double ql[4], qr[4], F[4];
          for (int i = 0; i < 4; ++i) {
            double sl = R[4 * i] * gl[0][m], sr_ = R[4 * i] * gr[0][m];
            for (int k = 1; k < 4; ++k) {
              sl = sl + R[4 * i + k] * gl[k][m];
              sr_ = sr_ + R[4 * i + k] * gr[k][m];
            }
            ql[i] = sl;
            qr[i] = sr_;
          }
          if (flux == FLUX_HLLC) E.hllc(dir, ql, qr, F);
          else E.rusanov(dir, ql, qr, L, R, F);
          for (int i = 0; i < 4; ++i) Fm[m][i] = K.gl3w[m] * F[i];
        }
        for (int i = 0; i < 4; ++i) {
          const double s = (Fm[0][i] + Fm[1][i]) + Fm[2][i];
          (dir == 1 ? fx : fy)[base + size_t(i) * stride] = s;
        }
      }
  }

  void residual() {  // rhs (:363-573)
    prim();
    faces(1);
    faces(2);
    fluxes(1);
    fluxes(2);
#pragma omp parallel for
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        for (int v = 0; v < 4; ++v)
          rhsu[c(v, i, j)] = ((fx[xf(v, i, j)] - fx[xf(v, i + 1, j)]) * dy +
                              (fy[yf(v, i, j)] - fy[yf(v, i, j + 1)]) * dx) / area + 0.0;
  }

  double compute_dt(double tFinal) {  // timeStepping (:622-645)
    Euler2<double> E(gamma);
    double mx = 0.0, my = 0.0;
    prim();
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double ww[4];
        for (int v = 0; v < 4; ++v) ww[v] = w[c(v, i, j)];
        mx = std::fmax(mx, E.maxSpeed(ww, 1));
        my = std::fmax(my, E.maxSpeed(ww, 2));
      }
    double d = cfl * std::pow(std::fmin(dx, dy), 3.0 / 3.0) / std::fmax(mx, my);
    return t + d > tFinal ? tFinal - t : d;
  }

  void rk3() {  // RungeKutta3 (:575-612)
    const size_t n = q.size();
    q0 = q;
    residual();
    for (size_t k = 0; k < n; ++k) q1[k] = ssprk3(q0[k], q0[k], rhsu[k], dt, 1);
    q = q1;
    residual();
    for (size_t k = 0; k < n; ++k) q1[k] = ssprk3(q0[k], q[k], rhsu[k], dt, 2);
    q = q1;
    residual();
    for (size_t k = 0; k < n; ++k) q1[k] = ssprk3(q0[k], q[k], rhsu[k], dt, 3);
    q = q1;
  }

  int run(int nsteps, double tFinal) {
    int s = 0;
    while (t < tFinal && s < nsteps) {
      dt = compute_dt(tFinal);
      rk3();
      t += dt;
      ++s;
    }
    return s;
  }
};

// FV::System1D (FV_System1D.cpp): rhs :158-241, RungeKutta3 :243-272, timeStepping :274-292.
// The reference ships teno5i + Rusanov (:200, :229-231); teno5 and HLLC are its commented
// alternatives (:233).  The KXRCF flag (:171-192) selects teno5i on both branches, so it has no
// effect and is not restated.
struct FV1D {
  int nx, bc, flux, recon;
  double dx, area, cfl, gamma, t = 0.0, dt = 0.0;
  std::vector<double> q, q0, q1, rhsu, F;  // q [3][nx]; F [3][nx+1]

  FV1D(int nx_, double x0, double x1, double cfl_, double g, int bc_ = BC_ZEROGRAD,
       int flux_ = FLUX_RUSANOV, int recon_ = RECON_TENO5I)
      : nx(nx_), bc(bc_), flux(flux_), recon(recon_), cfl(cfl_), gamma(g) {
    dx = (x1 - x0) / nx;
    area = dx;
    q.assign(3 * size_t(nx), 0.0); q0 = q; q1 = q; rhsu = q;
    F.assign(3 * size_t(nx + 1), 0.0);
  }
  double at(int v, int i) const { return q[size_t(v) * nx + bcmap(i, nx, bc)]; }

  void residual() {
    Euler1<double> E(gamma);
    for (int f = 0; f <= nx; ++f) {
      double wa[3], wb[3], qa[3], qb[3];
      for (int v = 0; v < 3; ++v) { qa[v] = at(v, f - 1); qb[v] = at(v, f); }
      E.primitive(qa, wa);
      E.primitive(qb, wb);
      double R[9], L[9];
      E.roe(wa, std::sqrt(std::fabs(wa[0])), (qa[2] + wa[2]) / wa[0], wb,
            std::sqrt(std::fabs(wb[0])), (qb[2] + wb[2]) / wb[0], R, L);
      double ch[3][6];
      for (int m = 0; m < 6; ++m)
        for (int r = 0; r < 3; ++r) {
          double s = L[3 * r] * at(0, f - 3 + m);
          for (int k = 1; k < 3; ++k) s = s + L[3 * r + k] * at(k, f - 3 + m);
          ch[r][m] = s;
        }
      double cl[3], cr[3];
      for (int r = 0; r < 3; ++r) {
        double o[2];
        lagrange_recon(recon, ch[r], o);
        cl[r] = o[0];
        cr[r] = o[1];
      }
      double ql[3], qr[3], Ff[3];
      for (int i = 0; i < 3; ++i) {  // transformToConservative (FV_System1D.h:48-51)
        double sl = R[3 * i] * cl[0], sr_ = R[3 * i] * cr[0];
        for (int k = 1; k < 3; ++k) {
          sl = sl + R[3 * i + k] * cl[k];
          sr_ = sr_ + R[3 * i + k] * cr[k];
        }
        ql[i] = sl;
        qr[i] = sr_;
      }
      if (flux == FLUX_HLLC) E.hllc(ql, qr, Ff);
      else E.rusanov(ql, qr, L, R, Ff);
      for (int v = 0; v < 3; ++v) F[size_t(v) * (nx + 1) + f] = Ff[v];
    }
    for (int i = 0; i < nx; ++i)
      for (int v = 0; v < 3; ++v)
        rhsu[size_t(v) * nx + i] = (F[size_t(v) * (nx + 1) + i] - F[size_t(v) * (nx + 1) + i + 1]) / area;
  }
  double compute_dt(double tFinal) {
    Euler1<double> E(gamma);
    double mx = 0.0;
    for (int i = 0; i < nx; ++i) {
      double qq[3] = {at(0, i), at(1, i), at(2, i)}, ww[3];
      E.primitive(qq, ww);
      mx = std::fmax(mx, E.maxSpeed(ww));
    }
    double d = cfl * std::pow(dx, 3.0 / 3.0) / mx;
    return t + d > tFinal ? tFinal - t : d;
  }
  void rk3() {
    const size_t n = q.size();
    q0 = q;
    residual();
    for (size_t k = 0; k < n; ++k) q1[k] = ssprk3(q0[k], q0[k], rhsu[k], dt, 1);
    q = q1;
    residual();
    for (size_t k = 0; k < n; ++k) q1[k] = ssprk3(q0[k], q[k], rhsu[k], dt, 2);
    q = q1;
    residual();
    for (size_t k = 0; k < n; ++k) q1[k] = ssprk3(q0[k], q[k], rhsu[k], dt, 3);
    q = q1;
  }
  int run(int nsteps, double tFinal) {
    int s = 0;
    while (t < tFinal && s < nsteps) {
      dt = compute_dt(tFinal);
      rk3();
      t += dt;
      ++s;
    }
    return s;
  }
};

// FVHermite::System2D (FVHermite_System2D.cpp): u plus first moments v = d/dx, w = d/dy.
// rhs :429-731 (zeroGradBc, limitDerivatives, zeroGradBc, primitives, eigen2DEuler, HTENO on
// (u, v) in x and (u, w) in y, TENO5 for the cross moment, GL3 transverse for all of them,
// Rusanov for u and dRusanov for v, w); RungeKutta3 :733-782; timeStepping :784-819.
// The Hermite coefficients use dx for both directions (setGridSize(dx), :28).
// limitDerivatives (:393-427) updates v in place while sweeping i (and w while sweeping j);
// with one thread that is a Gauss-Seidel sweep, which is the semantics restated here.
struct Hermite2D {
  int nx, ny;
  double dx, dy, area, cfl, gamma, t = 0.0, dt = 0.0;
  HermiteCoef HK;
  std::vector<double> q, v, w, q0, v0, w0, ru, rv, rw;  // [4][ny][nx]

  Hermite2D(int nx_, int ny_, double xl0, double xr0, double yb, double yt, double cfl_, double g)
      : nx(nx_), ny(ny_), cfl(cfl_), gamma(g), HK((xr0 - xl0) / nx_) {
    dx = (xr0 - xl0) / nx;
    dy = (yt - yb) / ny;
    area = dx * dy;
    const size_t n = 4 * size_t(nx) * ny;
    q.assign(n, 0.0); v = q; w = q; q0 = q; v0 = q; w0 = q; ru = q; rv = q; rw = q;
  }
  size_t c(int var, int i, int j) const { return (size_t(var) * ny + j) * nx + i; }
  size_t cm(int var, int i, int j) const {
    return c(var, bcmap(i, nx, BC_ZEROGRAD), bcmap(j, ny, BC_ZEROGRAD));
  }

  void limit() {
    std::vector<double> vold = v, wold = w;
    // x: v along each row, i increasing; ghost neighbours hold the pre-sweep values
#pragma omp parallel for
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        for (int e = 0; e < 4; ++e) {
          double uu[3] = {q[cm(e, i - 1, j)], q[c(e, i, j)], q[cm(e, i + 1, j)]};
          double dd[3] = {i > 0 ? v[c(e, i - 1, j)] : vold[c(e, 0, j)], v[c(e, i, j)],
                          i + 1 < nx ? v[c(e, i + 1, j)] : vold[c(e, nx - 1, j)]};
          v[c(e, i, j)] = hermite_limiter(HK, uu, dd);
        }
    // y: w along each column, j increasing
#pragma omp parallel for
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int e = 0; e < 4; ++e) {
          double uu[3] = {q[cm(e, i, j - 1)], q[c(e, i, j)], q[cm(e, i, j + 1)]};
          double dd[3] = {j > 0 ? w[c(e, i, j - 1)] : wold[c(e, i, 0)], w[c(e, i, j)],
                          j + 1 < ny ? w[c(e, i, j + 1)] : wold[c(e, i, ny - 1)]};
          w[c(e, i, j)] = hermite_limiter(HK, uu, dd);
        }
  }

  void residual() {
    Euler2<double> E(gamma);
    const LagrangeCoef& K = lag();
    limit();
    // cell primitives
    std::vector<double> pw(4 * size_t(nx) * ny), psr(size_t(nx) * ny), ph(size_t(nx) * ny);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double qq[4], ww[4];
        for (int e = 0; e < 4; ++e) qq[e] = q[c(e, i, j)];
        E.primitive(qq, ww);
        for (int e = 0; e < 4; ++e) pw[c(e, i, j)] = ww[e];
        psr[c(0, i, j)] = std::sqrt(std::fabs(ww[0]));
        ph[c(0, i, j)] = (qq[3] + ww[3]) / ww[0];
      }
    // face reconstruction, both directions.  Per face: 6 characteristic arrays x 4 fields:
    // 0 u-, 1 u+, 2 dn- (moment along the sweep), 3 dn+, 4 dt- (cross moment), 5 dt+
    for (int dir = 1; dir <= 2; ++dir) {
      const int nf = dir == 1 ? nx + 1 : ny + 1, nt = dir == 1 ? ny : nx;
      std::vector<double> fc(size_t(24) * nf * nt), fR(size_t(16) * nf * nt), fL(size_t(16) * nf * nt);
      std::vector<double>& qn = dir == 1 ? v : w;   // moment along the sweep (HTENO)
      std::vector<double>& qt = dir == 1 ? w : v;   // cross moment (TENO5)
#pragma omp parallel for
      for (int t_ = 0; t_ < nt; ++t_)
        for (int f = 0; f < nf; ++f) {
          auto at = [&](int e, int s) { return dir == 1 ? cm(e, s, t_) : cm(e, t_, s); };
          double wa[4], wb[4], R[16], L[16];
          for (int e = 0; e < 4; ++e) { wa[e] = pw[at(e, f - 1)]; wb[e] = pw[at(e, f)]; }
          E.roe(dir, wa, psr[at(0, f - 1)], ph[at(0, f - 1)], wb, psr[at(0, f)], ph[at(0, f)], R, L);
          auto proj = [&](const std::vector<double>& src, int s, double* out4) {
            double x[4];
            for (int e = 0; e < 4; ++e) x[e] = src[at(e, s)];
            for (int r = 0; r < 4; ++r) {
              double acc = L[4 * r] * x[0];
              for (int k2 = 1; k2 < 4; ++k2) acc = acc + L[4 * r + k2] * x[k2];
              out4[r] = acc;
            }
          };
          double A[4][4], B[4][4], C6[4][6];
          for (int m = 0; m < 4; ++m) {
            double a4[4], b4[4];
            proj(q, f - 2 + m, a4);
            proj(qn, f - 2 + m, b4);
            for (int r = 0; r < 4; ++r) { A[r][m] = a4[r]; B[r][m] = b4[r]; }
          }
          for (int m = 0; m < 6; ++m) {
            double c4[4];
            proj(qt, f - 3 + m, c4);
            for (int r = 0; r < 4; ++r) C6[r][m] = c4[r];
          }
          const size_t o = size_t(t_) * nf + f, stride = size_t(nf) * nt;
          for (int r = 0; r < 4; ++r) {
            double hv[4], tv[2];
            hermite_recon(HK, 0, A[r], B[r], hv);
            lagrange_recon(RECON_TENO5, C6[r], tv);
            fc[(0 * 4 + r) * stride + o] = hv[0];
            fc[(1 * 4 + r) * stride + o] = hv[1];
            fc[(2 * 4 + r) * stride + o] = hv[2];
            fc[(3 * 4 + r) * stride + o] = hv[3];
            fc[(4 * 4 + r) * stride + o] = tv[0];
            fc[(5 * 4 + r) * stride + o] = tv[1];
          }
          for (int k2 = 0; k2 < 16; ++k2) { fR[k2 * stride + o] = R[k2]; fL[k2 * stride + o] = L[k2]; }
        }
      // transverse GL3 + fluxes
      std::vector<double> F(size_t(12) * nf * nt);  // [3 kinds][4][face]
#pragma omp parallel for
      for (int t_ = 0; t_ < nt; ++t_)
        for (int f = 0; f < nf; ++f) {
          const size_t stride = size_t(nf) * nt, o = size_t(t_) * nf + f;
          double G[6][4][3];
          for (int a = 0; a < 6; ++a)
            for (int r = 0; r < 4; ++r) {
              double u5[5];
              for (int m = 0; m < 5; ++m)
                u5[m] = fc[(a * 4 + r) * stride + size_t(bcmap(t_ - 2 + m, nt, BC_ZEROGRAD)) * nf + f];
              gl3(u5, G[a][r]);
            }
          double R[16], L[16];
          for (int k2 = 0; k2 < 16; ++k2) { R[k2] = fR[k2 * stride + o]; L[k2] = fL[k2 * stride + o]; }
          // conservative values at the Gauss points: transformToConservativeAtGQ
          double X[6][3][4];
          for (int a = 0; a < 6; ++a)
            for (int m = 0; m < 3; ++m)
              for (int i2 = 0; i2 < 4; ++i2) {
                double acc = R[4 * i2] * G[a][0][m];
                for (int k2 = 1; k2 < 4; ++k2) acc = acc + R[4 * i2 + k2] * G[a][k2][m];
                X[a][m][i2] = acc;
              }
          double Fu[3][4], Fn[3][4], Ft[3][4];
          for (int m = 0; m < 3; ++m) {
            double fu[4], fn[4], ft[4];
            E.rusanov(dir, X[0][m], X[1][m], L, R, fu);
            E.drusanov(dir, X[0][m], X[1][m], X[2][m], X[3][m], L, R, fn);
            E.drusanov(dir, X[0][m], X[1][m], X[4][m], X[5][m], L, R, ft);
            for (int i2 = 0; i2 < 4; ++i2) {
              Fu[m][i2] = K.gl3w[m] * fu[i2];
              Fn[m][i2] = K.gl3w[m] * fn[i2];
              Ft[m][i2] = K.gl3w[m] * ft[i2];
            }
          }
          for (int i2 = 0; i2 < 4; ++i2) {
            F[(0 * 4 + i2) * stride + o] = (Fu[0][i2] + Fu[1][i2]) + Fu[2][i2];
            F[(1 * 4 + i2) * stride + o] = (Fn[0][i2] + Fn[1][i2]) + Fn[2][i2];
            F[(2 * 4 + i2) * stride + o] = (Ft[0][i2] + Ft[1][i2]) + Ft[2][i2];
          }
        }
      // flux differences: kind 0 -> u, 1 -> moment along this sweep, 2 -> cross moment
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
          for (int e = 0; e < 4; ++e) {
            const size_t stride = size_t(nf) * nt;
            const int f0 = dir == 1 ? i : j, t0 = dir == 1 ? j : i;
            const size_t oa = size_t(t0) * nf + f0, ob = oa + 1;
            for (int kind = 0; kind < 3; ++kind) {
              const double d = F[(kind * 4 + e) * stride + oa] - F[(kind * 4 + e) * stride + ob];
              std::vector<double>& dst = kind == 0 ? ru : ((kind == 1) == (dir == 1) ? rv : rw);
              if (dir == 1) dst[c(e, i, j)] = d;  // (F(i-1) - F(i)), combined below
              else dst[c(e, i, j)] = (dst[c(e, i, j)] * dy + d * dx) / area + 0.0;
            }
          }
    }
  }

  double compute_dt(double tFinal) {
    Euler2<double> E(gamma);
    double mx = 0.0, my = 0.0;
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double qq[4], ww[4];
        for (int e = 0; e < 4; ++e) qq[e] = q[c(e, i, j)];
        E.primitive(qq, ww);
        mx = std::fmax(mx, E.maxSpeed(ww, 1));
        my = std::fmax(my, E.maxSpeed(ww, 2));
      }
    double d = cfl * std::pow(std::fmin(dx, dy), 3.0 / 3.0) / std::fmax(mx, my) / 1.0;
    return t + d > tFinal ? tFinal - t : d;
  }
  // RungeKutta3 (:733-782): save() runs after the first rhs(), so v0, w0 are the limited
  // moments; stages 2 and 3 combine with the unlimited stage values v1, v2 (cell.v1 / cell.v2).
  void rk3() {
    const size_t n = q.size();
    std::vector<double> qs = q, vs = v, ws = w;  // u_{s}, v_{s}, w_{s} as stored by update1/2
    for (int stage = 1; stage <= 3; ++stage) {
      residual();
      if (stage == 1) { q0 = q; v0 = v; w0 = w; qs = q0; vs = v0; ws = w0; }
      for (size_t k = 0; k < n; ++k) {
        qs[k] = ssprk3(q0[k], qs[k], ru[k], dt, stage);
        vs[k] = ssprk3(v0[k], vs[k], rv[k], dt, stage);
        ws[k] = ssprk3(w0[k], ws[k], rw[k], dt, stage);
      }
      q = qs; v = vs; w = ws;
    }
  }
  int run(int nsteps, double tFinal) {
    int s = 0;
    while (t < tFinal && s < nsteps) {
      dt = compute_dt(tFinal);
      rk3();
      t += dt;
      ++s;
    }
    return s;
  }
};

// FVHermite::System1D (FVHermite_System1D.cpp): periodic boundaries (:201), LMPE troubled-cell
// flags (:239-257) that start false and are never reset, the derivative limiter applied once
// over the padded range when any flag in [s+1, nxx-s-1) is set (:259-273; the loop reuses the
// outer index, so it runs at most once per rhs), htenoi on flagged cells and linear elsewhere
// (:278-291), Rusanov + dRusanov (:306-337), dt = cfl * dx^(5/3) / max speed (:396).
// Flags live on the ghost-padded index space [0, nx + 2k) exactly as in the reference.
struct Hermite1D {
  static const int k = 4, s = 1;
  int nx, nxx;
  double dx, area, cfl, gamma, t = 0.0, dt = 0.0;
  HermiteCoef HK;
  std::vector<double> u, v, u0, v0, ru, rv;  // padded [3][nxx]
  std::vector<unsigned char> flag;           // padded [nxx][3]

  Hermite1D(int nx_, double x0, double x1, double cfl_, double g)
      : nx(nx_), nxx(nx_ + 2 * k), cfl(cfl_), gamma(g), HK((x1 - x0) / nx_) {
    dx = (x1 - x0) / nx;
    area = dx;
    u.assign(3 * size_t(nxx), 0.0); v = u; u0 = u; v0 = u; ru = u; rv = u;
    flag.assign(3 * size_t(nxx), 0);
  }
  double& U(int e, int i) { return u[size_t(e) * nxx + i]; }
  double& V(int e, int i) { return v[size_t(e) * nxx + i]; }
  void periodic() {  // periodicBc (:161-170)
    for (int m = 0; m < k; ++m)
      for (int e = 0; e < 3; ++e) {
        U(e, k - 1 - m) = U(e, nx + k - 1 - m);
        U(e, nxx - 1 - m) = U(e, k + k - 1 - m);
        V(e, k - 1 - m) = V(e, nx + k - 1 - m);
        V(e, nxx - 1 - m) = V(e, k + k - 1 - m);
      }
  }
  void residual() {
    Euler1<double> E(gamma);
    periodic();
    // LMPE
    for (int e = 0; e < 3; ++e)
      for (int i = s + 1; i < nxx - s - 1; ++i) {
        if (flag[size_t(i) * 3 + e]) continue;
        double A = std::fabs(-U(e, i - 1) + 2.0 * U(e, i) - U(e, i + 1)) / 2.0;
        if (A > 0.5 * dx) {
          double xc = (-2. * U(e, i - 1) + 3. * U(e, i) - U(e, i + 1)) /
                      (-U(e, i - 1) + 2.0 * U(e, i) - U(e, i + 1)) * dx;
          if (0.0 <= xc && xc <= 3. * dx) {
            flag[size_t(i) * 3 + e] = 1;
            flag[size_t(i - 1) * 3 + e] = 1;
            flag[size_t(i + 1) * 3 + e] = 1;
          }
        }
      }
    bool any = false;
    for (int i = s + 1; i < nxx - s - 1 && !any; ++i)
      any = flag[size_t(i) * 3] || flag[size_t(i) * 3 + 1] || flag[size_t(i) * 3 + 2];
    if (any)
      for (int i = k - 1; i < nxx - k + 1; ++i) {
        double uu[3][3], vv[3][3];
        for (int m = 0; m < 3; ++m)
          for (int e = 0; e < 3; ++e) { uu[e][m] = U(e, i - 1 + m); vv[e][m] = V(e, i - 1 + m); }
        for (int e = 0; e < 3; ++e) V(e, i) = hermite_limiter(HK, uu[e], vv[e]);
      }
    periodic();
    // faces i in [k-1, nxx-k): between padded cells i and i+1
    std::vector<double> Fu(3 * size_t(nxx)), Fv(3 * size_t(nxx));
    for (int i = k - 1; i < nxx - k; ++i) {
      double qa[3], qb[3], wa[3], wb[3], R[9], L[9];
      for (int e = 0; e < 3; ++e) { qa[e] = U(e, i); qb[e] = U(e, i + 1); }
      E.primitive(qa, wa);
      E.primitive(qb, wb);
      E.roe(wa, std::sqrt(std::fabs(wa[0])), (qa[2] + wa[2]) / wa[0], wb,
            std::sqrt(std::fabs(wb[0])), (qb[2] + wb[2]) / wb[0], R, L);
      double A[3][4], B[3][4];
      for (int m = 0; m < 4; ++m)
        for (int r = 0; r < 3; ++r) {
          double a = L[3 * r] * U(0, i - 1 + m), b = L[3 * r] * V(0, i - 1 + m);
          for (int k2 = 1; k2 < 3; ++k2) {
            a = a + L[3 * r + k2] * U(k2, i - 1 + m);
            b = b + L[3 * r + k2] * V(k2, i - 1 + m);
          }
          A[r][m] = a;
          B[r][m] = b;
        }
      double cl[4][3];  // [u-, u+, v-, v+][field]
      for (int r = 0; r < 3; ++r) {
        double o[4];
        hermite_recon(HK, flag[size_t(i) * 3 + r] ? 1 : 2, A[r], B[r], o);
        for (int a = 0; a < 4; ++a) cl[a][r] = o[a];
      }
      double X[4][3];
      for (int a = 0; a < 4; ++a)
        for (int i2 = 0; i2 < 3; ++i2) {
          double acc = R[3 * i2] * cl[a][0];
          for (int k2 = 1; k2 < 3; ++k2) acc = acc + R[3 * i2 + k2] * cl[a][k2];
          X[a][i2] = acc;
        }
      double fu[3], fv[3];
      E.rusanov(X[0], X[1], L, R, fu);
      E.drusanov(X[0], X[1], X[2], X[3], L, R, fv);
      for (int e = 0; e < 3; ++e) { Fu[size_t(e) * nxx + i] = fu[e]; Fv[size_t(e) * nxx + i] = fv[e]; }
    }
    for (int i = k; i < nxx - k; ++i)
      for (int e = 0; e < 3; ++e) {
        ru[size_t(e) * nxx + i] = (Fu[size_t(e) * nxx + i - 1] - Fu[size_t(e) * nxx + i]) / area;
        rv[size_t(e) * nxx + i] = (Fv[size_t(e) * nxx + i - 1] - Fv[size_t(e) * nxx + i]) / area;
      }
  }
  double compute_dt(double tFinal) {
    Euler1<double> E(gamma);
    double mx = 0.0;
    for (int i = k; i < nxx - k; ++i) {
      double qq[3] = {U(0, i), U(1, i), U(2, i)}, ww[3];
      E.primitive(qq, ww);
      mx = std::fmax(mx, E.maxSpeed(ww));
    }
    double d = cfl * std::pow(dx, 5.0 / 3.0) / mx;
    return t + d > tFinal ? tFinal - t : d;
  }
  // RungeKutta3 (:345-381): save() after the first rhs() (v0 may be limited); stages 2 and 3
  // combine with the unlimited stage values v1, v2.
  void rk3() {
    std::vector<double> us = u, vs = v;
    for (int stage = 1; stage <= 3; ++stage) {
      residual();
      if (stage == 1) { u0 = u; v0 = v; us = u; vs = v; }
      for (int e = 0; e < 3; ++e)
        for (int i = k; i < nxx - k; ++i) {
          const size_t o = size_t(e) * nxx + i;
          us[o] = ssprk3(u0[o], us[o], ru[o], dt, stage);
          vs[o] = ssprk3(v0[o], vs[o], rv[o], dt, stage);
        }
      for (int e = 0; e < 3; ++e)
        for (int i = k; i < nxx - k; ++i) {
          const size_t o = size_t(e) * nxx + i;
          u[o] = us[o];
          v[o] = vs[o];
        }
    }
  }
  int run(int nsteps, double tFinal) {
    int st = 0;
    while (t < tFinal && st < nsteps) {
      dt = compute_dt(tFinal);
      rk3();
      t += dt;
      ++st;
    }
    return st;
  }
};

}  // namespace orc
