// Driver that links the reference solver's own, unmodified sources (built against the
// project-written Eigen-subset header in eigen_compat/) and exposes them through extern "C"
// entry points.  It is test infrastructure: its only users are the golden-fixture generator
// (tests/golden/make_golden.py) and the oracle-validation tests.  Build recipe: oracle/Makefile
// target `ref`, output oracle/_ref/libhteno_ref.so.
//
// The reference solvers keep their grid and time-stepping state private and offer no way to
// set an arbitrary initial state or to stop after N steps.  This driver therefore opens the
// class members (a textual `private`->`public` switch applied only while the reference headers
// are parsed here; the reference .cpp files are compiled unchanged) and restates the small
// time-stepping loop of each solver's timeStepping() so that a run can stop after N steps.
// Every numerical call made below is a reference function.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>
#include <omp.h>
#include <Eigen/Dense>

#define private public
#define protected public
#include "Equations_Euler1D.h"
#include "Equations_Euler2D.h"
#include "FVHermite_System1D.h"
#include "FVHermite_System2D.h"
#include "FV_System1D.h"
#include "FV_System2D.h"
#include "Schemes_Hermite.h"
#include "Schemes_Lagrange.h"
#include "Schemes_SSPRK.h"
#undef private
#undef protected

namespace {

// The reference prints progress to std::cout; silence it while a call runs.
struct Quiet {
  std::streambuf* old;
  std::ostringstream sink;
  Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~Quiet() { std::cout.rdbuf(old); }
};

template <int N>
Eigen::Matrix<double, N, 1> vec(const double* p) {
  Eigen::Matrix<double, N, 1> v;
  for (int k = 0; k < N; ++k) v(k) = p[k];
  return v;
}
template <int N>
void put(const Eigen::Matrix<double, N, 1>& v, double* p) {
  for (int k = 0; k < N; ++k) p[k] = v(k);
}
Eigen::Matrix4d mat4(const double* p) {  // row-major input
  Eigen::Matrix4d m;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) m(i, j) = p[4 * i + j];
  return m;
}

}  // namespace

extern "C" {

// ---- Schemes::Lagrange (Schemes_Lagrange.cpp) ----------------------------------------------
void ref_teno5(const double* u, double* out, long n) {
  Schemes::Lagrange L;
  for (long k = 0; k < n; ++k) put<2>(L.teno5(vec<6>(u + 6 * k)), out + 2 * k);
}
void ref_teno5i(const double* u, double* out, long n) {
  Schemes::Lagrange L;
  for (long k = 0; k < n; ++k) put<2>(L.teno5i(vec<6>(u + 6 * k)), out + 2 * k);
}
void ref_linear5(const double* u, double* out, long n) {
  Schemes::Lagrange L;
  for (long k = 0; k < n; ++k) put<2>(L.linear(vec<6>(u + 6 * k)), out + 2 * k);
}
// weno5JS / weno5Z / weno5N / teno5N / teno5a (Schemes_Lagrange.cpp:358-594, 1265-1294)
void ref_lagrange_alt(int kind, const double* u, double* out, long n) {
  Schemes::Lagrange L;
  for (long k = 0; k < n; ++k) {
    const auto v = vec<6>(u + 6 * k);
    switch (kind) {
      case 3: put<2>(L.weno5JS(v), out + 2 * k); break;
      case 4: put<2>(L.weno5Z(v), out + 2 * k); break;
      case 5: put<2>(L.weno5N(v), out + 2 * k); break;
      case 6: put<2>(L.teno5N(v), out + 2 * k); break;
      default: put<2>(L.teno5a(v), out + 2 * k); break;
    }
  }
}
void ref_gl3(const double* u, double* out, long n) {
  Schemes::Lagrange L;
  for (long k = 0; k < n; ++k) put<3>(L.weno5JS3PointsQuadrature(vec<5>(u + 5 * k)), out + 3 * k);
}

// ---- Schemes::Hermite (Schemes_Hermite.cpp) -------------------------------------------------
// kind: 0 hteno, 1 htenoi, 2 linear
void ref_hermite_recon(int kind, double dx, const double* u, const double* d, double* out, long n) {
  Quiet q;
  Schemes::Hermite H;
  H.setGridSize(dx);
  for (long k = 0; k < n; ++k) {
    Eigen::Vector4d r = kind == 0   ? H.hteno(vec<4>(u + 4 * k), vec<4>(d + 4 * k))
                        : kind == 1 ? H.htenoi(vec<4>(u + 4 * k), vec<4>(d + 4 * k))
                                    : H.linear(vec<4>(u + 4 * k), vec<4>(d + 4 * k));
    put<4>(r, out + 4 * k);
  }
}
void ref_hermite_limiter(double dx, const double* u, const double* d, double* out, long n) {
  Quiet q;
  Schemes::Hermite H;
  H.setGridSize(dx);
  for (long k = 0; k < n; ++k) out[k] = H.hermiteLimiter(vec<3>(u + 3 * k), vec<3>(d + 3 * k));
}

// ---- Schemes::SSPRK (Schemes_SSPRK.cpp) ------------------------------------------------------
void ref_ssprk3(const double* q0, const double* qn, const double* rhs, double dt, int stage,
                double* out, long n) {
  Schemes::SSPRK rk;
  for (long k = 0; k < n; ++k) out[k] = rk.RungeKuttaIII<double>(q0[k], qn[k], rhs[k], dt, stage);
}

// ---- Equations::Euler2D / Euler1D -------------------------------------------------------------
void ref_hllc2d(double gamma, int dir, const double* ql, const double* qr, double* out, long n) {
  Equations::Euler2D E(gamma);
  for (long k = 0; k < n; ++k) put<4>(E.HLLC(vec<4>(ql + 4 * k), vec<4>(qr + 4 * k), dir), out + 4 * k);
}
void ref_hllc1d(double gamma, const double* ql, const double* qr, double* out, long n) {
  Equations::Euler1D E(gamma);
  for (long k = 0; k < n; ++k) put<3>(E.HLLC(vec<3>(ql + 3 * k), vec<3>(qr + 3 * k)), out + 3 * k);
}
// Characteristic Rusanov flux exactly as called in FV_System2D.cpp:436-464:
// aM = maxLocalWaveSpeed(w(ql), w(qr), dir); Rusanov(ql, qr, w(ql), w(qr), L, R, aM, dir).
// L and R are row-major 4x4 per entry.
void ref_rusanov2d(double gamma, int dir, const double* ql, const double* qr, const double* Lm,
                   const double* Rm, double* out, long n) {
  Equations::Euler2D E(gamma);
  for (long k = 0; k < n; ++k) {
    Eigen::Vector4d a = vec<4>(ql + 4 * k), b = vec<4>(qr + 4 * k);
    Eigen::Vector4d wl = E.primitive(a), wr = E.primitive(b);
    Eigen::Vector4d aM = E.maxLocalWaveSpeed(wl, wr, dir) / 1.0;
    put<4>(E.Rusanov(a, b, wl, wr, mat4(Lm + 16 * k), mat4(Rm + 16 * k), aM, dir), out + 4 * k);
  }
}
// Derivative-moment flux as called in FVHermite_System2D.cpp:553-589.
void ref_drusanov2d(double gamma, int dir, const double* ql, const double* qr, const double* dql,
                    const double* dqr, const double* Lm, const double* Rm, double* out, long n) {
  Equations::Euler2D E(gamma);
  for (long k = 0; k < n; ++k) {
    Eigen::Vector4d a = vec<4>(ql + 4 * k), b = vec<4>(qr + 4 * k);
    Eigen::Vector4d wl = E.primitive(a), wr = E.primitive(b);
    Eigen::Matrix4d Al = dir == 1 ? E.dfluxx(a, wl) : E.dfluxy(a, wl);
    Eigen::Matrix4d Ar = dir == 1 ? E.dfluxx(b, wr) : E.dfluxy(b, wr);
    Eigen::Vector4d aM = E.maxLocalWaveSpeed(wl, wr, dir) / 1.0;
    put<4>(E.dRusanov(vec<4>(dql + 4 * k), vec<4>(dqr + 4 * k), wl, wr, mat4(Lm + 16 * k),
                      mat4(Rm + 16 * k), Al, Ar, aM),
           out + 4 * k);
  }
}
void ref_riemann2d_ic(double gamma, const double* x, const double* y, double* q, long n) {
  Equations::Euler2D E(gamma);
  for (long k = 0; k < n; ++k) put<4>(E.conservativeOfRiemann2D(x[k], y[k]), q + 4 * k);
}
void ref_taylor_ic(double gamma, const double* x, const double* y, double* q, long n) {
  Equations::Euler2D E(gamma);
  for (long k = 0; k < n; ++k) put<4>(E.conservativeOfTaylorIns2D(x[k], y[k]), q + 4 * k);
}
void ref_double_mach_ic(double gamma, const double* x, const double* y, double* q, long n) {
  Equations::Euler2D E(gamma);
  for (long k = 0; k < n; ++k) put<4>(E.conservativeOfDoubleMach2D(x[k], y[k]), q + 4 * k);
}
void ref_sod_ic(double gamma, const double* x, double* q, long n) {
  Equations::Euler1D E(gamma);
  for (long k = 0; k < n; ++k) put<3>(E.conservative(E.sodShock(x[k])), q + 3 * k);
}

// ---- FV::System2D (FV_System2D.cpp) -------------------------------------------------------------
// q_in/q_out: interior state, SoA [4][ny][nx].  Runs at most nsteps steps of the loop in
// timeStepping() (FV_System2D.cpp:614-651), stopping early at tFinal.  Returns steps taken.
int ref_fv2d_run(int nx, int ny, double xl, double xr, double yb, double yt, double cfl,
                 double gamma, double tFinal, int nsteps, const double* q_in, double* q_out,
                 double* t_out) {
  Quiet quiet;
  FV::System2D S(xl, xr, nx, yb, yt, ny, cfl, tFinal, 0.0, gamma);
  const int k = S.k;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int v = 0; v < 4; ++v) S.cell(i + k, j + k).u(v) = q_in[(size_t(v) * ny + j) * nx + i];
  S.zeroGradBc();
  S.periodicBc();
  S.calcPrimitiveVariable();
  int steps = 0;
  while (S.t < S.tFinal && steps < nsteps) {
    double mx = 0.0, my = 0.0;
    for (int i = k; i < S.nxx - k; i++)
      for (int j = k; j < S.nyy - k; j++) {
        mx = std::fmax(mx, S.eulObj.maxSpeed(S.cell(i, j).pvar, 1));
        my = std::fmax(my, S.eulObj.maxSpeed(S.cell(i, j).pvar, 2));
      }
    S.dt = S.cfl * std::pow(std::fmin(S.dx, S.dy), 3.0 / 3.0) / std::fmax(mx, my);
    S.dt = S.t + S.dt > S.tFinal ? S.tFinal - S.t : S.dt;
    S.RungeKutta3();
    S.t += S.dt;
    ++steps;
  }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int v = 0; v < 4; ++v) q_out[(size_t(v) * ny + j) * nx + i] = S.cell(i + k, j + k).u(v);
  *t_out = S.t;
  return steps;
}

// ---- FV::System1D (FV_System1D.cpp) -------------------------------------------------------------
int ref_fv1d_run(int nx, double xl, double xr, double cfl, double gamma, double tFinal, int nsteps,
                 const double* q_in, double* q_out, double* t_out) {
  Quiet quiet;
  FV::System1D S(xl, xr, nx, cfl, tFinal, 0.0, gamma);
  const int k = S.k;
  for (int i = 0; i < nx; ++i)
    for (int v = 0; v < 3; ++v) S.cell(i + k).u(v) = q_in[size_t(v) * nx + i];
  S.zeroGradBc();
  S.calcPrimitiveVariable();
  int steps = 0;
  while (S.t < S.tFinal && steps < nsteps) {
    double mx = 0.0;
    for (int i = k; i < S.nxx - k; i++) mx = std::fmax(mx, S.eulObj.maxSpeed(S.cell(i).pvar));
    S.dt = S.cfl * std::pow(S.dx, 3.0 / 3.0) / mx;
    S.dt = S.t + S.dt > S.tFinal ? S.tFinal - S.t : S.dt;
    S.RungeKutta3();
    S.t += S.dt;
    ++steps;
  }
  for (int i = 0; i < nx; ++i)
    for (int v = 0; v < 3; ++v) q_out[size_t(v) * nx + i] = S.cell(i + k).u(v);
  *t_out = S.t;
  return steps;
}

// ---- FVHermite::System2D (FVHermite_System2D.cpp) -----------------------------------------------
// q, v (= d/dx moments), w (= d/dy moments): interior SoA [4][ny][nx] each.
int ref_hermite2d_run(int nx, int ny, double xl, double xr, double yb, double yt, double cfl,
                      double gamma, double tFinal, int nsteps, const double* q_in,
                      const double* v_in, const double* w_in, double* q_out, double* v_out,
                      double* w_out, double* t_out) {
  Quiet quiet;
  omp_set_num_threads(1);  // limitDerivatives() sweeps in place; one thread makes it a
                           // deterministic Gauss-Seidel sweep (FVHermite_System2D.cpp:393-427)
  FVHermite::System2D S(xl, xr, nx, yb, yt, ny, cfl, tFinal, 0.0, gamma);
  const int k = S.k;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int c = 0; c < 4; ++c) {
        const size_t o = (size_t(c) * ny + j) * nx + i;
        S.cell(i + k, j + k).u(c) = q_in[o];
        S.cell(i + k, j + k).v(c) = v_in[o];
        S.cell(i + k, j + k).w(c) = w_in[o];
      }
  S.zeroGradBc();
  S.calcPrimitiveVariable();
  int steps = 0;
  while (S.t < S.tFinal && steps < nsteps) {
    double mx = 0.0, my = 0.0;
    for (int i = k; i < S.nxx - k; i++)
      for (int j = k; j < S.nyy - k; j++) {
        mx = std::fmax(mx, S.eulObj.maxSpeed(S.cell(i, j).pvar, 1));
        my = std::fmax(my, S.eulObj.maxSpeed(S.cell(i, j).pvar, 2));
      }
    S.dt = S.cfl * std::pow(std::fmin(S.dx, S.dy), 3.0 / 3.0) / std::fmax(mx, my) / 1.0;
    S.dt = S.t + S.dt > S.tFinal ? S.tFinal - S.t : S.dt;
    S.RungeKutta3();
    S.t += S.dt;
    ++steps;
  }
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int c = 0; c < 4; ++c) {
        const size_t o = (size_t(c) * ny + j) * nx + i;
        q_out[o] = S.cell(i + k, j + k).u(c);
        v_out[o] = S.cell(i + k, j + k).v(c);
        w_out[o] = S.cell(i + k, j + k).w(c);
      }
  *t_out = S.t;
  return steps;
}

// ---- FVHermite::System1D (FVHermite_System1D.cpp) -----------------------------------------------
// Periodic boundaries, LMPE-routed htenoi/linear reconstruction (as shipped).  The troubled-cell
// flags start false (fresh storage) and are never reset, as in the reference.
int ref_hermite1d_run(int nx, double xl, double xr, double cfl, double gamma, double tFinal,
                      int nsteps, const double* q_in, const double* v_in, double* q_out,
                      double* v_out, double* t_out) {
  Quiet quiet;
  FVHermite::System1D S(xl, xr, nx, cfl, tFinal, 0.0, gamma);
  const int k = S.k;
  for (int i = 0; i < S.nxx; ++i) S.cell(i).discontinue.setZero();
  for (int i = 0; i < nx; ++i)
    for (int c = 0; c < 3; ++c) {
      S.cell(i + k).u(c) = q_in[size_t(c) * nx + i];
      S.cell(i + k).v(c) = v_in[size_t(c) * nx + i];
    }
  S.periodicBc();
  S.calcPrimitiveVariable();
  int steps = 0;
  while (S.t < S.tFinal && steps < nsteps) {
    double mx = 0.0;
    for (int i = k; i < S.nxx - k; i++) mx = std::fmax(mx, S.eulObj.maxSpeed(S.cell(i).pvar));
    S.dt = S.cfl * std::pow(S.dx, 5.0 / 3.0) / mx;
    S.dt = S.t + S.dt > S.tFinal ? S.tFinal - S.t : S.dt;
    S.RungeKutta3();
    S.t += S.dt;
    ++steps;
  }
  for (int i = 0; i < nx; ++i)
    for (int c = 0; c < 3; ++c) {
      q_out[size_t(c) * nx + i] = S.cell(i + k).u(c);
      v_out[size_t(c) * nx + i] = S.cell(i + k).v(c);
    }
  *t_out = S.t;
  return steps;
}

// The reference's own smooth-solution initial data (cell averages by 9x9 Gauss quadrature),
// for the convergence and exactness tests: FV::System2D::entropyWave (FV_System2D.cpp:49-74).
void ref_fv2d_entropy_wave_ic(int nx, int ny, double xl, double xr, double yb, double yt,
                              double gamma, double* q_out) {
  Quiet quiet;
  FV::System2D S(xl, xr, nx, yb, yt, ny, 0.4, 1.0, 0.0, gamma);
  S.entropyWave();
  const int k = S.k;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int v = 0; v < 4; ++v) q_out[(size_t(v) * ny + j) * nx + i] = S.cell(i + k, j + k).u(v);
}

// Face eigenvectors of cell pairs computed by the reference's own eigen2DEuler()
// (FV_System2D.cpp:265-361): pair k sits in cells (2k, 2k+1) of a one-row (dir 1) or
// one-column (dir 2) grid.  R, L row-major [n][16].
void ref_roe2d(double gamma, int dir, const double* qa, const double* qb, double* Rout,
               double* Lout, long n) {
  Quiet quiet;
  const int m = int(2 * n);
  FV::System2D S(0.0, 1.0, dir == 1 ? m : 1, 0.0, 1.0, dir == 1 ? 1 : m, 0.4, 1.0, 0.0, gamma);
  const int k = S.k;
  for (long p = 0; p < n; ++p)
    for (int v = 0; v < 4; ++v) {
      if (dir == 1) {
        S.cell(k + 2 * p, k).u(v) = qa[4 * p + v];
        S.cell(k + 2 * p + 1, k).u(v) = qb[4 * p + v];
      } else {
        S.cell(k, k + 2 * p).u(v) = qa[4 * p + v];
        S.cell(k, k + 2 * p + 1).u(v) = qb[4 * p + v];
      }
    }
  S.calcPrimitiveVariable();
  S.eigen2DEuler();
  for (long p = 0; p < n; ++p) {
    const auto& c = dir == 1 ? S.cell(k + 2 * p, k) : S.cell(k, k + 2 * p);
    const Eigen::Matrix4d& R = dir == 1 ? c.rightEigenVectorX : c.rightEigenVectorY;
    const Eigen::Matrix4d& L = dir == 1 ? c.leftEigenVectorX : c.leftEigenVectorY;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        Rout[16 * p + 4 * i + j] = R(i, j);
        Lout[16 * p + 4 * i + j] = L(i, j);
      }
  }
}

}  // extern "C"
