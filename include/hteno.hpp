// hteno.hpp -- C++ host classes over the C-ABI (hteno.h) shaped like the reference solver's public
// interface (indrow/Hermite-TENO), so that a host written against the reference switches by
// changing the include and the namespace:
//
//   FV::System2D(xl, xr, nx, yb, yt, ny, cfl, tmax, tInit, gamma)      FV_System2D.h:12-20
//   FV::System1D(xl, xr, nx, cfl, tmax, tInit, gamma)                   FV_System1D.h:12-17
//   FVHermite::System2D(xl, xr, nx, yb, yt, ny, cfl, tmax, tInit, gamma) FVHermite_System2D.h:16-24
//   FVHermite::System1D(xl, xr, nx, cfl, tmax, tInit, gamma)            FVHermite_System1D.h:12-18
//
// with the initial conditions the reference's main.cpp uses (Riemann2D, sodShock; any other state
// through setState/setMoments), timeStepping() (advance to tmax) and write() in the reference's
// result-file layout
// (FV_System2D.cpp:668-715).  Scheme choices the reference makes by commenting code in or out
// (flux, reconstruction, boundary) are an Options argument whose defaults are the reference as
// shipped.  Header-only; link with libhteno.so.  Errors throw hteno::Error (the C-ABI below never
// throws).
#pragma once

#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <stdexcept>
#include <string>
#include <vector>

#include "hteno.h"

namespace hteno {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, hteno_solver* s = nullptr) {
  if (rc != HTENO_OK)
    throw Error(rc, std::string(hteno_status_string(rc)) + (s ? std::string(": ") + hteno_last_error(s) : ""));
}

struct Options {
  int recon = -1;  // -1: the reference's choice for the solver (teno5 in 2D, teno5i in FV 1D)
  int flux = HTENO_FLUX_RUSANOV;
  int bc = -1;     // -1: the reference's choice (zero-gradient; periodic for FVHermite 1D)
  int precision = HTENO_PREC_FP64;
};

// Common owner of a solver handle.
class SolverBase {
 public:
  SolverBase(const SolverBase&) = delete;
  SolverBase& operator=(const SolverBase&) = delete;
  ~SolverBase() {
    if (h_) hteno_destroy(h_);
  }
  // Conserved state, SoA [nvar][ny][nx] (host memory).
  void setState(const std::vector<double>& q) {
    check(hteno_set_state(h_, q.data(), HTENO_HOST), h_);
    t_ = cfg_.t_init;
  }
  std::vector<double> state() const {
    std::vector<double> q(size());
    check(hteno_get_state(h_, q.data(), HTENO_HOST), h_);
    return q;
  }
  // Advance to tmax (the reference's timeStepping loop).
  void timeStepping() { advance(1 << 30, tmax_); }
  // Advance at most n steps (never beyond tmax).
  void advance(int n, double tmax) {
    check(hteno_step(h_, n, tmax), h_);
    long steps = 0;
    check(hteno_get_time(h_, &t_, &steps, nullptr), h_);
  }
  double time() const { return t_; }
  hteno_solver* handle() { return h_; }
  size_t size() const { return size_t(nvar_) * cfg_.nx * cfg_.ny; }

 protected:
  SolverBase(const hteno_config& c, double tmax) : cfg_(c), tmax_(tmax), t_(c.t_init) {
    nvar_ = c.dims == 2 ? 4 : 3;
    if (c.dims == 1) cfg_.ny = 1;
    check(hteno_create(&cfg_, &h_));
  }
  double x(int i) const { return cfg_.xl + (i + 0.5) * (cfg_.xr - cfg_.xl) / cfg_.nx; }
  double y(int j) const { return cfg_.yb + (j + 0.5) * (cfg_.yt - cfg_.yb) / cfg_.ny; }
  hteno_config cfg_;
  hteno_solver* h_ = nullptr;
  double tmax_, t_;
  int nvar_;
};

inline hteno_config make_cfg(int dims, int scheme, double xl, double xr, int nx, double yb, double yt,
                             int ny, double cfl, double tInit, double gamma, const Options& o,
                             int recon_default, int bc_default) {
  hteno_config c;
  hteno_config_default(&c);
  c.dims = dims;
  c.scheme = scheme;
  c.xl = xl; c.xr = xr; c.nx = nx;
  c.yb = yb; c.yt = yt; c.ny = ny;
  c.cfl = cfl;
  c.t_init = tInit;
  c.gamma = gamma;
  c.recon = o.recon < 0 ? recon_default : o.recon;
  c.flux = o.flux;
  c.bc = o.bc < 0 ? bc_default : o.bc;
  c.precision = o.precision;
  return c;
}

// Euler2D::conservative (Equations_Euler2D.cpp:28-34)
inline void conservative2(double g, const double* w, double* q) {
  q[0] = w[0];
  q[1] = w[0] * w[1];
  q[2] = w[0] * w[2];
  q[3] = w[3] / (g - 1.0) + 0.5 * (q[1] * w[1] + q[2] * w[2]);
}

namespace FV {

class System2D : public SolverBase {
 public:
  System2D(double xl, double xr, int nx, double yb, double yt, int ny, double cflnumber,
           double tmax, double tInit, double specificHeatRatio, const Options& o = Options())
      : SolverBase(make_cfg(2, HTENO_SCHEME_FV, xl, xr, nx, yb, yt, ny, cflnumber, tInit,
                            specificHeatRatio, o, HTENO_RECON_TENO5, HTENO_BC_ZEROGRAD),
                   tmax) {}

  // FV::System2D::Riemann2D (FV_System2D.cpp:101-112) initialises with
  // conservativeOfTaylorIns2D (Equations_Euler2D.cpp:619-634), not the Riemann configuration.
  void Riemann2D() {
    const double g = cfg_.gamma, pi = 4.0 * std::atan(1.0);
    std::vector<double> q(size());
    const size_t n = size_t(cfg_.nx) * cfg_.ny;
    for (int j = 0; j < cfg_.ny; ++j)
      for (int i = 0; i < cfg_.nx; ++i) {
        const double xx = x(i), yy = y(j);
        double w[4], qq[4];
        w[0] = yy < 0.5 ? 2.0 : 1.0;
        w[1] = 0.0;
        w[3] = yy < 0.5 ? 1.0 + 2.0 * yy : yy + 1.5;
        w[2] = -0.025 * std::sqrt(g * w[3] / w[0]) * std::cos(8.0 * pi * xx);
        conservative2(g, w, qq);
        for (int v = 0; v < 4; ++v) q[v * n + size_t(j) * cfg_.nx + i] = qq[v];
      }
    setState(q);
  }

  // Result file in the reference's layout (write(), FV_System2D.cpp:668-715): a "t:" line, a
  // header of x y Density Ux Uy Pressure in width-20 columns, then one row per interior cell
  // (j outer, i inner) holding x, y and the four conserved variables, precision 8.
  void write(const std::string& filename) const {
    std::ofstream out(filename);
    if (!out.good()) throw Error(HTENO_ERR_INVALID_ARG, "cannot open " + filename);
    const std::vector<double> q = state();
    const size_t n = size_t(cfg_.nx) * cfg_.ny;
    out << "t: " << t_ << "\n";
    for (const char* h : {"x", "y", "Density", "Ux", "Uy", "Pressure"})
      out << std::right << std::setw(20) << std::setfill(' ') << h;
    out << "\n";
    for (int j = 0; j < cfg_.ny; ++j) {
      for (int i = 0; i < cfg_.nx; ++i) {
        out << std::right << std::setw(20) << std::setprecision(8) << x(i);
        out << std::right << std::setw(20) << std::setprecision(8) << y(j);
        for (int v = 0; v < 4; ++v)
          out << std::right << std::setw(20) << std::setprecision(8) << q[v * n + size_t(j) * cfg_.nx + i];
        out << "\n";
      }
    }
  }
};

class System1D : public SolverBase {
 public:
  System1D(double xl, double xr, int nx, double cflnumber, double tmax, double tInit,
           double specificHeatRatio, const Options& o = Options())
      : SolverBase(make_cfg(1, HTENO_SCHEME_FV, xl, xr, nx, 0.0, 1.0, 1, cflnumber, tInit,
                            specificHeatRatio, o, HTENO_RECON_TENO5I, HTENO_BC_ZEROGRAD),
                   tmax) {}
  // Sod's shock tube (sodShock, Equations_Euler1D.cpp:317-332)
  void sodShock() {
    const double g = cfg_.gamma;
    std::vector<double> q(size());
    const int n = cfg_.nx;
    for (int i = 0; i < n; ++i) {
      const bool left = x(i) < 0.5;
      const double rho = left ? 1.0 : 0.125, p = left ? 1.0 : 0.1;
      q[i] = rho;
      q[n + i] = 0.0;
      q[2 * n + i] = p / (g - 1.0);
    }
    setState(q);
  }
};

}  // namespace FV

namespace FVHermite {

class System2D : public SolverBase {
 public:
  System2D(double xl, double xr, int nx, double yb, double yt, int ny, double cflnumber,
           double tmax, double tInit, double specificHeatRatio, const Options& o = Options())
      : SolverBase(make_cfg(2, HTENO_SCHEME_HERMITE, xl, xr, nx, yb, yt, ny, cflnumber, tInit,
                            specificHeatRatio, o, HTENO_RECON_TENO5, HTENO_BC_ZEROGRAD),
                   tmax) {}
  void setMoments(const std::vector<double>& v, const std::vector<double>& w) {
    check(hteno_set_moments(h_, v.data(), w.data(), HTENO_HOST), h_);
  }
  // FVHermite::System2D::Riemann2D (FVHermite_System2D.cpp:89-107): conservativeOfRiemann2D
  // (Equations_Euler2D.cpp:530-617) and moments by face differences of it.
  void Riemann2D() {
    const double g = cfg_.gamma;
    const double dx = (cfg_.xr - cfg_.xl) / cfg_.nx, dy = (cfg_.yt - cfg_.yb) / cfg_.ny;
    auto riemann = [&](double xx, double yy, double* q) {
      double w[4];
      if (xx > 0.5 && yy > 0.5) { w[0] = 1.0; w[1] = 0.75; w[2] = -0.5; w[3] = 1.0; }
      else if (xx < 0.5 && yy > 0.5) { w[0] = 2.0; w[1] = 0.75; w[2] = 0.5; w[3] = 1.0; }
      else if (xx < 0.5 && yy < 0.5) { w[0] = 1.0; w[1] = -0.75; w[2] = 0.5; w[3] = 1.0; }
      else { w[0] = 3.0; w[1] = -0.75; w[2] = -0.5; w[3] = 1.0; }
      conservative2(g, w, q);
    };
    std::vector<double> q(size()), v(size()), w(size());
    const size_t n = size_t(cfg_.nx) * cfg_.ny;
    for (int j = 0; j < cfg_.ny; ++j)
      for (int i = 0; i < cfg_.nx; ++i) {
        double c[4], a[4], b[4];
        const size_t o = size_t(j) * cfg_.nx + i;
        riemann(x(i), y(j), c);
        for (int k = 0; k < 4; ++k) q[k * n + o] = c[k];
        riemann(x(i) + dx / 2.0, y(j), a);
        riemann(x(i) - dx / 2.0, y(j), b);
        for (int k = 0; k < 4; ++k) v[k * n + o] = (a[k] - b[k]) / dx;
        riemann(x(i), y(j) + dy / 2.0, a);
        riemann(x(i), y(j) - dy / 2.0, b);
        for (int k = 0; k < 4; ++k) w[k * n + o] = (a[k] - b[k]) / dy;
      }
    setState(q);
    setMoments(v, w);
  }
};

class System1D : public SolverBase {
 public:
  System1D(double xl, double xr, int nx, double cflnumber, double tmax, double tInit,
           double specificHeatRatio, const Options& o = Options())
      : SolverBase(make_cfg(1, HTENO_SCHEME_HERMITE, xl, xr, nx, 0.0, 1.0, 1, cflnumber, tInit,
                            specificHeatRatio, o, HTENO_RECON_TENO5, HTENO_BC_PERIODIC),
                   tmax) {}
  void setMoments(const std::vector<double>& v) {
    check(hteno_set_moments(h_, v.data(), nullptr, HTENO_HOST), h_);
  }
};

}  // namespace FVHermite
}  // namespace hteno
