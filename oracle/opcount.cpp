// Algorithmic operation counts of the reference's hot path, obtained by running the oracle's
// scheme functions on a counting scalar type.  Counted: +, -, *, / and sqrt (one flop each),
// pow (one call each, reported separately), comparisons and fabs/fmax/fmin are not flops.
// Output: JSON with per-call counts (averaged over seeded inputs for data-dependent branches)
// and the per-face / per-cell totals of one SSP-RK3 stage of FV::System2D, as used for the
// compute roofline.   Build and run:  make -C oracle opcount && oracle/build/opcount
#include <cmath>
#include <cstdio>
#include <random>

namespace orc {
struct Cnt {
  static thread_local long add, mul, div, sqrt_, pow_;
  double v = 0.0;
  Cnt() = default;
  Cnt(double x) : v(x) {}
};
thread_local long Cnt::add = 0, Cnt::mul = 0, Cnt::div = 0, Cnt::sqrt_ = 0, Cnt::pow_ = 0;
inline Cnt operator+(Cnt a, Cnt b) { ++Cnt::add; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { ++Cnt::add; return Cnt(a.v - b.v); }
inline Cnt operator*(Cnt a, Cnt b) { ++Cnt::mul; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { ++Cnt::div; return Cnt(a.v / b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline bool operator<(Cnt a, Cnt b) { return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { return a.v > b.v; }
inline bool operator<=(Cnt a, Cnt b) { return a.v <= b.v; }
inline bool operator>=(Cnt a, Cnt b) { return a.v >= b.v; }
inline Cnt fabs(Cnt a) { return Cnt(std::fabs(a.v)); }
inline Cnt fmax(Cnt a, Cnt b) { return Cnt(std::fmax(a.v, b.v)); }
inline Cnt fmin(Cnt a, Cnt b) { return Cnt(std::fmin(a.v, b.v)); }
inline Cnt sqrt(Cnt a) { ++Cnt::sqrt_; return Cnt(std::sqrt(a.v)); }
inline Cnt pow(Cnt a, Cnt b) { ++Cnt::pow_; return Cnt(std::pow(a.v, b.v)); }
inline bool isnan(Cnt a) { return std::isnan(a.v); }
}  // namespace orc

#include "oracle.hpp"

using orc::Cnt;

namespace {
struct Count {
  double add = 0, mul = 0, div = 0, sqrt_ = 0, pow_ = 0;
  double flops() const { return add + mul + div + sqrt_; }
};
void reset() { Cnt::add = Cnt::mul = Cnt::div = Cnt::sqrt_ = Cnt::pow_ = 0; }
Count snap(int n) {
  Count c;
  c.add = double(Cnt::add) / n;
  c.mul = double(Cnt::mul) / n;
  c.div = double(Cnt::div) / n;
  c.sqrt_ = double(Cnt::sqrt_) / n;
  c.pow_ = double(Cnt::pow_) / n;
  return c;
}
void print(const char* name, const Count& c, bool last = false) {
  std::printf("  \"%s\": {\"add\": %.2f, \"mul\": %.2f, \"div\": %.2f, \"sqrt\": %.2f, \"pow\": %.2f, \"flops\": %.2f}%s\n",
              name, c.add, c.mul, c.div, c.sqrt_, c.pow_, c.flops(), last ? "" : ",");
}
}  // namespace

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0), Rho(0.1, 1.5), P(0.03, 1.5);
  const int N = 20000;
  // teno5 (both sides) on a 6-cell stencil
  reset();
  for (int k = 0; k < N; ++k) {
    Cnt u[6], o[2];
    for (auto& x : u) x = Cnt(U(rng));
    orc::lagrange_recon(0, u, o);
  }
  Count teno = snap(N);
  reset();
  for (int k = 0; k < N; ++k) {
    Cnt u[5], o[3];
    for (auto& x : u) x = Cnt(U(rng));
    orc::gl3(u, o);
  }
  Count gl3 = snap(N);
  auto state = [&](Cnt* q) {
    double r = Rho(rng), u = U(rng), v = U(rng), p = P(rng);
    q[0] = r; q[1] = r * u; q[2] = r * v; q[3] = p / 0.4 + 0.5 * r * (u * u + v * v);
  };
  orc::Euler2<Cnt> E(1.4);
  reset();
  for (int k = 0; k < N; ++k) {
    Cnt ql[4], qr[4], F[4];
    state(ql);
    state(qr);
    E.hllc(1 + (k & 1), ql, qr, F);
  }
  Count hllc = snap(N);
  reset();
  Cnt Rm[16], Lm[16];
  for (int k = 0; k < N; ++k) {
    Cnt qa[4], qb[4], wa[4], wb[4];
    state(qa);
    state(qb);
    E.primitive(qa, wa);
    E.primitive(qb, wb);
    E.roe(1, wa, Cnt(1.0), Cnt(1.0), wb, Cnt(1.0), Cnt(1.0), Rm, Lm);
  }
  Count roe = snap(N);  // includes the two primitive recoveries
  reset();
  for (int k = 0; k < N; ++k) {
    Cnt ql[4], qr[4], F[4];
    state(ql);
    state(qr);
    E.rusanov(1, ql, qr, Lm, Rm, F);
  }
  Count rus = snap(N);
  // matrix-vector product 4x4 (projection or back-projection): 16 mul + 12 add
  Count mv;
  mv.mul = 16;
  mv.add = 12;
  // cell primitives: primitive (2 div, 4 mul, 3 add) + sqrt(|rho|) + H = (E + p)/rho
  reset();
  for (int k = 0; k < N; ++k) {
    Cnt q[4], w[4];
    state(q);
    E.primitive(q, w);
    Cnt s = sqrt(fabs(w[0]));
    Cnt h = (q[3] + w[3]) / w[0];
    (void)s;
    (void)h;
  }
  Count prim = snap(N);
  // E.primitive alone (the Roe measurement above includes two of them)
  reset();
  for (int k = 0; k < N; ++k) {
    Cnt q[4], w[4];
    state(q);
    E.primitive(q, w);
  }
  Count pr = snap(N);
  auto lin = [](const Count& a, double ka, const Count& b, double kb) {
    Count c;
    c.add = ka * a.add + kb * b.add;
    c.mul = ka * a.mul + kb * b.mul;
    c.div = ka * a.div + kb * b.div;
    c.sqrt_ = ka * a.sqrt_ + kb * b.sqrt_;
    c.pow_ = ka * a.pow_ + kb * b.pow_;
    return c;
  };
  const Count roe_only = lin(roe, 1.0, pr, -2.0);
  // GPU kernel split of one stage of FV::System2D, per face of one direction:
  //   faces kernel: Roe average + eigenvectors, 6 projections L*q, TENO5 on 4 fields
  //   flux kernel : 8 GL3 (4 fields x 2 sides), 6 back-projections R*c, 3 fluxes, quadrature
  //   update      : per cell, primitives, rhs (4 x [2 sub, 2 mul, 1 add, 1 div]), RK stage
  Count faces = lin(lin(roe_only, 1, mv, 6), 1, teno, 4);
  Count quad;
  quad.mul = 12;
  quad.add = 8;
  auto fluxk = [&](const Count& f) { return lin(lin(lin(gl3, 8, mv, 6), 1, f, 3), 1, quad, 1); };
  Count fh = fluxk(hllc), fr = fluxk(rus);
  Count upd;
  upd.add = prim.add + 12 + 8;
  upd.mul = prim.mul + 8 + 8;
  upd.div = prim.div + 4 + 1;
  upd.sqrt_ = prim.sqrt_;
  std::printf("{\n");
  print("teno5_pair", teno);
  print("gl3", gl3);
  print("hllc2d", hllc);
  print("rusanov2d", rus);
  print("roe_pair_with_prims", roe);
  print("cell_prim", prim);
  print("faces_kernel_per_face", faces);
  print("flux_kernel_per_face_hllc", fh);
  print("flux_kernel_per_face_rusanov", fr);
  print("update_kernel_per_cell", upd, true);
  std::printf("}\n");
  return 0;
}
