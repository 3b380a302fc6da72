// extern "C" surface of the CPU oracle (test infrastructure; see oracle.hpp).  Array layouts
// match the CUDA library's C-ABI (include/hteno.h) so that tests compare like with like.
#include "oracle.hpp"

#include <cstring>

using namespace orc;

extern "C" {

void orc_lagrange_recon(int kind, const double* u, double* out, long n) {
#pragma omp parallel for if (n > 4096)
  for (long k = 0; k < n; ++k) lagrange_recon(kind, u + 6 * k, out + 2 * k);
}
void orc_gl3(const double* u, double* out, long n) {
#pragma omp parallel for if (n > 4096)
  for (long k = 0; k < n; ++k) gl3(u + 5 * k, out + 3 * k);
}
void orc_hermite_recon(int kind, double dx, const double* u, const double* d, double* out, long n) {
  HermiteCoef K(dx);
  for (long k = 0; k < n; ++k) hermite_recon(K, kind, u + 4 * k, d + 4 * k, out + 4 * k);
}
void orc_hermite_limiter(double dx, const double* u, const double* d, double* out, long n) {
  HermiteCoef K(dx);
  for (long k = 0; k < n; ++k) out[k] = hermite_limiter(K, u + 3 * k, d + 3 * k);
}
void orc_ssprk3(const double* q0, const double* qn, const double* rhs, double dt, int stage,
                double* out, long n) {
  for (long k = 0; k < n; ++k) out[k] = ssprk3(q0[k], qn[k], rhs[k], dt, stage);
}
void orc_hllc2d(double gamma, int dir, const double* ql, const double* qr, double* out, long n) {
  Euler2<double> E(gamma);
  for (long k = 0; k < n; ++k) E.hllc(dir, ql + 4 * k, qr + 4 * k, out + 4 * k);
}
void orc_hllc1d(double gamma, const double* ql, const double* qr, double* out, long n) {
  Euler1<double> E(gamma);
  for (long k = 0; k < n; ++k) E.hllc(ql + 3 * k, qr + 3 * k, out + 3 * k);
}
void orc_rusanov2d(double gamma, int dir, const double* ql, const double* qr, const double* L,
                   const double* R, double* out, long n) {
  Euler2<double> E(gamma);
  for (long k = 0; k < n; ++k) E.rusanov(dir, ql + 4 * k, qr + 4 * k, L + 16 * k, R + 16 * k, out + 4 * k);
}
void orc_drusanov2d(double gamma, int dir, const double* ql, const double* qr, const double* dql,
                    const double* dqr, const double* L, const double* R, double* out, long n) {
  Euler2<double> E(gamma);
  for (long k = 0; k < n; ++k)
    E.drusanov(dir, ql + 4 * k, qr + 4 * k, dql + 4 * k, dqr + 4 * k, L + 16 * k, R + 16 * k, out + 4 * k);
}
// Roe-averaged face eigenvectors from two cell states (eigen2DEuler), row-major.
void orc_roe2d(double gamma, int dir, const double* qa, const double* qb, double* R, double* L, long n) {
  Euler2<double> E(gamma);
  for (long k = 0; k < n; ++k) {
    double wa[4], wb[4];
    E.primitive(qa + 4 * k, wa);
    E.primitive(qb + 4 * k, wb);
    E.roe(dir, wa, std::sqrt(std::fabs(wa[0])), (qa[4 * k + 3] + wa[3]) / wa[0], wb,
          std::sqrt(std::fabs(wb[0])), (qb[4 * k + 3] + wb[3]) / wb[0], R + 16 * k, L + 16 * k);
  }
}

// FV 2D: q [4][ny][nx] in/out.  Returns steps taken.
int orc_fv2d_run(int nx, int ny, double xl, double xr, double yb, double yt, double cfl,
                 double gamma, int bc, int flux, int recon, double tFinal, int nsteps,
                 const double* q_in, double* q_out, double* t_out) {
  FV2D S(nx, ny, xl, xr, yb, yt, cfl, gamma, bc, flux, recon);
  std::memcpy(S.q.data(), q_in, sizeof(double) * S.q.size());
  int s = S.run(nsteps, tFinal);
  std::memcpy(q_out, S.q.data(), sizeof(double) * S.q.size());
  *t_out = S.t;
  return s;
}
// One residual evaluation (rhs) of the 2D scheme at state q: out [4][ny][nx].
void orc_fv2d_rhs(int nx, int ny, double xl, double xr, double yb, double yt, double gamma,
                  int bc, int flux, int recon, const double* q_in, double* rhs_out) {
  FV2D S(nx, ny, xl, xr, yb, yt, 0.4, gamma, bc, flux, recon);
  std::memcpy(S.q.data(), q_in, sizeof(double) * S.q.size());
  S.residual();
  std::memcpy(rhs_out, S.rhsu.data(), sizeof(double) * S.q.size());
}
int orc_fv1d_run(int nx, double xl, double xr, double cfl, double gamma, int bc, int flux,
                 int recon, double tFinal, int nsteps, const double* q_in, double* q_out,
                 double* t_out) {
  FV1D S(nx, xl, xr, cfl, gamma, bc, flux, recon);
  std::memcpy(S.q.data(), q_in, sizeof(double) * S.q.size());
  int s = S.run(nsteps, tFinal);
  std::memcpy(q_out, S.q.data(), sizeof(double) * S.q.size());
  *t_out = S.t;
  return s;
}

int orc_hermite2d_run(int nx, int ny, double xl, double xr, double yb, double yt, double cfl,
                      double gamma, int bc, double tFinal, int nsteps, const double* q_in,
                      const double* v_in, const double* w_in, double* q_out, double* v_out,
                      double* w_out, double* t_out) {
  (void)bc;  // the reference's Hermite 2D rhs uses zero-gradient boundaries
  Hermite2D S(nx, ny, xl, xr, yb, yt, cfl, gamma);
  const size_t n = S.q.size();
  std::memcpy(S.q.data(), q_in, sizeof(double) * n);
  std::memcpy(S.v.data(), v_in, sizeof(double) * n);
  std::memcpy(S.w.data(), w_in, sizeof(double) * n);
  int s = S.run(nsteps, tFinal);
  std::memcpy(q_out, S.q.data(), sizeof(double) * n);
  std::memcpy(v_out, S.v.data(), sizeof(double) * n);
  std::memcpy(w_out, S.w.data(), sizeof(double) * n);
  *t_out = S.t;
  return s;
}
int orc_hermite1d_run(int nx, double xl, double xr, double cfl, double gamma, double tFinal,
                      int nsteps, const double* q_in, const double* v_in, double* q_out,
                      double* v_out, double* t_out) {
  Hermite1D S(nx, xl, xr, cfl, gamma);
  for (int e = 0; e < 3; ++e)
    for (int i = 0; i < nx; ++i) {
      S.U(e, i + Hermite1D::k) = q_in[size_t(e) * nx + i];
      S.V(e, i + Hermite1D::k) = v_in[size_t(e) * nx + i];
    }
  int s = S.run(nsteps, tFinal);
  for (int e = 0; e < 3; ++e)
    for (int i = 0; i < nx; ++i) {
      q_out[size_t(e) * nx + i] = S.U(e, i + Hermite1D::k);
      v_out[size_t(e) * nx + i] = S.V(e, i + Hermite1D::k);
    }
  *t_out = S.t;
  return s;
}

}  // extern "C"
