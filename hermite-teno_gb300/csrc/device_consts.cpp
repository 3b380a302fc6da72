// Host-side construction of the device constant block.  Every coefficient is computed with the
// expression the reference uses in its constructors (Schemes_Lagrange.cpp:6-304,
// Schemes_Hermite.cpp:5-92), in double, with floating-point contraction disabled for this file,
// so the device sees the same bits the reference computes.
#include "dev_const.h"

#include <cmath>
#include <limits>

namespace hteno {

namespace {
// Normalised weights of each TENO cut-off pattern: w_k = s_k d_k / sum_j(s_j d_j), summed left
// to right and divided, as the reference does after cutOff() (Schemes_Lagrange.cpp:490-492).
// Pattern 0 cannot occur (the largest weight is always >= 1/3); it yields 0/0 = NaN there too.
void pattern_table(const double* d, double tab[8][3]) {
  for (int pat = 0; pat < 8; ++pat) {
    double w[3];
    for (int k = 0; k < 3; ++k) w[k] = ((pat >> k) & 1 ? 1.0 : 0.0) * d[k];
    double s = (w[0] + w[1]) + w[2];
    for (int k = 0; k < 3; ++k) tab[pat][k] = w[k] / s;
  }
}
template <int N, int M>
void to_float(const double (&a)[N][M], float (&b)[N][M]) {
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < M; ++j) b[i][j] = static_cast<float>(a[i][j]);
}
template <int N>
void to_float(const double (&a)[N], float (&b)[N]) {
  for (int i = 0; i < N; ++i) b[i] = static_cast<float>(a[i]);
}
}  // namespace

void fill_bc_consts(double gamma, double q[4][4], double* ctan, double* c16, double* s3) {
  // Euler2D::conservative (Equations_Euler2D.cpp:28-34)
  const double g1 = gamma - 1.0;
  auto cons = [&](double r, double u, double v, double p, double* o) {
    o[0] = r;
    o[1] = r * u;
    o[2] = r * v;
    o[3] = p / g1 + 0.5 * (o[1] * u + o[2] * v);
  };
  cons(2.0, 0.0, 0.0, 1.0, q[0]);  // TaylorInstBc wb, wu (:169-172)
  cons(1.0, 0.0, 0.0, 2.5, q[1]);
  *s3 = std::sqrt(3.0);
  cons(8.0, 8.25 * 0.5 * *s3, -8.25 * 0.5, 116.5, q[2]);  // conservativeOfDoubleMach2D (:637-655)
  cons(1.4, 0.0, 0.0, 1.0, q[3]);
  *c16 = 1.0 / 6.0;
  const double pi = 4.0 * std::atan(1.0);  // doubleMachBc (:189-190)
  *ctan = std::tan(pi / 6.0);
}

void fill_dev_const(DevConst* c) {
  const double sq15 = std::sqrt(15.0);
  // crjgp3L / crjgm3L (Schemes_Lagrange.cpp:65-83)
  c->gp[0][0] = 1.0 / 30.0 + sq15 / 20.0;
  c->gp[1][0] = -1.0 / 15.0 - sq15 / 5.0;
  c->gp[2][0] = 31.0 / 30.0 + 3.0 * sq15 / 20.0;
  c->gp[0][1] = 1.0 / 30.0 - sq15 / 20.0;
  c->gp[1][1] = 14.0 / 15.0;
  c->gp[2][1] = 1.0 / 30.0 + sq15 / 20.0;
  c->gp[0][2] = 31.0 / 30.0 - 3.0 * sq15 / 20.0;
  c->gp[1][2] = -1.0 / 15.0 + sq15 / 5.0;
  c->gp[2][2] = 1.0 / 30.0 - sq15 / 20.0;
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) c->gm[r][k] = c->gp[2 - r][2 - k];
  // linear weights of the three Gauss-Legendre points (:86-104)
  const double lin0[3] = {-9.0 / 80.0, 49.0 / 40.0, -9.0 / 80.0};
  for (int i = 0; i < 3; ++i) {
    c->linw0p[i] = 0.5 * (lin0[i] + 3.0 * std::fabs(lin0[i]));
    c->linw0m[i] = c->linw0p[i] - lin0[i];
  }
  c->sumw0p = (c->linw0p[0] + c->linw0p[1]) + c->linw0p[2];
  c->sumw0m = (c->linw0m[0] + c->linw0m[1]) + c->linw0m[2];
  for (int i = 0; i < 3; ++i) {
    c->linw0p[i] = c->linw0p[i] / c->sumw0p;
    c->linw0m[i] = c->linw0m[i] / c->sumw0m;
  }
  double den = 15720.0 * sq15 + 10480.0;
  c->linwp[0] = (2882.0 * sq15 - 1179.0) / den;
  c->linwp[1] = (9672.0 * sq15 + 6448.0) / den;
  c->linwp[2] = (3166.0 * sq15 + 5211.0) / den;
  den = 15720.0 * sq15 - 10480.0;
  c->linwm[0] = (2882.0 * sq15 + 1179.0) / den;
  c->linwm[1] = (9672.0 * sq15 - 6448.0) / den;
  c->linwm[2] = (3166.0 * sq15 - 5211.0) / den;
  {
    // weights of weno5JS3PointsQuadrature when all three indicators vanish, with the device's
    // operations: s = (eps + 0)^2, w_k = lw_k / s, normalised by the left-to-right sum
    const double e = 1e-6 + 0.0, s2 = e * e;
    const double* sets[4] = {c->linwp, c->linw0p, c->linw0m, c->linwm};
    for (int m = 0; m < 4; ++m) {
      double w[3];
      for (int k = 0; k < 3; ++k) w[k] = sets[m][k] / s2;
      const double sum = (w[0] + w[1]) + w[2];
      for (int k = 0; k < 3; ++k) c->gl3flat[m][k] = w[k] / sum;
    }
  }
  c->gl3w[0] = 5.0 / 9.0 / 2.0;
  c->gl3w[1] = 8.0 / 9.0 / 2.0;
  c->gl3w[2] = 5.0 / 9.0 / 2.0;
  // crj (:125-136), dkm / dkp (:140-142)
  const double crj[3][4] = {{11.0 / 6.0, 1.0 / 3.0, -1.0 / 6.0, 1.0 / 3.0},
                            {-7.0 / 6.0, 5.0 / 6.0, 5.0 / 6.0, -7.0 / 6.0},
                            {1.0 / 3.0, -1.0 / 6.0, 1.0 / 3.0, 11.0 / 6.0}};
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 4; ++k) c->crj[r][k] = crj[r][k];
  c->dkm[0] = 0.3; c->dkm[1] = 0.6; c->dkm[2] = 0.1;
  c->dkp[0] = 0.1; c->dkp[1] = 0.6; c->dkp[2] = 0.3;
  pattern_table(c->dkm, c->wtab_m);
  pattern_table(c->dkp, c->wtab_p);
  // Hermite optimal weights (Schemes_Hermite.cpp:57-72)
  c->hdkm[0] = 9.0 / 80.0; c->hdkm[1] = 42.0 / 80.0; c->hdkm[2] = 29.0 / 80.0;
  c->hdkp[0] = c->hdkm[1]; c->hdkp[1] = c->hdkm[0]; c->hdkp[2] = c->hdkm[2];
  c->hdkmd[0] = 1.0 / 18.0; c->hdkmd[1] = 5.0 / 6.0; c->hdkmd[2] = 1.0 / 9.0;
  c->hdkpd[0] = c->hdkmd[1]; c->hdkpd[1] = c->hdkmd[0]; c->hdkpd[2] = c->hdkmd[2];
  pattern_table(c->hdkm, c->hwtab_m);
  pattern_table(c->hdkp, c->hwtab_p);
  pattern_table(c->hdkmd, c->hwtab_md);
  pattern_table(c->hdkpd, c->hwtab_pd);

  to_float(c->crj, c->f_crj);
  to_float(c->gp, c->f_gp);
  to_float(c->gm, c->f_gm);
  to_float(c->linwp, c->f_linwp);
  to_float(c->linwm, c->f_linwm);
  to_float(c->linw0p, c->f_linw0p);
  to_float(c->linw0m, c->f_linw0m);
  c->f_sumw0p = static_cast<float>(c->sumw0p);
  c->f_sumw0m = static_cast<float>(c->sumw0m);
  to_float(c->gl3w, c->f_gl3w);
  to_float(c->wtab_m, c->f_wtab_m);
  to_float(c->wtab_p, c->f_wtab_p);
  to_float(c->hwtab_m, c->f_hwtab_m);
  to_float(c->hwtab_p, c->f_hwtab_p);
  to_float(c->hwtab_md, c->f_hwtab_md);
  to_float(c->hwtab_pd, c->f_hwtab_pd);
}

}  // namespace hteno
