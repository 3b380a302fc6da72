// Constant block of the device numerics.  Plain C++ so that the host file that fills it
// (device_consts.cpp) is compiled by the host compiler alone.
#pragma once

namespace hteno {

// Filled by the host from the reference's constructor formulas.
struct DevConst {
  // Schemes::Lagrange (Schemes_Lagrange.cpp:6-304)
  double crj[3][4];
  double gp[3][3], gm[3][3];          // crjgp3L / crjgm3L
  double linwp[3], linwm[3], linw0p[3], linw0m[3], sumw0p, sumw0m;
  double gl3w[3];                     // Gauss-Legendre weights / 2 (FV_System2D.cpp:28)
  // normalised GL3 weights when every smoothness indicator is zero (constant data): the sets
  // linwp, linw0p, linw0m, linwm divided by (eps + 0)^2 and normalised, in that order
  double gl3flat[4][3];
  double wtab_m[8][3], wtab_p[8][3];  // TENO5 weights per cut-off pattern (dkm / dkp)
  double dkm[3], dkp[3];
  // Schemes::Hermite (Schemes_Hermite.cpp:5-92, grid-size independent part)
  double hdkm[3], hdkp[3], hdkmd[3], hdkpd[3];
  double hwtab_m[8][3], hwtab_p[8][3], hwtab_md[8][3], hwtab_pd[8][3];
  // float copies of the most used tables for the mixed path
  float f_crj[3][4], f_gp[3][3], f_gm[3][3];
  float f_linwp[3], f_linwm[3], f_linw0p[3], f_linw0m[3], f_sumw0p, f_sumw0m, f_gl3w[3];
  float f_wtab_m[8][3], f_wtab_p[8][3];
  float f_hwtab_m[8][3], f_hwtab_p[8][3], f_hwtab_md[8][3], f_hwtab_pd[8][3];
};

void fill_dev_const(DevConst* c);  // host side, device_consts.cpp

// Fixed states and constants of the TaylorInstBc / doubleMachBc ghost rules (FV_System2D.cpp:
// 154-224), computed on the host as the reference computes them: q[0] bottom and q[1] top state
// of TaylorInstBc, q[2] post-shock and q[3] pre-shock state of conservativeOfDoubleMach2D; tan(pi/6)
// with pi = 4 atan(1); 1/6; sqrt(3).  host side, device_consts.cpp
void fill_bc_consts(double gamma, double q[4][4], double* ctan, double* c16, double* s3);

}  // namespace hteno
