// Barotropic subcycle of the precision form (B grid): the same predictor,
// momentum and corrector as pred_corr_tropic_depth_bgrid
// (ocean_barotropic.F90:3255-3575), in FP64 but with the step constants folded
// into per-column coefficients once per baroclinic step and the products
// contracted into FMAs.  The result is FP64-accurate (not bit-identical to the
// reference order); the exact drop-in keeps the bodies of fp64_bodies.cuh.
// Included by translation units built with FMA contraction on.
//
// Coefficients (planes of BtArgs::btf, each (ni+2)(nj+2)):
//   KG = -dtbt_gamma_rho0r*tmask*datr   SG = dtbt_gamma_rho0r*steady   (predictor)
//   KC = -dtbt_rho0r*tmask*datr         SC = dtbt_rho0r*steady         (corrector)
//   A  = dtbt*f/2
//   BX = -dtbt*thicku*dxur*umask/2, BY = -dtbt*thicku*dyur*umask/2 on compute
//        points (0 elsewhere: no pressure gradient there)
//   FU = dtbt*forcing_u, FV = dtbt*forcing_v
// so that, with D the undivided DIV_UD numerator and P the undivided corner
// differences of ps,
//   eta(new) = eta(old) + S + K*D
//   u(new)   = cori2*(t1 + cori1*t2), t1 = u + A*v + BX*Px + FU, t2 = v - A*u + BY*Py + FV.
#pragma once

#include "internal.h"

namespace mom5 {
namespace btfast {

#define DEVI __device__ __forceinline__

enum { KG = 0, SG, KC, SC, A, BX, BY, FU, FV, NPLANES };

DEVI long I2(const Geo& g, int i, int j) { return (long)j * g.nxd + i; }

// same rule as the exact path: a halo point takes its periodic image's value
// when the single-PE halo update would copy it, else it keeps its own
DEVI bool halo_image(const Geo& g, int& i, int& j) {
  bool hx = (i == 0 || i == g.ni + 1), hy = (j == 0 || j == g.nj + 1);
  if (!hx && !hy) return true;
  if (hx && hy) {
    if (!(g.cx && g.cy)) return false;
  } else if (hx && !g.cx) {
    return false;
  } else if (hy && !g.cy) {
    return false;
  }
  if (i == 0) i = g.ni;
  else if (i == g.ni + 1) i = 1;
  if (j == 0) j = g.nj;
  else if (j == g.nj + 1) j = 1;
  return true;
}

// undivided DIV_UD numerator from the stored products uh = u*dyu, vh = v*dxu
// (the backward averages' 1/2 is folded into the coefficients K)
DEVI double div_num(const Geo& g, const double* uh, const double* vh, int i, int j) {
  if (i < 1 || j < 1) return 0.0;
  long q = I2(g, i, j), qw = q - 1, qs = q - g.nxd, qsw = qs - 1;
  return ((uh[q] + uh[qs]) - (uh[qw] + uh[qsw])) + ((vh[q] + vh[qw]) - (vh[qs] + vh[qsw]));
}

DEVI void prep_body(const BtArgs& a, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x, j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j), n2 = g.n2;
  double* c = a.btf;
  double tmd = a.tmask1[q] * a.datr[q];
  c[KG * n2 + q] = -a.dtbt_gamma_rho0r * tmd * 0.5;
  c[SG * n2 + q] = a.dtbt_gamma_rho0r * a.steady[q];
  c[KC * n2 + q] = -a.dtbt_rho0r * tmd * 0.5;
  c[SC * n2 + q] = a.dtbt_rho0r * a.steady[q];
  c[A * n2 + q] = a.dtbt * a.f[q] * 0.5;
  bool comp = i <= g.ni && j <= g.nj;
  double th = a.dtbt * a.thicku[q] * a.umask1[q] * 0.5;
  c[BX * n2 + q] = comp ? -th * a.dxur[q] : 0.0;
  c[BY * n2 + q] = comp ? -th * a.dyur[q] : 0.0;
  c[FU * n2 + q] = a.dtbt * a.forcing_u[q];
  c[FV * n2 + q] = a.dtbt * a.forcing_v[q];
}

// with reuse, D of level so is the previous corrector's D of the same arrays (dvs)
DEVI void pred_body(const BtArgs& a, int so, int sn, int reuse, int bx, int by) {
  const Geo& g = a.g;
  int i0 = bx * blockDim.x + threadIdx.x, j0 = by;
  if (i0 > g.ni + 1) return;
  int i = i0, j = j0;
  if (!halo_image(g, i, j)) {
    i = i0;
    j = j0;
  }
  long q = I2(g, i, j), n2 = g.n2;
  double en = a.eta_bt[so * n2 + q];
  if (a.gamma > 0.0) {
    double D = reuse ? a.dvs[q] : div_num(g, a.uhb + so * n2, a.vhb + so * n2, i, j);
    en = fma(a.btf[KG * n2 + q], D, en + a.btf[SG * n2 + q]);
  }
  long q0 = I2(g, i0, j0);
  a.eta_bt[sn * n2 + q0] = en;
  a.ps[q0] = fma(a.rho_g[q0], en, a.patm[q0]);
}

DEVI void mom_body(const BtArgs& a, int so, int sn, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x, j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j), n2 = g.n2;
  const double* c = a.btf;
  double px = 0.0, py = 0.0;
  if (i <= g.ni && j <= g.nj) {
    const double* ps = a.ps;
    double p00 = ps[q], p10 = ps[q + 1], p01 = ps[q + g.nxd], p11 = ps[q + g.nxd + 1];
    px = (p10 + p11) - (p00 + p01);
    py = (p01 + p11) - (p00 + p10);
  }
  double uo = a.ubt[so * n2 + q], vo = a.vbt[so * n2 + q];
  double hf = c[A * n2 + q];
  double t1 = uo + fma(hf, vo, fma(c[BX * n2 + q], px, c[FU * n2 + q]));
  double t2 = vo + fma(-hf, uo, fma(c[BY * n2 + q], py, c[FV * n2 + q]));
  double c1 = a.cori1[q], c2 = a.cori2[q];
  double un = c2 * fma(c1, t2, t1);
  double vn = c2 * fma(-c1, t1, t2);
  a.ubt[sn * n2 + q] = un;
  a.vbt[sn * n2 + q] = vn;
  a.uhb[sn * n2 + q] = un * a.dyu[q];
  a.vhb[sn * n2 + q] = vn * a.dxu[q];
}

DEVI void corr_body(const BtArgs& a, int so, int sn, double wgt, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x, j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j), n2 = g.n2;
  double D = div_num(g, a.uhb + sn * n2, a.vhb + sn * n2, i, j);
  a.dvs[q] = D;
  double en = fma(a.btf[KC * n2 + q], D, a.eta_bt[so * n2 + q] + a.btf[SC * n2 + q]);
  a.eta_bt[sn * n2 + q] = en;
  a.eta_bar[q] += en;
  double un = a.ubt[sn * n2 + q], vn = a.vbt[sn * n2 + q];
  if (a.stepB) {
    a.udrho_u[q] = fma(wgt, un, a.udrho_u[q]);
    a.udrho_v[q] = fma(wgt, vn, a.udrho_v[q]);
  } else {
    a.udrho_u[q] += un;
    a.udrho_v[q] += vn;
  }
}

}  // namespace btfast
}  // namespace mom5
