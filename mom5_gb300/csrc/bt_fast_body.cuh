// Barotropic subcycle of the precision form (B grid): the same predictor,
// momentum and corrector as pred_corr_tropic_depth_bgrid
// (ocean_barotropic.F90:3255-3575) with the state (eta, udrho, the transports
// u*dyu, v*dxu and the time sums) in FP64 and each subcycle's increments in
// FP32, the form's "FP32 fluxes, FP64 state" split.  The exact drop-in keeps
// the bodies of fp64_bodies.cuh.
//
// Step coefficients, FP32 planes of BtArgs::btf (each (ni+2)(nj+2) floats),
// formed in FP64 once per baroclinic step and rounded to FP32:
//   KG = -dtbt_gamma_rho0r*tmask*datr/2   SG = dtbt_gamma_rho0r*steady   (predictor)
//   KC = -dtbt_rho0r*tmask*datr/2         SC = dtbt_rho0r*steady         (corrector)
//   A  = dtbt*f/2
//   BX = -dtbt*thicku*dxur*umask/2, BY = -dtbt*thicku*dyur*umask/2 on compute
//        points (0 elsewhere: no pressure gradient there)
//   G1 = cori2 - 1, G2 = cori2*cori1            (the Coriolis rotation as an increment)
//   PX = BX*Px(patm + rho_g*E) + dtbt*forcing_u, PY = BY*Py(patm + rho_g*E) + dtbt*forcing_v
//        (the pressure gradient of the step's initial surface E, an FP64 plane, and
//        the forcing, each rounded to FP32 and summed in FP32)
//   RG = rho_g
// With D the undivided DIV_UD numerator of the transports and Px, Py the
// undivided corner differences of rho_g*(eta - E) (a float plane PS written by
// the predictor: the departure from E, small, keeps its FP32 rounding small
// against the gradient), a subcycle is
//   eta(new) = eta(old) + [S + K*D]
//   u(new)   = u + [d1 + G1*t1 + G2*t2],  v(new) = v + [d2 + G1*t2 - G2*t1]
//   d1 = A*v + BX*Px + PX,  d2 = -A*u + BY*Py + PY,  t1 = u + d1,  t2 = v + d2
// (algebraically u(new) = cori2*(t1 + cori1*t2), v(new) = cori2*(t2 - cori1*t1)),
// the brackets in FP32 and each added to the FP64 state with one FP64 add.  D
// is formed from four FP64 differences of neighbouring transports summed in
// FP32.  The increments are small against the state (Coriolis and pressure
// terms of one short subcycle), so their FP32 rounding stays near 1e-7 of the
// increment and far below the form's 1e-6 bound on the state.
#pragma once

#include "internal.h"
#include "mixed_body.cuh"

namespace mom5 {
namespace btfast {

#define DEVI __device__ __forceinline__

enum { KG = 0, SG, KC, SC, A, BX, BY, G1, G2, PX, PY, RG, PS, DV, E0, E1, DV1, NPLANES };
static_assert(E0 % 2 == 0, "the FP64 plane E starts on an 8-byte boundary");
static_assert(NPLANES <= 2 * kBtFastPlanes, "float planes of the precision-form subcycle");

DEVI long I2(const Geo& g, int i, int j) { return (long)j * g.nxd + i; }
DEVI float* plane(const BtArgs& a, int p) { return reinterpret_cast<float*>(a.btf) + (long)p * a.g.n2; }
// E: the FP64 plane over float planes E0, E1 (8-byte aligned: n2 floats per plane, E0 even)
DEVI double* eref(const BtArgs& a) { return reinterpret_cast<double*>(plane(a, E0)); }

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

// undivided DIV_UD numerator of a point from the stored transports uh = u*dyu,
// vh = v*dxu at the point (c) and its west (w), south (s) and south-west (sw)
// neighbours (the backward averages' 1/2 is folded into K): four FP64
// differences, rounded to FP32 and summed
DEVI float div_sum(double uc, double uw, double us, double usw, double vc, double vw, double vs, double vsw) {
  float d1 = mixed::d2f_rn(uc - uw), d2 = mixed::d2f_rn(us - usw);
  float d3 = mixed::d2f_rn(vc - vs), d4 = mixed::d2f_rn(vw - vsw);
  return (d1 + d2) + (d3 + d4);
}
DEVI float div_num(const Geo& g, const double* uh, const double* vh, int i, int j) {
  if (i < 1 || j < 1) return 0.0f;
  long q = I2(g, i, j), qw = q - 1, qs = q - g.nxd, qsw = qs - 1;
  return div_sum(uh[q], uh[qw], uh[qs], uh[qsw], vh[q], vh[qw], vh[qs], vh[qsw]);
}

// The arithmetic of one point of the predictor, the momentum step and the
// corrector, shared by the three-launch subcycle and the one-launch subcycle so
// that both give the same bits.
//
// predictor of point (i0, j0): the predicted eta (en, from the point's image
// under the halo rule) and the returned surface-pressure departure PS; dv is the
// divergence plane the previous corrector wrote (read when reuse)
DEVI float pred_point(const BtArgs& a, int so, int reuse, const float* dv, int i0, int j0, double& en) {
  const Geo& g = a.g;
  int i = i0, j = j0;
  if (!halo_image(g, i, j)) {
    i = i0;
    j = j0;
  }
  long q = I2(g, i, j), n2 = g.n2;
  en = a.eta_bt[so * n2 + q];
  if (a.gamma > 0.0) {
    float D = reuse ? dv[q] : div_num(g, a.uhb + so * n2, a.vhb + so * n2, i, j);
    en += mixed::f2d(fmaf(plane(a, KG)[q], D, plane(a, SG)[q]));
  }
  long q0 = I2(g, i0, j0);
  return plane(a, RG)[q0] * mixed::d2f_rn(en - eref(a)[q0]);
}
// undivided corner differences of PS around a U point
DEVI void ps_diff(float p00, float p10, float p01, float p11, float& px, float& py) {
  px = (p10 + p11) - (p00 + p01);
  py = (p01 + p11) - (p00 + p10);
}
// momentum step of point q from its PS differences: the new transports un, vn
DEVI void mom_point(const BtArgs& a, int so, long q, float px, float py, double& un, double& vn) {
  const long n2 = a.g.n2;
  double uo = a.ubt[so * n2 + q], vo = a.vbt[so * n2 + q];
  float uf = mixed::d2f_rn(uo), vf = mixed::d2f_rn(vo), hf = plane(a, A)[q];
  float d1 = fmaf(hf, vf, fmaf(plane(a, BX)[q], px, plane(a, PX)[q]));
  float d2 = fmaf(-hf, uf, fmaf(plane(a, BY)[q], py, plane(a, PY)[q]));
  float t1 = uf + d1, t2 = vf + d2, g1 = plane(a, G1)[q], g2 = plane(a, G2)[q];
  un = uo + mixed::f2d(d1 + fmaf(g1, t1, g2 * t2));
  vn = vo + mixed::f2d(d2 + fmaf(g1, t2, -g2 * t1));
}
// time sums of the transports of point q, formed where the new transports are
// (the momentum step; the corrector does not change them)
DEVI void sum_point(const BtArgs& a, double wgt, long q, double un, double vn) {
  if (a.stepB) {
    a.udrho_u[q] = fma(wgt, un, a.udrho_u[q]);
    a.udrho_v[q] = fma(wgt, vn, a.udrho_v[q]);
  } else {
    a.udrho_u[q] += un;
    a.udrho_v[q] += vn;
  }
}
// corrector of point q from its divergence D, with the time sum of eta
DEVI double corr_point(const BtArgs& a, int so, int sn, long q, float D) {
  const long n2 = a.g.n2;
  double en = a.eta_bt[so * n2 + q] + mixed::f2d(fmaf(plane(a, KC)[q], D, plane(a, SC)[q]));
  a.eta_bt[sn * n2 + q] = en;
  a.eta_bar[q] += en;
  return en;
}

DEVI void prep_body(const BtArgs& a, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x, j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double tmd = a.tmask1[q] * a.datr[q];
  plane(a, KG)[q] = (float)(-a.dtbt_gamma_rho0r * tmd * 0.5);
  plane(a, SG)[q] = (float)(a.dtbt_gamma_rho0r * a.steady[q]);
  plane(a, KC)[q] = (float)(-a.dtbt_rho0r * tmd * 0.5);
  plane(a, SC)[q] = (float)(a.dtbt_rho0r * a.steady[q]);
  plane(a, A)[q] = (float)(a.dtbt * a.f[q] * 0.5);
  bool comp = i <= g.ni && j <= g.nj;
  double th = a.dtbt * a.thicku[q] * a.umask1[q] * 0.5;
  double bxq = comp ? -th * a.dxur[q] : 0.0, byq = comp ? -th * a.dyur[q] : 0.0;
  plane(a, BX)[q] = (float)bxq;
  plane(a, BY)[q] = (float)byq;
  plane(a, G1)[q] = (float)(a.cori2[q] - 1.0);
  plane(a, G2)[q] = (float)(a.cori2[q] * a.cori1[q]);
  // E = eta_bt at the first subcycle's old level (eta_t_bar(tau), set by the init kernel)
  const double* e = a.eta_bt + g.n2;
  eref(a)[q] = e[q];
  double pxa = 0.0, pya = 0.0;
  if (comp) {
    auto P = [&](long r) { return a.patm[r] + a.rho_g[r] * e[r]; };
    double p00 = P(q), p10 = P(q + 1), p01 = P(q + g.nxd), p11 = P(q + g.nxd + 1);
    pxa = bxq * ((p10 + p11) - (p00 + p01));
    pya = byq * ((p01 + p11) - (p00 + p10));
  }
  plane(a, PX)[q] = (float)pxa + (float)(a.dtbt * a.forcing_u[q]);
  plane(a, PY)[q] = (float)pya + (float)(a.dtbt * a.forcing_v[q]);
  plane(a, RG)[q] = (float)a.rho_g[q];
}

// with reuse, D of level so is the previous corrector's D of the same arrays
DEVI void pred_body(const BtArgs& a, int so, int sn, int reuse, int bx, int by) {
  const Geo& g = a.g;
  int i0 = bx * blockDim.x + threadIdx.x, j0 = by;
  if (i0 > g.ni + 1) return;
  double en;
  const float ps = pred_point(a, so, reuse, plane(a, DV), i0, j0, en);
  long q0 = I2(g, i0, j0);
  a.eta_bt[sn * g.n2 + q0] = en;
  plane(a, PS)[q0] = ps;
}

DEVI void mom_body(const BtArgs& a, int so, int sn, double wgt, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x, j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j), n2 = g.n2;
  float px = 0.0f, py = 0.0f;
  if (i <= g.ni && j <= g.nj) {
    const float* ps = plane(a, PS);
    ps_diff(ps[q], ps[q + 1], ps[q + g.nxd], ps[q + g.nxd + 1], px, py);
  }
  double un, vn;
  mom_point(a, so, q, px, py, un, vn);
  a.ubt[sn * n2 + q] = un;
  a.vbt[sn * n2 + q] = vn;
  a.uhb[sn * n2 + q] = un * a.dyu[q];
  a.vhb[sn * n2 + q] = vn * a.dxu[q];
  sum_point(a, wgt, q, un, vn);
}

DEVI void corr_body(const BtArgs& a, int so, int sn, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x, j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j), n2 = g.n2;
  float D = div_num(g, a.uhb + sn * n2, a.vhb + sn * n2, i, j);
  plane(a, DV)[q] = D;
  corr_point(a, so, sn, q, D);
}

// Corrector of subcycle t and predictor of subcycle t+1 in one launch.  The
// predictor of a point reads only that point's corrected eta and divergence (or,
// for a halo point in a periodic direction, its image's), so the thread of a
// point forms its next PS from the values it has just computed, and the thread
// of a compute point also forms the PS of the periodic halo points whose image
// it is.  The predicted eta is not stored (the next corrector overwrites it
// unread), nor is the divergence.  Same arithmetic as corr_body then pred_body
// with reuse, so the same bits.
DEVI void corr_pred_body(const BtArgs& a, int so, int sn, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x, j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j), n2 = g.n2;
  const float D = div_num(g, a.uhb + sn * n2, a.vhb + sn * n2, i, j);
  double en = corr_point(a, so, sn, q, D);
  // the next subcycle's predictor at this point (pred_point with reuse)
  if (a.gamma > 0.0) en += mixed::f2d(fmaf(plane(a, KG)[q], D, plane(a, SG)[q]));
  float* ps = plane(a, PS);
  const float* rg = plane(a, RG);
  const double* e0 = eref(a);
  int ii = i, jj = j;
  if (!halo_image(g, ii, jj) || (ii == i && jj == j)) ps[q] = rg[q] * mixed::d2f_rn(en - e0[q]);
  if (i < 1 || i > g.ni || j < 1 || j > g.nj) return;
  // periodic halo points whose image this compute point is
  int hx[2], nhx = 0, hy[2], nhy = 0;
  if (g.cx) {
    if (i == g.ni) hx[nhx++] = 0;
    if (i == 1) hx[nhx++] = g.ni + 1;
  }
  if (g.cy) {
    if (j == g.nj) hy[nhy++] = 0;
    if (j == 1) hy[nhy++] = g.nj + 1;
  }
  for (int u = 0; u < nhx; ++u) {
    const long r = I2(g, hx[u], j);
    ps[r] = rg[r] * mixed::d2f_rn(en - e0[r]);
  }
  for (int v = 0; v < nhy; ++v) {
    const long r = I2(g, i, hy[v]);
    ps[r] = rg[r] * mixed::d2f_rn(en - e0[r]);
  }
  if (g.cx && g.cy)
    for (int u = 0; u < nhx; ++u)
      for (int v = 0; v < nhy; ++v) {
        const long r = I2(g, hx[u], hy[v]);
        ps[r] = rg[r] * mixed::d2f_rn(en - e0[r]);
      }
}

// One whole subcycle -- predictor, momentum, corrector -- in one launch on a
// tile of TX x TY data-domain points.  The tile recomputes what its corrector
// needs from its neighbours in shared memory: PS on the tile and a ring of one
// (west and south for the momentum's west and south ring, east and north for
// the corner differences), the momentum on the tile and its west and south
// ring.  No PS plane and no predicted eta go through global memory; the
// divergence the next predictor reuses goes to plane DV or DV1 by parity (a
// neighbouring tile may still be reading the other one).  Each point's
// arithmetic is the three-launch subcycle's (the point helpers above), so the
// results are the same bits.
template <int TX, int TY>
DEVI void fused_body(const BtArgs& a, int so, int sn, int reuse, double wgt, int bx, int by) {
  constexpr int PXN = TX + 2, PYN = TY + 2;  // PS: points x0-1 .. x0+TX, y0-1 .. y0+TY
  constexpr int MX = TX + 1, MY = TY + 1;    // momentum: points x0-1 .. x0+TX-1, y0-1 .. y0+TY-1
  __shared__ float ps_s[PYN * PXN];
  __shared__ double uh_s[MY * MX], vh_s[MY * MX];
  const Geo& g = a.g;
  const long n2 = g.n2;
  const int x0 = bx * TX, y0 = by * TY;
  const float* dv_o = plane(a, so ? DV1 : DV);
  float* dv_n = plane(a, sn ? DV1 : DV);
  // ---- predictor: PS on the tile and its ring ----
  for (int e = threadIdx.x; e < PXN * PYN; e += blockDim.x) {
    const int i0 = x0 - 1 + e % PXN, j0 = y0 - 1 + e / PXN;
    if (i0 < 0 || i0 > g.ni + 1 || j0 < 0 || j0 > g.nj + 1) continue;  // never read
    double en;
    ps_s[e] = pred_point(a, so, reuse, dv_o, i0, j0, en);
  }
  __syncthreads();
  // ---- momentum on the tile and its west and south ring ----
  for (int e = threadIdx.x; e < MX * MY; e += blockDim.x) {
    const int li = e % MX, lj = e / MX;
    const int i = x0 - 1 + li, j = y0 - 1 + lj;
    if (i < 0 || i > g.ni + 1 || j < 0 || j > g.nj + 1) continue;  // never read
    const long q = I2(g, i, j);
    float px = 0.0f, py = 0.0f;
    if (i <= g.ni && j <= g.nj) {
      const int pe = lj * PXN + li;  // PS point (i, j)
      ps_diff(ps_s[pe], ps_s[pe + 1], ps_s[pe + PXN], ps_s[pe + PXN + 1], px, py);
    }
    double un, vn;
    mom_point(a, so, q, px, py, un, vn);
    const double uh = un * a.dyu[q], vh = vn * a.dxu[q];
    uh_s[e] = uh;
    vh_s[e] = vh;
    if (li >= 1 && lj >= 1) {  // the tile's own points: the state the next subcycle reads
      a.ubt[sn * n2 + q] = un;
      a.vbt[sn * n2 + q] = vn;
      a.uhb[sn * n2 + q] = uh;
      a.vhb[sn * n2 + q] = vh;
      sum_point(a, wgt, q, un, vn);
    }
  }
  __syncthreads();
  // ---- corrector and the time sum of eta on the tile ----
  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    const int li = e % TX + 1, lj = e / TX + 1;  // in the momentum arrays
    const int i = x0 - 1 + li, j = y0 - 1 + lj;
    if (i > g.ni + 1 || j > g.nj + 1) continue;
    const long q = I2(g, i, j);
    const int m = lj * MX + li, mw = m - 1, ms = m - MX, msw = ms - 1;
    const float D = (i >= 1 && j >= 1)
                        ? div_sum(uh_s[m], uh_s[mw], uh_s[ms], uh_s[msw], vh_s[m], vh_s[mw], vh_s[ms], vh_s[msw])
                        : 0.0f;
    dv_n[q] = D;
    corr_point(a, so, sn, q, D);
  }
}

}  // namespace btfast
}  // namespace mom5
