// MDPPM (advect_tracer_mdppm, ocean_tracer_advect.F90:5990-6507): direction-split
// piecewise-parabolic advection, z then x then y, with the edge limiter chosen
// per tracer (ppm_hlimiter: 1 Colella-Woodward 1984 :6510-6538, 2 improved full
// constraint :6555-6580, 3 Suresh-Huynh 1997 :6601-6660; the reference applies
// it in all three directions).  FP64 in the reference's operation order; built
// with --fmad=false.
//
// The horizontal passes stream along a line of cells (one thread per line):
// at the step that reads cell i the thread forms the slope of cell i-2, the
// limited edge values and curvature of cell i-3, the flux through face i-4
// and the update of cell i-4, keeping a sliding window of the values each
// needs.  Values outside the compute domain come from the halo of width 4 by
// the single-PE rules (periodic image, else 0), as tracer_mdppm and
// tmask_mdppm hold them (mdppm_init :1702-1735).
#pragma once

#include "fp64_select.cuh"
#include "internal.h"

namespace mom5 {
namespace ppm {

#define DEVI __device__ __forceinline__

constexpr double kR12 = 1.0 / 12.0, kSixth = 1.0 / 6.0, kTwoThirds = 2.0 / 3.0, kFourThirds = 4.0 / 3.0;

// a > b ? a : b and a < b ? a : b, compared on the integer pipe
DEVI double mx(double a, double b) { return sel::gt_max(a, b); }
DEVI double mn(double a, double b) { return sel::lt_min(a, b); }

// slope of the centre cell of S[0..4] (offsets -2..+2) and its one-sided differences
DEVI void slope(const double* S, const double* M, double& da, double& d1m, double& d1p, double& d1mm, double& d1pp) {
  double Sim2 = S[0], Sim1 = S[1], Si = S[2], Sip1 = S[3], Sip2 = S[4];
  double mskm2 = M[0], mskm1 = M[1], msk0 = M[2], mskp1 = M[3], mskp2 = M[4];
  double da2 = 0.5 * (Sip1 - Sim1);
  double da3m = kR12 * (2. * Sim2 - 12. * Sim1 + 6. * Si + 4. * Sip1);
  double da3p = kR12 * (-(4. * Sim1) - 6. * Si + 12. * Sip1 - 2. * Sip2);
  double a = ((mskm2 * (1. - 0.5 * mskp2) * da3m + mskp2 * (1. - 0.5 * mskm2) * da3p) +
              (1. - mskm2) * (1. - mskp2) * da2);
  double dMx = mx(mx(Sip1, Sim1), Si) - Si;
  double dMn = Si - mn(mn(Sip1, Sim1), Si);
  da = copysign(1., a) * mn(fabs(a), 2. * mn(dMx, dMn)) * mskm1 * mskp1 * msk0;
  d1m = (Si - Sim1) * mskm1;
  d1p = (Sip1 - Si) * mskp1;
  d1mm = (Sim1 - Sim2) * mskm1 * mskm2;
  d1pp = (Sip2 - Sip1) * mskp1 * mskp2;
}

DEVI void limit(int lim, double Si, double da, double d1m, double d1p, double d1mm, double d1pp, double& aL,
                double& aR) {
  if (lim == 1) {
    if (!sel::gt0((aR - Si) * (Si - aL))) {
      aL = Si;
      aR = Si;
    }
    double da2 = aR - aL, da4 = 0.5 * (aR + aL);
    double da3m = 6. * da2 * (Si - da4), da3p = da2 * da2;
    if (sel::ord0(da3m) > sel::ord0(da3p)) aL = 3. * Si - 2. * aR;
    if (sel::ord0(da3m) < sel::ord0(-da3p)) aR = 3. * Si - 2. * aL;
  } else if (lim == 2) {
    double ada = fabs(da), sda = copysign(1., da);
    aL = Si - sda * mn(ada, fabs(aL - Si));
    aR = Si + sda * mn(ada, fabs(aR - Si));
  } else {
    double Sim1 = Si - d1m, Sip1 = Si + d1p;
    double z = d1m - d1mm, w = d1p - d1m;
    double x = 4. * w - z, y = 4. * z - w;
    double dM4m = mx(0., mn(mn(mn(x, y), z), w)) + mn(0., mx(mx(mx(x, y), z), w));
    z = d1pp - d1p;
    x = 4. * w - z;
    y = 4. * z - w;
    double dM4p = mx(0., mn(mn(mn(x, y), z), w)) + mn(0., mx(mx(mx(x, y), z), w));
    double qAV = 0.5 * (Si + Sip1);
    x = d1p;
    y = 3. * d1m;
    double qMP = Si + mx(0., mn(x, y)) + mn(0., mx(x, y));
    double qUL = Si + y;
    double qLC = (Si + 0.5 * d1m) + kFourThirds * dM4m;
    double qMD = qAV - 0.5 * dM4p;
    double qMin = mx(mn(mn(qMD, Si), Sip1), mn(mn(Si, qUL), qLC));
    double qMax = mn(mx(mx(qMD, Si), Sip1), mx(mx(Si, qUL), qLC));
    if (sel::ord0((aR - Si) * (aR - qMP)) > sel::ord0(1.e-10)) aR = mn(mx(aR, qMin), qMax);
    qAV = 0.5 * (Si + Sim1);
    x = -d1m;
    y = -3. * d1p;
    qMP = Si + mx(0., mn(x, y)) + mn(0., mx(x, y));
    qUL = Si + y;
    qLC = (Si - 0.5 * d1p) + kFourThirds * dM4p;
    qMD = qAV - 0.5 * dM4m;
    qMin = mx(mn(mn(qMD, Si), Sim1), mn(mn(Si, qUL), qLC));
    qMax = mn(mx(mx(qMD, Si), Sim1), mx(mx(Si, qUL), qLC));
    if (sel::ord0((aL - Si) * (aL - qMP)) > sel::ord0(1.e-10)) aL = mn(mx(aL, qMin), qMax);
  }
}

// flux through the face between a cell with edge data (aL0, aR0, a60) and mask m0 and
// its neighbour (aL1, aR1, a61), mask m1, in the horizontal passes (:6293-6305,
// :6470-6482); the masks multiply in the reference's order
DEVI double hflux(double massflux, double m0, double m1, double cfl, double aL0, double aR0, double a60, double aL1,
                  double aR1, double a61) {
  if (sel::ge0(massflux))
    return massflux * m0 * m1 * (aR0 + 0.5 * cfl * ((aL0 - aR0) + (1. - kTwoThirds * cfl) * a60));
  return massflux * m0 * m1 * (aL1 - 0.5 * cfl * ((aR1 - aL1) + (1. + kTwoThirds * cfl) * a61));
}

// Stream one line of n compute cells (positions 1..n).  S(pos), M(pos) give the
// tracer and mask of any position in [-3, n+4];
// face(pos, m0, m1, aL0, aR0, a60, aL1, aR1, a61) returns the flux through face pos
// (between cells pos and pos+1, whose masks and edge data are passed);
// upd(pos, S, m, Fw, Fe) applies the update of cell pos (its tracer and mask, the
// fluxes through its west/south and east/north faces).
template <class FS, class FM, class FF, class FU>
DEVI void stream_line(int n, int lim, FS S, FM M, FF face, FU upd) {
  double sw[5], mw[5];        // tracer and mask at i-4..i
  double daw[3];              // slope at i-4..i-2
  double d1[2][4];            // d1m, d1p, d1mm, d1pp at i-3, i-2
  double eL[2], eR[2], e6[2];  // edge values and curvature at i-4, i-3
  double fprev = 0.0;         // flux through face i-5
#pragma unroll
  for (int q = 0; q < 5; ++q) sw[q] = mw[q] = 0.0;
#pragma unroll
  for (int q = 0; q < 3; ++q) daw[q] = 0.0;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    eL[q] = eR[q] = e6[q] = 0.0;
    d1[q][0] = d1[q][1] = d1[q][2] = d1[q][3] = 0.0;
  }
  for (int i = -3; i <= n + 4; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      sw[q] = sw[q + 1];
      mw[q] = mw[q + 1];
    }
    sw[4] = S(i);
    mw[4] = M(i);
    // slope of cell i-2 (needed for i-2 in [-1, n+2])
    daw[0] = daw[1];
    daw[1] = daw[2];
#pragma unroll
    for (int c = 0; c < 4; ++c) d1[0][c] = d1[1][c];
    if (i >= 1) slope(sw, mw, daw[2], d1[1][0], d1[1][1], d1[1][2], d1[1][3]);
    // edge values of cell i-3 (needed for i-3 in [0, n+1])
    eL[0] = eL[1];
    eR[0] = eR[1];
    e6[0] = e6[1];
    if (i >= 3) {
      double Si = sw[1];
      double Sim1 = Si - d1[0][0], Sip1 = Si + d1[0][1];
      double al = 0.5 * (Sim1 + Si) + kSixth * (daw[0] - daw[1]);
      double ar = 0.5 * (Si + Sip1) + kSixth * (daw[1] - daw[2]);
      limit(lim, Si, daw[1], d1[0][0], d1[0][1], d1[0][2], d1[0][3], al, ar);
      eL[1] = al;
      eR[1] = ar;
      e6[1] = 6. * Si - 3. * (ar + al);
    }
    // flux through face i-4 (faces 0..n) and update of cell i-4 (cells 1..n)
    if (i >= 4) {
      double f = face(i - 4, mw[0], mw[1], eL[0], eR[0], e6[0], eL[1], eR[1], e6[1]);
      if (i >= 5) upd(i - 4, sw[0], mw[0], fprev, f);
      fprev = f;
    }
  }
}

// The same computation as stream_line with one thread per position: a segment
// of L positions p0 .. p0+L-1 of BI lines (lane = the line's slot) forms, stage
// by stage with a barrier between stages, the slopes, the limited edge values,
// the fluxes and the updates; cells p0+4 .. p0+L-5 are updated (the first and
// last four positions only supply their neighbours).  sm holds the stages'
// values: tracer, mask, slope, edge values, curvature and face flux.
template <int L, int BI, class FS, class FM, class FF, class FU>
DEVI void tile_line(int n, int lim, int p0, int t, int lane, bool lane_ok, double (*sm)[L][BI], FS S, FM M, FF face,
                    FU upd) {
  enum { QS, QM, QDA, QL, QR, Q6, QF };
  const int p = p0 + t;
  double sv = 0.0, mv = 0.0;
  if (lane_ok && p >= -3 && p <= n + 4) {
    sv = S(p);
    mv = M(p);
  }
  sm[QS][t][lane] = sv;
  sm[QM][t][lane] = mv;
  __syncthreads();
  // slope and one-sided differences of positions -1 .. n+2
  double da = 0.0, d1m = 0.0, d1p = 0.0, d1mm = 0.0, d1pp = 0.0;
  if (lane_ok && t >= 2 && t <= L - 3 && p >= -1 && p <= n + 2) {
    double Sw[5], Mw[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      Sw[q] = sm[QS][t - 2 + q][lane];
      Mw[q] = sm[QM][t - 2 + q][lane];
    }
    slope(Sw, Mw, da, d1m, d1p, d1mm, d1pp);
  }
  sm[QDA][t][lane] = da;
  __syncthreads();
  // limited edge values and curvature of cells 0 .. n+1
  double el = 0.0, er = 0.0, e6 = 0.0;
  if (lane_ok && t >= 3 && t <= L - 4 && p >= 0 && p <= n + 1) {
    double Si = sv;
    double Sim1 = Si - d1m, Sip1 = Si + d1p;
    double al = 0.5 * (Sim1 + Si) + kSixth * (sm[QDA][t - 1][lane] - da);
    double ar = 0.5 * (Si + Sip1) + kSixth * (da - sm[QDA][t + 1][lane]);
    limit(lim, Si, da, d1m, d1p, d1mm, d1pp, al, ar);
    el = al;
    er = ar;
    e6 = 6. * Si - 3. * (ar + al);
  }
  sm[QL][t][lane] = el;
  sm[QR][t][lane] = er;
  sm[Q6][t][lane] = e6;
  __syncthreads();
  // flux through face p (between positions p and p+1), faces 0 .. n
  double f = 0.0;
  if (lane_ok && t >= 3 && t <= L - 5 && p >= 0 && p <= n)
    f = face(p, mv, sm[QM][t + 1][lane], el, er, e6, sm[QL][t + 1][lane], sm[QR][t + 1][lane], sm[Q6][t + 1][lane]);
  sm[QF][t][lane] = f;
  __syncthreads();
  // update of cells 1 .. n
  if (lane_ok && t >= 4 && t <= L - 5 && p >= 1 && p <= n) upd(p, sv, mv, sm[QF][t - 1][lane], f);
}

}  // namespace ppm
}  // namespace mom5
