// FP64 MDFL Sweby and barotropic kernel bodies, shared by the one-domain
// kernels (k_fp64.cu) and the batched kernels (k_batch64.cu).  Included only by
// translation units built with --fmad=false: every product and sum is rounded
// on its own, in the reference's order (see k_fp64.cu).
#pragma once
#include <math.h>

#include "internal.h"
#include "fp64_div.cuh"

namespace mom5 {
namespace fp64 {

#define DEVI __device__ __forceinline__

DEVI long I2(const Geo& g, int i, int j) { return (long)j * g.nxd + i; }
DEVI long I3(const Geo& g, int i, int j, int k) { return (long)k * g.n2 + (long)j * g.nxd + i; }
// index into a (ni+4)(nj+4)nk halo-2 array; i, j in data-domain coordinates (isc = 1)
DEVI long IM(const Geo& g, int i, int j, int k) { return ((long)k * (g.nj + 4) + (j + 1)) * (g.ni + 4) + (i + 1); }

constexpr double kOneSixth = 1.0 / 6.0;  // ocean_parameters.F90:92

// max(0, x) and min(a, b) on the integer pipe (ordered-integer comparison of
// the bit patterns; equal to the FP comparison for all non-NaN operands).  The
// bit patterns are taken through bits_of so that the compiler keeps the tests
// integer.
DEVI long long ordbits(double x) {
  long long b = bits_of(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
DEVI double dmin(double a, double b) { return ordbits(a) <= ordbits(b) ? a : b; }
DEVI double dmax0(double x) { return bits_of(x) > 0 ? x : 0.0; }
DEVI bool dpos(double x) {  // x > 0 (false for NaN)
  long long b = bits_of(x);
  return b > 0 && b <= 0x7ff0000000000000LL;
}

// Exact shortcuts that keep work off the FP64 pipe (GB300 issues FP64 at
// 1/64 of the FP32 rate; integer operations are cheap).  Each returns the
// bit pattern the FP64 operation would produce.
DEVI bool is_one(double m) { return bits_of(m) == 0x3ff0000000000000LL; }
DEVI bool is_zero(double m) { return (bits_of(m) << 1) == 0; }
// x*m for a mask value m: 1 -> x (x*1 == x), +-0 -> 0.0 as the callers' selects do
DEVI double mask_mul(double x, double m) {
  if (is_one(m)) return x;
  return x * m;
}
// x + 0.0: the same value except that -0 becomes +0
DEVI double plus_zero(double x) { return bits_of(x) == (long long)0x8000000000000000ULL ? 0.0 : x; }
// -x (the sign bit flipped) when flip, on the integer pipe
DEVI double neg_if(double x, bool flip) {
  return double_of(bits_of(x) ^ (flip ? (long long)0x8000000000000000ULL : 0LL));
}
// 0.5*x: for a normal x whose exponent field is at least 2 the product is the
// exponent lowered by one; +-0 is unchanged.  Subnormals, the smallest normals,
// Inf and NaN take the multiply (decided per warp, so the common case issues no
// FP64 instruction).
DEVI double half_exact(double x) {
  long long b = bits_of(x);
  unsigned e = (unsigned)((unsigned long long)b >> 52) & 0x7ffu;
  bool normal = e - 2u < 0x7fdu;  // 2 <= e <= 0x7fe
  bool fast = normal || (b << 1) == 0;
  long long r = normal ? b - (1LL << 52) : b;
  if (__all_sync(__activemask(), fast)) return double_of(r);
  return fast ? double_of(r) : 0.5 * x;
}

// Arithmetic policy of the MDFL bodies: the FP64 instructions.  (Integer-pipe
// emulation of the FP64 additions and products was measured on C2 and was
// 13-90% slower than the FP64 pipe at this occupancy, so none is used.)
struct HwArith {
  static DEVI double add(double a, double b) { return a + b; }
  static DEVI double sub(double a, double b) { return a - b; }
  static DEVI double mul(double a, double b) { return a * b; }
};
using MdflFaceArith = HwArith;
using MdflUpdArith = HwArith;

// Sweby limiter psi (ocean_tracer_advect.F90:3868-3878).  With the limiter on
// the reference forms psi*(1-1) + max(...)*1, with it off psi*1 + max(...)*0;
// for finite psi both reduce to the selected term exactly.
template <bool SWEBY, class Ar>
DEVI double limiter(double theta, double d0, double d1, double c) {
  double lin = Ar::add(d0, Ar::mul(d1, theta));
  if (!SWEBY) return lin;
  double a = dmin(1.0, lin);
  return dmax0(dmin(a, Ar::mul(c, theta)));
}

// Flux of one face given the upwind-side data.  Reference form
// 0.5*((mf+|mf|)*(Tup + psiP*Rj) + (mf-|mf|)*(Tdn - psiM*Rj)): for mf > 0 the
// second product is an exact zero and 0.5*(2mf*X) == mf*X exactly; for mf < 0
// the first is.  Both signs share one division and one limiter evaluation (the
// operands are selected first), so a warp whose faces carry both signs runs
// the division once, not once per branch; Tdn - p is computed as Tdn + (-p),
// which IEEE defines to be the same operation, with -p formed on the integer
// pipe.
template <bool SWEBY, class Ar>
DEVI double face_flux(double mf, double Rjm, double Rj, double Rjp, double Tp, double Tm, double d0, double d1,
                      double c) {
  long long b = bits_of(mf);
  bool pos = b > 0;                                                 // mf > 0
  bool neg = b < 0 && b != (long long)0x8000000000000000ULL;        // mf < 0
  double theta = div_seeded(pos ? Rjm : Rjp, add_1em30(Rj));
  double psi = limiter<SWEBY, Ar>(theta, d0, d1, c);
  double p = Ar::mul(psi, Rj);
  double r = Ar::mul(mf, Ar::add(pos ? Tp : Tm, neg_if(p, !pos)));
  return (pos || neg) ? r : 0.0;
}

// Per-tracer running values live in shared memory, [tracer][thread], so the
// tracer loops stay rolled (one copy of the loop body in the instruction cache).
constexpr int kMdflThreads = 128;

// Face terms of the bottom face of level k of one column: w(k+1), the mass flux
// and the limiter coefficients of the Courant number (ocean_tracer_advect.F90:
// 3860-3866), evaluated the same way wherever a level's face is formed.
struct ZFace {
  double wk, massflux, d0, d1, c, rdz;
};
DEVI ZFace z_face(const MdflArgs& a, const Geo& g, int i, int j, int k, double dat) {
  ZFace f;
  f.wk = a.w[I3(g, i, j, k + 1)];
  f.rdz = a.rdz[I3(g, i, j, k)];
  f.massflux = dat * f.wk;
  double cfl = fabs(div_seeded(f.wk * a.dtime, f.rdz));
  f.d0 = (2.0 - cfl) * (1.0 - cfl) * kOneSixth;
  f.d1 = (1.0 - cfl * cfl) * kOneSixth;
  f.c = div_seeded(1.0 - cfl, add_1em30(cfl));
  return f;
}
// R(m) = (m(m) && m(m1)) ? T(m) - T(m1) : 0 with m1 = min(m+1, nk-1): the masked
// vertical difference that the column march forms once per level
template <class Ar>
DEVI double z_rdiff(const MdflArgs& a, const Geo& g, const double* T, int i, int j, int m) {
  const int m1 = m + 1 < g.nk ? m + 1 : g.nk - 1;
  return (a.mask2[IM(g, i, j, m)] && a.mask2[IM(g, i, j, m1)]) ? Ar::sub(T[I3(g, i, j, m)], T[I3(g, i, j, m1)])
                                                                 : 0.0;
}

// z pass: one thread per column, march down levels k0..k1-1 (SEG; else the whole
// column).  A segment that starts below the surface first forms what the march
// from the surface would carry into level k0 -- the flux through its top face
// (the bottom face of level k0-1) and R(k0-1), R(k0) -- with the same
// operations, so every segment length gives the same bits.
template <bool ALL, bool SWEBY, int MAXN, class Ar = MdflFaceArith, class Au = MdflUpdArith, bool SEG = false>
DEVI void mdfl_z_body(MdflArgs a, int bx, int by, int k0 = 0, int k1 = -1) {
  // ftp: flux through the top face; Rp, Rc: the masked differences R(k-1), R(k),
  // R(k) = (m(k) && m(k1)) ? T(k) - T(k1) : 0 with k1 = min(k+1, nk-1).  The
  // reference's Rjp at level k is R(k-1) (+0 at k = 0) and its Rjm is R(k+1), so
  // each difference is formed once and carried down the column.
  __shared__ double ftp[MAXN][kMdflThreads], Rp[MAXN][kMdflThreads], Rc[MAXN][kMdflThreads];
  const Geo& g = a.g;
  const int t = threadIdx.x;
  int i = bx * blockDim.x + t + 1;
  int j = by + 1;
  if (i > g.ni) return;
  if (!SEG) k0 = 0, k1 = g.nk;  // whole columns: the segment code is not compiled in
  if (k1 < 0 || k1 > g.nk) k1 = g.nk;
  double wk_top = 0.0;  // w at the top face of level k0 (0 at the surface)
  if (!SEG || k0 == 0) {
    const int k1s = g.nk > 1 ? 1 : 0;
    const bool m0 = a.mask2[IM(g, i, j, 0)], m1 = a.mask2[IM(g, i, j, k1s)];
#pragma unroll 1
    for (int n = 0; n < a.ntr; ++n) {
      const double* T = a.T + n * a.tstride;
      ftp[n][t] = 0.0;
      Rp[n][t] = 0.0;
      Rc[n][t] = (m0 && m1) ? Ar::sub(T[I3(g, i, j, 0)], T[I3(g, i, j, k1s)]) : 0.0;
    }
  } else {
    // the bottom face of level kq = k0-1, as the march forms it there
    const int kq = k0 - 1;
    const ZFace f = z_face(a, g, i, j, kq, a.dat[I2(g, i, j)]);
    const bool fm = a.mask2[IM(g, i, j, k0)] && a.mask2[IM(g, i, j, kq)];
#pragma unroll 1
    for (int n = 0; n < a.ntr; ++n) {
      const double* T = a.T + n * a.tstride;
      const double Rjp = kq > 0 ? z_rdiff<Ar>(a, g, T, i, j, kq - 1) : 0.0;
      const double Rj = z_rdiff<Ar>(a, g, T, i, j, kq);
      const double Rjm = z_rdiff<Ar>(a, g, T, i, j, k0);
      ftp[n][t] = fm ? face_flux<SWEBY, Ar>(f.massflux, Rjm, Rj, Rjp, T[I3(g, i, j, k0)], T[I3(g, i, j, kq)], f.d0,
                                             f.d1, f.c)
                     : 0.0;
      Rp[n][t] = Rj;
      Rc[n][t] = Rjm;
    }
    wk_top = f.wk;
  }
  double wkm1 = wk_top;
  const double dat = a.dat[I2(g, i, j)];
  const double datr = a.datr[I2(g, i, j)];
  for (int k = k0; k < k1; ++k) {
    int kp1 = k + 1 < g.nk ? k + 1 : g.nk - 1;
    int kp2 = k + 2 < g.nk ? k + 2 : g.nk - 1;
    bool mk = a.mask2[IM(g, i, j, k)];
    bool mkp1 = a.mask2[IM(g, i, j, kp1)], mkp2 = a.mask2[IM(g, i, j, kp2)];
    // the face terms as z_face forms them
    double wk = a.w[I3(g, i, j, k + 1)];
    double rdz = a.rdz[I3(g, i, j, k)];
    double massflux = dat * wk;
    double cfl = fabs(div_seeded(wk * a.dtime, rdz));
    double d0 = (2.0 - cfl) * (1.0 - cfl) * kOneSixth;
    double d1 = (1.0 - cfl * cfl) * kOneSixth;
    double c = div_seeded(1.0 - cfl, add_1em30(cfl));
    double dtr = ALL ? 0.0 : div_seeded(a.dtime, rdz);
    double wdiff = wkm1 - wk;
    bool fm = mkp1 && mk;
    long p = I3(g, i, j, k);
#pragma unroll 1
    for (int n = 0; n < a.ntr; ++n) {
      const double* T = a.T + n * a.tstride;
      double Tk = T[p];
      double Tkp1 = T[I3(g, i, j, kp1)], Tkp2 = T[I3(g, i, j, kp2)];
      double Rjp = Rp[n][t];
      double Rj = Rc[n][t];
      double Rjm = (mkp1 && mkp2) ? Ar::sub(Tkp1, Tkp2) : 0.0;
      Rp[n][t] = Rj;
      Rc[n][t] = Rjm;
      double fbt = fm ? face_flux<SWEBY, Ar>(massflux, Rjm, Rj, Rjp, Tkp1, Tk, d0, d1, c) : 0.0;
      double div = Au::add(Au::mul(datr, Au::sub(fbt, ftp[n][t])), Au::mul(Tk, wdiff));
      double tm;
      if (!ALL) {
        tm = Au::add(Tk, Au::mul(dtr, div));
      } else {
        tm = Au::add(Tk, div_seeded(Au::mul(div, a.dtime), rdz));
      }
      a.tz[n * g.n3 + p] = tm;
      ftp[n][t] = fbt;
    }
    wkm1 = wk;
  }
}

// tracer_mdfl after the x halo update (XUPDATE): compute rows only.
DEVI double tm_xhalo(const Geo& g, const double* a, int i, int j, int k) {
  if (i < 1) {
    if (!g.cx) return 0.0;
    i += g.ni;
  } else if (i > g.ni) {
    if (!g.cx) return 0.0;
    i -= g.ni;
  }
  return a[I3(g, i, j, k)];
}
DEVI double tm_yhalo(const Geo& g, const double* a, int i, int j, int k) {
  if (j < 1) {
    if (!g.cy) return 0.0;
    j += g.nj;
  } else if (j > g.nj) {
    if (!g.cy) return 0.0;
    j -= g.nj;
  }
  return a[I3(g, i, j, k)];
}

// tracer_mdfl of tracer n at a halo column or row: from the strip a
// neighbouring subdomain's exchange filled (decomposed domains), else by the
// single-PE rule above.
DEVI double tz_halo(const MdflArgs& a, int n, int i, int j, int k) {
  const Geo& g = a.g;
  if ((i < 1 || i > g.ni) && (a.nbr & (i < 1 ? 1 : 2))) {
    const int s = i < 1 ? i + 1 : i - g.ni + 1;  // -1, 0, ni+1, ni+2 -> 0..3
    return a.hz[(((long)n * g.nk + k) * g.nj + (j - 1)) * 4 + s];
  }
  return tm_xhalo(g, a.tz + n * g.n3, i, j, k);
}
DEVI double tx_halo(const MdflArgs& a, int n, int i, int j, int k) {
  const Geo& g = a.g;
  if ((j < 1 || j > g.nj) && (a.nbr & (j < 1 ? 4 : 8))) {
    const int s = j < 1 ? j + 1 : j - g.nj + 1;
    return a.hx[(((long)n * g.nk + k) * 4 + s) * g.ni + (i - 1)];
  }
  return tm_yhalo(g, a.tx + n * g.n3, i, j, k);
}

constexpr int kTX = 128;

// x-face i of row (j,k): fluxes of every tracer into sm[n][slot].  Rs[n][r-1..r+1]
// hold the masked differences R of faces i-1, i, i+1 (the reference's Rjm, Rj,
// Rjp), each formed once per block.
template <bool SWEBY, int MAXN, class Ar>
DEVI void x_face(const MdflArgs& a, int i, int j, int k, double (*sm)[kTX + 1], int slot,
                 const double (*Rs)[kTX + 3], int r) {
  const Geo& g = a.g;
  bool m1 = a.mask2[IM(g, i, j, k)], m2 = a.mask2[IM(g, i + 1, j, k)];
  double u = a.uh[I3(g, i, j, k)];
  double massflux = a.dyte[I2(g, i, j)] * u;
  double cfl = fabs(div_seeded(u * a.dtime * 2.0, (a.rdz[I3(g, i, j, k)] + a.rdz[I3(g, i + 1, j, k)]) * a.dxte[I2(g, i, j)]));
  double d0 = (2.0 - cfl) * (1.0 - cfl) * kOneSixth;
  double d1 = (1.0 - cfl * cfl) * kOneSixth;
  double c = div_seeded(1.0 - cfl, add_1em30(cfl));
  bool fm = m1 && m2;
#pragma unroll 1
  for (int n = 0; n < a.ntr; ++n) {
    double tB = tz_halo(a, n, i, j, k), tC = tz_halo(a, n, i + 1, j, k);
    sm[n][slot] = fm ? face_flux<SWEBY, Ar>(massflux, Rs[n][r - 1], Rs[n][r], Rs[n][r + 1], tB, tC, d0, d1, c) : 0.0;
  }
}

template <bool ALL, bool SWEBY, int MAXN, class Ar = MdflFaceArith, class Au = MdflUpdArith>
DEVI void mdfl_x_body(MdflArgs a, int bx, int by, int bz) {
  __shared__ double sm[MAXN][kTX + 1], Rs[MAXN][kTX + 3];
  const Geo& g = a.g;
  int i0 = bx * kTX + 1;
  int j = by + 1;
  int k = bz;
  int t = threadIdx.x;
  int i = i0 + t;
  // R(f) = (m(f) && m(f+1)) ? tz(f+1) - tz(f) : 0 for faces f = i0-2 .. i0+128 (slot f-i0+2)
  for (int sl = t; sl < kTX + 3; sl += kTX) {
    int f = i0 - 2 + sl;
    if (f > g.ni + 1) continue;
    bool ma = a.mask2[IM(g, f, j, k)], mb = a.mask2[IM(g, f + 1, j, k)];
#pragma unroll 1
    for (int n = 0; n < a.ntr; ++n) {
      Rs[n][sl] = (mb && ma) ? Ar::sub(tz_halo(a, n, f + 1, j, k), tz_halo(a, n, f, j, k)) : 0.0;
    }
  }
  __syncthreads();
  if (i <= g.ni) x_face<SWEBY, MAXN, Ar>(a, i, j, k, sm, t + 1, Rs, t + 2);
  if (t == 0) x_face<SWEBY, MAXN, Ar>(a, i0 - 1, j, k, sm, 0, Rs, 1);
  __syncthreads();
  if (i > g.ni) return;
  bool mk = a.mask2[IM(g, i, j, k)];
  double datr = a.datr[I2(g, i, j)];
  double rdz = a.rdz[I3(g, i, j, k)];
  double divx = a.dyte[I2(g, i, j)] * a.uh[I3(g, i, j, k)] - a.dyte[I2(g, i - 1, j)] * a.uh[I3(g, i - 1, j, k)];
  // dtime*tmask*datr/rho_dzt (:3960-3961); tmask_mdfl*datr (:4277)
  double coef = ALL ? 0.0 : (mk ? div_seeded(a.dtime * datr, rdz) : 0.0);
  long p = I3(g, i, j, k);
#pragma unroll 1
  for (int n = 0; n < a.ntr; ++n) {
    double Tk = a.T[n * a.tstride + p];
    double tm = a.tz[n * g.n3 + p];
    double s = Au::add(Au::sub(sm[n][t], sm[n][t + 1]), Au::mul(Tk, divx));
    if (!ALL) {
      tm = Au::add(tm, Au::mul(coef, s));
    } else {
      double w1 = mk ? Au::mul(datr, s) : 0.0;
      tm = Au::add(tm, div_seeded(Au::mul(w1, a.dtime), rdz));
    }
    a.tx[n * g.n3 + p] = tm;
  }
}

// y pass + closing divergence correction + tendency: one thread per (i,k) and a
// strip of TJ rows, marching north; th_tendency += result.  Ra, Rb carry the
// masked differences R of faces j-1 and j (R(f) = (m(f) && m(f+1)) ?
// tx(f+1) - tx(f) : 0, the reference's Rjm and Rj of face j); face j forms only
// R(j+1), its Rjp.
//
// Tracer-independent terms of face j (between rows j and j+1).
struct YFace {
  bool m2, m3, fm;
  double massflux, d0, d1, c;
};
DEVI YFace y_geom(const MdflArgs& a, int i, int j, int k, bool& m0, bool& m1) {
  const Geo& g = a.g;
  YFace f;
  m0 = a.mask2[IM(g, i, j - 1, k)];
  m1 = a.mask2[IM(g, i, j, k)];
  f.m2 = a.mask2[IM(g, i, j + 1, k)];
  f.m3 = a.mask2[IM(g, i, j + 2, k)];
  double v = a.vh[I3(g, i, j, k)];
  f.massflux = a.dxtn[I2(g, i, j)] * v;
  double cfl = fabs(div_seeded(v * a.dtime * 2.0, (a.rdz[I3(g, i, j, k)] + a.rdz[I3(g, i, j + 1, k)]) * a.dytn[I2(g, i, j)]));
  f.d0 = (2.0 - cfl) * (1.0 - cfl) * kOneSixth;
  f.d1 = (1.0 - cfl * cfl) * kOneSixth;
  f.c = div_seeded(1.0 - cfl, add_1em30(cfl));
  f.fm = m1 && f.m2;
  return f;
}
// Flux of tracer n through face j, carrying Ra/Rb; tB returns tx at row j.
template <bool SWEBY, class Ar>
DEVI double y_flux(const MdflArgs& a, const YFace& f, int i, int j, int k, int n, int t, double (*Ra)[kMdflThreads],
                   double (*Rb)[kMdflThreads], double& tB) {
  tB = tx_halo(a, n, i, j, k);
  double tC = tx_halo(a, n, i, j + 1, k), tD = tx_halo(a, n, i, j + 2, k);
  double Rjm = Ra[n][t], Rj = Rb[n][t];
  double Rjp = (f.m3 && f.m2) ? Ar::sub(tD, tC) : 0.0;
  Ra[n][t] = Rj;
  Rb[n][t] = Rjp;
  return f.fm ? face_flux<SWEBY, Ar>(f.massflux, Rjm, Rj, Rjp, tB, tC, f.d0, f.d1, f.c) : 0.0;
}

// Each tracer's face flux is formed and used in the same iteration (the
// flux of the row's north face in a register, the south face's from the
// previous row in shared memory), so the per-tracer shared state is fprev, Ra
// and Rb only.
template <bool ALL, bool SWEBY, int MAXN, class Ar = MdflFaceArith, class Au = MdflUpdArith>
DEVI void mdfl_y_body(MdflArgs a, int TJ, int bx, int by, int bz) {
  __shared__ double fprev[MAXN][kMdflThreads];
  __shared__ double Ra[MAXN][kMdflThreads], Rb[MAXN][kMdflThreads];
  const Geo& g = a.g;
  const int t = threadIdx.x;
  int i = bx * blockDim.x + t + 1;
  int j0 = by * TJ + 1;
  int k = bz;
  if (i > g.ni) return;
  int j1 = j0 + TJ - 1;
  if (j1 > g.nj) j1 = g.nj;
  double rdt_h, rdt_l;  // two-term reciprocal of dtime
  recip_pair(a.dtime, rdt_h, rdt_l);
  {
    // the face below the strip: its flux and the two carried differences
    bool m0, m1;
    const YFace f = y_geom(a, i, j0 - 1, k, m0, m1);
#pragma unroll 1
    for (int n = 0; n < a.ntr; ++n) {
      double tA = tx_halo(a, n, i, j0 - 2, k), tB = tx_halo(a, n, i, j0 - 1, k);
      double tC = tx_halo(a, n, i, j0, k);
      Ra[n][t] = (m1 && m0) ? Ar::sub(tB, tA) : 0.0;
      Rb[n][t] = (f.m2 && m1) ? Ar::sub(tC, tB) : 0.0;
      double tb;
      fprev[n][t] = y_flux<SWEBY, Ar>(a, f, i, j0 - 1, k, n, t, Ra, Rb, tb);
    }
  }
  for (int j = j0; j <= j1; ++j) {
    bool m0, m1;
    const YFace f = y_geom(a, i, j, k, m0, m1);
    long p = I3(g, i, j, k);
    bool mk = a.mask2[IM(g, i, j, k)];
    double datr = a.datr[I2(g, i, j)];
    double rdz = a.rdz[p];
    double wk = a.w[I3(g, i, j, k + 1)];
    double wkm1j = k > 0 ? a.w[I3(g, i, j, k)] : 0.0;  // bottom face of level k-1; 0 at the surface
    double corr = (wk - wkm1j) + datr * (a.dyte[I2(g, i - 1, j)] * a.uh[I3(g, i - 1, j, k)] -
                                         a.dyte[I2(g, i, j)] * a.uh[p]);
    double coef = ALL ? 0.0 : (mk ? div_seeded(a.dtime * datr, rdz) : 0.0);
    double rr_h, rr_l;  // two-term reciprocal of rho_dzt, shared by every tracer's divisions
    recip_pair(rdz, rr_h, rr_l);
#pragma unroll 1
    for (int n = 0; n < a.ntr; ++n) {
      double tm;  // tracer_mdfl after the x pass at (i, j, k)
      double fc = y_flux<SWEBY, Ar>(a, f, i, j, k, n, t, Ra, Rb, tm);
      double Tk = a.T[n * a.tstride + p];
      double fp = fprev[n][t];
      double out;
      if (!ALL) {
        tm = Au::add(tm, Au::mul(coef, Au::sub(fp, fc)));
        tm = Au::add(tm, Au::mul(div_pair(Au::mul(a.dtime, Tk), rdz, rr_h, rr_l), corr));
      } else {
        double w1 = Au::add(mk ? Au::mul(datr, Au::sub(fp, fc)) : 0.0, Au::mul(Tk, corr));
        tm = Au::add(tm, div_pair(Au::mul(w1, a.dtime), rdz, rr_h, rr_l));
      }
      out = mk ? div_pair(Au::mul(rdz, Au::sub(tm, Tk)), a.dtime, rdt_h, rdt_l) : 0.0;
      double* th = a.th + n * g.n3;
      th[p] = a.th_fresh ? plus_zero(out) : Au::add(th[p], out);  // +0 + out == plus_zero(out)
      fprev[n][t] = fc;
    }
  }
}



// DIV_UD at (i,j) (ocean_operators.F90:507-608), halo_in = halo_out = 1.
DEVI double div_ud(const BtArgs& a, const double* u, const double* v, int i, int j) {
  const Geo& g = a.g;
  if (i < 1 || j < 1) return 0.0;
  if (a.cgrid) {
    double uhim = u[I2(g, i - 1, j)] * a.dat[I2(g, i - 1, j)] * a.dxter[I2(g, i - 1, j)];
    double vhjm = v[I2(g, i, j - 1)] * a.dat[I2(g, i, j - 1)] * a.dytnr[I2(g, i, j - 1)];
    double uh = u[I2(g, i, j)] * a.dat[I2(g, i, j)] * a.dxter[I2(g, i, j)];
    double vh = v[I2(g, i, j)] * a.dat[I2(g, i, j)] * a.dytnr[I2(g, i, j)];
    return ((uh - uhim) + (vh - vhjm)) * a.datr[I2(g, i, j)];
  }
  double uh = u[I2(g, i, j)] * a.dyu[I2(g, i, j)];
  double vh = v[I2(g, i, j)] * a.dxu[I2(g, i, j)];
  double uhjm = u[I2(g, i, j - 1)] * a.dyu[I2(g, i, j - 1)];
  double vhjm = v[I2(g, i, j - 1)] * a.dxu[I2(g, i, j - 1)];
  double uhim = u[I2(g, i - 1, j)] * a.dyu[I2(g, i - 1, j)];
  double vhim = v[I2(g, i - 1, j)] * a.dxu[I2(g, i - 1, j)];
  double uhimjm = u[I2(g, i - 1, j - 1)] * a.dyu[I2(g, i - 1, j - 1)];
  double vhimjm = v[I2(g, i - 1, j - 1)] * a.dxu[I2(g, i - 1, j - 1)];
  double uh_bay = 0.5 * (uh + uhjm);
  double vh_bax = 0.5 * (vh + vhim);
  double uhim_bay = 0.5 * (uhim + uhimjm);
  double vhjm_bax = 0.5 * (vhjm + vhimjm);
  return ((uh_bay - uhim_bay) + (vh_bax - vhjm_bax)) * a.datr[I2(g, i, j)];
}

// B-grid DIV_UD from the stored products uh = u*dyu, vh = v*dxu: the same
// operations as div_ud on the same values, without recomputing the products.
DEVI double div_ud_bh(const BtArgs& a, const double* uh, const double* vh, int i, int j) {
  const Geo& g = a.g;
  if (i < 1 || j < 1) return 0.0;
  long q = I2(g, i, j), qw = q - 1, qs = q - g.nxd, qsw = qs - 1;
  double uh_bay = half_exact(uh[q] + uh[qs]);
  double vh_bax = half_exact(vh[q] + vh[qw]);
  double uhim_bay = half_exact(uh[qw] + uh[qsw]);
  double vhjm_bax = half_exact(vh[qs] + vh[qsw]);
  return ((uh_bay - uhim_bay) + (vh_bax - vhjm_bax)) * a.datr[q];
}

// image of a halo point under the single-PE full halo update; returns false
// when the point is left untouched (non-cyclic wall, or a corner of a domain
// cyclic in one direction only).
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

DEVI void bt_init_body(BtArgs a, const double* eta_bar_tau, const double* eta_tau, const double* ud_tau,
                          const double* vd_tau, const double* pme, const double* river, const double* source,
                          const double* eta_smooth, int initsum_with_bar, int bx, int by) {
  long q = bx * (long)blockDim.x + threadIdx.x;
  if (q >= a.g.n2) return;
  a.eta_bar[q] = initsum_with_bar ? eta_bar_tau[q] : eta_tau[q];
  a.udrho_u[q] = 0.0;
  a.udrho_v[q] = 0.0;
  // fstau = mod(1,2)+1 = 2 -> plane 1
  a.eta_bt[a.g.n2 + q] = eta_bar_tau[q];
  a.ubt[a.g.n2 + q] = ud_tau[q];
  a.vbt[a.g.n2 + q] = vd_tau[q];
  if (!a.cgrid) {
    a.uhb[a.g.n2 + q] = ud_tau[q] * a.dyu[q];
    a.vhb[a.g.n2 + q] = vd_tau[q] * a.dxu[q];
  }
  a.steady[q] = a.tmask1[q] * (pme[q] + river[q] + source[q] - eta_smooth[q]);
}

// C-grid: initial Adams-Bashforth Coriolis history (:3707-3730)
DEVI void bt_cgrid_init_body(BtArgs a, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x + 1;
  int j = by + 1;
  if (i > g.ni) return;
  const double abm0 = 23.0 / 12.0, abm1 = -16.0 / 12.0, abm2 = 5.0 / 12.0;
  const int itime = 1;
  int m2 = (itime + 0) % 3, m1 = (itime + 1) % 3, m0 = (itime + 2) % 3;
  const double* u = a.ubt + g.n2;
  const double* v = a.vbt + g.n2;
  long n2 = g.n2;
  long q = I2(g, i, j);
  double c0 = 0.25 * (a.f[q] * (v[q] + v[I2(g, i + 1, j)]) + a.f[I2(g, i, j - 1)] * (v[I2(g, i, j - 1)] + v[I2(g, i + 1, j - 1)]));
  a.cf[(m0 * 2 + 0) * n2 + q] = c0;
  a.cf[(m1 * 2 + 0) * n2 + q] = c0;
  a.cf[(m2 * 2 + 0) * n2 + q] = c0;
  a.ca[q] = abm0 * c0 + abm1 * c0 + abm2 * c0;
  double c1 = -0.25 * (a.f[q] * (u[q] + u[I2(g, i, j + 1)]) + a.f[I2(g, i - 1, j)] * (u[I2(g, i - 1, j)] + u[I2(g, i - 1, j + 1)]));
  a.cf[(m0 * 2 + 1) * n2 + q] = c1;
  a.cf[(m1 * 2 + 1) * n2 + q] = c1;
  a.cf[(m2 * 2 + 1) * n2 + q] = c1;
  a.ca[n2 + q] = abm0 * c1 + abm1 * c1 + abm2 * c1;
}

// predictor + ps (both grids).  With reuse the divergence of the transports at
// level so is the one the previous subcycle's corrector formed from the same
// arrays (its level sn), stored in dvs: the same values, read instead of formed.
DEVI void bt_pred_body(BtArgs a, int so, int sn, int reuse, int bx, int by) {
  const Geo& g = a.g;
  int i0 = bx * blockDim.x + threadIdx.x;
  int j0 = by;
  if (i0 > g.ni + 1) return;
  int i = i0, j = j0;
  // B-grid legacy halos: eta(fstaup1) is halo-updated right after the predictor,
  // so a halo point takes the value computed at its periodic image.
  if (!a.cgrid) {
    if (!halo_image(g, i, j)) {
      i = i0;
      j = j0;
    }
  }
  const double* eo = a.eta_bt + so * g.n2;
  long q = I2(g, i, j);
  double en;
  if (dpos(a.gamma)) {
    double dv = reuse ? a.dvs[q]
                      : (a.cgrid ? div_ud(a, a.ubt + so * g.n2, a.vbt + so * g.n2, i, j)
                                 : div_ud_bh(a, a.uhb + so * g.n2, a.vhb + so * g.n2, i, j));
    double tm = a.tmask1[q];
    double tmp = is_zero(tm) ? 0.0 : mask_mul(-dv, tm);
    en = eo[q] + a.dtbt_gamma_rho0r * (tmp + a.steady[q]);
  } else {
    en = eo[q];
  }
  long q0 = I2(g, i0, j0);
  a.eta_bt[sn * g.n2 + q0] = en;
  a.ps[q0] = a.rho_g[q0] * en + a.patm[q0];
}

// momentum update, B grid (:3466-3485)
DEVI void bt_mom_b_body(BtArgs a, int so, int sn, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x;
  int j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double gx = 0.0, gy = 0.0;
  if (i <= g.ni && j <= g.nj) {
    const double* ps = a.ps;
    double um = a.umask1[q];
    if (!is_zero(um)) {
      double p00 = ps[q], p10 = ps[I2(g, i + 1, j)], p01 = ps[I2(g, i, j + 1)], p11 = ps[I2(g, i + 1, j + 1)];
      double p_fay = half_exact(p00 + p01);
      double p_fax = half_exact(p00 + p10);
      double pip_fay = half_exact(p10 + p11);
      double pjp_fax = half_exact(p01 + p11);
      gx = mask_mul((pip_fay - p_fay) * a.dxur[q], um);
      gy = mask_mul((pjp_fax - p_fax) * a.dyur[q], um);
    }
  }
  double pf1 = -a.thicku[q] * gx;
  double pf2 = -a.thicku[q] * gy;
  double uo = a.ubt[so * g.n2 + q], vo = a.vbt[so * g.n2 + q];
  double hf = half_exact(a.f[q]);  // 0.5*f; -0.5*f is its negation
  double t1 = uo + a.dtbt * plus_zero(hf * vo + pf1 + a.forcing_u[q]);
  double t2 = vo + a.dtbt * plus_zero((-hf) * uo + pf2 + a.forcing_v[q]);
  double un = a.cori2[q] * (t1 + a.cori1[q] * t2);
  double vn = a.cori2[q] * (t2 - a.cori1[q] * t1);
  a.ubt[sn * g.n2 + q] = un;
  a.vbt[sn * g.n2 + q] = vn;
  a.uhb[sn * g.n2 + q] = un * a.dyu[q];
  a.vhb[sn * g.n2 + q] = vn * a.dxu[q];
}

// C grid: Coriolis (compute domain) + gradient + momentum (:3780-3830)
DEVI void bt_mom_c_body(BtArgs a, int so, int sn, int itime, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x;
  int j = by;
  if (i > g.ni + 1) return;
  long n2 = g.n2;
  long q = I2(g, i, j);
  const double abm0 = 23.0 / 12.0, abm1 = -16.0 / 12.0, abm2 = 5.0 / 12.0;
  int m2 = (itime + 0) % 3, m1 = (itime + 1) % 3, m0 = (itime + 2) % 3;
  double ca0 = 0.0, ca1 = 0.0;
  if (i >= 1 && i <= g.ni && j >= 1 && j <= g.nj) {
    const double* u = a.ubt + so * n2;
    const double* v = a.vbt + so * n2;
    double c0 = 0.25 * (a.f[q] * (v[q] + v[I2(g, i + 1, j)]) + a.f[I2(g, i, j - 1)] * (v[I2(g, i, j - 1)] + v[I2(g, i + 1, j - 1)]));
    a.cf[(m0 * 2 + 0) * n2 + q] = c0;
    ca0 = abm0 * c0 + abm1 * a.cf[(m1 * 2 + 0) * n2 + q] + abm2 * a.cf[(m2 * 2 + 0) * n2 + q];
    double c1 = -0.25 * (a.f[q] * (u[q] + u[I2(g, i, j + 1)]) + a.f[I2(g, i - 1, j)] * (u[I2(g, i - 1, j)] + u[I2(g, i - 1, j + 1)]));
    a.cf[(m0 * 2 + 1) * n2 + q] = c1;
    ca1 = abm0 * c1 + abm1 * a.cf[(m1 * 2 + 1) * n2 + q] + abm2 * a.cf[(m2 * 2 + 1) * n2 + q];
  }
  double gx = 0.0, gy = 0.0;
  if (i <= g.ni && j <= g.nj) {
    gx = (a.ps[I2(g, i + 1, j)] - a.ps[q]) * a.dxter[q] * a.tmen_e[q];
    gy = (a.ps[I2(g, i, j + 1)] - a.ps[q]) * a.dytnr[q] * a.tmen_n[q];
  }
  double pf1 = -a.thicken_e[q] * gx;
  double pf2 = -a.thicken_n[q] * gy;
  double uo = a.ubt[so * n2 + q], vo = a.vbt[so * n2 + q];
  a.ubt[sn * n2 + q] = uo + a.dtbt * a.tmen_e[q] * (ca0 + pf1 + a.forcing_u[q] + 0.0);
  a.vbt[sn * n2 + q] = vo + a.dtbt * a.tmen_n[q] * (ca1 + pf2 + a.forcing_v[q] + 0.0);
}

// corrector + accumulation
DEVI void bt_corr_body(BtArgs a, int so, int sn, double wgt, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x;
  int j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double dv = a.cgrid ? div_ud(a, a.ubt + sn * g.n2, a.vbt + sn * g.n2, i, j)
                      : div_ud_bh(a, a.uhb + sn * g.n2, a.vhb + sn * g.n2, i, j);
  a.dvs[q] = dv;
  double tm = a.tmask1[q];
  double tmp = is_zero(tm) ? 0.0 : mask_mul(-dv, tm);
  double en = a.eta_bt[so * g.n2 + q] + a.dtbt_rho0r * (tmp + a.steady[q]);
  a.eta_bt[sn * g.n2 + q] = en;
  a.eta_bar[q] = a.eta_bar[q] + en;
  double un = a.ubt[sn * g.n2 + q], vn = a.vbt[sn * g.n2 + q];
  if (a.stepB) {
    a.udrho_u[q] = a.udrho_u[q] + wgt * un;
    a.udrho_v[q] = a.udrho_v[q] + wgt * vn;
  } else {
    a.udrho_u[q] = a.udrho_u[q] + un;
    a.udrho_v[q] = a.udrho_v[q] + vn;
  }
}

// B grid: the corrector of subcycle t and the predictor of subcycle t+1 in one
// pass.  With reuse the predictor of a point reads only the divergence and the
// corrected eta of that point (or, for a halo point in a periodic direction, of
// its image), so the thread of a point forms the next surface pressure from the
// values it has just computed, and the thread of a compute point also forms it
// at the periodic halo points whose image it is.  The predicted eta is not
// stored (the next corrector overwrites it unread), nor is the divergence.  The
// operations are bt_corr_body's and bt_pred_body's, so the bits are theirs.
DEVI void bt_corr_pred_body(BtArgs a, int so, int sn, double wgt, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x;
  int j = by;
  if (i > g.ni + 1) return;
  const long n2 = g.n2;
  long q = I2(g, i, j);
  double dv = div_ud_bh(a, a.uhb + sn * n2, a.vhb + sn * n2, i, j);
  double tm = a.tmask1[q];
  double tmp = is_zero(tm) ? 0.0 : mask_mul(-dv, tm);
  const double st = tmp + a.steady[q];
  double en = a.eta_bt[so * n2 + q] + a.dtbt_rho0r * st;
  a.eta_bt[sn * n2 + q] = en;
  a.eta_bar[q] = a.eta_bar[q] + en;
  double un = a.ubt[sn * n2 + q], vn = a.vbt[sn * n2 + q];
  if (a.stepB) {
    a.udrho_u[q] = a.udrho_u[q] + wgt * un;
    a.udrho_v[q] = a.udrho_v[q] + wgt * vn;
  } else {
    a.udrho_u[q] = a.udrho_u[q] + un;
    a.udrho_v[q] = a.udrho_v[q] + vn;
  }
  // the next subcycle's predictor (bt_pred_body with reuse)
  const double ep = dpos(a.gamma) ? en + a.dtbt_gamma_rho0r * st : en;
  int ii = i, jj = j;
  if (!halo_image(g, ii, jj) || (ii == i && jj == j)) a.ps[q] = a.rho_g[q] * ep + a.patm[q];
  if (i < 1 || i > g.ni || j < 1 || j > g.nj) return;
  int hx[2], nhx = 0, hy[2], nhy = 0;  // periodic halo points whose image this is
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
    a.ps[r] = a.rho_g[r] * ep + a.patm[r];
  }
  for (int v = 0; v < nhy; ++v) {
    const long r = I2(g, i, hy[v]);
    a.ps[r] = a.rho_g[r] * ep + a.patm[r];
  }
  if (g.cx && g.cy)
    for (int u = 0; u < nhx; ++u)
      for (int v = 0; v < nhy; ++v) {
        const long r = I2(g, hx[u], hy[v]);
        a.ps[r] = a.rho_g[r] * ep + a.patm[r];
      }
}

// One whole B-grid subcycle -- predictor, momentum, corrector -- in one launch
// on a tile of TX x TY data-domain points: the predictor's surface pressure on
// the tile and a ring of one (west and south one wider, east and north the
// +1 the pressure gradient reads) and the momentum on the tile and its west and
// south ring are recomputed by each tile that needs them, in shared memory, so
// the corrector of the tile needs nothing from another block in this launch.
// Every point's arithmetic is that of bt_pred_body, bt_mom_b_body and
// bt_corr_body, in the same order, so the results are the same bits.  The
// divergence the predictor reuses comes from plane `so` of a.dvs and the
// corrector writes plane `sn` (two planes: a neighbouring tile may still be
// reading the previous one).  For domains where three launches per subcycle
// cost more than the ring recompute.
template <int TX, int TY>
DEVI void bt_fused_body(BtArgs a, int so, int sn, int reuse, double wgt, int bx, int by) {
  constexpr int PX = TX + 2, PY = TY + 2;  // pressure: points x0-1 .. x0+TX, y0-1 .. y0+TY
  constexpr int MX = TX + 1, MY = TY + 1;  // momentum: points x0-1 .. x0+TX-1, y0-1 .. y0+TY-1
  __shared__ double ps_s[PY * PX];
  __shared__ double un_s[MY * MX], vn_s[MY * MX], uh_s[MY * MX], vh_s[MY * MX];
  const Geo& g = a.g;
  const long n2 = g.n2;
  const int x0 = bx * TX, y0 = by * TY;
  const double* dvs_o = a.dvs + (long)so * n2;
  // ---- predictor and surface pressure (bt_pred_body) ----
  for (int e = threadIdx.x; e < PX * PY; e += blockDim.x) {
    const int i0 = x0 - 1 + e % PX, j0 = y0 - 1 + e / PX;
    if (i0 < 0 || i0 > g.ni + 1 || j0 < 0 || j0 > g.nj + 1) continue;
    int i = i0, j = j0;
    if (!halo_image(g, i, j)) {
      i = i0;
      j = j0;
    }
    const double* eo = a.eta_bt + so * n2;
    const long q = I2(g, i, j);
    double en;
    if (dpos(a.gamma)) {
      double dv = reuse ? dvs_o[q] : div_ud_bh(a, a.uhb + so * n2, a.vhb + so * n2, i, j);
      double tm = a.tmask1[q];
      double tmp = is_zero(tm) ? 0.0 : mask_mul(-dv, tm);
      en = eo[q] + a.dtbt_gamma_rho0r * (tmp + a.steady[q]);
    } else {
      en = eo[q];
    }
    const long q0 = I2(g, i0, j0);
    ps_s[e] = a.rho_g[q0] * en + a.patm[q0];
  }
  __syncthreads();
  // ---- momentum (bt_mom_b_body) ----
  for (int e = threadIdx.x; e < MX * MY; e += blockDim.x) {
    const int li = e % MX, lj = e / MX;
    const int i = x0 - 1 + li, j = y0 - 1 + lj;
    if (i < 0 || i > g.ni + 1 || j < 0 || j > g.nj + 1) continue;
    const long q = I2(g, i, j);
    double gx = 0.0, gy = 0.0;
    if (i <= g.ni && j <= g.nj) {
      double um = a.umask1[q];
      if (!is_zero(um)) {
        const int pe = lj * PX + li;  // pressure point (i, j)
        double p00 = ps_s[pe], p10 = ps_s[pe + 1], p01 = ps_s[pe + PX], p11 = ps_s[pe + PX + 1];
        double p_fay = half_exact(p00 + p01);
        double p_fax = half_exact(p00 + p10);
        double pip_fay = half_exact(p10 + p11);
        double pjp_fax = half_exact(p01 + p11);
        gx = mask_mul((pip_fay - p_fay) * a.dxur[q], um);
        gy = mask_mul((pjp_fax - p_fax) * a.dyur[q], um);
      }
    }
    double pf1 = -a.thicku[q] * gx;
    double pf2 = -a.thicku[q] * gy;
    double uo = a.ubt[so * n2 + q], vo = a.vbt[so * n2 + q];
    double hf = half_exact(a.f[q]);
    double t1 = uo + a.dtbt * plus_zero(hf * vo + pf1 + a.forcing_u[q]);
    double t2 = vo + a.dtbt * plus_zero((-hf) * uo + pf2 + a.forcing_v[q]);
    double un = a.cori2[q] * (t1 + a.cori1[q] * t2);
    double vn = a.cori2[q] * (t2 - a.cori1[q] * t1);
    double uh = un * a.dyu[q], vh = vn * a.dxu[q];
    un_s[e] = un;
    vn_s[e] = vn;
    uh_s[e] = uh;
    vh_s[e] = vh;
    if (li >= 1 && lj >= 1) {  // the tile's own points: the state the next subcycle reads
      a.ubt[sn * n2 + q] = un;
      a.vbt[sn * n2 + q] = vn;
      a.uhb[sn * n2 + q] = uh;
      a.vhb[sn * n2 + q] = vh;
    }
  }
  __syncthreads();
  // ---- corrector and accumulation (bt_corr_body) ----
  double* dvs_n = a.dvs + (long)sn * n2;
  for (int e = threadIdx.x; e < TX * TY; e += blockDim.x) {
    const int li = e % TX + 1, lj = e / TX + 1;  // in the momentum arrays
    const int i = x0 - 1 + li, j = y0 - 1 + lj;
    if (i > g.ni + 1 || j > g.nj + 1) continue;
    const long q = I2(g, i, j);
    const int m = lj * MX + li, mw = m - 1, ms = m - MX, msw = ms - 1;
    double dv = 0.0;
    if (i >= 1 && j >= 1) {  // div_ud_bh
      double uh_bay = half_exact(uh_s[m] + uh_s[ms]);
      double vh_bax = half_exact(vh_s[m] + vh_s[mw]);
      double uhim_bay = half_exact(uh_s[mw] + uh_s[msw]);
      double vhjm_bax = half_exact(vh_s[ms] + vh_s[msw]);
      dv = ((uh_bay - uhim_bay) + (vh_bax - vhjm_bax)) * a.datr[q];
    }
    dvs_n[q] = dv;
    double tm = a.tmask1[q];
    double tmp = is_zero(tm) ? 0.0 : mask_mul(-dv, tm);
    double en = a.eta_bt[so * n2 + q] + a.dtbt_rho0r * (tmp + a.steady[q]);
    a.eta_bt[sn * n2 + q] = en;
    a.eta_bar[q] = a.eta_bar[q] + en;
    double un = un_s[m], vn = vn_s[m];
    if (a.stepB) {
      a.udrho_u[q] = a.udrho_u[q] + wgt * un;
      a.udrho_v[q] = a.udrho_v[q] + wgt * vn;
    } else {
      a.udrho_u[q] = a.udrho_u[q] + un;
      a.udrho_v[q] = a.udrho_v[q] + vn;
    }
  }
}

DEVI void bt_post2_body(BtArgs a, double* conv, double* eta_u, double* ps_out, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x;
  int j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  conv[q] = -div_ud(a, a.udrho_u, a.udrho_v, i, j);
  double r = 0.0;
  if (i <= g.ni && j <= g.nj) {
    const double* e = a.eta_bar;
    r = (e[q] * a.dte[q] * a.dus[q] + e[I2(g, i + 1, j)] * a.dtw[I2(g, i + 1, j)] * a.dus[q] +
         e[I2(g, i, j + 1)] * a.dte[I2(g, i, j + 1)] * a.dun[q] +
         e[I2(g, i + 1, j + 1)] * a.dtw[I2(g, i + 1, j + 1)] * a.dun[q]) *
        a.daur[q];
  }
  eta_u[q] = a.umask1[q] != 0.0 ? a.umask1[q] * r : 0.0;
  ps_out[q] = a.rho_g[q] * a.eta_bar[q] + a.patm[q];
}

DEVI void bt_post3_body(BtArgs a, const double* ps, double* gxo, double* gyo, int bx, int by) {
  const Geo& g = a.g;
  int i = bx * blockDim.x + threadIdx.x;
  int j = by;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double gx = 0.0, gy = 0.0;
  if (i <= g.ni && j <= g.nj) {
    if (!a.cgrid) {
      double p_fay = 0.5 * (ps[q] + ps[I2(g, i, j + 1)]);
      double p_fax = 0.5 * (ps[q] + ps[I2(g, i + 1, j)]);
      double pip_fay = 0.5 * (ps[I2(g, i + 1, j)] + ps[I2(g, i + 1, j + 1)]);
      double pjp_fax = 0.5 * (ps[I2(g, i, j + 1)] + ps[I2(g, i + 1, j + 1)]);
      bool um = a.umask1[q] != 0.0;
      gx = um ? (pip_fay - p_fay) * a.dxur[q] * a.umask1[q] : 0.0;
      gy = um ? (pjp_fax - p_fax) * a.dyur[q] * a.umask1[q] : 0.0;
    } else {
      gx = (ps[I2(g, i + 1, j)] - ps[q]) * a.dxter[q] * a.tmen_e[q];
      gy = (ps[I2(g, i, j + 1)] - ps[q]) * a.dytnr[q] * a.tmen_n[q];
    }
  }
  gxo[q] = gx;
  gyo[q] = gy;
}


}  // namespace fp64
}  // namespace mom5
