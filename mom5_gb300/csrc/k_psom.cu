// PSOM tracer advection: advect_tracer_psom (ocean_tracer_advect.F90:4549-4660)
// with psom_x (:4662-4917), psom_y (:4919-5174) and psom_z (:5176-5420):
// Prather's second-order moments, the sweep order set by mod(itt0, 6), and
// the Merryfield-Holloway or Prather moment limiter.  FP64 in the reference's
// operation order; built with --fmad=false.
//
// Work layout.  In the reference each direction is an outflow sweep over every
// face, a halo update, an inflow sweep over every face in the same order and a
// full halo update.  A cell is touched by two faces of a direction, always the
// one on its low side first, so both sweeps are per-cell computations: a cell
// sends through its low face (if the flow there leaves it), then through its
// high face; once every cell has sent, it receives through its low face, then
// its high face.  One kernel per direction runs both sweeps for segments of
// L-2 cells on BI lines: each thread owns a cell, stores the in-transit
// moments of the faces it is upstream of in shared memory and, after one
// barrier, applies the inflows.  The two end threads of a segment run the
// outflow of the neighbouring cells only to supply the segment's end faces.
// A periodic direction is a ring (the halo update makes each halo cell a copy
// of its image before it is used), and the boundary face of a closed direction
// carries nothing: its velocity is masked to zero, which makes the halo cell
// the upstream cell with a zero transfer fraction.  Along z the line runs
// upwards (s = nk - k), so that a positive vertical velocity moves towards
// higher s as positive u and v do along x and y.
//
// The moments sx..syz of each tracer live in HBM over the compute domain
// (data-domain layout, halo not maintained); the mass sm and the face fluxes
// are per-domain scratch.
#include <math.h>

#include "fp64_div.cuh"
#include "fp64_select.cuh"
#include "internal.h"

namespace mom5 {
namespace psom {

#define DEVI __device__ __forceinline__

DEVI long I2(const Geo& g, int i, int j) { return (long)j * g.nxd + i; }
DEVI long I3(const Geo& g, int i, int j, int k) { return (long)k * g.n2 + (long)j * g.nxd + i; }
// a > b ? a : b and a < b ? a : b, compared on the integer pipe
DEVI double mx(double a, double b) { return sel::gt_max(a, b); }
DEVI double mn(double a, double b) { return sel::lt_min(a, b); }

constexpr double kEpsln = 1.0e-20;  // constants_mod epsln

// moments in the order of the MOM5GPU_PSOM_SX.. fields
enum { SX, SXX, SY, SYY, SZ, SZZ, SXY, SXZ, SYZ, NMOM };
// in-transit moments of a face
enum { F0, FA, FAA, FB1, FB2, FC1, FC2, FBB1, FBB2, FBC, FM, NF };
// roles of the moments in a sweep: first and second along the direction, the
// other two firsts, the two cross moments with the direction, the other two
// seconds, the cross moment of the other two
enum { RA, RAA, RB1, RB2, RC1, RC2, RBB1, RBB2, RBC, NROLE };

struct Args {
  Geo g;
  double dtime, dtimer;
  int limit, prather, first;
  const double *tmask, *dat, *datr, *dxtn, *dyte, *uh, *vh, *w, *rdz, *T;
  double *sm, *s0;
  double* mr[NROLE];  // the moments in role order for this direction
  double *fx, *fy, *fz;
  double* th;
};

struct Cell {
  double sm, s0, a, aa, b1, b2, c1, c2, bb1, bb2, bc;
};

// T or tmask at any position: the periodic image, else 0 (halo of a closed edge)
DEVI double tq(const Geo& g, const double* T, int i, int j, int k) {
  if (i < 1) {
    if (!g.cx) return 0.0;
    i += g.ni;
  } else if (i > g.ni) {
    if (!g.cx) return 0.0;
    i -= g.ni;
  }
  if (j < 1) {
    if (!g.cy) return 0.0;
    j += g.nj;
  } else if (j > g.nj) {
    if (!g.cy) return 0.0;
    j -= g.nj;
  }
  return T[I3(g, i, j, k)];
}

// Prather's limiter (psom_x :4676-4692)
DEVI void limit_prather(Cell& c) {
  double slpmax = 0.0;
  if (sel::gt0(c.s0)) slpmax = c.s0;
  double s1max = 1.5 * slpmax;
  double s1new = mn(s1max, mx(-s1max, c.a));
  double s2new = mn(slpmax + slpmax - 0.3334 * fabs(s1new), mx(fabs(s1new) - slpmax, c.aa));
  c.c1 = mn(slpmax, mx(-slpmax, c.c1));
  c.c2 = mn(slpmax, mx(-slpmax, c.c2));
  c.a = s1new;
  c.aa = s2new;
}

// Merryfield-Holloway limiter (psom_x :4696-4741): the cell's tracer and mask
// (fc, mc) and its two neighbours along the direction (fm, mm), (fp, mp)
DEVI void limit_mh(Cell& c, double fc, double mc, double fm, double mm, double fp, double mp) {
  double s0max1 = fc * mc;
  if (sel::gt0(mm)) s0max1 = mx(fm, s0max1);
  if (sel::gt0(mp)) s0max1 = mx(fp, s0max1);
  s0max1 = s0max1 * c.sm;
  double slpmax = -c.s0 + s0max1;
  double s1max = 1.5 * slpmax;
  double s1new = mn(s1max, mx(-s1max, -c.a));
  double s2new = mn(slpmax + slpmax - 0.3334 * fabs(s1new), mx(fabs(s1new) - slpmax, -c.aa));
  c.c1 = -mn(slpmax, mx(-slpmax, -c.c1));
  c.c2 = -mn(slpmax, mx(-slpmax, -c.c2));
  c.a = -s1new;
  c.aa = -s2new;
  double s0min1 = fc * mc;
  if (sel::gt0(mm)) s0min1 = mn(fm, s0min1);
  if (sel::gt0(mp)) s0min1 = mn(fp, s0min1);
  s0min1 = s0min1 * c.sm;
  slpmax = c.s0 - s0min1;
  s1max = 1.5 * slpmax;
  s1new = mn(s1max, mx(-s1max, c.a));
  s2new = mn(slpmax + slpmax - 0.3334 * fabs(s1new), mx(fabs(s1new) - slpmax, c.aa));
  c.c1 = mn(slpmax, mx(-slpmax, c.c1));
  c.c2 = mn(slpmax, mx(-slpmax, c.c2));
  c.a = s1new;
  c.aa = s2new;
}

// outflow through a face (psom_x :4756-4828): pos = through the high face
// (velocity >= 0), else through the low face
DEVI void out_op(Cell& c, double velocity, double dv, double dtime, bool pos, double* f) {
  f[FM] = pos ? velocity * dtime * dv : -velocity * dtime * dv;
  double alf = fp64::div_seeded(f[FM], c.sm + kEpsln);
  double alfq = alf * alf, alf1 = 1.0 - alf, alf1q = alf1 * alf1;
  if (pos) {
    f[F0] = alf * (c.s0 + alf1 * (c.a + (alf1 - alf) * c.aa));
    f[FA] = alfq * (c.a + 3.0 * alf1 * c.aa);
    f[FB1] = alf * (c.b1 + alf1 * c.c1);
    f[FB2] = alf * (c.b2 + alf1 * c.c2);
  } else {
    f[F0] = alf * (c.s0 - alf1 * (c.a - (alf1 - alf) * c.aa));
    f[FA] = alfq * (c.a - 3.0 * alf1 * c.aa);
    f[FB1] = alf * (c.b1 - alf1 * c.c1);
    f[FB2] = alf * (c.b2 - alf1 * c.c2);
  }
  f[FAA] = alf * alfq * c.aa;
  f[FC1] = alfq * c.c1;
  f[FC2] = alfq * c.c2;
  f[FBB1] = alf * c.bb1;
  f[FBB2] = alf * c.bb2;
  f[FBC] = alf * c.bc;
  c.sm = c.sm - f[FM];
  c.s0 = c.s0 - f[F0];
  if (pos) c.a = alf1q * (c.a - 3.0 * alf * c.aa);
  else c.a = alf1q * (c.a + 3.0 * alf * c.aa);
  c.aa = alf1 * alf1q * c.aa;
  c.b1 = c.b1 - f[FB1];
  c.bb1 = c.bb1 - f[FBB1];
  c.b2 = c.b2 - f[FB2];
  c.bb2 = c.bb2 - f[FBB2];
  c.c1 = alf1q * c.c1;
  c.c2 = alf1q * c.c2;
  c.bc = c.bc - f[FBC];
}

// inflow through a face (psom_x :4857-4891): pos = through the low face
// (velocity >= 0), else through the high face
DEVI void in_op(Cell& c, bool pos, const double* f) {
  c.sm = c.sm + f[FM];
  double alf = fp64::div_seeded(f[FM], c.sm + kEpsln), alf1 = 1.0 - alf;
  if (pos) {
    double temptm = alf * c.s0 - alf1 * f[F0];
    c.s0 = c.s0 + f[F0];
    c.aa = alf * alf * f[FAA] + alf1 * alf1 * c.aa + 5.0 * (alf * alf1 * (c.a - f[FA]) - (alf1 - alf) * temptm);
    c.a = alf * f[FA] + alf1 * c.a + 3.0 * temptm;
    c.c1 = alf * f[FC1] + alf1 * c.c1 + 3.0 * (-alf1 * f[FB1] + alf * c.b1);
    c.c2 = alf * f[FC2] + alf1 * c.c2 + 3.0 * (-alf1 * f[FB2] + alf * c.b2);
  } else {
    double temptm = -alf * c.s0 + alf1 * f[F0];
    c.s0 = c.s0 + f[F0];
    c.aa = alf * alf * f[FAA] + alf1 * alf1 * c.aa + 5.0 * (alf * alf1 * (-c.a + f[FA]) + (alf1 - alf) * temptm);
    c.a = alf * f[FA] + alf1 * c.a + 3.0 * temptm;
    c.c1 = alf * f[FC1] + alf1 * c.c1 + 3.0 * (alf1 * f[FB1] - alf * c.b1);
    c.c2 = alf * f[FC2] + alf1 * c.c2 + 3.0 * (alf1 * f[FB2] - alf * c.b2);
  }
  c.b1 = c.b1 + f[FB1];
  c.bb1 = c.bb1 + f[FBB1];
  c.b2 = c.b2 + f[FB2];
  c.bb2 = c.bb2 + f[FBB2];
  c.bc = c.bc + f[FBC];
}

// Geometry of direction DIR (1 x, 2 y, 3 z) for a line through (i, j) or (i, k)
template <int DIR>
struct Line {
  const Geo& g;
  int i, j, k;  // the two coordinates across the line (the one along it unused)
  int N;
  bool cyc;
  DEVI Line(const Geo& g_, int i_, int j_, int k_)
      : g(g_), i(i_), j(j_), k(k_), N(DIR == 1 ? g_.ni : DIR == 2 ? g_.nj : g_.nk),
        cyc(DIR == 1 ? g_.cx != 0 : DIR == 2 ? g_.cy != 0 : false) {}
  // cell at line position s: its canonical position, false if it holds no state
  DEVI bool cell(int s, int& sc) const {
    if (s >= 1 && s <= N) {
      sc = s;
      return true;
    }
    if (cyc && (s == 0 || s == N + 1)) {
      sc = s == 0 ? N : 1;
      return true;
    }
    return false;
  }
  DEVI long index(int sc) const {
    if (DIR == 1) return I3(g, sc, j, k);
    if (DIR == 2) return I3(g, i, sc, k);
    return I3(g, i, j, g.nk - sc);
  }
  // face f joins positions f and f+1
  DEVI bool face(int f, int& fc) const {
    if (DIR == 3) {
      fc = f;
      return f >= 1 && f <= N - 1;
    }
    if (cyc) {  // only faces -1..N+1 are asked for (cells 0..N+1)
      fc = ((f - 1) % N + N) % N + 1;
      return true;
    }
    fc = f;
    return f >= 0 && f <= N;
  }
  // velocity * mask and the face length of a canonical face
  DEVI void face_vel(const Args& a, int fc, double& v, double& dv) const {
    if (DIR == 1) {
      v = a.uh[I3(g, fc, j, k)] * mn(tq(g, a.tmask, fc, j, k), tq(g, a.tmask, fc + 1, j, k));
      dv = a.dyte[I2(g, fc, j)];
    } else if (DIR == 2) {
      v = a.vh[I3(g, i, fc, k)] * mn(tq(g, a.tmask, i, fc, k), tq(g, a.tmask, i, fc + 1, k));
      dv = a.dxtn[I2(g, i, fc)];
    } else {
      long q = I3(g, i, j, g.nk - fc);  // wrho_bt at the bottom of the upper cell; tmask of the lower
      v = a.w[q] * a.tmask[q];
      dv = a.dat[I2(g, i, j)];
    }
  }
  // where the flux through face f is stored (flux_x(i), flux_y(j), flux_z(upper k))
  DEVI long flux_index(int f) const {
    if (DIR == 1) return I3(g, f, j, k);
    if (DIR == 2) return I3(g, i, f, k);
    return I3(g, i, j, g.nk - 1 - f);
  }
  DEVI void limit(const Args& a, int sc, long p, Cell& c) const {
    if (a.prather) {
      limit_prather(c);
      return;
    }
    double fm, mm, fp, mp;
    if (DIR == 1) {
      fm = tq(g, a.T, sc - 1, j, k), mm = tq(g, a.tmask, sc - 1, j, k);
      fp = tq(g, a.T, sc + 1, j, k), mp = tq(g, a.tmask, sc + 1, j, k);
    } else if (DIR == 2) {
      fm = tq(g, a.T, i, sc - 1, k), mm = tq(g, a.tmask, i, sc - 1, k);
      fp = tq(g, a.T, i, sc + 1, k), mp = tq(g, a.tmask, i, sc + 1, k);
    } else {
      int kk = g.nk - sc, km1 = kk > 0 ? kk - 1 : 0, kp1 = kk < g.nk - 1 ? kk + 1 : g.nk - 1;
      fm = a.T[I3(g, i, j, km1)], mm = a.tmask[I3(g, i, j, km1)];
      fp = a.T[I3(g, i, j, kp1)], mp = a.tmask[I3(g, i, j, kp1)];
    }
    limit_mh(c, a.T[p], a.tmask[p], fm, mm, fp, mp);
  }
};

// Both sweeps of one direction for segments of L-2 cells on BI lines.
template <int DIR, int BI, int L>
__global__ void __launch_bounds__(BI* L) k_psom_dir(Args a) {
  __shared__ double slot[NF][L - 1][BI];
  const Geo& g = a.g;
  const int lane = threadIdx.x, t = threadIdx.y;
  int i = 0, j = 0, k = 0, seg;
  bool lane_ok = true;
  if (DIR == 1) {
    seg = blockIdx.x, j = blockIdx.y + 1, k = blockIdx.z;
  } else if (DIR == 2) {
    i = blockIdx.x * BI + lane + 1, seg = blockIdx.y, k = blockIdx.z;
    lane_ok = i <= g.ni;
  } else {
    i = blockIdx.x * BI + lane + 1, j = blockIdx.y + 1, seg = blockIdx.z;
    lane_ok = i <= g.ni;
  }
  const Line<DIR> ln(g, i, j, k);
  const int s0 = seg * (L - 2), s = s0 + t;
  int sc = 0;
  const bool valid = lane_ok && ln.cell(s, sc);
  Cell c;
  long p = 0;
  if (valid) {
    p = ln.index(sc);
    if (a.first) {
      long q = DIR == 1 ? I2(g, sc, j) : DIR == 2 ? I2(g, i, sc) : I2(g, i, j);
      c.sm = a.rdz[p] * a.dat[q];
      c.s0 = a.T[p] * c.sm * a.tmask[p];
    } else {
      c.sm = a.sm[p];
      c.s0 = a.s0[p];
    }
    c.a = a.mr[RA][p], c.aa = a.mr[RAA][p], c.b1 = a.mr[RB1][p], c.b2 = a.mr[RB2][p];
    c.c1 = a.mr[RC1][p], c.c2 = a.mr[RC2][p], c.bb1 = a.mr[RBB1][p], c.bb2 = a.mr[RBB2][p];
    c.bc = a.mr[RBC][p];
    if (a.limit) ln.limit(a, sc, p, c);
  }
  int fwc = 0, fec = 0;
  // faces of cells holding state; past the ends of a ring a segment's spare
  // threads have none, while the halo cell of a closed edge keeps its (empty) face
  const bool asks = lane_ok && (valid || !ln.cyc);
  const bool hw = asks && ln.face(s - 1, fwc), he = asks && ln.face(s, fec);
  double vw = 0.0, ve = 0.0, dvw = 0.0, dve = 0.0;
  if (hw) ln.face_vel(a, fwc, vw, dvw);
  if (he) ln.face_vel(a, fec, ve, dve);
  double f[NF];
  // outflow sweep: low face first, then high face
  if (hw && sel::lt0(vw)) {
    if (valid) out_op(c, vw, dvw, a.dtime, false, f);
    else
      for (int q = 0; q < NF; ++q) f[q] = 0.0;
    int sl = s - 1 - s0;
    if (sl >= 0 && sl <= L - 2)
      for (int q = 0; q < NF; ++q) slot[q][sl][lane] = f[q];
  }
  if (he && sel::ge0(ve)) {
    if (valid) out_op(c, ve, dve, a.dtime, true, f);
    else
      for (int q = 0; q < NF; ++q) f[q] = 0.0;  // halo cell of a closed edge: nothing in transit
    int sl = s - s0;
    if (sl >= 0 && sl <= L - 2)
      for (int q = 0; q < NF; ++q) slot[q][sl][lane] = f[q];
  }
  __syncthreads();
  if (!valid || t < 1 || t > L - 2 || s < 1 || s > ln.N) return;
  // inflow sweep: low face first, then high face
  if (hw && sel::ge0(vw)) {
    for (int q = 0; q < NF; ++q) f[q] = slot[q][t - 1][lane];
    in_op(c, true, f);
  }
  if (he && sel::lt0(ve)) {
    for (int q = 0; q < NF; ++q) f[q] = slot[q][t][lane];
    in_op(c, false, f);
  }
  a.sm[p] = c.sm;
  a.s0[p] = c.s0;
  a.mr[RA][p] = c.a, a.mr[RAA][p] = c.aa, a.mr[RB1][p] = c.b1, a.mr[RB2][p] = c.b2;
  a.mr[RC1][p] = c.c1, a.mr[RC2][p] = c.c2, a.mr[RBB1][p] = c.bb1, a.mr[RBB2][p] = c.bb2;
  a.mr[RBC][p] = c.bc;
  // fluxes (flux_x(i,j,k) = +-f0/dtime) of the high face, and of face 0 in the first cell
  double* flux = DIR == 1 ? a.fx : DIR == 2 ? a.fy : a.fz;
  if (he) {
    double f0 = slot[F0][t][lane];
    flux[ln.flux_index(s)] = sel::ge0(ve) ? f0 * a.dtimer : -f0 * a.dtimer;
  }
  if (DIR != 3 && s == 1 && hw) {
    double f0 = slot[F0][t - 1][lane];
    flux[ln.flux_index(0)] = sel::ge0(vw) ? f0 * a.dtimer : -f0 * a.dtimer;
  }
}

// the tendency (:4627-4642): th += -tmask*(flux divergence)*datr
__global__ void __launch_bounds__(128) k_psom_tendency(Args a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z;
  if (i > g.ni) return;
  long p = I3(g, i, j, k);
  double ft1 = k > 0 ? a.fz[p - g.n2] : 0.0;
  double fzk = k < g.nk - 1 ? a.fz[p] : 0.0;  // flux_z(nk) stays at its reset value 0
  double advect = a.tmask[p] * (a.fx[p] - a.fx[p - 1] + a.fy[p] - a.fy[p - g.nxd] + ft1 - fzk) * a.datr[I2(g, i, j)];
  a.th[p] = a.th[p] + (-advect);
}

}  // namespace psom

using namespace psom;

int launch_psom(mom5gpu_domain* d, int n, int taum1, double dtime) {
  const Geo& g = d->geo;
  size_t n3 = (size_t)g.n3;
  if (!d->psom_scr) {
    cudaError_t e = cudaMalloc(&d->psom_scr, sizeof(double) * 4 * n3);
    if (e != cudaSuccess) return fail(d, MOM5GPU_ENOMEM, "psom scratch: %s", cudaGetErrorString(e));
    d->bytes += sizeof(double) * 4 * n3;
    cudaMemsetAsync(d->psom_scr, 0, sizeof(double) * 4 * n3, d->stream);
  }
  Args a;
  a.g = g;
  a.dtime = dtime;
  a.dtimer = 1.0 / dtime;
  a.limit = d->scheme[n - 1].psom_limit;
  a.prather = d->opt.psom_limit_prather != 0;
  a.tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  a.dat = fptr(d, MOM5GPU_DAT, 0, 0);
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a.dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a.uh = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a.vh = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a.w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  a.rdz = fptr(d, MOM5GPU_RHO_DZT, 0, taum1);
  a.T = fptr(d, MOM5GPU_TRACER, n, taum1);
  a.th = fptr(d, MOM5GPU_TH_TENDENCY, n, 0);
  a.sm = d->psom_scr;
  a.fx = d->psom_scr + n3;
  a.fy = d->psom_scr + 2 * n3;
  a.fz = d->psom_scr + 3 * n3;
  a.s0 = fptr(d, MOM5GPU_PSOM_S0, n, 0);
  double* m[NMOM];
  for (int q = 0; q < NMOM; ++q) m[q] = fptr(d, MOM5GPU_PSOM_SX + q, n, 0);
  const void* need[] = {a.tmask, a.dat, a.datr, a.dxtn, a.dyte, a.uh, a.vh, a.w, a.rdz, a.T, a.th, a.s0};
  for (const void* p : need)
    if (!p) return fail(d, MOM5GPU_ESTATE, "psom: a required field was never set");
  for (double* p : m)
    if (!p) return fail(d, MOM5GPU_ENOMEM, "psom: moment storage");
  // roles per direction: along (first, second), other firsts, cross with the
  // direction, other seconds, cross of the other two
  static const int roles[3][NROLE] = {{SX, SXX, SY, SZ, SXY, SXZ, SYY, SZZ, SYZ},
                                      {SY, SYY, SX, SZ, SXY, SYZ, SXX, SZZ, SXZ},
                                      {SZ, SZZ, SX, SY, SXZ, SYZ, SXX, SYY, SXY}};
  // ocean_tracer_advect.F90:4592-4621
  static const int order[6][3] = {{1, 2, 3}, {3, 1, 2}, {2, 3, 1}, {1, 3, 2}, {2, 1, 3}, {3, 2, 1}};
  ClockScope clk(d, SEC_MDFL);
  cudaStream_t s = d->stream;
  const int* o = order[d->itt0 % 6];
  constexpr int LX = 128, BI = 16, LYZ = 32;
  for (int st = 0; st < 3; ++st) {
    int dir = o[st];
    a.first = st == 0;
    for (int r = 0; r < NROLE; ++r) a.mr[r] = m[roles[dir - 1][r]];
    if (dir == 1) {
      dim3 grid((g.ni + LX - 3) / (LX - 2), g.nj, g.nk);
      k_psom_dir<1, 1, LX><<<grid, dim3(1, LX), 0, s>>>(a);
    } else if (dir == 2) {
      dim3 grid((g.ni + BI - 1) / BI, (g.nj + LYZ - 3) / (LYZ - 2), g.nk);
      k_psom_dir<2, BI, LYZ><<<grid, dim3(BI, LYZ), 0, s>>>(a);
    } else {
      dim3 grid((g.ni + BI - 1) / BI, g.nj, (g.nk + LYZ - 3) / (LYZ - 2));
      k_psom_dir<3, BI, LYZ><<<grid, dim3(BI, LYZ), 0, s>>>(a);
    }
  }
  dim3 gt((g.ni + 127) / 128, g.nj, g.nk);
  k_psom_tendency<<<gt, 128, 0, s>>>(a);
  count_launches(d, 4);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "psom");
}

}  // namespace mom5
