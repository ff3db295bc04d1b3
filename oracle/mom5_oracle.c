/*
 * mom5_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64, line-by-line restatement of the MOM5 routines on the
 * tracer-advection and split-explicit barotropic path.  It exists to check the
 * CUDA implementation; nothing in the shipped library links, loads or calls
 * it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * use it.
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists in
 * the build container, so this restatement cannot be diffed against a compiled
 * reference there; the reference tree holds no golden vectors for these
 * routines (its only regression data are whole-model checksums that need
 * missing experiment inputs).  Parity of this file is therefore pinned by the
 * analytic and property tests in tests/test_oracle_*.py (among them known
 * answers of the advection equation: exact translation of polynomial profiles
 * in uniform flow, tests/analytic.py).  No Fortran compiler exists on the GPU
 * host either.
 *
 * Conventions (mirroring the Fortran arrays of the reference):
 *   - compute domain i = 1..ni, j = 1..nj (isc=1, iec=ni); the data domain has
 *     a halo of one cell, so C indices run 0..ni+1 and 0..nj+1 (isd=0).
 *   - arrays are column-major: i fastest, then j, then k (k = 0..nk-1 for
 *     Fortran k = 1..nk), then any further index (component, tracer).
 *   - wrho_bt has levels 0..nk (Fortran dimension 0:nk).
 *   - one processor element owns the whole domain, so mpp_update_domains
 *     reduces to a periodic copy in cyclic directions and to "leave the halo
 *     alone" at non-cyclic walls (halo_update_* below).
 * Build with -O2 -ffp-contract=off so that no multiply-add is fused: the
 * reference's gfortran build evaluates every product and sum separately.
 */
#define _POSIX_C_SOURCE 199309L
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct {
  int ni, nj, nk;
  int cyclic_x, cyclic_y;
} orc_dims;

typedef struct orc_mdfl_ws orc_mdfl_ws;
void orc_advect_mdfl_sweby_ws(orc_mdfl_ws* ws, double sweby_limiter, double dtime, const double* dat,
                              const double* datr, const double* dxte, const double* dyte, const double* dxtn,
                              const double* dytn, const double* uhrho_et, const double* vhrho_nt,
                              const double* wrho_bt, const double* rho_dzt, const double* T, double* wrk1);

#define NXD(d) ((d)->ni + 2)
#define NYD(d) ((d)->nj + 2)
#define I2(d, i, j) ((size_t)(j) * NXD(d) + (size_t)(i))
#define I3(d, i, j, k) (((size_t)(k) * NYD(d) + (size_t)(j)) * NXD(d) + (size_t)(i))

static inline double fmaxd(double a, double b) { return a > b ? a : b; }
static inline double fmind(double a, double b) { return a < b ? a : b; }

/* Built with -fopenmp (the CPU baseline's build only), the loops marked
 * OMP_FOR run their iterations on all host cores; every marked loop has
 * independent iterations, so the results are those of the serial build. */
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

#ifdef _OPENMP
#include <omp.h>
#endif

/* Threads of the OpenMP build's parallel loops (no effect in the serial build). */
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

static void zero_par(double* a, size_t n) {
  const size_t chunk = 1 << 16;
  long nc = (long)((n + chunk - 1) / chunk);
  OMP_FOR
  for (long c = 0; c < nc; ++c) {
    size_t lo = (size_t)c * chunk, hi = lo + chunk < n ? lo + chunk : n;
    memset(a + lo, 0, sizeof(double) * (hi - lo));
  }
}

/* ocean_parameters.F90:92 onesixth = 1.0/6.0; :194-195 rho0, rho0r */
static const double onesixth = 1.0 / 6.0;

/* ------------------------------------------------------------------------- */
/* Halo update of a data-domain (halo 1) field on a single-PE domain.        */
/* flags: 1 = east/west halo (XUPDATE), 2 = north/south (YUPDATE), 3 = both. */
/* mpp_update_domains semantics: src/shared/mpp/include/mpp_do_update.h;     */
/* corners are filled only when both directions are cyclic.                  */
/* ------------------------------------------------------------------------- */
void orc_halo_update_3d(const orc_dims* d, double* a, int nlev, int flags) {
  int ni = d->ni, nj = d->nj;
  for (int k = 0; k < nlev; ++k) {
    if ((flags & 1) && d->cyclic_x) {
      for (int j = 1; j <= nj; ++j) {
        a[I3(d, 0, j, k)] = a[I3(d, ni, j, k)];
        a[I3(d, ni + 1, j, k)] = a[I3(d, 1, j, k)];
      }
    }
    if ((flags & 2) && d->cyclic_y) {
      for (int i = 1; i <= ni; ++i) {
        a[I3(d, i, 0, k)] = a[I3(d, i, nj, k)];
        a[I3(d, i, nj + 1, k)] = a[I3(d, i, 1, k)];
      }
    }
    if (flags == 3 && d->cyclic_x && d->cyclic_y) {
      a[I3(d, 0, 0, k)] = a[I3(d, ni, nj, k)];
      a[I3(d, ni + 1, 0, k)] = a[I3(d, 1, nj, k)];
      a[I3(d, 0, nj + 1, k)] = a[I3(d, ni, 1, k)];
      a[I3(d, ni + 1, nj + 1, k)] = a[I3(d, 1, 1, k)];
    }
  }
}

void orc_halo_update_2d(const orc_dims* d, double* a, int flags) { orc_halo_update_3d(d, a, 1, flags); }

/* Halo-2 arrays (isc-2:iec+2, jsc-2:jec+2, nk) used by mdfl and quicker.    */
#define NX2(d) ((d)->ni + 4)
#define NY2(d) ((d)->nj + 4)
/* i, j in data-domain coordinates (isc = 1), so i = -1 is isc-2. */
#define H3(d, i, j, k) (((size_t)(k) * NY2(d) + (size_t)((j) + 1)) * NX2(d) + (size_t)((i) + 1))

static void halo2_update(const orc_dims* d, double* a, int flags) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  for (int k = 0; k < nk; ++k) {
    if ((flags & 1) && d->cyclic_x) {
      for (int j = 1; j <= nj; ++j)
        for (int h = 1; h <= 2; ++h) {
          a[H3(d, 1 - h, j, k)] = a[H3(d, ni + 1 - h, j, k)];
          a[H3(d, ni + h, j, k)] = a[H3(d, h, j, k)];
        }
    }
    if ((flags & 2) && d->cyclic_y) {
      for (int i = 1; i <= ni; ++i)
        for (int h = 1; h <= 2; ++h) {
          a[H3(d, i, 1 - h, k)] = a[H3(d, i, nj + 1 - h, k)];
          a[H3(d, i, nj + h, k)] = a[H3(d, i, h, k)];
        }
    }
    if (flags == 3 && d->cyclic_x && d->cyclic_y) {
      for (int hj = 1; hj <= 2; ++hj)
        for (int hi = 1; hi <= 2; ++hi) {
          a[H3(d, 1 - hi, 1 - hj, k)] = a[H3(d, ni + 1 - hi, nj + 1 - hj, k)];
          a[H3(d, ni + hi, 1 - hj, k)] = a[H3(d, hi, nj + 1 - hj, k)];
          a[H3(d, 1 - hi, nj + hj, k)] = a[H3(d, ni + 1 - hi, hj, k)];
          a[H3(d, ni + hi, nj + hj, k)] = a[H3(d, hi, hj, k)];
        }
    }
  }
}

/* tmask copied into a halo-2 array and halo-updated: mdfl_init
 * (ocean_tracer_advect.F90:1644-1691) and quicker_init (:1478-1487). */
void orc_mask_halo2(const orc_dims* d, const double* tmask, double* mask2) {
  memset(mask2, 0, sizeof(double) * NX2(d) * NY2(d) * d->nk);
  for (int k = 0; k < d->nk; ++k)
    for (int j = 1; j <= d->nj; ++j)
      for (int i = 1; i <= d->ni; ++i) mask2[H3(d, i, j, k)] = tmask[I3(d, i, j, k)];
  halo2_update(d, mask2, 3);
}

/* ------------------------------------------------------------------------- */
/* Upwind: ocean_tracer_advect.F90:2238-2294 (horizontal), :2792-2824 (vert). */
/* Outputs wrk1 = -scheme(...) on the compute domain (horz_advect_tracer     */
/* :1935-1936 negates the function result), zero elsewhere.                  */
/* ------------------------------------------------------------------------- */
void orc_horz_advect_upwind(const orc_dims* d, const double* tmask, const double* dyte, const double* dxtn,
                            const double* datr, const double* uhrho_et, const double* vhrho_nt, const double* T,
                            double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* fe = (double*)calloc(n2, sizeof(double));
  double* fn = (double*)calloc(n2, sizeof(double));
  memset(wrk1, 0, sizeof(double) * n2 * nk);
  for (int k = 0; k < nk; ++k) {
    for (int j = 1; j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        double velocity = 0.5 * uhrho_et[I3(d, i, j, k)];
        double upos = velocity + fabs(velocity);
        double uneg = velocity - fabs(velocity);
        fe[I2(d, i, j)] = dyte[I2(d, i, j)] * (upos * T[I3(d, i, j, k)] + uneg * T[I3(d, i + 1, j, k)]) *
                          tmask[I3(d, i, j, k)] * tmask[I3(d, i + 1, j, k)];
      }
    for (int j = 0; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double velocity = 0.5 * vhrho_nt[I3(d, i, j, k)];
        double upos = velocity + fabs(velocity);
        double uneg = velocity - fabs(velocity);
        fn[I2(d, i, j)] = dxtn[I2(d, i, j)] * (upos * T[I3(d, i, j, k)] + uneg * T[I3(d, i, j + 1, k)]) *
                          tmask[I3(d, i, j, k)] * tmask[I3(d, i, j + 1, k)];
      }
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double r = tmask[I3(d, i, j, k)] *
                   (fe[I2(d, i, j)] - fe[I2(d, i - 1, j)] + fn[I2(d, i, j)] - fn[I2(d, i, j - 1)]) *
                   datr[I2(d, i, j)];
        wrk1[I3(d, i, j, k)] = -r;
      }
  }
  free(fe);
  free(fn);
}

void orc_vert_advect_upwind(const orc_dims* d, const double* tmask, const double* wrho_bt, const double* T,
                            double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* ft1 = (double*)calloc(n2, sizeof(double));
  memset(wrk1, 0, sizeof(double) * n2 * nk);
  for (int k = 0; k < nk; ++k) {
    int kp1 = k + 1 < nk ? k + 1 : nk - 1;
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        /* wrho_bt(i,j,k) for Fortran level k = C level k+1 of the 0:nk array */
        double velocity = 0.5 * wrho_bt[I3(d, i, j, k + 1)];
        double wpos = velocity + fabs(velocity);
        double wneg = velocity - fabs(velocity);
        double ft2 = (wneg * T[I3(d, i, j, k)] + wpos * T[I3(d, i, j, kp1)]) * tmask[I3(d, i, j, k)] *
                     tmask[I3(d, i, j, kp1)];
        double r = tmask[I3(d, i, j, k)] * (ft1[I2(d, i, j)] - ft2);
        wrk1[I3(d, i, j, k)] = -r;
        ft1[I2(d, i, j)] = ft2;
      }
  }
  free(ft1);
}

/* ------------------------------------------------------------------------- */
/* Centred schemes: 2nd order (:2306-2352, :2836-2864), 4th order            */
/* (:2361-2435, :2873-2907), 6th order (:2444-2529, :2916-2972), with        */
/* a4, b4, a6, b6, c6 (:349-350).  The 4th/6th-order horizontal schemes read */
/* tracer_fourth/sixth and tmask_fourth/sixth (fourth_sixth_init             */
/* :1597-1636): the compute-domain values with a halo of 2/3 filled by the   */
/* single-PE halo update (periodic image in cyclic directions, else 0).      */
/* Outputs wrk1 = -scheme(...) on the compute domain, zero elsewhere.        */
/* ------------------------------------------------------------------------- */
static const double c_a4 = 7.0 / 12.0, c_b4 = -1.0 / 12.0;
static const double c_a6 = 37.0 / 60.0, c_b6 = -2.0 / 15.0, c_c6 = 1.0 / 60.0;

/* value of a compute-domain field at (i,j,k) after a halo update of any width */
static double halo_value(const orc_dims* d, const double* a, int i, int j, int k) {
  if (i < 1 || i > d->ni) {
    if (!d->cyclic_x) return 0.0;
    i = i < 1 ? i + d->ni : i - d->ni;
  }
  if (j < 1 || j > d->nj) {
    if (!d->cyclic_y) return 0.0;
    j = j < 1 ? j + d->nj : j - d->nj;
  }
  return a[I3(d, i, j, k)];
}

/* 2-D version (one level of a data-domain array) */
static double halo_value2d(const orc_dims* d, const double* a, int i, int j) {
  if (i < 1 || i > d->ni) {
    if (!d->cyclic_x) return 0.0;
    i = i < 1 ? i + d->ni : i - d->ni;
  }
  if (j < 1 || j > d->nj) {
    if (!d->cyclic_y) return 0.0;
    j = j < 1 ? j + d->nj : j - d->nj;
  }
  return a[I2(d, i, j)];
}

void orc_horz_advect_centred(const orc_dims* d, int order, const double* tmask, const double* dyte,
                             const double* dxtn, const double* datr, const double* uhrho_et, const double* vhrho_nt,
                             const double* T, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* fx = (double*)calloc(n2, sizeof(double));
  double* fy = (double*)calloc(n2, sizeof(double));
  memset(wrk1, 0, sizeof(double) * n2 * nk);
#define TT(i, j) halo_value(d, T, (i), (j), k)
#define TM(i, j) halo_value(d, tmask, (i), (j), k)
  for (int k = 0; k < nk; ++k) {
    memset(fx, 0, sizeof(double) * n2);
    memset(fy, 0, sizeof(double) * n2);
    for (int j = (order == 2 ? 0 : 1); j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        double u = uhrho_et[I3(d, i, j, k)], f;
        if (order == 2) {
          f = dyte[I2(d, i, j)] * u * 0.5 * (T[I3(d, i + 1, j, k)] + T[I3(d, i, j, k)]);
        } else if (order == 4 || TM(i - 2, j) * TM(i - 1, j) == 0.0 || TM(i + 3, j) * TM(i + 2, j) == 0.0) {
          int im1 = (int)(TM(i - 1, j) * (i - 1) + (1.0 - TM(i - 1, j)) * i);
          int ip2 = (int)(TM(i + 2, j) * (i + 2) + (1.0 - TM(i + 2, j)) * (i + 1));
          f = dyte[I2(d, i, j)] * u * (c_a4 * (TT(i + 1, j) + TT(i, j)) + c_b4 * (TT(ip2, j) + TT(im1, j)));
        } else {
          f = dyte[I2(d, i, j)] * u *
              (c_a6 * (TT(i + 1, j) + TT(i, j)) + c_b6 * (TT(i + 2, j) + TT(i - 1, j)) +
               c_c6 * (TT(i + 3, j) + TT(i - 2, j)));
        }
        fx[I2(d, i, j)] = f;
      }
    for (int j = 0; j <= nj; ++j)
      for (int i = (order == 2 ? 0 : 1); i <= ni; ++i) {
        double v = vhrho_nt[I3(d, i, j, k)], f;
        if (order == 2) {
          f = dxtn[I2(d, i, j)] * v * 0.5 * (T[I3(d, i, j + 1, k)] + T[I3(d, i, j, k)]);
        } else if (order == 4 || TM(i, j - 2) * TM(i, j - 1) == 0.0 || TM(i, j + 3) * TM(i, j + 2) == 0.0) {
          int jm1 = (int)(TM(i, j - 1) * (j - 1) + (1.0 - TM(i, j - 1)) * j);
          int jp2 = (int)(TM(i, j + 2) * (j + 2) + (1.0 - TM(i, j + 2)) * (j + 1));
          f = dxtn[I2(d, i, j)] * v * (c_a4 * (TT(i, j + 1) + TT(i, j)) + c_b4 * (TT(i, jp2) + TT(i, jm1)));
        } else {
          f = dxtn[I2(d, i, j)] * v *
              (c_a6 * (TT(i, j + 1) + TT(i, j)) + c_b6 * (TT(i, j + 2) + TT(i, j - 1)) +
               c_c6 * (TT(i, j + 3) + TT(i, j - 2)));
        }
        fy[I2(d, i, j)] = f;
      }
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double r = tmask[I3(d, i, j, k)] *
                   (fx[I2(d, i, j)] - fx[I2(d, i - 1, j)] + fy[I2(d, i, j)] - fy[I2(d, i, j - 1)]) *
                   datr[I2(d, i, j)];
        wrk1[I3(d, i, j, k)] = -r;
      }
  }
#undef TT
#undef TM
  free(fx);
  free(fy);
}

void orc_vert_advect_centred(const orc_dims* d, int order, const double* tmask, const int* kmt,
                             const double* wrho_bt, const double* T, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  memset(wrk1, 0, sizeof(double) * n2 * nk);
  for (int j = 1; j <= nj; ++j)
    for (int i = 1; i <= ni; ++i) {
      double ft1 = 0.0;
      for (int K = 1; K <= nk; ++K) { /* Fortran level numbers */
        int k = K - 1;
        double w = wrho_bt[I3(d, i, j, K)];
        int p1 = K + 1 < nk ? K + 1 : nk, p2 = K + 2 < nk ? K + 2 : nk, km1 = K - 1 > 1 ? K - 1 : 1;
#define TV(L) T[I3(d, i, j, (L) - 1)]
        double ft2;
        if (order == 2) {
          ft2 = w * 0.5 * (TV(K) + TV(p1));
        } else {
          double tp2 = tmask[I3(d, i, j, p2 - 1)];
          int kp2 = (int)nearbyint(tp2 * p2 + (1.0 - tp2) * p1);
          if (order == 6 && !(K <= 2 || K >= nk - 1) && K < kmt[I2(d, i, j)] - 2)
            ft2 = w * (c_a6 * (TV(K) + TV(p1)) + c_b6 * (TV(km1) + TV(kp2)) + c_c6 * (TV(K - 2) + TV(K + 3)));
          else
            ft2 = w * (c_a4 * (TV(K) + TV(p1)) + c_b4 * (TV(km1) + TV(kp2)));
        }
#undef TV
        double r = tmask[I3(d, i, j, k)] * (ft1 - ft2);
        wrk1[I3(d, i, j, k)] = -r;
        ft1 = ft2;
      }
    }
}

/* ------------------------------------------------------------------------- */
/* PSOM: advect_tracer_psom (ocean_tracer_advect.F90:4549-4660) with psom_x  */
/* (:4662-4917), psom_y (:4919-5174), psom_z (:5176-5420): Prather's second- */
/* order moments, direction order by mod(itt0, 6), optional moment limiters. */
/* The nine moments sx..syz are prognostic (in/out); s0 and the mass sm are  */
/* formed from the tracer at lag = taum1.  Every array is data-domain sized. */
/* Returns wrk1 = -advect.                                                    */
/* ------------------------------------------------------------------------- */
enum { P_SX, P_SXX, P_SY, P_SYY, P_SZ, P_SZZ, P_SXY, P_SXZ, P_SYZ, P_N };
static const double psom_epsln = 1.0e-20; /* constants_mod epsln */

typedef struct {
  double *sm, *s0, *m[P_N];
} psom_state;

static void psom_full_update(const orc_dims* d, psom_state* st) {
  orc_halo_update_3d(d, st->sm, d->nk, 3);
  orc_halo_update_3d(d, st->s0, d->nk, 3);
  for (int q = 0; q < P_N; ++q) orc_halo_update_3d(d, st->m[q], d->nk, 3);
}

/* limiter of the moments along one direction before transport (:4676-4748 and the
 * y/z analogues); a = first moment along the direction, aa = second, c1, c2 = the
 * two cross moments with it; nb selects the neighbours (1 x, 2 y, 3 z). */
static void psom_limit(const orc_dims* d, int prather, int dir, const double* tmask, const double* field,
                       psom_state* st, int a, int aa, int c1, int c2) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  double *A = st->m[a], *AA = st->m[aa], *C1 = st->m[c1], *C2 = st->m[c2];
  if (prather) {
    for (int k = 0; k < nk; ++k)
      for (int j = 0; j <= nj + 1; ++j)
        for (int i = 0; i <= ni + 1; ++i) {
          size_t p = I3(d, i, j, k);
          double slpmax = 0.0;
          if (st->s0[p] > 0.0) slpmax = st->s0[p];
          double s1max = 1.5 * slpmax;
          double s1new = fmind(s1max, fmaxd(-s1max, A[p]));
          double s2new = fmind(slpmax + slpmax - 0.3334 * fabs(s1new), fmaxd(fabs(s1new) - slpmax, AA[p]));
          C1[p] = fmind(slpmax, fmaxd(-slpmax, C1[p]));
          C2[p] = fmind(slpmax, fmaxd(-slpmax, C2[p]));
          A[p] = s1new;
          AA[p] = s2new;
        }
    return;
  }
  int i0 = dir == 1 ? 1 : 0, i1 = dir == 1 ? ni : ni + 1;
  int j0 = dir == 2 ? 1 : 0, j1 = dir == 2 ? nj : nj + 1;
  for (int k = 0; k < nk; ++k) {
    int km1 = k - 1 > 0 ? k - 1 : 0, kp1 = k + 1 < nk ? k + 1 : nk - 1;
    for (int j = j0; j <= j1; ++j)
      for (int i = i0; i <= i1; ++i) {
        size_t p = I3(d, i, j, k), pm, pp;
        if (dir == 1) {
          pm = I3(d, i - 1, j, k);
          pp = I3(d, i + 1, j, k);
        } else if (dir == 2) {
          pm = I3(d, i, j - 1, k);
          pp = I3(d, i, j + 1, k);
        } else {
          pm = I3(d, i, j, km1);
          pp = I3(d, i, j, kp1);
        }
        double s0max1 = field[p] * tmask[p];
        if (tmask[pm] > 0.) s0max1 = fmaxd(field[pm], s0max1);
        if (tmask[pp] > 0.) s0max1 = fmaxd(field[pp], s0max1);
        s0max1 = s0max1 * st->sm[p];
        double slpmax = -st->s0[p] + s0max1;
        double s1max = 1.5 * slpmax;
        double s1new = fmind(s1max, fmaxd(-s1max, -A[p]));
        double s2new = fmind(slpmax + slpmax - 0.3334 * fabs(s1new), fmaxd(fabs(s1new) - slpmax, -AA[p]));
        C1[p] = -fmind(slpmax, fmaxd(-slpmax, -C1[p]));
        C2[p] = -fmind(slpmax, fmaxd(-slpmax, -C2[p]));
        A[p] = -s1new;
        AA[p] = -s2new;
        double s0min1 = field[p] * tmask[p];
        if (tmask[pm] > 0.) s0min1 = fmind(field[pm], s0min1);
        if (tmask[pp] > 0.) s0min1 = fmind(field[pp], s0min1);
        s0min1 = s0min1 * st->sm[p];
        slpmax = st->s0[p] - s0min1;
        s1max = 1.5 * slpmax;
        s1new = fmind(s1max, fmaxd(-s1max, A[p]));
        s2new = fmind(slpmax + slpmax - 0.3334 * fabs(s1new), fmaxd(fabs(s1new) - slpmax, AA[p]));
        C1[p] = fmind(slpmax, fmaxd(-slpmax, C1[p]));
        C2[p] = fmind(slpmax, fmaxd(-slpmax, C2[p]));
        A[p] = s1new;
        AA[p] = s2new;
      }
  }
  if (dir != 3) { /* Dom_flux full halo update of the four limited moments */
    orc_halo_update_3d(d, A, nk, 3);
    orc_halo_update_3d(d, AA, nk, 3);
    orc_halo_update_3d(d, C1, nk, 3);
    orc_halo_update_3d(d, C2, nk, 3);
  }
}

/* One face of a transport sweep.  Along the direction: a, aa (first and second
 * moment), cross moments c1 = (a x other1), c2 = (a x other2) with the other two
 * first moments b1, b2 and their second moments bb1, bb2, and the cross moment
 * between the two others bc.  fl[0..10] = f0, fa, faa, fb1, fb2, fc1, fc2, fbb1, fbb2, fbc, fm. */
enum { F0, FA, FAA, FB1, FB2, FC1, FC2, FBB1, FBB2, FBC, FM, NF };

static void psom_out(double velocity, double dv, double dtime, psom_state* st, size_t up, int sgn, const int* ix,
                     double* fl) {
  /* ix: indices of a, aa, b1, b2, c1, c2, bb1, bb2, bc in st->m */
  double *sm = st->sm, *s0 = st->s0;
  double *A = st->m[ix[0]], *AA = st->m[ix[1]], *B1 = st->m[ix[2]], *B2 = st->m[ix[3]];
  double *C1 = st->m[ix[4]], *C2 = st->m[ix[5]], *BB1 = st->m[ix[6]], *BB2 = st->m[ix[7]], *BC = st->m[ix[8]];
  fl[FM] = sgn > 0 ? velocity * dtime * dv : -velocity * dtime * dv;
  double alf = fl[FM] / (sm[up] + psom_epsln), alfq = alf * alf, alf1 = 1.0 - alf, alf1q = alf1 * alf1;
  if (sgn > 0) {
    fl[F0] = alf * (s0[up] + alf1 * (A[up] + (alf1 - alf) * AA[up]));
    fl[FA] = alfq * (A[up] + 3.0 * alf1 * AA[up]);
    fl[FB1] = alf * (B1[up] + alf1 * C1[up]);
    fl[FB2] = alf * (B2[up] + alf1 * C2[up]);
  } else {
    fl[F0] = alf * (s0[up] - alf1 * (A[up] - (alf1 - alf) * AA[up]));
    fl[FA] = alfq * (A[up] - 3.0 * alf1 * AA[up]);
    fl[FB1] = alf * (B1[up] - alf1 * C1[up]);
    fl[FB2] = alf * (B2[up] - alf1 * C2[up]);
  }
  fl[FAA] = alf * alfq * AA[up];
  fl[FC1] = alfq * C1[up];
  fl[FC2] = alfq * C2[up];
  fl[FBB1] = alf * BB1[up];
  fl[FBB2] = alf * BB2[up];
  fl[FBC] = alf * BC[up];
  sm[up] = sm[up] - fl[FM];
  s0[up] = s0[up] - fl[F0];
  if (sgn > 0) A[up] = alf1q * (A[up] - 3.0 * alf * AA[up]);
  else A[up] = alf1q * (A[up] + 3.0 * alf * AA[up]);
  AA[up] = alf1 * alf1q * AA[up];
  B1[up] = B1[up] - fl[FB1];
  BB1[up] = BB1[up] - fl[FBB1];
  B2[up] = B2[up] - fl[FB2];
  BB2[up] = BB2[up] - fl[FBB2];
  C1[up] = alf1q * C1[up];
  C2[up] = alf1q * C2[up];
  BC[up] = BC[up] - fl[FBC];
}

static void psom_in(psom_state* st, size_t dn, int sgn, const int* ix, const double* fl) {
  double *sm = st->sm, *s0 = st->s0;
  double *A = st->m[ix[0]], *AA = st->m[ix[1]], *B1 = st->m[ix[2]], *B2 = st->m[ix[3]];
  double *C1 = st->m[ix[4]], *C2 = st->m[ix[5]], *BB1 = st->m[ix[6]], *BB2 = st->m[ix[7]], *BC = st->m[ix[8]];
  sm[dn] = sm[dn] + fl[FM];
  double alf = fl[FM] / (sm[dn] + psom_epsln), alf1 = 1.0 - alf;
  if (sgn > 0) {
    double temptm = alf * s0[dn] - alf1 * fl[F0];
    s0[dn] = s0[dn] + fl[F0];
    AA[dn] = alf * alf * fl[FAA] + alf1 * alf1 * AA[dn] + 5.0 * (alf * alf1 * (A[dn] - fl[FA]) - (alf1 - alf) * temptm);
    A[dn] = alf * fl[FA] + alf1 * A[dn] + 3.0 * temptm;
    C1[dn] = alf * fl[FC1] + alf1 * C1[dn] + 3.0 * (-alf1 * fl[FB1] + alf * B1[dn]);
    C2[dn] = alf * fl[FC2] + alf1 * C2[dn] + 3.0 * (-alf1 * fl[FB2] + alf * B2[dn]);
  } else {
    double temptm = -alf * s0[dn] + alf1 * fl[F0];
    s0[dn] = s0[dn] + fl[F0];
    AA[dn] = alf * alf * fl[FAA] + alf1 * alf1 * AA[dn] + 5.0 * (alf * alf1 * (-A[dn] + fl[FA]) + (alf1 - alf) * temptm);
    A[dn] = alf * fl[FA] + alf1 * A[dn] + 3.0 * temptm;
    C1[dn] = alf * fl[FC1] + alf1 * C1[dn] + 3.0 * (alf1 * fl[FB1] - alf * B1[dn]);
    C2[dn] = alf * fl[FC2] + alf1 * C2[dn] + 3.0 * (alf1 * fl[FB2] - alf * B2[dn]);
  }
  B1[dn] = B1[dn] + fl[FB1];
  BB1[dn] = BB1[dn] + fl[FBB1];
  B2[dn] = B2[dn] + fl[FB2];
  BB2[dn] = BB2[dn] + fl[FBB2];
  BC[dn] = BC[dn] + fl[FBC];
}

/* moment roles per direction: along (a, aa), other firsts (b1, b2), cross (c1 = a*b1,
 * c2 = a*b2), other seconds (bb1, bb2), other cross (bc) */
static const int psom_roles[3][9] = {
    {P_SX, P_SXX, P_SY, P_SZ, P_SXY, P_SXZ, P_SYY, P_SZZ, P_SYZ}, /* psom_x */
    {P_SY, P_SYY, P_SX, P_SZ, P_SXY, P_SYZ, P_SXX, P_SZZ, P_SXZ}, /* psom_y */
    {P_SZ, P_SZZ, P_SX, P_SY, P_SXZ, P_SYZ, P_SXX, P_SYY, P_SXY}, /* psom_z */
};

/* Transport sweeps of one direction.  A face joins cell a (upstream when the
 * velocity is >= 0) and cell b: x (i, i+1), y (j, j+1), z (k+1, k) with k the
 * upper cell.  Outflow sweep over every face, halo update of the in-transit
 * moments (XUPDATE without fm in x, YUPDATE with fm in y, none in z), inflow
 * sweep in the same face order, full halo update. */
static void psom_sweep(const orc_dims* d, int dir, double dtime, const double* tmask, const double* dat,
                       const double* dxtn, const double* dyte, const double* uhrho_et, const double* vhrho_nt,
                       const double* wrho_bt, psom_state* st, double* flux, double* fb) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n3 = (size_t)NXD(d) * NYD(d) * nk;
  const int* ix = psom_roles[dir - 1];
  double dtimer = 1.0 / dtime, fl[NF];
  for (int pass = 0; pass < 2; ++pass) {
    if (dir == 3) {
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i)
          for (int kf = nk - 2; kf >= 0; --kf) {
            size_t pa = I3(d, i, j, kf + 1), pb = I3(d, i, j, kf), pf = I3(d, i, j, kf);
            double velocity = wrho_bt[I3(d, i, j, kf + 1)] * tmask[I3(d, i, j, kf + 1)];
            if (pass == 0) {
              if (velocity >= 0.0) {
                psom_out(velocity, dat[I2(d, i, j)], dtime, st, pa, 1, ix, fl);
                flux[pf] = fl[F0] * dtimer;
              } else {
                psom_out(velocity, dat[I2(d, i, j)], dtime, st, pb, -1, ix, fl);
                flux[pf] = -fl[F0] * dtimer;
              }
              for (int q = 0; q < NF; ++q) fb[q * n3 + pf] = fl[q];
            } else {
              for (int q = 0; q < NF; ++q) fl[q] = fb[q * n3 + pf];
              if (velocity >= 0.0) psom_in(st, pb, 1, ix, fl);
              else psom_in(st, pa, -1, ix, fl);
            }
          }
    } else {
      int i0 = dir == 1 ? 0 : 1, j0 = dir == 2 ? 0 : 1;
      for (int k = 0; k < nk; ++k)
        for (int j = j0; j <= nj; ++j)
          for (int i = i0; i <= ni; ++i) {
            size_t pa = I3(d, i, j, k), pf = pa;
            size_t pb = dir == 1 ? I3(d, i + 1, j, k) : I3(d, i, j + 1, k);
            double velocity, dv;
            if (dir == 1) {
              velocity = uhrho_et[pa] * fmind(tmask[pa], tmask[pb]);
              dv = dyte[I2(d, i, j)];
            } else {
              velocity = vhrho_nt[pa] * fmind(tmask[pa], tmask[pb]);
              dv = dxtn[I2(d, i, j)];
            }
            if (pass == 0) {
              if (velocity >= 0.0) {
                psom_out(velocity, dv, dtime, st, pa, 1, ix, fl);
                flux[pf] = fl[F0] * dtimer;
              } else {
                psom_out(velocity, dv, dtime, st, pb, -1, ix, fl);
                flux[pf] = -fl[F0] * dtimer;
              }
              for (int q = 0; q < NF; ++q) fb[q * n3 + pf] = fl[q];
            } else {
              for (int q = 0; q < NF; ++q) fl[q] = fb[q * n3 + pf];
              if (velocity >= 0.0) psom_in(st, pb, 1, ix, fl);
              else psom_in(st, pa, -1, ix, fl);
            }
          }
    }
    if (pass == 0 && dir != 3) {
      int fl_flag = dir == 1 ? 1 : 2;
      for (int q = 0; q < NF; ++q)
        if (q != FM || dir == 2) orc_halo_update_3d(d, fb + q * n3, nk, fl_flag);
      orc_halo_update_3d(d, flux, nk, fl_flag);
      orc_halo_update_3d(d, st->sm, nk, fl_flag);
      orc_halo_update_3d(d, st->s0, nk, fl_flag);
      for (int q = 0; q < P_N; ++q) orc_halo_update_3d(d, st->m[q], nk, fl_flag);
    }
  }
  psom_full_update(d, st);
}

/* mom: the nine moments sx, sxx, sy, syy, sz, szz, sxy, sxz, syz (each data-domain
 * sized, in/out); s0: out; rho_dzt and field at taum1. */
void orc_advect_psom(const orc_dims* d, long itt0, int limit, int prather, double dtime, const double* tmask,
                     const double* dat, const double* datr, const double* dxtn, const double* dyte,
                     const double* uhrho_et, const double* vhrho_nt, const double* wrho_bt, const double* rho_dzt,
                     const double* field, double* s0, double* mom, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d), n3 = n2 * nk;
  psom_state st;
  st.sm = (double*)calloc(n3, sizeof(double));
  st.s0 = s0;
  for (int q = 0; q < P_N; ++q) st.m[q] = mom + q * n3;
  double* fx = (double*)calloc(n3, sizeof(double));
  double* fy = (double*)calloc(n3, sizeof(double));
  double* fz = (double*)calloc(n3, sizeof(double));
  double* fb = (double*)calloc(NF * n3, sizeof(double));
  for (int k = 0; k < nk; ++k)
    for (int j = 0; j <= nj + 1; ++j)
      for (int i = 0; i <= ni + 1; ++i) {
        size_t p = I3(d, i, j, k);
        st.sm[p] = rho_dzt[p] * dat[I2(d, i, j)];
        s0[p] = field[p] * st.sm[p] * tmask[p];
      }
  static const int order[6][3] = {{1, 2, 3}, {3, 1, 2}, {2, 3, 1}, {1, 3, 2}, {2, 1, 3}, {3, 2, 1}};
  const int* o = order[itt0 % 6];
  for (int s = 0; s < 3; ++s) {
    int dir = o[s];
    if (limit) {
      if (dir == 1) psom_limit(d, prather, 1, tmask, field, &st, P_SX, P_SXX, P_SXY, P_SXZ);
      else if (dir == 2) psom_limit(d, prather, 2, tmask, field, &st, P_SY, P_SYY, P_SXY, P_SYZ);
      else psom_limit(d, prather, 3, tmask, field, &st, P_SZ, P_SZZ, P_SXZ, P_SYZ);
    }
    double* flux = dir == 1 ? fx : dir == 2 ? fy : fz;
    psom_sweep(d, dir, dtime, tmask, dat, dxtn, dyte, uhrho_et, vhrho_nt, wrho_bt, &st, flux, fb);
  }
  memset(wrk1, 0, sizeof(double) * n3);
  for (int j = 1; j <= nj; ++j)
    for (int i = 1; i <= ni; ++i) {
      double ft1 = 0.0;
      for (int k = 0; k < nk; ++k) {
        size_t p = I3(d, i, j, k);
        double fzk = k < nk - 1 ? fz[p] : 0.0; /* flux_z = 0 on entry; the bottom face is never written */
        double advect = tmask[p] * (fx[p] - fx[I3(d, i - 1, j, k)] + fy[p] - fy[I3(d, i, j - 1, k)] + ft1 - fzk) *
                        datr[I2(d, i, j)];
        wrk1[p] = -advect;
        ft1 = fzk;
      }
    }
  free(st.sm);
  free(fx);
  free(fy);
  free(fz);
  free(fb);
}

/* ------------------------------------------------------------------------- */
/* MDFL Super-B: advect_tracer_mdfl_sup_b (ocean_tracer_advect.F90:3189-3466),*/
/* split level by level: z flux on the tracer, update, halo update of the    */
/* level, x fluxes on the z-updated level, update, halo update, y fluxes,    */
/* update, divergence correction.  Superbee limiter on Cr = R/Rj (R*1e20 for */
/* Rj = 0).  tmask_mdfl is the halo-2 mask.  Returns wrk1 = -advect.        */
/* ------------------------------------------------------------------------- */
static double superbee(double Cr) { return fmaxd(0.0, fmaxd(fmind(1.0, 2.0 * Cr), fmind(2.0, Cr))); }

void orc_advect_mdfl_sup_b(const orc_dims* d, double dtime, const double* tmask, const double* dat,
                           const double* datr, const double* dxte, const double* dyte, const double* dxtn,
                           const double* dytn, const double* uhrho_et, const double* vhrho_nt, const double* wrho_bt,
                           const double* rho_dzt, const double* T, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d), n3 = n2 * nk;
  double* mk = (double*)calloc((size_t)NX2(d) * NY2(d) * nk, sizeof(double)); /* tmask_mdfl, halo 2 */
  orc_mask_halo2(d, tmask, mk);
#define TM2(i, j, k) mk[H3(d, i, j, k)]
  double* ftp = (double*)calloc(n2, sizeof(double));
  double* wkm1 = (double*)calloc(n2, sizeof(double));
  double* tz = (double*)calloc(n2, sizeof(double)); /* tmp_updated_tracer, one level */
  double* tx = (double*)calloc(n2, sizeof(double));
  double* fe = (double*)calloc(n2, sizeof(double));
  double* fn = (double*)calloc(n2, sizeof(double));
  memset(wrk1, 0, sizeof(double) * n3);
  for (int k = 0; k < nk; ++k) {
    int kp1 = k + 1 < nk ? k + 1 : nk - 1, kp2 = k + 2 < nk ? k + 2 : nk - 1, km1 = k > 0 ? k - 1 : 0;
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        size_t q = I2(d, i, j);
        double Tk = T[I3(d, i, j, k)], Tkp1 = T[I3(d, i, j, kp1)];
        double Rjp = (T[I3(d, i, j, km1)] - Tk) * TM2(i, j, km1) * TM2(i, j, k);
        double Rj = (Tk - Tkp1) * TM2(i, j, k) * TM2(i, j, kp1);
        double Rjm = (Tkp1 - T[I3(d, i, j, kp2)]) * TM2(i, j, kp1) * TM2(i, j, kp2);
        double w = wrho_bt[I3(d, i, j, k + 1)];
        double massflux = dat[q] * w;
        double cfl = fabs(w * dtime / rho_dzt[I3(d, i, j, k)]);
        double Cr;
        if (Rj != 0.0) Cr = massflux > 0.0 ? Rjm / Rj : Rjp / Rj;
        else Cr = massflux > 0.0 ? Rjm * 1.0e20 : Rjp * 1.0e20;
        Cr = superbee(Cr);
        double fbt = 0.5 * (massflux * (Tk + Tkp1) - fabs(massflux) * (1.0 + (cfl - 1) * Cr) * Rj) *
                     TM2(i, j, kp1) * TM2(i, j, k);
        tz[q] = Tk + dtime / rho_dzt[I3(d, i, j, k)] * (datr[q] * (fbt - ftp[q]) + Tk * (wkm1[q] - w));
        ftp[q] = fbt;
      }
    /* halo update of the level: periodic image of the compute values, else the
     * (zero) halo the array was created with */
#define HV(a, i, j) halo_value2d(d, a, i, j)
    for (int j = 1; j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        double Rjp = (HV(tz, i + 2, j) - HV(tz, i + 1, j)) * TM2(i + 2, j, k) * TM2(i + 1, j, k);
        double Rj = (HV(tz, i + 1, j) - HV(tz, i, j)) * TM2(i + 1, j, k) * TM2(i, j, k);
        double Rjm = (HV(tz, i, j) - HV(tz, i - 1, j)) * TM2(i, j, k) * TM2(i - 1, j, k);
        double u = uhrho_et[I3(d, i, j, k)];
        double massflux = dyte[I2(d, i, j)] * u;
        double cfl = fabs(u * dtime * 2.0 / ((rho_dzt[I3(d, i, j, k)] + rho_dzt[I3(d, i + 1, j, k)]) * dxte[I2(d, i, j)]));
        double Cr;
        if (Rj != 0.0) Cr = massflux > 0.0 ? Rjm / Rj : Rjp / Rj;
        else Cr = massflux > 0.0 ? Rjm * 1.0e20 : Rjp * 1.0e20;
        Cr = superbee(Cr);
        fe[I2(d, i, j)] = 0.5 * (massflux * (HV(tz, i + 1, j) + HV(tz, i, j)) -
                                 fabs(massflux) * (1.0 + (cfl - 1) * Cr) * Rj) *
                          TM2(i, j, k) * TM2(i + 1, j, k);
      }
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        size_t q = I2(d, i, j);
        size_t p = I3(d, i, j, k);
        tx[q] = tz[q] + dtime * TM2(i, j, k) * datr[q] / rho_dzt[p] *
                            (fe[I2(d, i - 1, j)] - fe[q] +
                             T[p] * (dyte[q] * uhrho_et[p] - dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)]));
      }
    for (int j = 0; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double Rjp = (HV(tx, i, j + 2) - HV(tx, i, j + 1)) * TM2(i, j + 2, k) * TM2(i, j + 1, k);
        double Rj = (HV(tx, i, j + 1) - HV(tx, i, j)) * TM2(i, j + 1, k) * TM2(i, j, k);
        double Rjm = (HV(tx, i, j) - HV(tx, i, j - 1)) * TM2(i, j, k) * TM2(i, j - 1, k);
        double v = vhrho_nt[I3(d, i, j, k)];
        double massflux = dxtn[I2(d, i, j)] * v;
        double cfl = fabs(v * dtime * 2.0 / ((rho_dzt[I3(d, i, j, k)] + rho_dzt[I3(d, i, j + 1, k)]) * dytn[I2(d, i, j)]));
        double Cr;
        if (Rj != 0.0) Cr = massflux > 0.0 ? Rjm / Rj : Rjp / Rj;
        else Cr = massflux > 0.0 ? Rjm * 1.0e20 : Rjp * 1.0e20;
        Cr = superbee(Cr);
        fn[I2(d, i, j)] = 0.5 * (massflux * (HV(tx, i, j + 1) + HV(tx, i, j)) -
                                 fabs(massflux) * (1.0 + (cfl - 1.0) * Cr) * Rj) *
                          TM2(i, j, k) * TM2(i, j + 1, k);
      }
#undef HV
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        size_t q = I2(d, i, j);
        size_t p = I3(d, i, j, k);
        double t = tx[q] + dtime * tmask[p] * datr[q] / rho_dzt[p] * (fn[I2(d, i, j - 1)] - fn[q]);
        t = t + dtime * T[p] / rho_dzt[p] *
                    (wrho_bt[I3(d, i, j, k + 1)] - wkm1[q] +
                     datr[q] * ((dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)] - dyte[q] * uhrho_et[p])));
        double advect = -rho_dzt[p] * (t - T[p]) / dtime * TM2(i, j, k);
        wrk1[p] = -advect;
        wkm1[q] = wrho_bt[I3(d, i, j, k + 1)];
      }
  }
#undef TM2
  free(mk);
  free(ftp);
  free(wkm1);
  free(tz);
  free(tx);
  free(fe);
  free(fn);
}

/* ------------------------------------------------------------------------- */
/* MDPPM: advect_tracer_mdppm (ocean_tracer_advect.F90:5990-6507) with the   */
/* edge limiters ppm_limit_cw84 (:6510-6538), ppm_limit_ifc (:6555-6580) and */
/* ppm_limit_sh (:6601-6660) selected by ppm_hlimiter (1, 2, 3) for all      */
/* three directions, as the reference does; tracer_mdppm and tmask_mdppm     */
/* carry a halo of 4 (mdppm_init :1702-1735).  Returns wrk1 = -advect.       */
/* ------------------------------------------------------------------------- */
static const double ppm_r12 = 1.0 / 12.0, ppm_sixth = 1.0 / 6.0, ppm_2_3 = 2.0 / 3.0, ppm_4_3 = 4.0 / 3.0;

static double fmax3(double a, double b, double c) { return fmaxd(fmaxd(a, b), c); }
static double fmin3(double a, double b, double c) { return fmind(fmind(a, b), c); }
static double fmax4(double a, double b, double c, double e) { return fmaxd(fmaxd(fmaxd(a, b), c), e); }
static double fmin4(double a, double b, double c, double e) { return fmind(fmind(fmind(a, b), c), e); }

/* slope da (Lin 1994 B2 with the masked 3rd/2nd-order estimate) and the differences d1* of cell S[2] */
static void ppm_slope(const double* S, const double* M, double* da, double* d1m, double* d1p, double* d1mm,
                      double* d1pp) {
  /* S, M: values at offsets -2..+2 (index 0..4); M already includes the level-collapse factors */
  double Sim2 = S[0], Sim1 = S[1], Si = S[2], Sip1 = S[3], Sip2 = S[4];
  double mskm2 = M[0], mskm1 = M[1], msk0 = M[2], mskp1 = M[3], mskp2 = M[4];
  double da2 = 0.5 * (Sip1 - Sim1);
  double da3m = ppm_r12 * (2. * Sim2 - 12. * Sim1 + 6. * Si + 4. * Sip1);
  double da3p = ppm_r12 * (-(4. * Sim1) - 6. * Si + 12. * Sip1 - 2. * Sip2);
  double a = ((mskm2 * (1. - 0.5 * mskp2) * da3m + mskp2 * (1. - 0.5 * mskm2) * da3p) +
              (1. - mskm2) * (1. - mskp2) * da2);
  double dMx = fmax3(Sip1, Sim1, Si) - Si;
  double dMn = Si - fmin3(Sip1, Sim1, Si);
  *da = copysign(1., a) * fmind(fabs(a), 2. * fmind(dMx, dMn)) * mskm1 * mskp1 * msk0;
  *d1m = (Si - Sim1) * mskm1;
  *d1p = (Sip1 - Si) * mskp1;
  *d1mm = (Sim1 - Sim2) * mskm1 * mskm2;
  *d1pp = (Sip2 - Sip1) * mskp1 * mskp2;
}

static void ppm_limit(int lim, double Si, double da, double d1m, double d1p, double d1mm, double d1pp, double* aL,
                      double* aR) {
  if (lim == 1) { /* Colella and Woodward 1984, Eq. 1.10 */
    if ((*aR - Si) * (Si - *aL) <= 0.) {
      *aL = Si;
      *aR = Si;
    }
    double da2 = *aR - *aL, da4 = 0.5 * (*aR + *aL);
    double da3m = 6. * da2 * (Si - da4), da3p = da2 * da2;
    if (da3m > da3p) *aL = 3. * Si - 2. * *aR;
    if (da3m < -da3p) *aR = 3. * Si - 2. * *aL;
  } else if (lim == 2) { /* improved full constraint, Lin 2004 */
    double ada = fabs(da), sda = copysign(1., da);
    *aL = Si - sda * fmind(ada, fabs(*aL - Si));
    *aR = Si + sda * fmind(ada, fabs(*aR - Si));
  } else { /* Suresh and Huynh 1997 */
    double Sim1 = Si - d1m, Sip1 = Si + d1p;
    double z = d1m - d1mm, w = d1p - d1m;
    double x = 4. * w - z, y = 4. * z - w;
    double dM4m = fmaxd(0., fmin4(x, y, z, w)) + fmind(0., fmax4(x, y, z, w));
    z = d1pp - d1p;
    x = 4. * w - z;
    y = 4. * z - w;
    double dM4p = fmaxd(0., fmin4(x, y, z, w)) + fmind(0., fmax4(x, y, z, w));
    double qAV = 0.5 * (Si + Sip1);
    x = d1p;
    y = 3. * d1m;
    double qMP = Si + fmaxd(0., fmind(x, y)) + fmind(0., fmaxd(x, y));
    double qUL = Si + y;
    double qLC = (Si + 0.5 * d1m) + ppm_4_3 * dM4m;
    double qMD = qAV - 0.5 * dM4p;
    double qMin = fmaxd(fmin3(qMD, Si, Sip1), fmin3(Si, qUL, qLC));
    double qMax = fmind(fmax3(qMD, Si, Sip1), fmax3(Si, qUL, qLC));
    if ((*aR - Si) * (*aR - qMP) > 1.e-10) *aR = fmind(fmaxd(*aR, qMin), qMax);
    qAV = 0.5 * (Si + Sim1);
    x = -d1m;
    y = -3. * d1p;
    qMP = Si + fmaxd(0., fmind(x, y)) + fmind(0., fmaxd(x, y));
    qUL = Si + y;
    qLC = (Si - 0.5 * d1p) + ppm_4_3 * dM4p;
    qMD = qAV - 0.5 * dM4m;
    qMin = fmaxd(fmin3(qMD, Si, Sim1), fmin3(Si, qUL, qLC));
    qMax = fmind(fmax3(qMD, Si, Sim1), fmax3(Si, qUL, qLC));
    if ((*aL - Si) * (*aL - qMP) > 1.e-10) *aL = fmind(fmaxd(*aL, qMin), qMax);
  }
}

/* edge values, limited, and the curvature of a line of cells; S and M are indexed by
 * position p = 0..n-1 with a 4-cell margin at each end; results for p = 3..n-4 */
static void ppm_line(int n, int lim, const double* S, const double* M, double* aL, double* aR, double* a6) {
  double *da = calloc(n, sizeof(double)), *d1m = calloc(n, sizeof(double)), *d1p = calloc(n, sizeof(double));
  double *d1mm = calloc(n, sizeof(double)), *d1pp = calloc(n, sizeof(double));
  for (int q = 2; q < n - 2; ++q) ppm_slope(S + q - 2, M + q - 2, &da[q], &d1m[q], &d1p[q], &d1mm[q], &d1pp[q]);
  for (int q = 3; q < n - 3; ++q) {
    double Si = S[q], Sim1 = Si - d1m[q], Sip1 = Si + d1p[q];
    aL[q] = 0.5 * (Sim1 + Si) + ppm_sixth * (da[q - 1] - da[q]);
    aR[q] = 0.5 * (Si + Sip1) + ppm_sixth * (da[q] - da[q + 1]);
    ppm_limit(lim, Si, da[q], d1m[q], d1p[q], d1mm[q], d1pp[q], &aL[q], &aR[q]);
    a6[q] = 6. * Si - 3. * (aR[q] + aL[q]);
  }
  free(da);
  free(d1m);
  free(d1p);
  free(d1mm);
  free(d1pp);
}

void orc_advect_mdppm(const orc_dims* d, int lim, double dtime, const double* tmask, const double* dat,
                      const double* datr, const double* dxte, const double* dyte, const double* dxtn,
                      const double* dytn, const double* uhrho_et, const double* vhrho_nt, const double* wrho_bt,
                      const double* rho_dzt, const double* T, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d), n3 = n2 * nk;
  double* tm = (double*)malloc(sizeof(double) * n3); /* tracer_mdppm on the compute domain (+ halo by image) */
  double* fz = (double*)calloc(n3, sizeof(double));
  memset(wrk1, 0, sizeof(double) * n3);
  memcpy(tm, T, sizeof(double) * n3);
#define W(i, j, K) wrho_bt[I3(d, i, j, K)] /* Fortran face index K = 0..nk */
#define MK(i, j, K) tmask[I3(d, i, j, (K) - 1)] /* Fortran level K = 1..nk */
#define TV(i, j, K) T[I3(d, i, j, (K) - 1)]
  int L = nk + 8;
  double *S = calloc(L, sizeof(double)), *M = calloc(L, sizeof(double));
  double *aL = calloc(L, sizeof(double)), *aR = calloc(L, sizeof(double)), *a6 = calloc(L, sizeof(double));
  double* dak = calloc(L, sizeof(double));
  /* ---- vertical ---- */
  for (int j = 1; j <= nj; ++j)
    for (int i = 1; i <= ni; ++i) {
      /* slopes dak(k) for all k (:6064-6099); positions q = K + 3 */
      for (int K = 1; K <= nk; ++K) {
        int km2 = K - 2 > 1 ? K - 2 : 1, km1 = K - 1 > 1 ? K - 1 : 1, kp1 = K + 1 < nk ? K + 1 : nk,
            kp2 = K + 2 < nk ? K + 2 : nk;
        double Sv[5] = {TV(i, j, km2), TV(i, j, km1), TV(i, j, K), TV(i, j, kp1), TV(i, j, kp2)};
        double Mv[5] = {MK(i, j, km2) * (double)(km1 - km2), MK(i, j, km1) * (double)(K - km1), MK(i, j, K),
                        MK(i, j, kp1) * (double)(kp1 - K), MK(i, j, kp2) * (double)(kp2 - kp1)};
        double t0, t1, t2, t3;
        ppm_slope(Sv, Mv, &dak[K], &t0, &t1, &t2, &t3);
      }
      for (int K = 1; K <= nk; ++K) {
        int km2 = K - 2 > 1 ? K - 2 : 1, km1 = K - 1 > 1 ? K - 1 : 1, kp1 = K + 1 < nk ? K + 1 : nk,
            kp2 = K + 2 < nk ? K + 2 : nk;
        double mskp2 = MK(i, j, kp2) * (double)(kp2 - kp1), mskp1 = MK(i, j, kp1) * (double)(kp1 - K);
        double msk0 = MK(i, j, K), mskm1 = MK(i, j, km1) * (double)(K - km1);
        double mskm2 = MK(i, j, km2) * (double)(km1 - km2);
        double Sip2 = TV(i, j, kp2), Sip1 = TV(i, j, kp1), Si = TV(i, j, K), Sim1 = TV(i, j, km1),
               Sim2 = TV(i, j, km2);
        double d1m = (Si - Sim1) * mskm1, d1p = (Sip1 - Si) * mskp1;
        double d1mm = (Sim1 - Sim2) * mskm1 * mskm2, d1pp = (Sip2 - Sip1) * mskp1 * mskp2;
        Sim1 = Si - d1m;
        Sip1 = Si + d1p;
        double al = 0.5 * (Sim1 + Si) + ppm_sixth * (dak[km1] - dak[K]);
        double ar = 0.5 * (Si + Sip1) + ppm_sixth * (dak[K] - dak[kp1]);
        ppm_limit(lim, Si, dak[K], d1m, d1p, d1mm, d1pp, &al, &ar);
        double c6 = 6. * Si - 3. * (ar + al);
        double massflux = dat[I2(d, i, j)] * W(i, j, K) * msk0 * mskp1;
        if (massflux <= 0.0) {
          double cfl = fabs(W(i, j, K) * dtime / rho_dzt[I3(d, i, j, K - 1)]);
          fz[I3(d, i, j, K - 1)] = massflux * (ar + 0.5 * cfl * ((al - ar) + (1. - ppm_2_3 * cfl) * c6));
        }
        massflux = dat[I2(d, i, j)] * W(i, j, km1) * msk0 * mskm1;
        if (massflux > 0.0) {
          double cfl = fabs(W(i, j, km1) * dtime / rho_dzt[I3(d, i, j, km1 - 1)]);
          fz[I3(d, i, j, km1 - 1)] = massflux * (al + 0.5 * cfl * ((ar - al) + (1. - ppm_2_3 * cfl) * c6));
        }
      }
      for (int K = 1; K <= nk; ++K) {
        int km1 = K - 1 > 1 ? K - 1 : 1;
        double mskm1 = (double)(K - km1);
        size_t p = I3(d, i, j, K - 1);
        tm[p] = tm[p] + dtime / rho_dzt[p] *
                            (datr[I2(d, i, j)] * (fz[p] - mskm1 * fz[I3(d, i, j, km1 - 1)]) +
                             T[p] * (mskm1 * W(i, j, km1) - W(i, j, K)));
      }
    }
  /* ---- x: lines along i of compute rows, halo of 4 by image (XUPDATE) ---- */
  int Lx = ni + 8;
  double *Sx = calloc(Lx, sizeof(double)), *Mx = calloc(Lx, sizeof(double)), *fx = calloc(Lx, sizeof(double));
  double *aLx = calloc(Lx, sizeof(double)), *aRx = calloc(Lx, sizeof(double)), *a6x = calloc(Lx, sizeof(double));
  double* tx = (double*)malloc(sizeof(double) * n3);
  memcpy(tx, tm, sizeof(double) * n3);
  for (int k = 0; k < nk; ++k)
    for (int j = 1; j <= nj; ++j) {
      for (int q = 0; q < Lx; ++q) { /* position q <-> i = q - 3 */
        Sx[q] = halo_value(d, tm, q - 3, j, k);
        Mx[q] = halo_value(d, tmask, q - 3, j, k);
      }
      ppm_line(Lx, lim, Sx, Mx, aLx, aRx, a6x);
      for (int i = 0; i <= ni; ++i) { /* face i+1/2, q = i + 3 */
        int q = i + 3;
        double u = uhrho_et[I3(d, i, j, k)];
        double massflux = dyte[I2(d, i, j)] * u;
        double cfl = u * dtime * 2.0 / ((rho_dzt[I3(d, i, j, k)] + rho_dzt[I3(d, i + 1, j, k)]) * dxte[I2(d, i, j)]);
        if (massflux >= 0.0)
          fx[q] = massflux * Mx[q] * Mx[q + 1] *
                  (aRx[q] + 0.5 * cfl * ((aLx[q] - aRx[q]) + (1. - ppm_2_3 * cfl) * a6x[q]));
        else
          fx[q] = massflux * Mx[q] * Mx[q + 1] *
                  (aLx[q + 1] - 0.5 * cfl * ((aRx[q + 1] - aLx[q + 1]) + (1. + ppm_2_3 * cfl) * a6x[q + 1]));
      }
      for (int i = 1; i <= ni; ++i) {
        size_t p = I3(d, i, j, k);
        int q = i + 3;
        tx[p] = tm[p] + dtime * Mx[q] * datr[I2(d, i, j)] / rho_dzt[p] *
                            (fx[q - 1] - fx[q] +
                             T[p] * (dyte[I2(d, i, j)] * uhrho_et[p] - dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)]));
      }
    }
  /* ---- y: lines along j of compute columns, halo of 4 by image (YUPDATE) ---- */
  int Ly = nj + 8;
  double *Sy = calloc(Ly, sizeof(double)), *My = calloc(Ly, sizeof(double)), *fy = calloc(Ly, sizeof(double));
  double *aLy = calloc(Ly, sizeof(double)), *aRy = calloc(Ly, sizeof(double)), *a6y = calloc(Ly, sizeof(double));
  for (int k = 0; k < nk; ++k)
    for (int i = 1; i <= ni; ++i) {
      for (int q = 0; q < Ly; ++q) {
        Sy[q] = halo_value(d, tx, i, q - 3, k);
        My[q] = halo_value(d, tmask, i, q - 3, k);
      }
      ppm_line(Ly, lim, Sy, My, aLy, aRy, a6y);
      for (int j = 0; j <= nj; ++j) {
        int q = j + 3;
        double v = vhrho_nt[I3(d, i, j, k)];
        double massflux = dxtn[I2(d, i, j)] * v;
        double cfl = v * dtime * 2.0 / ((rho_dzt[I3(d, i, j, k)] + rho_dzt[I3(d, i, j + 1, k)]) * dytn[I2(d, i, j)]);
        if (massflux >= 0.0)
          fy[q] = massflux * My[q] * My[q + 1] *
                  (aRy[q] + 0.5 * cfl * ((aLy[q] - aRy[q]) + (1. - 2. / 3. * cfl) * a6y[q]));
        else
          fy[q] = massflux * My[q] * My[q + 1] *
                  (aLy[q + 1] - 0.5 * cfl * ((aRy[q + 1] - aLy[q + 1]) + (1. + 2. / 3. * cfl) * a6y[q + 1]));
      }
      for (int j = 1; j <= nj; ++j) {
        size_t p = I3(d, i, j, k);
        int q = j + 3;
        double t = tx[p] + dtime * tmask[p] * datr[I2(d, i, j)] / rho_dzt[p] * (fy[q - 1] - fy[q]);
        double wkm1 = k > 0 ? wrho_bt[I3(d, i, j, k)] : 0.0;
        t = t + dtime * T[p] / rho_dzt[p] *
                    (wrho_bt[I3(d, i, j, k + 1)] - wkm1 +
                     datr[I2(d, i, j)] * ((dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)] -
                                           dyte[I2(d, i, j)] * uhrho_et[p])));
        double advect = -rho_dzt[p] * (t - T[p]) / dtime * My[q];
        wrk1[p] = -advect;
      }
    }
#undef W
#undef MK
#undef TV
  free(tm);
  free(tx);
  free(fz);
  free(S);
  free(M);
  free(aL);
  free(aR);
  free(a6);
  free(dak);
  free(Sx);
  free(Mx);
  free(fx);
  free(aLx);
  free(aRx);
  free(a6x);
  free(Sy);
  free(My);
  free(fy);
  free(aLy);
  free(aRy);
  free(a6y);
}

/* ------------------------------------------------------------------------- */
/* Quicker: quicker_init :1442-1586, horz :2538-2653, vert :2981-3031.       */
/* Weight arrays are data-domain 2-D arrays with a trailing component index: */
/* quick_x(·,·,2), curv_xp(·,·,3) ...; quick_z(nk,2), curv_zp(nk,3).         */
/* ------------------------------------------------------------------------- */
typedef struct {
  double *quick_x, *quick_y, *curv_xp, *curv_xn, *curv_yp, *curv_yn; /* data domain × 2 or × 3 */
  double *quick_z, *curv_zp, *curv_zn;                                /* nk × 2 or nk × 3 (k fastest) */
  double *tmask_quick;                                                /* halo-2 array */
} orc_quicker;

/* 2-D halo-2 index */
#define H2(d, i, j) ((size_t)((j) + 1) * NX2(d) + (size_t)((i) + 1))

void orc_quicker_init(const orc_dims* d, const double* dxt, const double* dyt, const double* dzt,
                      const double* tmask, orc_quicker* q) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  memset(q->quick_x, 0, sizeof(double) * n2 * 2);
  memset(q->quick_y, 0, sizeof(double) * n2 * 2);
  memset(q->curv_xp, 0, sizeof(double) * n2 * 3);
  memset(q->curv_xn, 0, sizeof(double) * n2 * 3);
  memset(q->curv_yp, 0, sizeof(double) * n2 * 3);
  memset(q->curv_yn, 0, sizeof(double) * n2 * 3);
  orc_mask_halo2(d, tmask, q->tmask_quick);

  size_t nh = (size_t)NX2(d) * NY2(d);
  double* dxq = (double*)calloc(nh, sizeof(double));
  double* dyq = (double*)calloc(nh, sizeof(double));
  for (int i = 1; i <= ni; ++i)
    for (int j = 1; j <= nj; ++j) {
      dxq[H2(d, i, j)] = dxt[I2(d, i, j)];
      dyq[H2(d, i, j)] = dyt[I2(d, i, j)];
    }
  /* boundary fill (:1489-1507): x-halo columns replicate isc / iec; dxt only
   * for the compute rows, dyt for all rows; then the y-halo rows replicate
   * jsc / jec over the whole (halo-2) row. */
  for (int i = -1; i <= 0; ++i) {
    for (int j = 1; j <= nj; ++j) dxq[H2(d, i, j)] = dxq[H2(d, 1, j)];
    for (int j = -1; j <= nj + 2; ++j) dyq[H2(d, i, j)] = dyq[H2(d, 1, j)];
  }
  for (int i = ni + 1; i <= ni + 2; ++i) {
    for (int j = 1; j <= nj; ++j) dxq[H2(d, i, j)] = dxq[H2(d, ni, j)];
    for (int j = -1; j <= nj + 2; ++j) dyq[H2(d, i, j)] = dyq[H2(d, ni, j)];
  }
  for (int j = -1; j <= 0; ++j)
    for (int i = -1; i <= ni + 2; ++i) {
      dxq[H2(d, i, j)] = dxq[H2(d, i, 1)];
      dyq[H2(d, i, j)] = dyq[H2(d, i, 1)];
    }
  for (int j = nj + 1; j <= nj + 2; ++j)
    for (int i = -1; i <= ni + 2; ++i) {
      dxq[H2(d, i, j)] = dxq[H2(d, i, nj)];
      dyq[H2(d, i, j)] = dyq[H2(d, i, nj)];
    }
  /* mpp_update_domains(dxt_quick / dyt_quick) with halo 2 (:1508-1509) */
  {
    orc_dims d1 = *d;
    d1.nk = 1;
    halo2_update(&d1, dxq, 3);
    halo2_update(&d1, dyq, 3);
  }
#define DX(i, j) dxq[H2(d, (i), (j))]
#define DY(i, j) dyq[H2(d, (i), (j))]
#define W2(a, i, j, m) (a)[(size_t)(m) * n2 + I2(d, (i), (j))]
  for (int i = 0; i <= ni; ++i)
    for (int j = 0; j <= nj; ++j) {
      W2(q->quick_x, i, j, 0) = DX(i + 1, j) / (DX(i + 1, j) + DX(i, j));
      W2(q->quick_x, i, j, 1) = DX(i, j) / (DX(i + 1, j) + DX(i, j));
      W2(q->quick_y, i, j, 0) = DY(i, j + 1) / (DY(i, j + 1) + DY(i, j));
      W2(q->quick_y, i, j, 1) = DY(i, j) / (DY(i, j + 1) + DY(i, j));

      W2(q->curv_xp, i, j, 0) =
          DX(i, j) * DX(i + 1, j) / ((DX(i - 1, j) + 2.0 * DX(i, j) + DX(i + 1, j)) * (DX(i, j) + DX(i + 1, j)));
      W2(q->curv_xp, i, j, 1) =
          -DX(i, j) * DX(i + 1, j) / ((DX(i, j) + DX(i + 1, j)) * (DX(i - 1, j) + DX(i, j)));
      W2(q->curv_xp, i, j, 2) =
          DX(i, j) * DX(i + 1, j) / ((DX(i - 1, j) + 2.0 * DX(i, j) + DX(i + 1, j)) * (DX(i - 1, j) + DX(i, j)));

      W2(q->curv_xn, i, j, 0) = DX(i, j) * DX(i + 1, j) /
                                ((DX(i, j) + 2.0 * DX(i + 1, j) + DX(i + 2, j)) * (DX(i + 1, j) + DX(i + 2, j)));
      W2(q->curv_xn, i, j, 1) =
          -DX(i, j) * DX(i + 1, j) / ((DX(i + 1, j) + DX(i + 2, j)) * (DX(i, j) + DX(i + 1, j)));
      W2(q->curv_xn, i, j, 2) =
          DX(i, j) * DX(i + 1, j) / ((DX(i, j) + 2.0 * DX(i + 1, j) + DX(i + 2, j)) * (DX(i, j) + DX(i + 1, j)));

      W2(q->curv_yp, i, j, 0) =
          DY(i, j) * DY(i, j + 1) / ((DY(i, j - 1) + 2.0 * DY(i, j) + DY(i, j + 1)) * (DY(i, j) + DY(i, j + 1)));
      W2(q->curv_yp, i, j, 1) =
          -DY(i, j) * DY(i, j + 1) / ((DY(i, j) + DY(i, j + 1)) * (DY(i, j - 1) + DY(i, j)));
      W2(q->curv_yp, i, j, 2) =
          DY(i, j) * DY(i, j + 1) / ((DY(i, j - 1) + 2.0 * DY(i, j) + DY(i, j + 1)) * (DY(i, j - 1) + DY(i, j)));

      W2(q->curv_yn, i, j, 0) = DY(i, j) * DY(i, j + 1) /
                                ((DY(i, j) + 2.0 * DY(i, j + 1) + DY(i, j + 2)) * (DY(i, j + 1) + DY(i, j + 2)));
      W2(q->curv_yn, i, j, 1) =
          -DY(i, j) * DY(i, j + 1) / ((DY(i, j + 1) + DY(i, j + 2)) * (DY(i, j) + DY(i, j + 1)));
      W2(q->curv_yn, i, j, 2) =
          DY(i, j) * DY(i, j + 1) / ((DY(i, j) + 2.0 * DY(i, j + 1) + DY(i, j + 2)) * (DY(i, j) + DY(i, j + 1)));
    }
#undef DX
#undef DY
  for (int k = 0; k < nk; ++k) {
    int kp2 = k + 2 < nk ? k + 2 : nk - 1;
    int kp1 = k + 1 < nk ? k + 1 : nk - 1;
    int km1 = k - 1 > 0 ? k - 1 : 0;
    q->quick_z[k] = dzt[kp1] / (dzt[kp1] + dzt[k]);
    q->quick_z[nk + k] = dzt[k] / (dzt[kp1] + dzt[k]);
    q->curv_zp[k] = dzt[k] * dzt[kp1] / ((dzt[km1] + 2.0 * dzt[k] + dzt[kp1]) * (dzt[k] + dzt[kp1]));
    q->curv_zp[nk + k] = -dzt[k] * dzt[kp1] / ((dzt[k] + dzt[kp1]) * (dzt[km1] + dzt[k]));
    q->curv_zp[2 * nk + k] = dzt[k] * dzt[kp1] / ((dzt[km1] + 2.0 * dzt[k] + dzt[kp1]) * (dzt[km1] + dzt[k]));
    q->curv_zn[k] = dzt[k] * dzt[kp1] / ((dzt[k] + 2.0 * dzt[kp1] + dzt[kp2]) * (dzt[kp1] + dzt[kp2]));
    q->curv_zn[nk + k] = -dzt[k] * dzt[kp1] / ((dzt[kp1] + dzt[kp2]) * (dzt[k] + dzt[kp1]));
    q->curv_zn[2 * nk + k] = dzt[k] * dzt[kp1] / ((dzt[k] + 2.0 * dzt[kp1] + dzt[kp2]) * (dzt[k] + dzt[kp1]));
  }
  free(dxq);
  free(dyq);
}

/* horz_advect_tracer_quickmom3 (ocean_tracer_advect.F90:2665-2780): the Quicker
 * weights with the upwind-biased terms switched off by mask products instead of
 * the coast masks, and the northern second neighbour clamped to jec (jp2 =
 * min(j+2, jec), :2703-2705) for a single-PE domain. */
void orc_horz_advect_quickmom3(const orc_dims* d, int limit_with_upwind, const orc_quicker* q, const double* tmask,
                               const double* tmask_limit, const double* dyte, const double* dxtn, const double* datr,
                               const double* uhrho_et, const double* vhrho_nt, const double* T_taum1,
                               const double* T_tau, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  size_t nh = (size_t)NX2(d) * NY2(d) * nk;
  double* tq = (double*)calloc(nh, sizeof(double));
  double* fx = (double*)calloc(n2 * nk, sizeof(double));
  double* fy = (double*)calloc(n2 * nk, sizeof(double));
  const double* tmq = q->tmask_quick;
  memset(wrk1, 0, sizeof(double) * n2 * nk);
  for (int k = 0; k < nk; ++k)
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) tq[H3(d, i, j, k)] = T_taum1[I3(d, i, j, k)];
  halo2_update(d, tq, 3);
#define TQ(i, j, k) tq[H3(d, (i), (j), (k))]
#define MQ(i, j, k) tmq[H3(d, (i), (j), (k))]
  for (int k = 0; k < nk; ++k) {
    for (int j = 0; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        int jp2 = j + 2 < nj ? j + 2 : nj;
        double vel = dxtn[I2(d, i, j)] * vhrho_nt[I3(d, i, j, k)];
        double upos = 0.5 * (vel + fabs(vel)) * MQ(i, j - 1, k) * MQ(i, j, k) * MQ(i, j + 1, k);
        double uneg = 0.5 * (vel - fabs(vel)) * MQ(i, jp2, k) * MQ(i, j + 1, k) * MQ(i, j, k);
        fy[I3(d, i, j, k)] =
            vel * (W2(q->quick_y, i, j, 0) * T_tau[I3(d, i, j, k)] + W2(q->quick_y, i, j, 1) * T_tau[I3(d, i, j + 1, k)]) -
            upos * (W2(q->curv_yp, i, j, 0) * TQ(i, j + 1, k) + W2(q->curv_yp, i, j, 1) * TQ(i, j, k) +
                    W2(q->curv_yp, i, j, 2) * TQ(i, j - 1, k)) -
            uneg * (W2(q->curv_yn, i, j, 0) * TQ(i, jp2, k) + W2(q->curv_yn, i, j, 1) * TQ(i, j + 1, k) +
                    W2(q->curv_yn, i, j, 2) * TQ(i, j, k));
      }
    for (int j = 1; j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        double vel = dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)];
        double upos = 0.5 * (vel + fabs(vel)) * MQ(i - 1, j, k) * MQ(i, j, k) * MQ(i + 1, j, k);
        double uneg = 0.5 * (vel - fabs(vel)) * MQ(i + 2, j, k) * MQ(i + 1, j, k) * MQ(i, j, k);
        fx[I3(d, i, j, k)] =
            vel * (W2(q->quick_x, i, j, 0) * T_tau[I3(d, i, j, k)] + W2(q->quick_x, i, j, 1) * T_tau[I3(d, i + 1, j, k)]) -
            upos * (W2(q->curv_xp, i, j, 0) * TQ(i + 1, j, k) + W2(q->curv_xp, i, j, 1) * TQ(i, j, k) +
                    W2(q->curv_xp, i, j, 2) * TQ(i - 1, j, k)) -
            uneg * (W2(q->curv_xn, i, j, 0) * TQ(i + 2, j, k) + W2(q->curv_xn, i, j, 1) * TQ(i + 1, j, k) +
                    W2(q->curv_xn, i, j, 2) * TQ(i, j, k));
      }
    if (limit_with_upwind) {
      for (int j = 1; j <= nj; ++j)
        for (int i = 0; i <= ni; ++i)
          if (tmask_limit[I3(d, i, j, k)] == 1.0) {
            double vel = uhrho_et[I3(d, i, j, k)];
            double upos = 0.5 * (vel + fabs(vel));
            double uneg = 0.5 * (vel - fabs(vel));
            fx[I3(d, i, j, k)] = dyte[I2(d, i, j)] *
                                 (upos * T_taum1[I3(d, i, j, k)] + uneg * T_taum1[I3(d, i + 1, j, k)]) *
                                 tmask[I3(d, i, j, k)] * tmask[I3(d, i + 1, j, k)];
          }
      for (int j = 0; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i)
          if (tmask_limit[I3(d, i, j, k)] == 1.0) {
            double vel = vhrho_nt[I3(d, i, j, k)];
            double upos = 0.5 * (vel + fabs(vel));
            double uneg = 0.5 * (vel - fabs(vel));
            fy[I3(d, i, j, k)] = dxtn[I2(d, i, j)] *
                                 (upos * T_taum1[I3(d, i, j, k)] + uneg * T_taum1[I3(d, i, j + 1, k)]) *
                                 tmask[I3(d, i, j, k)] * tmask[I3(d, i, j + 1, k)];
          }
    }
  }
#undef TQ
#undef MQ
  for (int k = 0; k < nk; ++k)
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double r = tmask[I3(d, i, j, k)] *
                   (fx[I3(d, i, j, k)] - fx[I3(d, i - 1, j, k)] + fy[I3(d, i, j, k)] - fy[I3(d, i, j - 1, k)]) *
                   datr[I2(d, i, j)];
        wrk1[I3(d, i, j, k)] = -r;
      }
  free(tq);
  free(fx);
  free(fy);
}

void orc_horz_advect_quicker(const orc_dims* d, int limit_with_upwind, const orc_quicker* q, const double* tmask,
                             const double* tmask_limit, const double* dyte, const double* dxtn, const double* datr,
                             const double* uhrho_et, const double* vhrho_nt, const double* T_taum1,
                             const double* T_tau, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  size_t nh = (size_t)NX2(d) * NY2(d) * nk;
  double* tq = (double*)calloc(nh, sizeof(double));
  double* fx = (double*)calloc(n2 * nk, sizeof(double));
  double* fy = (double*)calloc(n2 * nk, sizeof(double));
  const double* tmq = q->tmask_quick;
  memset(wrk1, 0, sizeof(double) * n2 * nk);
  for (int k = 0; k < nk; ++k)
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) tq[H3(d, i, j, k)] = T_taum1[I3(d, i, j, k)];
  halo2_update(d, tq, 3);
#define TQ(i, j, k) tq[H3(d, (i), (j), (k))]
#define MQ(i, j, k) tmq[H3(d, (i), (j), (k))]
  for (int k = 0; k < nk; ++k) {
    for (int j = 0; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double vel = dxtn[I2(d, i, j)] * vhrho_nt[I3(d, i, j, k)];
        double upos = 0.5 * (vel + fabs(vel));
        double uneg = 0.5 * (vel - fabs(vel));
        double rnormsk = MQ(i, j, k) * (1 - MQ(i, j - 1, k));
        double soutmsk = MQ(i, j + 1, k) * (1 - MQ(i, j + 2, k));
        fy[I3(d, i, j, k)] =
            vel * (W2(q->quick_y, i, j, 0) * T_tau[I3(d, i, j, k)] + W2(q->quick_y, i, j, 1) * T_tau[I3(d, i, j + 1, k)]) -
            upos * (W2(q->curv_yp, i, j, 0) * TQ(i, j + 1, k) + W2(q->curv_yp, i, j, 1) * TQ(i, j, k) +
                    W2(q->curv_yp, i, j, 2) * (TQ(i, j - 1, k) * (1 - rnormsk) + TQ(i, j, k) * rnormsk)) -
            uneg * (W2(q->curv_yn, i, j, 0) * (TQ(i, j + 2, k) * (1 - soutmsk) + TQ(i, j + 1, k) * soutmsk) +
                    W2(q->curv_yn, i, j, 1) * TQ(i, j + 1, k) + W2(q->curv_yn, i, j, 2) * TQ(i, j, k));
      }
    for (int j = 1; j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        double vel = dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)];
        double upos = 0.5 * (vel + fabs(vel));
        double uneg = 0.5 * (vel - fabs(vel));
        double eastmsk = MQ(i, j, k) * (1 - MQ(i - 1, j, k));
        double westmsk = MQ(i + 1, j, k) * (1 - MQ(i + 2, j, k));
        fx[I3(d, i, j, k)] =
            vel * (W2(q->quick_x, i, j, 0) * T_tau[I3(d, i, j, k)] + W2(q->quick_x, i, j, 1) * T_tau[I3(d, i + 1, j, k)]) -
            upos * (W2(q->curv_xp, i, j, 0) * TQ(i + 1, j, k) + W2(q->curv_xp, i, j, 1) * TQ(i, j, k) +
                    W2(q->curv_xp, i, j, 2) * (TQ(i - 1, j, k) * (1 - eastmsk) + TQ(i, j, k) * eastmsk)) -
            uneg * (W2(q->curv_xn, i, j, 0) * (TQ(i + 2, j, k) * (1 - westmsk) + TQ(i + 1, j, k) * westmsk) +
                    W2(q->curv_xn, i, j, 1) * TQ(i + 1, j, k) + W2(q->curv_xn, i, j, 2) * TQ(i, j, k));
      }
    if (limit_with_upwind) {
      for (int j = 1; j <= nj; ++j)
        for (int i = 0; i <= ni; ++i)
          if (tmask_limit[I3(d, i, j, k)] == 1.0) {
            double vel = uhrho_et[I3(d, i, j, k)];
            double upos = 0.5 * (vel + fabs(vel));
            double uneg = 0.5 * (vel - fabs(vel));
            fx[I3(d, i, j, k)] = dyte[I2(d, i, j)] *
                                 (upos * T_taum1[I3(d, i, j, k)] + uneg * T_taum1[I3(d, i + 1, j, k)]) *
                                 tmask[I3(d, i, j, k)] * tmask[I3(d, i + 1, j, k)];
          }
      for (int j = 0; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i)
          if (tmask_limit[I3(d, i, j, k)] == 1.0) {
            double vel = vhrho_nt[I3(d, i, j, k)];
            double upos = 0.5 * (vel + fabs(vel));
            double uneg = 0.5 * (vel - fabs(vel));
            fy[I3(d, i, j, k)] = dxtn[I2(d, i, j)] *
                                 (upos * T_taum1[I3(d, i, j, k)] + uneg * T_taum1[I3(d, i, j + 1, k)]) *
                                 tmask[I3(d, i, j, k)] * tmask[I3(d, i, j + 1, k)];
          }
    }
  }
  for (int k = 0; k < nk; ++k)
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double r = tmask[I3(d, i, j, k)] *
                   (fx[I3(d, i, j, k)] - fx[I3(d, i - 1, j, k)] + fy[I3(d, i, j, k)] - fy[I3(d, i, j - 1, k)]) *
                   datr[I2(d, i, j)];
        wrk1[I3(d, i, j, k)] = -r;
      }
#undef TQ
#undef MQ
  free(tq);
  free(fx);
  free(fy);
}

void orc_vert_advect_quicker(const orc_dims* d, const orc_quicker* q, const double* tmask,
                             const double* tmask_limit, const double* wrho_bt, const double* T_taum1,
                             const double* T_tau, double* wrk1) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* ft1 = (double*)calloc(n2, sizeof(double));
  double* ft2 = (double*)calloc(n2, sizeof(double));
  memset(wrk1, 0, sizeof(double) * n2 * nk);
  for (int k = 0; k < nk; ++k) {
    int km1 = k - 1 > 0 ? k - 1 : 0;
    int kp1 = k + 1 < nk ? k + 1 : nk - 1;
    int p2 = k + 2 < nk ? k + 2 : nk - 1;
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double vel = wrho_bt[I3(d, i, j, k + 1)];
        double upos = 0.5 * (vel + fabs(vel));
        double uneg = 0.5 * (vel - fabs(vel));
        double f;
        if (tmask_limit[I3(d, i, j, k)] == 1.0) {
          f = (uneg * T_taum1[I3(d, i, j, k)] + upos * T_taum1[I3(d, i, j, kp1)]) * tmask[I3(d, i, j, k)] *
              tmask[I3(d, i, j, kp1)];
        } else {
          /* kp2 = nint(tmask(p2)*p2 + (1-tmask(p2))*kp1), Fortran 1-based levels */
          double mp2 = tmask[I3(d, i, j, p2)];
          int kp2 = (int)lround(mp2 * (double)(p2 + 1) + (1.0 - mp2) * (double)(kp1 + 1)) - 1;
          double upmsk = tmask[I3(d, i, j, k)] * (1 - tmask[I3(d, i, j, km1)]);
          f = vel * (q->quick_z[k] * T_tau[I3(d, i, j, k)] + q->quick_z[nk + k] * T_tau[I3(d, i, j, kp1)]) -
              uneg * (q->curv_zp[k] * T_taum1[I3(d, i, j, kp1)] + q->curv_zp[nk + k] * T_taum1[I3(d, i, j, k)] +
                      q->curv_zp[2 * nk + k] * T_taum1[I3(d, i, j, km1)]) -
              upos * (q->curv_zn[k] * T_taum1[I3(d, i, j, kp2)] + q->curv_zn[nk + k] * T_taum1[I3(d, i, j, kp1)] +
                      q->curv_zn[2 * nk + k] *
                          (T_taum1[I3(d, i, j, k)] * (1 - upmsk) + T_taum1[I3(d, i, j, kp1)] * upmsk));
        }
        ft2[I2(d, i, j)] = f;
        double r = tmask[I3(d, i, j, k)] * (ft1[I2(d, i, j)] - f);
        wrk1[I3(d, i, j, k)] = -r;
      }
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) ft1[I2(d, i, j)] = ft2[I2(d, i, j)];
  }
  free(ft1);
  free(ft2);
}
#undef W2

/* ------------------------------------------------------------------------- */
/* MDFL Sweby, one tracer: advect_tracer_mdfl_sweby :3806-4066.              */
/* wrk1 receives -advect_tracer_mdfl_sweby (horz_advect_tracer :1953-1959).  */
/* sweby_limiter = 1 for ADVECT_MDFL_SWEBY, 0 for ADVECT_DST_LINEAR.         */
/* ------------------------------------------------------------------------- */
/* The module scratch of the MDFL scheme, allocated once as mdfl_init does
 * (ocean_tracer_advect.F90:1644-1669; flux_x/flux_y :548-553): tmask_mdfl is
 * built once, the rest is zeroed at the top of every call (:3833-3838). */
struct orc_mdfl_ws {
  orc_dims d;
  double *tm, *mk, *ftp, *fbt, *wkm1, *fx, *fy;
};

orc_mdfl_ws* orc_mdfl_ws_create(const orc_dims* d, const double* tmask) {
  orc_mdfl_ws* ws = (orc_mdfl_ws*)calloc(1, sizeof(orc_mdfl_ws));
  size_t n2 = (size_t)NXD(d) * NYD(d);
  size_t nh = (size_t)NX2(d) * NY2(d) * d->nk;
  ws->d = *d;
  ws->tm = (double*)calloc(nh, sizeof(double)); /* tracer_mdfl */
  ws->mk = (double*)calloc(nh, sizeof(double)); /* tmask_mdfl  */
  ws->ftp = (double*)calloc(n2, sizeof(double));
  ws->fbt = (double*)calloc(n2, sizeof(double));
  ws->wkm1 = (double*)calloc(n2, sizeof(double));
  ws->fx = (double*)calloc(n2 * d->nk, sizeof(double)); /* flux_x */
  ws->fy = (double*)calloc(n2 * d->nk, sizeof(double)); /* flux_y */
  orc_mask_halo2(d, tmask, ws->mk);
  return ws;
}

void orc_mdfl_ws_destroy(orc_mdfl_ws* ws) {
  if (!ws) return;
  free(ws->tm);
  free(ws->mk);
  free(ws->ftp);
  free(ws->fbt);
  free(ws->wkm1);
  free(ws->fx);
  free(ws->fy);
  free(ws);
}

void orc_advect_mdfl_sweby(const orc_dims* d, double sweby_limiter, double dtime, const double* tmask,
                           const double* dat, const double* datr, const double* dxte, const double* dyte,
                           const double* dxtn, const double* dytn, const double* uhrho_et,
                           const double* vhrho_nt, const double* wrho_bt, const double* rho_dzt,
                           const double* T, double* wrk1) {
  orc_mdfl_ws* ws = orc_mdfl_ws_create(d, tmask);
  orc_advect_mdfl_sweby_ws(ws, sweby_limiter, dtime, dat, datr, dxte, dyte, dxtn, dytn, uhrho_et, vhrho_nt,
                           wrho_bt, rho_dzt, T, wrk1);
  orc_mdfl_ws_destroy(ws);
}

void orc_advect_mdfl_sweby_ws(orc_mdfl_ws* ws, double sweby_limiter, double dtime, const double* dat,
                              const double* datr, const double* dxte, const double* dyte, const double* dxtn,
                              const double* dytn, const double* uhrho_et, const double* vhrho_nt,
                              const double* wrho_bt, const double* rho_dzt, const double* T, double* wrk1) {
  const orc_dims* d = &ws->d;
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  size_t nh = (size_t)NX2(d) * NY2(d) * nk;
  double* tm = ws->tm;
  const double* mk = ws->mk;
  double* ftp = ws->ftp;
  double* fbt = ws->fbt;
  double* wkm1 = ws->wkm1;
  double* fx = ws->fx;
  double* fy = ws->fy;
  /* :3833-3838 */
  zero_par(ftp, n2);
  zero_par(fbt, n2);
  zero_par(wkm1, n2);
  zero_par(tm, nh);
  zero_par(fx, n2 * nk);
  zero_par(fy, n2 * nk);
  /* horz_advect_tracer :1925-1931 */
  zero_par(wrk1, n2 * nk);
#define TM(i, j, k) tm[H3(d, (i), (j), (k))]
#define MK(i, j, k) mk[H3(d, (i), (j), (k))]
#define TF(i, j, k) T[I3(d, (i), (j), (k))]
#define RDZ(i, j, k) rho_dzt[I3(d, (i), (j), (k))]
#define WB(i, j, k) wrho_bt[I3(d, (i), (j), (k) + 1)]
  for (int k = 0; k < nk; ++k) {
    OMP_FOR
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) TM(i, j, k) = TF(i, j, k);
    int kp1 = k + 1 < nk ? k + 1 : nk - 1;
    int kp2 = k + 2 < nk ? k + 2 : nk - 1;
    int km1 = k - 1 > 0 ? k - 1 : 0;
    OMP_FOR
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double Rjp = (TF(i, j, km1) - TF(i, j, k)) * MK(i, j, km1) * MK(i, j, k);
        double Rj = (TF(i, j, k) - TF(i, j, kp1)) * MK(i, j, k) * MK(i, j, kp1);
        double Rjm = (TF(i, j, kp1) - TF(i, j, kp2)) * MK(i, j, kp1) * MK(i, j, kp2);
        double massflux = dat[I2(d, i, j)] * WB(i, j, k);
        double cfl = fabs(WB(i, j, k) * dtime / RDZ(i, j, k));
        double d0 = (2.0 - cfl) * (1.0 - cfl) * onesixth;
        double d1 = (1.0 - cfl * cfl) * onesixth;
        double thetaP = Rjm / (1.0e-30 + Rj);
        double thetaM = Rjp / (1.0e-30 + Rj);
        double psiP = d0 + d1 * thetaP;
        psiP = psiP * (1.0 - sweby_limiter) +
               fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaP), (1.0 - cfl) / (1.0e-30 + cfl) * thetaP)) * sweby_limiter;
        double psiM = d0 + d1 * thetaM;
        psiM = psiM * (1.0 - sweby_limiter) +
               fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaM), (1.0 - cfl) / (1.0e-30 + cfl) * thetaM)) * sweby_limiter;
        fbt[I2(d, i, j)] = 0.5 * ((massflux + fabs(massflux)) * (TF(i, j, kp1) + psiP * Rj) +
                                  (massflux - fabs(massflux)) * (TF(i, j, k) - psiM * Rj)) *
                           MK(i, j, kp1) * MK(i, j, k);
        TM(i, j, k) = TM(i, j, k) + dtime / RDZ(i, j, k) *
                                        (datr[I2(d, i, j)] * (fbt[I2(d, i, j)] - ftp[I2(d, i, j)]) +
                                         TF(i, j, k) * (wkm1[I2(d, i, j)] - WB(i, j, k)));
        ftp[I2(d, i, j)] = fbt[I2(d, i, j)];
      }
    OMP_FOR
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) wkm1[I2(d, i, j)] = WB(i, j, k);
  }
  halo2_update(d, tm, 1); /* XUPDATE :3912 */

  OMP_FOR
  for (int k = 0; k < nk; ++k) {
    for (int j = 1; j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        double Rjp = (TM(i + 2, j, k) - TM(i + 1, j, k)) * MK(i + 2, j, k) * MK(i + 1, j, k);
        double Rj = (TM(i + 1, j, k) - TM(i, j, k)) * MK(i + 1, j, k) * MK(i, j, k);
        double Rjm = (TM(i, j, k) - TM(i - 1, j, k)) * MK(i, j, k) * MK(i - 1, j, k);
        double massflux = dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)];
        double cfl = fabs(uhrho_et[I3(d, i, j, k)] * dtime * 2.0 /
                          ((RDZ(i, j, k) + RDZ(i + 1, j, k)) * dxte[I2(d, i, j)]));
        double d0 = (2.0 - cfl) * (1.0 - cfl) * onesixth;
        double d1 = (1.0 - cfl * cfl) * onesixth;
        double thetaP = Rjm / (1.0e-30 + Rj);
        double thetaM = Rjp / (1.0e-30 + Rj);
        double psiP = d0 + d1 * thetaP;
        psiP = psiP * (1.0 - sweby_limiter) +
               fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaP), (1.0 - cfl) / (1.0e-30 + cfl) * thetaP)) * sweby_limiter;
        double psiM = d0 + d1 * thetaM;
        psiM = psiM * (1.0 - sweby_limiter) +
               fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaM), (1.0 - cfl) / (1.0e-30 + cfl) * thetaM)) * sweby_limiter;
        fx[I3(d, i, j, k)] = 0.5 * ((massflux + fabs(massflux)) * (TM(i, j, k) + psiP * Rj) +
                                    (massflux - fabs(massflux)) * (TM(i + 1, j, k) - psiM * Rj)) *
                             MK(i, j, k) * MK(i + 1, j, k);
      }
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        TM(i, j, k) = TM(i, j, k) + dtime * MK(i, j, k) * datr[I2(d, i, j)] / RDZ(i, j, k) *
                                        (fx[I3(d, i - 1, j, k)] - fx[I3(d, i, j, k)] +
                                         TF(i, j, k) * (dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)] -
                                                        dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)]));
      }
  }
  halo2_update(d, tm, 2); /* YUPDATE :3970 */

  memset(wkm1, 0, sizeof(double) * n2);
  for (int k = 0; k < nk; ++k) {
    OMP_FOR
    for (int j = 0; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        double Rjp = (TM(i, j + 2, k) - TM(i, j + 1, k)) * MK(i, j + 2, k) * MK(i, j + 1, k);
        double Rj = (TM(i, j + 1, k) - TM(i, j, k)) * MK(i, j + 1, k) * MK(i, j, k);
        double Rjm = (TM(i, j, k) - TM(i, j - 1, k)) * MK(i, j, k) * MK(i, j - 1, k);
        double massflux = dxtn[I2(d, i, j)] * vhrho_nt[I3(d, i, j, k)];
        double cfl = fabs(vhrho_nt[I3(d, i, j, k)] * dtime * 2.0 /
                          ((RDZ(i, j, k) + RDZ(i, j + 1, k)) * dytn[I2(d, i, j)]));
        double d0 = (2.0 - cfl) * (1.0 - cfl) * onesixth;
        double d1 = (1.0 - cfl * cfl) * onesixth;
        double thetaP = Rjm / (1.0e-30 + Rj);
        double thetaM = Rjp / (1.0e-30 + Rj);
        double psiP = d0 + d1 * thetaP;
        psiP = psiP * (1.0 - sweby_limiter) +
               fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaP), (1.0 - cfl) / (1.0e-30 + cfl) * thetaP)) * sweby_limiter;
        double psiM = d0 + d1 * thetaM;
        psiM = psiM * (1.0 - sweby_limiter) +
               fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaM), (1.0 - cfl) / (1.0e-30 + cfl) * thetaM)) * sweby_limiter;
        fy[I3(d, i, j, k)] = 0.5 * ((massflux + fabs(massflux)) * (TM(i, j, k) + psiP * Rj) +
                                    (massflux - fabs(massflux)) * (TM(i, j + 1, k) - psiM * Rj)) *
                             MK(i, j, k) * MK(i, j + 1, k);
      }
    OMP_FOR
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i)
        TM(i, j, k) = TM(i, j, k) + dtime * MK(i, j, k) * datr[I2(d, i, j)] / RDZ(i, j, k) *
                                        (fy[I3(d, i, j - 1, k)] - fy[I3(d, i, j, k)]);
    OMP_FOR
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        TM(i, j, k) = TM(i, j, k) + dtime * TF(i, j, k) / RDZ(i, j, k) *
                                        (WB(i, j, k) - wkm1[I2(d, i, j)] +
                                         datr[I2(d, i, j)] * ((dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)] -
                                                               dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)])));
        double adv = -RDZ(i, j, k) * (TM(i, j, k) - TF(i, j, k)) / dtime * MK(i, j, k);
        wrk1[I3(d, i, j, k)] = -adv;
      }
    OMP_FOR
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) wkm1[I2(d, i, j)] = WB(i, j, k);
  }
#undef TM
#undef MK
#undef TF
#undef RDZ
#undef WB
}

/* ------------------------------------------------------------------------- */
/* MDFL Sweby for all tracers at once: advect_tracer_sweby_all :4104-4511.   */
/* T and wrk1 hold ntr consecutive data-domain 3-D blocks.  Differs from the */
/* one-tracer routine in the grouping of the update products (:4194-4195,    */
/* :4277-4284, :4386-4399) and in merging the y-pass with the closing        */
/* divergence correction.                                                    */
/* ------------------------------------------------------------------------- */
void orc_advect_sweby_all(const orc_dims* d, int ntr, double dtime, const double* tmask, const double* dat,
                          const double* datr, const double* dxte, const double* dyte, const double* dxtn,
                          const double* dytn, const double* uhrho_et, const double* vhrho_nt,
                          const double* wrho_bt, const double* rho_dzt, const double* Tall, double* wrk1_all) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  size_t n3 = n2 * nk;
  size_t nh = (size_t)NX2(d) * NY2(d) * nk;
  double* tma = (double*)calloc(nh * ntr, sizeof(double));
  double* mk = (double*)calloc(nh, sizeof(double));
  double* ftp = (double*)calloc(n2, sizeof(double));
  double* fbt = (double*)calloc(n2, sizeof(double));
  double* wkm1 = (double*)calloc(n2, sizeof(double));
  double* fx = (double*)calloc(n3, sizeof(double));
  double* fy = (double*)calloc(n3, sizeof(double));
  double* wrk1 = (double*)calloc(n3, sizeof(double));
  orc_mask_halo2(d, tmask, mk);
  memset(wrk1_all, 0, sizeof(double) * n3 * ntr);
#define MK(i, j, k) mk[H3(d, (i), (j), (k))]
#define RDZ(i, j, k) rho_dzt[I3(d, (i), (j), (k))]
#define WB(i, j, k) wrho_bt[I3(d, (i), (j), (k) + 1)]
  for (int n = 0; n < ntr; ++n) {
    const double* T = Tall + n3 * n;
    double* tm = tma + nh * n;
#define TM(i, j, k) tm[H3(d, (i), (j), (k))]
#define TF(i, j, k) T[I3(d, (i), (j), (k))]
    memset(ftp, 0, sizeof(double) * n2);
    memset(wkm1, 0, sizeof(double) * n2);
    for (int k = 0; k < nk; ++k) {
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) TM(i, j, k) = TF(i, j, k);
      int kp1 = k + 1 < nk ? k + 1 : nk - 1;
      int kp2 = k + 2 < nk ? k + 2 : nk - 1;
      int km1 = k - 1 > 0 ? k - 1 : 0;
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
          double Rjp = (TF(i, j, km1) - TF(i, j, k)) * MK(i, j, km1) * MK(i, j, k);
          double Rj = (TF(i, j, k) - TF(i, j, kp1)) * MK(i, j, k) * MK(i, j, kp1);
          double Rjm = (TF(i, j, kp1) - TF(i, j, kp2)) * MK(i, j, kp1) * MK(i, j, kp2);
          double massflux = dat[I2(d, i, j)] * WB(i, j, k);
          double cfl = fabs(WB(i, j, k) * dtime / RDZ(i, j, k));
          double d0 = (2.0 - cfl) * (1.0 - cfl) * onesixth;
          double d1 = (1.0 - cfl * cfl) * onesixth;
          double thetaP = Rjm / (1.0e-30 + Rj);
          double thetaM = Rjp / (1.0e-30 + Rj);
          double psiP = fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaP), (1.0 - cfl) / (1.0e-30 + cfl) * thetaP));
          double psiM = fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaM), (1.0 - cfl) / (1.0e-30 + cfl) * thetaM));
          fbt[I2(d, i, j)] = 0.5 * ((massflux + fabs(massflux)) * (TF(i, j, kp1) + psiP * Rj) +
                                    (massflux - fabs(massflux)) * (TF(i, j, k) - psiM * Rj)) *
                             MK(i, j, kp1) * MK(i, j, k);
          double w1 = datr[I2(d, i, j)] * (fbt[I2(d, i, j)] - ftp[I2(d, i, j)]) +
                      TF(i, j, k) * (wkm1[I2(d, i, j)] - WB(i, j, k));
          TM(i, j, k) = TM(i, j, k) + w1 * dtime / RDZ(i, j, k);
          ftp[I2(d, i, j)] = fbt[I2(d, i, j)];
        }
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) wkm1[I2(d, i, j)] = WB(i, j, k);
    }
    halo2_update(d, tm, 1);
#undef TM
#undef TF
  }
  for (int n = 0; n < ntr; ++n) {
    const double* T = Tall + n3 * n;
    double* tm = tma + nh * n;
#define TM(i, j, k) tm[H3(d, (i), (j), (k))]
#define TF(i, j, k) T[I3(d, (i), (j), (k))]
    for (int k = 0; k < nk; ++k) {
      for (int j = 1; j <= nj; ++j)
        for (int i = 0; i <= ni; ++i) {
          double Rjp = (TM(i + 2, j, k) - TM(i + 1, j, k)) * MK(i + 2, j, k) * MK(i + 1, j, k);
          double Rj = (TM(i + 1, j, k) - TM(i, j, k)) * MK(i + 1, j, k) * MK(i, j, k);
          double Rjm = (TM(i, j, k) - TM(i - 1, j, k)) * MK(i, j, k) * MK(i - 1, j, k);
          double massflux = dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)];
          double cfl = fabs(uhrho_et[I3(d, i, j, k)] * dtime * 2.0 /
                            ((RDZ(i, j, k) + RDZ(i + 1, j, k)) * dxte[I2(d, i, j)]));
          double d0 = (2.0 - cfl) * (1.0 - cfl) * onesixth;
          double d1 = (1.0 - cfl * cfl) * onesixth;
          double thetaP = Rjm / (1.0e-30 + Rj);
          double thetaM = Rjp / (1.0e-30 + Rj);
          double psiP = fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaP), (1.0 - cfl) / (1.0e-30 + cfl) * thetaP));
          double psiM = fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaM), (1.0 - cfl) / (1.0e-30 + cfl) * thetaM));
          fx[I3(d, i, j, k)] = 0.5 * ((massflux + fabs(massflux)) * (TM(i, j, k) + psiP * Rj) +
                                      (massflux - fabs(massflux)) * (TM(i + 1, j, k) - psiM * Rj)) *
                               MK(i, j, k) * MK(i + 1, j, k);
        }
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
          double w1 = MK(i, j, k) * datr[I2(d, i, j)] *
                      (fx[I3(d, i - 1, j, k)] - fx[I3(d, i, j, k)] +
                       TF(i, j, k) * (dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)] -
                                      dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)]));
          TM(i, j, k) = TM(i, j, k) + w1 * dtime / RDZ(i, j, k);
        }
    }
    halo2_update(d, tm, 2);
#undef TM
#undef TF
  }
  for (int n = 0; n < ntr; ++n) {
    const double* T = Tall + n3 * n;
    double* tm = tma + nh * n;
    double* out = wrk1_all + n3 * n;
#define TM(i, j, k) tm[H3(d, (i), (j), (k))]
#define TF(i, j, k) T[I3(d, (i), (j), (k))]
    memset(wkm1, 0, sizeof(double) * n2);
    for (int k = 0; k < nk; ++k) {
      for (int j = 0; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
          double Rjp = (TM(i, j + 2, k) - TM(i, j + 1, k)) * MK(i, j + 2, k) * MK(i, j + 1, k);
          double Rj = (TM(i, j + 1, k) - TM(i, j, k)) * MK(i, j + 1, k) * MK(i, j, k);
          double Rjm = (TM(i, j, k) - TM(i, j - 1, k)) * MK(i, j, k) * MK(i, j - 1, k);
          double massflux = dxtn[I2(d, i, j)] * vhrho_nt[I3(d, i, j, k)];
          double cfl = fabs(vhrho_nt[I3(d, i, j, k)] * dtime * 2.0 /
                            ((RDZ(i, j, k) + RDZ(i, j + 1, k)) * dytn[I2(d, i, j)]));
          double d0 = (2.0 - cfl) * (1.0 - cfl) * onesixth;
          double d1 = (1.0 - cfl * cfl) * onesixth;
          double thetaP = Rjm / (1.0e-30 + Rj);
          double thetaM = Rjp / (1.0e-30 + Rj);
          double psiP = fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaP), (1.0 - cfl) / (1.0e-30 + cfl) * thetaP));
          double psiM = fmaxd(0.0, fmind(fmind(1.0, d0 + d1 * thetaM), (1.0 - cfl) / (1.0e-30 + cfl) * thetaM));
          fy[I3(d, i, j, k)] = 0.5 * ((massflux + fabs(massflux)) * (TM(i, j, k) + psiP * Rj) +
                                      (massflux - fabs(massflux)) * (TM(i, j + 1, k) - psiM * Rj)) *
                               MK(i, j, k) * MK(i, j + 1, k);
        }
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
          double w1 = MK(i, j, k) * datr[I2(d, i, j)] * (fy[I3(d, i, j - 1, k)] - fy[I3(d, i, j, k)]) +
                      TF(i, j, k) * (WB(i, j, k) - wkm1[I2(d, i, j)] +
                                     datr[I2(d, i, j)] * (dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)] -
                                                          dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)]));
          TM(i, j, k) = TM(i, j, k) + w1 * dtime / RDZ(i, j, k);
          out[I3(d, i, j, k)] = RDZ(i, j, k) * (TM(i, j, k) - TF(i, j, k)) / dtime * MK(i, j, k);
        }
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) wkm1[I2(d, i, j)] = WB(i, j, k);
    }
#undef TM
#undef TF
  }
#undef MK
#undef RDZ
#undef WB
  free(tma);
  free(mk);
  free(ftp);
  free(fbt);
  free(wkm1);
  free(fx);
  free(fy);
  free(wrk1);
}

/* ------------------------------------------------------------------------- */
/* Explicit tracer update: ocean_tracer.F90:2341-2350 / :2640-2647.          */
/* Compute domain only; the caller halo-updates T(taup1) afterwards          */
/* (ocean_model.F90:1903-1911).                                              */
/* ------------------------------------------------------------------------- */
void orc_update_tracer(const orc_dims* d, double dtime, const double* rho_dzt_taum1, const double* rho_dztr,
                       const double* T_taum1, const double* th_tendency, double* T_taup1) {
  OMP_FOR
  for (int k = 0; k < d->nk; ++k)
    for (int j = 1; j <= d->nj; ++j)
      for (int i = 1; i <= d->ni; ++i) {
        size_t p = I3(d, i, j, k);
        T_taup1[p] = (rho_dzt_taum1[p] * T_taum1[p] + dtime * th_tendency[p]) * rho_dztr[p];
      }
}

/* compute_tmask_limit, one tracer: ocean_tracer.F90:2804-2851. */
void orc_compute_tmask_limit(const orc_dims* d, const double* tmask, const double* T_tau, double tmin,
                             double tmax, double* tmask_limit) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  for (int k = 0; k < nk; ++k)
    for (int j = 0; j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        size_t p = I3(d, i, j, k);
        tmask_limit[p] = 0.0;
        if (tmask[p] == 1.0 && (T_tau[p] < tmin || T_tau[p] > tmax)) tmask_limit[p] = tmask[p];
        size_t pe = I3(d, i + 1, j, k);
        if (tmask[pe] == 1.0 && (T_tau[pe] < tmin || T_tau[pe] > tmax)) tmask_limit[p] = tmask[p];
        size_t pn = I3(d, i, j + 1, k);
        if (tmask[pn] == 1.0 && (T_tau[pn] < tmin || T_tau[pn] > tmax)) tmask_limit[p] = tmask[p];
      }
  for (int k = 0; k < nk - 1; ++k)
    for (int j = 0; j <= nj; ++j)
      for (int i = 0; i <= ni; ++i) {
        size_t p = I3(d, i, j, k);
        size_t pd = I3(d, i, j, k + 1);
        if (tmask[pd] == 1.0 && (T_tau[pd] < tmin || T_tau[pd] > tmax)) tmask_limit[p] = tmask[p];
      }
}

/* tmask_limit_ts_same (:2855-2867) */
void orc_tmask_limit_ts_same(const orc_dims* d, double* tl_temp, double* tl_salt) {
  for (int k = 0; k < d->nk; ++k)
    for (int j = 0; j <= d->nj; ++j)
      for (int i = 0; i <= d->ni; ++i) {
        size_t p = I3(d, i, j, k);
        if (tl_temp[p] == 1.0 || tl_salt[p] == 1.0) {
          tl_temp[p] = 1.0;
          tl_salt[p] = 1.0;
        }
      }
}

/* ------------------------------------------------------------------------- */
/* Operators on the barotropic domain (halo 1, halo_in = halo_out = 1).      */
/* ------------------------------------------------------------------------- */

/* DIV_UD, B-grid non-legacy branch: ocean_operators.F90:559-598, 605-606.   */
void orc_div_ud_bgrid(const orc_dims* d, const double* udu, const double* udv, const double* dyu,
                      const double* dxu, const double* datr, double* out) {
  int ni = d->ni, nj = d->nj;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  zero_par(out, n2);
  OMP_FOR
  for (int j = 1; j <= nj + 1; ++j) {
    int i = 1;
    double uhim = udu[I2(d, i - 1, j)] * dyu[I2(d, i - 1, j)];
    double vhim = udv[I2(d, i - 1, j)] * dxu[I2(d, i - 1, j)];
    double uhimjm = udu[I2(d, i - 1, j - 1)] * dyu[I2(d, i - 1, j - 1)];
    double vhimjm = udv[I2(d, i - 1, j - 1)] * dxu[I2(d, i - 1, j - 1)];
    double uhim_bay = 0.5 * (uhim + uhimjm);
    for (i = 1; i <= ni + 1; ++i) {
      double uh = udu[I2(d, i, j)] * dyu[I2(d, i, j)];
      double vh = udv[I2(d, i, j)] * dxu[I2(d, i, j)];
      double uhjm = udu[I2(d, i, j - 1)] * dyu[I2(d, i, j - 1)];
      double vhjm = udv[I2(d, i, j - 1)] * dxu[I2(d, i, j - 1)];
      double uh_bay = 0.5 * (uh + uhjm);
      double vh_bax = 0.5 * (vh + vhim);
      double vhjm_bax = 0.5 * (vhjm + vhimjm);
      out[I2(d, i, j)] = ((uh_bay - uhim_bay) + (vh_bax - vhjm_bax)) * datr[I2(d, i, j)];
      uhim = uh;
      vhim = vh;
      uhimjm = uhjm;
      vhimjm = vhjm;
      uhim_bay = uh_bay;
    }
  }
}

/* DIV_UD, C-grid branch: ocean_operators.F90:526-535. */
void orc_div_ud_cgrid(const orc_dims* d, const double* udu, const double* udv, const double* dat,
                      const double* dxter, const double* dytnr, const double* datr, double* out) {
  int ni = d->ni, nj = d->nj;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  zero_par(out, n2);
  OMP_FOR
  for (int j = 1; j <= nj + 1; ++j)
    for (int i = 1; i <= ni + 1; ++i) {
      double uhim = udu[I2(d, i - 1, j)] * dat[I2(d, i - 1, j)] * dxter[I2(d, i - 1, j)];
      double vhjm = udv[I2(d, i, j - 1)] * dat[I2(d, i, j - 1)] * dytnr[I2(d, i, j - 1)];
      double uh = udu[I2(d, i, j)] * dat[I2(d, i, j)] * dxter[I2(d, i, j)];
      double vh = udv[I2(d, i, j)] * dat[I2(d, i, j)] * dytnr[I2(d, i, j)];
      out[I2(d, i, j)] = ((uh - uhim) + (vh - vhjm)) * datr[I2(d, i, j)];
    }
}

/* GRAD_BAROTROPIC_P: ocean_operators.F90:643-674. */
void orc_grad_baro_p(const orc_dims* d, int cgrid, const double* press, const double* rx, const double* ry,
                     const double* mx, const double* my, double* gx, double* gy) {
  int ni = d->ni, nj = d->nj;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  zero_par(gx, n2);
  zero_par(gy, n2);
  OMP_FOR
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i <= ni; ++i) {
      if (!cgrid) {
        double p_fay = 0.5 * (press[I2(d, i, j)] + press[I2(d, i, j + 1)]);
        double p_fax = 0.5 * (press[I2(d, i, j)] + press[I2(d, i + 1, j)]);
        double pip_fay = 0.5 * (press[I2(d, i + 1, j)] + press[I2(d, i + 1, j + 1)]);
        double pjp_fax = 0.5 * (press[I2(d, i, j + 1)] + press[I2(d, i + 1, j + 1)]);
        gx[I2(d, i, j)] = (pip_fay - p_fay) * rx[I2(d, i, j)] * mx[I2(d, i, j)];
        gy[I2(d, i, j)] = (pjp_fax - p_fax) * ry[I2(d, i, j)] * mx[I2(d, i, j)];
      } else {
        gx[I2(d, i, j)] = (press[I2(d, i + 1, j)] - press[I2(d, i, j)]) * rx[I2(d, i, j)] * mx[I2(d, i, j)];
        gy[I2(d, i, j)] = (press[I2(d, i, j + 1)] - press[I2(d, i, j)]) * ry[I2(d, i, j)] * my[I2(d, i, j)];
      }
    }
}

/* REMAP_BT_TO_BU: ocean_operators.F90:462-477 (halo 1). */
void orc_remap_bt_to_bu(const orc_dims* d, const double* a, const double* dte, const double* dtw,
                        const double* dus, const double* dun, const double* daur, double* out) {
  int ni = d->ni, nj = d->nj;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  memset(out, 0, sizeof(double) * n2);
  for (int j = 0; j <= nj; ++j)
    for (int i = 0; i <= ni; ++i)
      out[I2(d, i, j)] = (a[I2(d, i, j)] * dte[I2(d, i, j)] * dus[I2(d, i, j)] +
                          a[I2(d, i + 1, j)] * dtw[I2(d, i + 1, j)] * dus[I2(d, i, j)] +
                          a[I2(d, i, j + 1)] * dte[I2(d, i, j + 1)] * dun[I2(d, i, j)] +
                          a[I2(d, i + 1, j + 1)] * dtw[I2(d, i + 1, j + 1)] * dun[I2(d, i, j)]) *
                         daur[I2(d, i, j)];
}

/* ------------------------------------------------------------------------- */
/* Barotropic step: pred_corr_tropic_depth_bgrid :3225-3579 (legacy halos,   */
/* barotropic_halo = 1, no OBC, tides, geoid, smoothing or friction),         */
/* pred_corr_tropic_depth_cgrid :3601-3965 and the splitting branch of       */
/* update_ocean_barotropic :2793-2985.                                        */
/* ------------------------------------------------------------------------- */
typedef struct {
  int nts;
  double dtbt;
  double pred_corr_gamma;
  double rho0;
  int time_stepping_B; /* 0: barotropic_time_stepping_A, 1: _B */
  int initsum_with_bar;
  int cgrid;
} orc_baro_params;

typedef struct {
  /* grid, data domain */
  const double *tmask1, *umask1, *f, *dxu, *dyu, *dxur, *dyur, *dat, *datr, *dxter, *dytnr;
  const double *tmasken_e, *tmasken_n, *dte, *dtw, *dus, *dun, *daur;
  /* inputs constant over the step */
  const double *patm, *pme, *river, *source, *eta_smooth, *thicku, *thicken_e, *thicken_n;
  const double *forcing_u, *forcing_v, *rho_g;
  /* state at tau */
  const double *eta_t_tau, *eta_t_bar_tau, *udrho_u_tau, *udrho_v_tau;
  /* outputs at taup1 */
  double *eta_t_bar, *udrho_u, *udrho_v, *conv_rho_ud_t, *eta_u, *ps, *grad_ps_x, *grad_ps_y;
} orc_baro_io;

typedef struct orc_baro_ws orc_baro_ws;
void orc_update_ocean_barotropic_ws(orc_baro_ws* ws, const orc_baro_params* p, const orc_baro_io* io);

static void div_ud_any(const orc_dims* d, const orc_baro_params* p, const orc_baro_io* io, const double* u,
                       const double* v, double* out) {
  if (p->cgrid)
    orc_div_ud_cgrid(d, u, v, io->dat, io->dxter, io->dytnr, io->datr, out);
  else
    orc_div_ud_bgrid(d, u, v, io->dyu, io->dxu, io->datr, out);
}

/* The barotropic module arrays, allocated once as ocean_barotropic_init does
 * (ocean_barotropic.F90:1249-1256); every call starts them from zero. */
struct orc_baro_ws {
  orc_dims d;
  double* buf;
};

orc_baro_ws* orc_baro_ws_create(const orc_dims* d) {
  orc_baro_ws* ws = (orc_baro_ws*)calloc(1, sizeof(orc_baro_ws));
  ws->d = *d;
  ws->buf = (double*)calloc((size_t)NXD(d) * NYD(d) * 21, sizeof(double));
  return ws;
}

void orc_baro_ws_destroy(orc_baro_ws* ws) {
  if (!ws) return;
  free(ws->buf);
  free(ws);
}

void orc_update_ocean_barotropic(const orc_dims* d, const orc_baro_params* p, const orc_baro_io* io) {
  orc_baro_ws* ws = orc_baro_ws_create(d);
  orc_update_ocean_barotropic_ws(ws, p, io);
  orc_baro_ws_destroy(ws);
}

void orc_update_ocean_barotropic_ws(orc_baro_ws* ws, const orc_baro_params* p, const orc_baro_io* io) {
  const orc_dims* d = &ws->d;
  int ni = d->ni, nj = d->nj, nts = p->nts;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double rho0r = 1.0 / p->rho0;
  double dtbt = p->dtbt;
  /* ocean_barotropic_init :1195-1197 */
  double dtbt_gamma_rho0r = dtbt * p->pred_corr_gamma * rho0r;
  double dtbt_rho0r = dtbt * rho0r;
  /* AB3 weights :617-619, onefourth */
  const double abtau_m0 = 23.0 / 12.0, abtau_m1 = -16.0 / 12.0, abtau_m2 = 5.0 / 12.0, onefourth = 0.25;

  memset(ws->buf, 0, sizeof(double) * n2 * 21);
  double* eta_bt = ws->buf;
  double* ubt = eta_bt + n2 * 2;
  double* vbt = ubt + n2 * 2;
  double* steady = vbt + n2 * 2;
  double* tmp = steady + n2;
  double* ps = tmp + n2;
  double* gx = ps + n2;
  double* gy = gx + n2;
  double* cori1 = gy + n2;
  double* cori2 = cori1 + n2;
  double* cf = cori2 + n2; /* coriolis_force_bt(·,·,2,3) */
  double* ca = cf + n2 * 6; /* coriolis_accel_bt(·,·,2) */
#define CF(i, j, c, l) cf[((size_t)(l) * 2 + (c)) * n2 + I2(d, (i), (j))]
#define CA(i, j, c) ca[(size_t)(c) * n2 + I2(d, (i), (j))]
  /* :1283-1288 */
  for (size_t q = 0; q < n2; ++q) {
    cori1[q] = 0.5 * dtbt * io->f[q];
    cori2[q] = 1.0 / (1.0 + cori1[q] * cori1[q]);
  }
  int itime = 1;
  int fstau = (itime + 0) % 2, fstaup1 = (itime + 1) % 2; /* 0-based versions of mod(itime,2)+1 */
  for (size_t q = 0; q < n2; ++q) {
    io->eta_t_bar[q] = p->initsum_with_bar ? io->eta_t_bar_tau[q] : io->eta_t_tau[q];
    io->udrho_u[q] = 0.0;
    io->udrho_v[q] = 0.0;
  }
  for (size_t q = 0; q < n2; ++q) {
    eta_bt[fstau * n2 + q] = io->eta_t_bar_tau[q];
    ubt[fstau * n2 + q] = io->udrho_u_tau[q];
    vbt[fstau * n2 + q] = io->udrho_v_tau[q];
    steady[q] = io->tmask1[q] * (io->pme[q] + io->river[q] + io->source[q] - io->eta_smooth[q]);
  }
  if (p->cgrid) {
    int m2 = (itime + 0) % 3, m1 = (itime + 1) % 3, m0 = (itime + 2) % 3;
    const double* u = ubt + fstau * n2;
    const double* v = vbt + fstau * n2;
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) {
        CF(i, j, 0, m0) = onefourth * (io->f[I2(d, i, j)] * (v[I2(d, i, j)] + v[I2(d, i + 1, j)]) +
                                       io->f[I2(d, i, j - 1)] * (v[I2(d, i, j - 1)] + v[I2(d, i + 1, j - 1)]));
        CF(i, j, 0, m1) = CF(i, j, 0, m0);
        CF(i, j, 0, m2) = CF(i, j, 0, m0);
        CA(i, j, 0) = abtau_m0 * CF(i, j, 0, m0) + abtau_m1 * CF(i, j, 0, m1) + abtau_m2 * CF(i, j, 0, m2);
        CF(i, j, 1, m0) = -onefourth * (io->f[I2(d, i, j)] * (u[I2(d, i, j)] + u[I2(d, i, j + 1)]) +
                                        io->f[I2(d, i - 1, j)] * (u[I2(d, i - 1, j)] + u[I2(d, i - 1, j + 1)]));
        CF(i, j, 1, m1) = CF(i, j, 1, m0);
        CF(i, j, 1, m2) = CF(i, j, 1, m0);
        CA(i, j, 1) = abtau_m0 * CF(i, j, 1, m0) + abtau_m1 * CF(i, j, 1, m1) + abtau_m2 * CF(i, j, 1, m2);
      }
    orc_halo_update_2d(d, ca, 3);
    orc_halo_update_2d(d, ca + n2, 3);
  }

  for (itime = 1; itime <= nts; ++itime) {
    fstau = (itime + 0) % 2;
    fstaup1 = (itime + 1) % 2;
    double* eo = eta_bt + fstau * n2;
    double* en = eta_bt + fstaup1 * n2;
    double* uo = ubt + fstau * n2;
    double* un = ubt + fstaup1 * n2;
    double* vo = vbt + fstau * n2;
    double* vn = vbt + fstaup1 * n2;
    /* predictor */
    if (p->pred_corr_gamma > 0.0) {
      div_ud_any(d, p, io, uo, vo, tmp);
      OMP_FOR
      for (size_t q = 0; q < n2; ++q) tmp[q] = -tmp[q] * io->tmask1[q];
      OMP_FOR
      for (size_t q = 0; q < n2; ++q) en[q] = eo[q] + dtbt_gamma_rho0r * (tmp[q] + steady[q]);
    } else {
      OMP_FOR
      for (size_t q = 0; q < n2; ++q) en[q] = eo[q];
    }
    if (!p->cgrid) orc_halo_update_2d(d, en, 3); /* use_legacy_barotropic_halos (B-grid only) */
    OMP_FOR
    for (size_t q = 0; q < n2; ++q) ps[q] = io->rho_g[q] * en[q] + io->patm[q];
    if (!p->cgrid) {
      orc_grad_baro_p(d, 0, ps, io->dxur, io->dyur, io->umask1, io->umask1, gx, gy);
      OMP_FOR
      for (int j = 0; j <= nj + 1; ++j)
        for (int i = 0; i <= ni + 1; ++i) {
          size_t q = I2(d, i, j);
          double pf1 = -io->thicku[q] * gx[q];
          double pf2 = -io->thicku[q] * gy[q];
          double t1 = uo[q] + dtbt * (0.5 * io->f[q] * vo[q] + pf1 + io->forcing_u[q] + 0.0);
          double t2 = vo[q] + dtbt * (-0.5 * io->f[q] * uo[q] + pf2 + io->forcing_v[q] + 0.0);
          un[q] = cori2[q] * (t1 + cori1[q] * t2);
          vn[q] = cori2[q] * (t2 - cori1[q] * t1);
        }
    } else {
      int m2 = (itime + 0) % 3, m1 = (itime + 1) % 3, m0 = (itime + 2) % 3;
      memset(ca, 0, sizeof(double) * n2 * 2);
      OMP_FOR
      for (int j = 1; j <= nj; ++j)
        for (int i = 1; i <= ni; ++i) {
          CF(i, j, 0, m0) = onefourth * (io->f[I2(d, i, j)] * (vo[I2(d, i, j)] + vo[I2(d, i + 1, j)]) +
                                         io->f[I2(d, i, j - 1)] * (vo[I2(d, i, j - 1)] + vo[I2(d, i + 1, j - 1)]));
          CA(i, j, 0) = abtau_m0 * CF(i, j, 0, m0) + abtau_m1 * CF(i, j, 0, m1) + abtau_m2 * CF(i, j, 0, m2);
          CF(i, j, 1, m0) = -onefourth * (io->f[I2(d, i, j)] * (uo[I2(d, i, j)] + uo[I2(d, i, j + 1)]) +
                                          io->f[I2(d, i - 1, j)] * (uo[I2(d, i - 1, j)] + uo[I2(d, i - 1, j + 1)]));
          CA(i, j, 1) = abtau_m0 * CF(i, j, 1, m0) + abtau_m1 * CF(i, j, 1, m1) + abtau_m2 * CF(i, j, 1, m2);
        }
      orc_grad_baro_p(d, 1, ps, io->dxter, io->dytnr, io->tmasken_e, io->tmasken_n, gx, gy);
      OMP_FOR
      for (int j = 0; j <= nj + 1; ++j)
        for (int i = 0; i <= ni + 1; ++i) {
          size_t q = I2(d, i, j);
          double pf1 = -io->thicken_e[q] * gx[q];
          double pf2 = -io->thicken_n[q] * gy[q];
          un[q] = uo[q] + dtbt * io->tmasken_e[q] * (CA(i, j, 0) + pf1 + io->forcing_u[q] + 0.0);
          vn[q] = vo[q] + dtbt * io->tmasken_n[q] * (CA(i, j, 1) + pf2 + io->forcing_v[q] + 0.0);
        }
      orc_halo_update_2d(d, un, 3);
      orc_halo_update_2d(d, vn, 3);
    }
    /* corrector */
    div_ud_any(d, p, io, un, vn, tmp);
    OMP_FOR
    for (size_t q = 0; q < n2; ++q) tmp[q] = -tmp[q] * io->tmask1[q];
    OMP_FOR
    for (size_t q = 0; q < n2; ++q) en[q] = eo[q] + dtbt_rho0r * (tmp[q] + steady[q]);
    /* accumulate */
    double wgt = p->time_stepping_B ? (double)(nts - itime + 1) : 1.0;
    OMP_FOR
    for (size_t q = 0; q < n2; ++q) {
      io->eta_t_bar[q] = io->eta_t_bar[q] + en[q];
      if (p->time_stepping_B) {
        io->udrho_u[q] = io->udrho_u[q] + wgt * un[q];
        io->udrho_v[q] = io->udrho_v[q] + wgt * vn[q];
      } else {
        io->udrho_u[q] = io->udrho_u[q] + un[q];
        io->udrho_v[q] = io->udrho_v[q] + vn[q];
      }
    }
  }
#undef CF
#undef CA
  /* update_ocean_barotropic, splitting branch :2803-2811, :2846-2901, :2969-2985 */
  double rntsp1 = 1.0 / ((double)nts + 1.0);
  double rnts = p->time_stepping_B ? 2.0 / ((double)nts * (double)(nts + 1)) : 1.0 / (double)nts;
  for (size_t q = 0; q < n2; ++q) io->eta_t_bar[q] = rntsp1 * io->eta_t_bar[q];
  orc_halo_update_2d(d, io->eta_t_bar, 3);
  for (size_t q = 0; q < n2; ++q) io->udrho_u[q] = rnts * io->udrho_u[q];
  for (size_t q = 0; q < n2; ++q) io->udrho_v[q] = rnts * io->udrho_v[q];
  orc_halo_update_2d(d, io->udrho_u, 3);
  orc_halo_update_2d(d, io->udrho_v, 3);
  div_ud_any(d, p, io, io->udrho_u, io->udrho_v, tmp);
  for (size_t q = 0; q < n2; ++q) io->conv_rho_ud_t[q] = -tmp[q];
  orc_halo_update_2d(d, io->conv_rho_ud_t, 3);
  orc_remap_bt_to_bu(d, io->eta_t_bar, io->dte, io->dtw, io->dus, io->dun, io->daur, tmp);
  for (size_t q = 0; q < n2; ++q) io->eta_u[q] = io->umask1[q] * tmp[q];
  orc_halo_update_2d(d, io->eta_u, 3);
  /* twolevel: itime = taup1 (:2797-2801) */
  for (size_t q = 0; q < n2; ++q) io->ps[q] = io->rho_g[q] * io->eta_t_bar[q] + io->patm[q];
  if (!p->cgrid)
    orc_grad_baro_p(d, 0, io->ps, io->dxur, io->dyur, io->umask1, io->umask1, io->grad_ps_x, io->grad_ps_y);
  else
    orc_grad_baro_p(d, 1, io->ps, io->dxter, io->dytnr, io->tmasken_e, io->tmasken_n, io->grad_ps_x,
                    io->grad_ps_y);
}

/* eta_and_pbot_tendency, depth-based: ocean_barotropic.F90:2683-2690. */
void orc_eta_and_pbot_tendency(const orc_dims* d, double rho0, const double* tmask1, const double* conv_tau,
                               const double* pme, const double* river, const double* source, double* deta_dt) {
  double rho0r = 1.0 / rho0;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  for (size_t q = 0; q < n2; ++q)
    deta_dt[q] = tmask1[q] * rho0r * (conv_tau[q] + pme[q] + river[q] + source[q]);
}

/* eta_and_pbot_update, depth-based, no OBC: :2314-2330. */
void orc_eta_and_pbot_update(const orc_dims* d, double dtime, const double* eta_taum1, const double* deta_dt,
                             double* eta_taup1) {
  for (int j = 1; j <= d->nj; ++j)
    for (int i = 1; i <= d->ni; ++i) eta_taup1[I2(d, i, j)] = eta_taum1[I2(d, i, j)] + dtime * deta_dt[I2(d, i, j)];
  orc_halo_update_2d(d, eta_taup1, 3);
}

/* Continuity for the B-grid tracer vertical mass flux with rho_dzt_tendency =
 * mass_source = 0: ocean_advection_velocity.F90:600-606 (diverge_t from
 * BDX_ET/BDY_NT, ocean_operators.F90:951-956, :1236-1241) and :609-627.     */
void orc_continuity_w(const orc_dims* d, const double* tmask, const double* dyte, const double* dxtn,
                      const double* datr, const double* uhrho_et, const double* vhrho_nt, const double* pme,
                      const double* river, double* wrho_bt) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* bdx = (double*)calloc(n2, sizeof(double));
  double* bdy = (double*)calloc(n2, sizeof(double));
  for (size_t q = 0; q < n2; ++q) wrho_bt[q] = -(pme[q] + river[q]);
  for (int k = 0; k < nk; ++k) {
    memset(bdx, 0, sizeof(double) * n2);
    memset(bdy, 0, sizeof(double) * n2);
    for (int j = 0; j <= nj + 1; ++j)
      for (int i = 1; i <= ni + 1; ++i)
        bdx[I2(d, i, j)] = (dyte[I2(d, i, j)] * uhrho_et[I3(d, i, j, k)] -
                            dyte[I2(d, i - 1, j)] * uhrho_et[I3(d, i - 1, j, k)]) *
                           datr[I2(d, i, j)];
    for (int j = 1; j <= nj + 1; ++j)
      for (int i = 0; i <= ni + 1; ++i)
        bdy[I2(d, i, j)] = (dxtn[I2(d, i, j)] * vhrho_nt[I3(d, i, j, k)] -
                            dxtn[I2(d, i, j - 1)] * vhrho_nt[I3(d, i, j - 1, k)]) *
                           datr[I2(d, i, j)];
    for (size_t q = 0; q < n2; ++q) {
      double div = tmask[(size_t)k * n2 + q] * (bdx[q] + bdy[q]);
      wrho_bt[(size_t)(k + 1) * n2 + q] = (0.0 + div + wrho_bt[(size_t)k * n2 + q]) * tmask[(size_t)k * n2 + q];
    }
  }
  free(bdx);
  free(bdy);
}

/* ocean_advection_velocity (ocean_advection_velocity.F90:568-672), T-cell part,
 * no blobs, OBC or inflow.  B grid (:600-606): uhrho_et = BAY(u*dyu*rho_dzu)/dyte,
 * vhrho_nt = BAX(v*dxu*rho_dzu)/dxtn, with BAY/BAX (ocean_operators.F90:834-902)
 * zero on the first row/column of the data domain.  C grid (:645-654):
 * uhrho_et = u*rho_dzten_e*dxt_dxter*dyt_dyter, vhrho_nt = v*rho_dzten_n*dxt_dxtnr*dyt_dytnr.
 * Both: diverge_t = tmask*(BDX_ET(uhrho_et) + BDY_NT(vhrho_nt)) and
 * wrho_bt(0) = -(pme+river), wrho_bt(k) = ((rho_dzt_tendency-mass_source) + diverge_t
 * + wrho_bt(k-1))*tmask (:614-625, :657-662).  Unused pointers may be NULL. */
void orc_ocean_advection_velocity(const orc_dims* d, int cgrid, const double* u, const double* v,
                                  const double* rho_dzu, const double* rho_dzten_e, const double* rho_dzten_n,
                                  const double* dxu, const double* dyu, const double* dyte, const double* dxtn,
                                  const double* dxt_dxter, const double* dyt_dyter, const double* dxt_dxtnr,
                                  const double* dyt_dytnr, const double* datr, const double* tmask,
                                  const double* rho_dzt_tendency, const double* mass_source, const double* pme,
                                  const double* river, double* uhrho_et, double* vhrho_nt, double* diverge_t,
                                  double* wrho_bt) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* a = (double*)calloc(n2, sizeof(double));
  double* bdx = (double*)calloc(n2, sizeof(double));
  double* bdy = (double*)calloc(n2, sizeof(double));
  for (int k = 0; k < nk; ++k) {
    double* ue = uhrho_et + (size_t)k * n2;
    double* vn = vhrho_nt + (size_t)k * n2;
    const double* uk = u + (size_t)k * n2;
    const double* vk = v + (size_t)k * n2;
    if (!cgrid) {
      const double* rz = rho_dzu + (size_t)k * n2;
      for (size_t q = 0; q < n2; ++q) a[q] = uk[q] * dyu[q] * rz[q];
      for (int j = 0; j <= nj + 1; ++j)
        for (int i = 0; i <= ni + 1; ++i) {
          double bay = j >= 1 ? 0.5 * (a[I2(d, i, j)] + a[I2(d, i, j - 1)]) : 0.0;
          ue[I2(d, i, j)] = bay / dyte[I2(d, i, j)];
        }
      for (size_t q = 0; q < n2; ++q) a[q] = vk[q] * dxu[q] * rz[q];
      for (int j = 0; j <= nj + 1; ++j)
        for (int i = 0; i <= ni + 1; ++i) {
          double bax = i >= 1 ? 0.5 * (a[I2(d, i, j)] + a[I2(d, i - 1, j)]) : 0.0;
          vn[I2(d, i, j)] = bax / dxtn[I2(d, i, j)];
        }
    } else {
      const double* re = rho_dzten_e + (size_t)k * n2;
      const double* rn = rho_dzten_n + (size_t)k * n2;
      for (size_t q = 0; q < n2; ++q) {
        ue[q] = uk[q] * re[q] * dxt_dxter[q] * dyt_dyter[q];
        vn[q] = vk[q] * rn[q] * dxt_dxtnr[q] * dyt_dytnr[q];
      }
    }
    memset(bdx, 0, sizeof(double) * n2);
    memset(bdy, 0, sizeof(double) * n2);
    for (int j = 0; j <= nj + 1; ++j)
      for (int i = 1; i <= ni + 1; ++i)
        bdx[I2(d, i, j)] = (dyte[I2(d, i, j)] * ue[I2(d, i, j)] - dyte[I2(d, i - 1, j)] * ue[I2(d, i - 1, j)]) *
                           datr[I2(d, i, j)];
    for (int j = 1; j <= nj + 1; ++j)
      for (int i = 0; i <= ni + 1; ++i)
        bdy[I2(d, i, j)] = (dxtn[I2(d, i, j)] * vn[I2(d, i, j)] - dxtn[I2(d, i, j - 1)] * vn[I2(d, i, j - 1)]) *
                           datr[I2(d, i, j)];
    const double* tm = tmask + (size_t)k * n2;
    for (size_t q = 0; q < n2; ++q) diverge_t[(size_t)k * n2 + q] = tm[q] * (bdx[q] + bdy[q]);
  }
  for (size_t q = 0; q < n2; ++q) wrho_bt[q] = -(pme[q] + river[q]);
  for (int k = 0; k < nk; ++k)
    for (size_t q = 0; q < n2; ++q) {
      size_t p = (size_t)k * n2 + q;
      double tmp = rho_dzt_tendency[p] - mass_source[p];
      wrho_bt[(size_t)(k + 1) * n2 + q] = (tmp + diverge_t[p] + wrho_bt[(size_t)k * n2 + q]) * tmask[p];
    }
  free(a);
  free(bdx);
  free(bdy);
}

/* Surface and bottom source terms of the explicit tracer step, one tracer
 * (ocean_tracer.F90:2318-2336). kmt is the 2-D array of deepest wet levels. */
void orc_tracer_boundary_terms(const orc_dims* d, const double* tmask, const int* kmt, const double* pme,
                               const double* tpme, const double* eta_smooth, const double* pbot_smooth, double* th) {
  size_t n2 = (size_t)NXD(d) * NYD(d);
  for (int j = 1; j <= d->nj; ++j)
    for (int i = 1; i <= d->ni; ++i) {
      size_t q = I2(d, i, j);
      th[q] = th[q] + tmask[q] * (pme[q] * tpme[q] + eta_smooth[q]);
    }
  for (int j = 1; j <= d->nj; ++j)
    for (int i = 1; i <= d->ni; ++i) {
      size_t q = I2(d, i, j);
      int kbot = kmt[q];
      if (kbot > 0) {
        size_t p = (size_t)(kbot - 1) * n2 + q;
        th[p] = th[p] + tmask[p] * pbot_smooth[q];
      }
    }
}

/* ocean_barotropic_forcing (ocean_barotropic.F90:3058-3141), one component;
 * tmasken and accel are 3-D.  friction_lap and friction_bih (data domain) are the
 * component's barotropic frictions, or NULL for the reference's 0.0 (udrho_lap =
 * udrho_bih = .false., their default). */
void orc_ocean_barotropic_forcing_friction(const orc_dims* d, int zero_nonlinear, int zero_forcing,
                                           const double* tmasken, const double* accel, const double* smf,
                                           const double* bmf, const double* friction_lap,
                                           const double* friction_bih, double* forcing) {
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* wrk = (double*)calloc(n2, sizeof(double));
  for (size_t q = 0; q < n2; ++q) forcing[q] = 0.0;
  if (!zero_nonlinear)
    for (int k = 0; k < d->nk; ++k)
      for (int j = 1; j <= d->nj; ++j)
        for (int i = 1; i <= d->ni; ++i) {
          size_t q = I2(d, i, j);
          wrk[q] = wrk[q] + tmasken[(size_t)k * n2 + q] * accel[(size_t)k * n2 + q];
        }
  for (int j = 1; j <= d->nj; ++j)
    for (int i = 1; i <= d->ni; ++i) {
      size_t q = I2(d, i, j);
      forcing[q] = wrk[q] + tmasken[q] * (smf[q] - bmf[q]);
    }
  orc_halo_update_2d(d, forcing, 3);
  for (size_t q = 0; q < n2; ++q)
    forcing[q] = forcing[q] + (friction_lap ? friction_lap[q] : 0.0) + (friction_bih ? friction_bih[q] : 0.0);
  if (zero_forcing)
    for (size_t q = 0; q < n2; ++q) forcing[q] = 0.0;
  free(wrk);
}

void orc_ocean_barotropic_forcing(const orc_dims* d, int zero_nonlinear, int zero_forcing, const double* tmasken,
                                  const double* accel, const double* smf, const double* bmf, double* forcing) {
  orc_ocean_barotropic_forcing_friction(d, zero_nonlinear, zero_forcing, tmasken, accel, smf, bmf, NULL, NULL,
                                        forcing);
}

/* Background viscosities of the barotropic friction, as ocean_barotropic_init
 * forms them (ocean_barotropic.F90:1306-1341): all four start at 0.0;
 * smooth_lap_udrho = umask*udrho_lap_vel_micom*(2.0*dxu*dyu/(dxu+dyu)) and
 * smooth_bih_udrho = umask*udrho_bih_vel_micom*(...)**3 over the data domain
 * (x**3 evaluated as x*x*x, left to right); the east and north face averages
 * 0.5*(s(i,j)+s(i+1,j)), 0.5*(s(i,j)+s(i,j+1)) on the compute domain; the
 * halo update of each; then the square root of the two biharmonic ones over
 * the data domain. */
void orc_bt_friction_back(const orc_dims* d, const double* dxu, const double* dyu, const double* umask1,
                          double vel_lap, double vel_bih, double* lap_ceu, double* lap_cnu, double* bih_ceu,
                          double* bih_cnu) {
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* sl = (double*)malloc(n2 * sizeof(double));
  double* sb = (double*)malloc(n2 * sizeof(double));
  for (size_t q = 0; q < n2; ++q) {
    double x = 2.0 * dxu[q] * dyu[q] / (dxu[q] + dyu[q]);
    sl[q] = umask1[q] * vel_lap * x;
    sb[q] = umask1[q] * vel_bih * (x * x * x);
    lap_ceu[q] = lap_cnu[q] = bih_ceu[q] = bih_cnu[q] = 0.0;
  }
  for (int j = 1; j <= d->nj; ++j)
    for (int i = 1; i <= d->ni; ++i) {
      size_t q = I2(d, i, j), qe = I2(d, i + 1, j), qn = I2(d, i, j + 1);
      lap_ceu[q] = 0.5 * (sl[q] + sl[qe]);
      lap_cnu[q] = 0.5 * (sl[q] + sl[qn]);
      bih_ceu[q] = 0.5 * (sb[q] + sb[qe]);
      bih_cnu[q] = 0.5 * (sb[q] + sb[qn]);
    }
  orc_halo_update_2d(d, lap_ceu, 3);
  orc_halo_update_2d(d, lap_cnu, 3);
  orc_halo_update_2d(d, bih_ceu, 3);
  orc_halo_update_2d(d, bih_cnu, 3);
  for (size_t q = 0; q < n2; ++q) {
    bih_ceu[q] = sqrt(bih_ceu[q]);
    bih_cnu[q] = sqrt(bih_cnu[q]);
  }
  free(sl);
  free(sb);
}

/* The ocean_operators B-grid operators on the data domain, in the reference's
 * ranges (halo 1): FDX_U(a)(i,j) = (a(i+1,j)-a(i,j))*dxuer(i,j), 0.0 at ied
 * (ocean_operators.F90:973-986); FDY_U with dyunr, 0.0 at jed (:1258-1271);
 * BDX_EU(a)(i,j) = (dyue(i,j)*a(i,j) - dyue(i-1,j)*a(i-1,j))*daur(i,j), 0.0 at
 * isd (:917-930); BDY_NU with dxun, 0.0 at jsd (:1202-1215). */
static void op_fdx_u(const orc_dims* d, const double* dxuer, const double* a, double* out) {
  for (int j = 0; j <= d->nj + 1; ++j) {
    for (int i = 0; i <= d->ni; ++i) out[I2(d, i, j)] = (a[I2(d, i + 1, j)] - a[I2(d, i, j)]) * dxuer[I2(d, i, j)];
    out[I2(d, d->ni + 1, j)] = 0.0;
  }
}
static void op_fdy_u(const orc_dims* d, const double* dyunr, const double* a, double* out) {
  for (int j = 0; j <= d->nj; ++j)
    for (int i = 0; i <= d->ni + 1; ++i) out[I2(d, i, j)] = (a[I2(d, i, j + 1)] - a[I2(d, i, j)]) * dyunr[I2(d, i, j)];
  for (int i = 0; i <= d->ni + 1; ++i) out[I2(d, i, d->nj + 1)] = 0.0;
}
static void op_bdx_eu(const orc_dims* d, const double* dyue, const double* daur, const double* a, double* out) {
  for (int j = 0; j <= d->nj + 1; ++j) {
    for (int i = 1; i <= d->ni + 1; ++i)
      out[I2(d, i, j)] = (dyue[I2(d, i, j)] * a[I2(d, i, j)] - dyue[I2(d, i - 1, j)] * a[I2(d, i - 1, j)]) *
                         daur[I2(d, i, j)];
    out[I2(d, 0, j)] = 0.0;
  }
}
static void op_bdy_nu(const orc_dims* d, const double* dxun, const double* daur, const double* a, double* out) {
  for (int j = 1; j <= d->nj + 1; ++j)
    for (int i = 0; i <= d->ni + 1; ++i)
      out[I2(d, i, j)] = (dxun[I2(d, i, j)] * a[I2(d, i, j)] - dxun[I2(d, i, j - 1)] * a[I2(d, i, j - 1)]) *
                         daur[I2(d, i, j)];
  for (int i = 0; i <= d->ni + 1; ++i) out[I2(d, i, 0)] = 0.0;
}

/* tmp = BDX_EU((ce_back+ce_visc)*FDX_U(a)) + BDY_NU((cn_back+cn_visc)*FDY_U(a)) as
 * whole-array expressions; out = tmp*umask (negate: -tmp*umask) on the compute
 * domain of an array that was 0.0, then its halo update
 * (ocean_lap_friction.F90:433-443; ocean_bih_friction.F90:428-451). */
static void bt_friction_op(const orc_dims* d, const double* const* m, const double* ce_back, const double* ce_visc,
                           const double* cn_back, const double* cn_visc, const double* a, int negate, double* out) {
  const double *dyue = m[0], *dxuer = m[1], *dxun = m[2], *dyunr = m[3], *daur = m[4], *umask1 = m[5];
  size_t n2 = (size_t)NXD(d) * NYD(d);
  double* fx = (double*)malloc(n2 * sizeof(double));
  double* fy = (double*)malloc(n2 * sizeof(double));
  double* bx = (double*)malloc(n2 * sizeof(double));
  double* by = (double*)malloc(n2 * sizeof(double));
  op_fdx_u(d, dxuer, a, fx);
  op_fdy_u(d, dyunr, a, fy);
  for (size_t q = 0; q < n2; ++q) {
    fx[q] = (ce_back[q] + ce_visc[q]) * fx[q];
    fy[q] = (cn_back[q] + cn_visc[q]) * fy[q];
  }
  op_bdx_eu(d, dyue, daur, fx, bx);
  op_bdy_nu(d, dxun, daur, fy, by);
  for (size_t q = 0; q < n2; ++q) out[q] = 0.0;
  for (int j = 1; j <= d->nj; ++j)
    for (int i = 1; i <= d->ni; ++i) {
      size_t q = I2(d, i, j);
      double tmp = bx[q] + by[q];
      out[q] = (negate ? -tmp : tmp) * umask1[q];
    }
  orc_halo_update_2d(d, out, 3);
  free(fx);
  free(fy);
  free(bx);
  free(by);
}

/* The barotropic friction of one component a = udrho(:,:,n,tau) (ocean_barotropic.F90:
 * 3105-3113): friction_lap = lap_friction_barotropic (ocean_lap_friction.F90:423-446)
 * when lap, friction_bih = bih_friction_barotropic (ocean_bih_friction.F90:416-454:
 * del2_vel, then the negated second iteration) when bih; 0.0 otherwise.
 * m = {dyue, dxuer, dxun, dyunr, daur, umask1}; c = {lap_ceu_back, lap_cnu_back,
 * lap_visc_ceu, lap_visc_cnu, bih_ceu_back, bih_cnu_back, bih_visc_ceu,
 * bih_visc_cnu}; del2 receives del2_vel when bih. */
void orc_bt_friction(const orc_dims* d, int lap, int bih, const double* const* m, const double* const* c,
                     const double* a, double* friction_lap, double* friction_bih, double* del2) {
  size_t n2 = (size_t)NXD(d) * NYD(d);
  for (size_t q = 0; q < n2; ++q) friction_lap[q] = friction_bih[q] = 0.0;
  if (lap) bt_friction_op(d, m, c[0], c[2], c[1], c[3], a, 0, friction_lap);
  if (bih) {
    bt_friction_op(d, m, c[4], c[6], c[5], c[7], a, 0, del2);
    bt_friction_op(d, m, c[4], c[6], c[5], c[7], del2, 1, friction_bih);
  }
}

/* total_tracer (ocean_tracer_diag.F90:2395-2412) with conversion = 1: the
 * per-column sum over k in the reference order, then a global sum.  The
 * global sum here is Neumaier-compensated; result[0] = sum, result[1] = the
 * plain left-to-right sum in Fortran array order. */
void orc_total_tracer(const orc_dims* d, const double* tmask, const double* dat, const double* rho_dzt,
                      const double* T, double* result) {
  int ni = d->ni, nj = d->nj, nk = d->nk;
  double s = 0.0, c = 0.0, plain = 0.0;
  for (int j = 1; j <= nj; ++j)
    for (int i = 1; i <= ni; ++i) {
      double col = 0.0;
      for (int k = 0; k < nk; ++k) {
        size_t p = I3(d, i, j, k);
        col = col + 1.0 * tmask[p] * dat[I2(d, i, j)] * rho_dzt[p] * T[p];
      }
      plain += col;
      double t = s + col;
      if (fabs(s) >= fabs(col))
        c += (s - t) + col;
      else
        c += (col - t) + s;
      s = t;
    }
  result[0] = s + c;
  result[1] = plain;
}

/* mass integral used by the barotropic conservation test: sum of
 * tmask1 * dat * eta over the compute domain, Neumaier-compensated. */
double orc_area_integral(const orc_dims* d, const double* tmask1, const double* dat, const double* eta) {
  double s = 0.0, c = 0.0;
  for (int j = 1; j <= d->nj; ++j)
    for (int i = 1; i <= d->ni; ++i) {
      double x = tmask1[I2(d, i, j)] * dat[I2(d, i, j)] * eta[I2(d, i, j)];
      double t = s + x;
      if (fabs(s) >= fabs(x))
        c += (s - t) + x;
      else
        c += (x - t) + s;
      s = t;
    }
  return s + c;
}

/* update_ucell_thickness (ocean_thickness.F90:3507-3886), no blobs.
 * vcoord: 1 GEOPOTENTIAL, 3 ZSIGMA, 6 PSIGMA, any other value (ZSTAR, PRESSURE,
 * PSTAR) the branch that takes U-cell and face thicknesses as the minimum of
 * the neighbouring T cells (:3735-3763).  Arrays are data-domain [k][j][i];
 * dzwt and dzwu hold levels 0..nk (nk+1 planes).  kmu (Grid%kmu) is given.
 * Updated in place: dzu, dzwu, rho_dzu (level taup1), rho_dzur, dzten_e/n,
 * rho_dzten_e/n, depth_zu, depth_zwu; written: thicku and mass_u (level
 * taup1), thicken_e/n, mass_en_e/n.  Fortran min(a,b,c,d) is evaluated left to
 * right with a < b ? a : b; single-PE mpp_update_domains halos. */
void orc_update_ucell_thickness(const orc_dims* d, int vcoord, int linear_free_surface, int update_dzwu_k0,
                                double rho0, const double* umask, const double* tmasken_e, const double* tmasken_n,
                                const double* dzt, const double* dzwt, const double* rho_dzt, const double* depth_zt1,
                                const double* depth_zwt1, const double* eta_u, const int* kmu, double* dzu,
                                double* dzwu, double* rho_dzu, double* rho_dzur, double* dzten_e, double* dzten_n,
                                double* rho_dzten_e, double* rho_dzten_n, double* depth_zu, double* depth_zwu,
                                double* thicku, double* thicken_e, double* thicken_n, double* mass_u,
                                double* mass_en_e, double* mass_en_n) {
  const double epsln = 1.0e-20; /* constants_mod epsln */
  int ni = d->ni, nj = d->nj, nk = d->nk;
  size_t n2 = (size_t)NXD(d) * NYD(d);
#define MIN4(a, b, c, e) fmind(fmind(fmind((a), (b)), (c)), (e))
  if (vcoord == 1) {
    for (int j = 0; j <= nj + 1; ++j)
      for (int i = 0; i <= ni + 1; ++i) {
        size_t q = I2(d, i, j);
        double eu = linear_free_surface ? 0.0 : eta_u[q];
        dzwu[q] = linear_free_surface ? depth_zt1[q] : depth_zt1[q] + eu;             /* dzwu(:,:,0) */
        dzu[q] = linear_free_surface ? depth_zwt1[q] : depth_zwt1[q] + eu;            /* dzu(:,:,1) */
        rho_dzu[q] = rho0 * dzu[q];
        rho_dzur[q] = 1.0 / (rho_dzu[q] + epsln);
      }
  } else {
    if (vcoord == 3 || vcoord == 6) {
      for (int k = 0; k < nk; ++k)
        for (size_t q = 0; q < n2; ++q) {
          size_t p = (size_t)k * n2 + q;
          dzu[p] = dzt[p];
          dzten_e[p] = dzt[p];
          dzten_n[p] = dzt[p];
          dzwu[p + n2] = dzwt[p + n2];
          rho_dzu[p] = rho_dzt[p];
        }
      for (size_t q = 0; q < n2; ++q) dzwu[q] = dzwt[q];
    } else {
      for (int k = 0; k < nk; ++k)
        for (int j = 0; j <= nj; ++j)
          for (int i = 0; i <= ni; ++i) {
            size_t p = I3(d, i, j, k), pe = I3(d, i + 1, j, k), pn = I3(d, i, j + 1, k), pne = I3(d, i + 1, j + 1, k);
            dzu[p] = MIN4(dzt[p], dzt[pe], dzt[pn], dzt[pne]);
            dzwu[p + n2] = MIN4(dzwt[p + n2], dzwt[pe + n2], dzwt[pn + n2], dzwt[pne + n2]);
            rho_dzu[p] = MIN4(rho_dzt[p], rho_dzt[pe], rho_dzt[pn], rho_dzt[pne]);
            dzten_e[p] = fmind(dzt[p], dzt[pe]);
            dzten_n[p] = fmind(dzt[p], dzt[pn]);
            rho_dzten_e[p] = fmind(rho_dzt[p], rho_dzt[pe]);
            rho_dzten_n[p] = fmind(rho_dzt[p], rho_dzt[pn]);
          }
      if (update_dzwu_k0)
        for (int j = 0; j <= nj; ++j)
          for (int i = 0; i <= ni; ++i)
            dzwu[I2(d, i, j)] = MIN4(dzwt[I2(d, i, j)], dzwt[I2(d, i + 1, j)], dzwt[I2(d, i, j + 1)],
                                     dzwt[I2(d, i + 1, j + 1)]);
      orc_halo_update_3d(d, dzu, nk, 3);
      orc_halo_update_3d(d, dzwu, nk + 1, 3);
      orc_halo_update_3d(d, rho_dzu, nk, 3);
      orc_halo_update_3d(d, dzten_e, nk, 3);
      orc_halo_update_3d(d, dzten_n, nk, 3);
      orc_halo_update_3d(d, rho_dzten_e, nk, 3);
      orc_halo_update_3d(d, rho_dzten_n, nk, 3);
    }
    for (int k = 0; k < nk; ++k)
      for (size_t q = 0; q < n2; ++q) {
        size_t p = (size_t)k * n2 + q;
        rho_dzur[p] = umask[p] / (rho_dzu[p] + epsln);
      }
    for (size_t q = 0; q < n2; ++q) {
      depth_zu[q] = dzwu[q];
      depth_zwu[q] = dzu[q];
    }
    for (int k = 1; k < nk; ++k)
      for (size_t q = 0; q < n2; ++q) {
        size_t p = (size_t)k * n2 + q;
        depth_zu[p] = depth_zu[p - n2] + dzwu[p];          /* + dzwu(k-1): level k-1 of 0..nk is plane k */
        depth_zwu[p] = depth_zwu[p - n2] + dzu[p];
      }
  }
#undef MIN4
  for (size_t q = 0; q < n2; ++q) {
    int k = kmu[q];
    thicku[q] = k > 1 ? depth_zwu[(size_t)(k - 1) * n2 + q] : 0.0;
  }
  for (size_t q = 0; q < n2; ++q) {
    thicken_e[q] = 0.0;
    thicken_n[q] = 0.0;
    mass_u[q] = 0.0;
    mass_en_e[q] = 0.0;
    mass_en_n[q] = 0.0;
  }
  for (int k = 0; k < nk; ++k)
    for (size_t q = 0; q < n2; ++q) {
      size_t p = (size_t)k * n2 + q;
      thicken_e[q] = thicken_e[q] + dzten_e[p];
      thicken_n[q] = thicken_n[q] + dzten_n[p];
    }
  for (int k = 0; k < nk; ++k)
    for (size_t q = 0; q < n2; ++q) {
      size_t p = (size_t)k * n2 + q;
      mass_u[q] = mass_u[q] + umask[p] * rho_dzu[p];
    }
  for (int k = 0; k < nk; ++k)
    for (size_t q = 0; q < n2; ++q) {
      size_t p = (size_t)k * n2 + q;
      mass_en_e[q] = mass_en_e[q] + tmasken_e[p] * rho_dzten_e[p];
    }
  for (int k = 0; k < nk; ++k)
    for (size_t q = 0; q < n2; ++q) {
      size_t p = (size_t)k * n2 + q;
      mass_en_n[q] = mass_en_n[q] + tmasken_n[p] * rho_dzten_n[p];
    }
}

/* ------------------------------------------------------------------------- */
/* The CPU baseline's timed loop: warmup + steps two-level baroclinic steps  */
/* of one block with no host language in between.  Each step advects every  */
/* tracer by MDFL Sweby into a zeroed th_tendency (update_advection_only,    */
/* ocean_tracer.F90:2618-2649; horz_advect_tracer :1925-1936), updates it    */
/* explicitly (:2341-2350) and halo-updates T(taup1) (ocean_model.F90:       */
/* 1903-1911), then runs update_ocean_barotropic when p is not NULL.  The    */
/* scratch lives across steps as the reference's module arrays do (mdfl_init */
/* ocean_tracer_advect.F90:1644-1669, ocean_barotropic_init :1249-1256).  T  */
/* holds ntr data-domain blocks and ends at the last step's values; the      */
/* barotropic *_tau inputs and out_* outputs of io swap roles every step (a  */
/* local copy of io; the caller's arrays hold the last two steps).  Returns  */
/* the seconds of the timed steps (CLOCK_MONOTONIC).                         */
/* ------------------------------------------------------------------------- */
double orc_run_steps(const orc_dims* d, int ntr, int warmup, int steps, double dtts, const double* tmask,
                     const double* dat, const double* datr, const double* dxte, const double* dyte,
                     const double* dxtn, const double* dytn, const double* uhrho_et, const double* vhrho_nt,
                     const double* wrho_bt, const double* rho_dzt, const double* rho_dztr, double* T,
                     const orc_baro_params* p, const orc_baro_io* io_in) {
  size_t n3 = (size_t)NXD(d) * NYD(d) * d->nk;
  orc_mdfl_ws* ws = ntr > 0 ? orc_mdfl_ws_create(d, tmask) : NULL;
  orc_baro_ws* bws = p ? orc_baro_ws_create(d) : NULL;
  orc_baro_io io;
  if (io_in) io = *io_in;
  double* th = (double*)malloc(sizeof(double) * (n3 > 0 ? n3 : 1));
  double* wrk1 = (double*)malloc(sizeof(double) * (n3 > 0 ? n3 : 1));
  double* other = (double*)malloc(sizeof(double) * (n3 * (size_t)ntr + 1));
  if (ntr > 0) memcpy(other, T, sizeof(double) * n3 * (size_t)ntr);
  double* cur = T;
  double* nxt = other;
  struct timespec t0 = {0, 0}, t1;
  for (int s = 0; s < warmup + steps; ++s) {
    if (s == warmup) clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int n = 0; n < ntr; ++n) {
      zero_par(th, n3);
      orc_advect_mdfl_sweby_ws(ws, 1.0, dtts, dat, datr, dxte, dyte, dxtn, dytn, uhrho_et, vhrho_nt, wrho_bt,
                               rho_dzt, cur + n * n3, wrk1);
      OMP_FOR
      for (int k = 0; k < d->nk; ++k)
        for (int j = 1; j <= d->nj; ++j)
          for (int i = 1; i <= d->ni; ++i) th[I3(d, i, j, k)] = th[I3(d, i, j, k)] + wrk1[I3(d, i, j, k)];
      orc_update_tracer(d, dtts, rho_dzt, rho_dztr, cur + n * n3, th, nxt + n * n3);
      orc_halo_update_3d(d, nxt + n * n3, d->nk, 3);
    }
    double* sw = cur;
    cur = nxt;
    nxt = sw;
    if (p) {
      orc_update_ocean_barotropic_ws(bws, p, &io);
      /* the outputs become the next step's inputs; the old inputs take the next outputs */
      double* a;
      a = (double*)io.eta_t_bar_tau; io.eta_t_bar_tau = io.eta_t_bar; io.eta_t_bar = a;
      a = (double*)io.udrho_u_tau; io.udrho_u_tau = io.udrho_u; io.udrho_u = a;
      a = (double*)io.udrho_v_tau; io.udrho_v_tau = io.udrho_v; io.udrho_v = a;
    }
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (ntr > 0 && cur != T) memcpy(T, cur, sizeof(double) * n3 * (size_t)ntr);
  free(th);
  free(wrk1);
  free(other);
  orc_mdfl_ws_destroy(ws);
  orc_baro_ws_destroy(bws);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
