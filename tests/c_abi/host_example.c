/* A C host of the library (what a non-Python, non-Fortran caller writes): one
 * small closed basin, uniform tracers in a flow at rest, one baroclinic step of
 * MDFL advection plus the barotropic subcycle, then the status-code contract.
 * Prints "ok" and exits 0 when every check holds. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "mom5gpu.h"

#define NI 20
#define NJ 16
#define NK 6
#define NTR 2

static int fail_count = 0;
#define CHECK(cond, ...)               \
  do {                                 \
    if (!(cond)) {                     \
      fprintf(stderr, __VA_ARGS__);    \
      fputc('\n', stderr);             \
      ++fail_count;                    \
    }                                  \
  } while (0)

static int set(mom5gpu_domain* d, int f, int n, int lv, const double* a) {
  int st = mom5gpu_set_field(d, f, n, lv, a, 0);
  if (st) fprintf(stderr, "set_field %d: %s\n", f, mom5gpu_last_error(d));
  return st;
}

int main(void) {
  const int nxd = NI + 2, nyd = NJ + 2;
  const size_t n2 = (size_t)nxd * nyd, n3 = n2 * NK, n3w = n2 * (NK + 1);
  mom5gpu_dims dims = {NI, NJ, NK, 0, 0, NTR, MOM5GPU_BGRID};
  mom5gpu_options opt;
  mom5gpu_default_options(&opt);
  opt.barotropic_time_stepping_B = 1;
  mom5gpu_domain* d = NULL;
  if (mom5gpu_create(&dims, &opt, &d) != MOM5GPU_OK) {
    fprintf(stderr, "create: %s\n", mom5gpu_last_error(NULL));
    return 2;
  }
  double* a2 = calloc(n2, sizeof(double));
  double* a3 = calloc(n3w, sizeof(double));
  double* tm = calloc(n3, sizeof(double));
  int* kmt = calloc(n2, sizeof(int));
  double dzt[NK], zw[NK];
  for (int k = 0; k < NK; ++k) {
    dzt[k] = 100.0;
    zw[k] = 100.0 * (k + 1);
  }
  /* uniform 10 km metrics */
  const int metrics[] = {MOM5GPU_DXT, MOM5GPU_DYT, MOM5GPU_DXU, MOM5GPU_DYU, MOM5GPU_DXTE, MOM5GPU_DYTE,
                         MOM5GPU_DXTN, MOM5GPU_DYTN, MOM5GPU_DTE, MOM5GPU_DTW, MOM5GPU_DUS, MOM5GPU_DUN};
  for (size_t q = 0; q < n2; ++q) a2[q] = 1.0e4;
  for (size_t m = 0; m < sizeof(metrics) / sizeof(metrics[0]); ++m) set(d, metrics[m], 0, 0, a2);
  for (size_t q = 0; q < n2; ++q) a2[q] = 1.0e8;
  set(d, MOM5GPU_DAT, 0, 0, a2);
  for (size_t q = 0; q < n2; ++q) a2[q] = 1.0e-8;
  set(d, MOM5GPU_DATR, 0, 0, a2);
  set(d, MOM5GPU_DAUR, 0, 0, a2);
  for (size_t q = 0; q < n2; ++q) a2[q] = 1.0e-4;
  const int recips[] = {MOM5GPU_DXUR, MOM5GPU_DYUR, MOM5GPU_DXTER, MOM5GPU_DYTNR, MOM5GPU_CORIOLIS_F};
  for (size_t m = 0; m < sizeof(recips) / sizeof(recips[0]); ++m) set(d, recips[m], 0, 0, a2);
  /* a closed basin: wet interior, walls on the halo; kmt = NK */
  for (int j = 1; j <= NJ; ++j)
    for (int i = 1; i <= NI; ++i) {
      kmt[j * nxd + i] = NK;
      for (int k = 0; k < NK; ++k) tm[(size_t)k * n2 + j * nxd + i] = 1.0;
    }
  set(d, MOM5GPU_TMASK, 0, 0, tm);
  for (size_t q = 0; q < n2; ++q) a2[q] = tm[q];
  set(d, MOM5GPU_TMASKEN_E1, 0, 0, a2);
  set(d, MOM5GPU_TMASKEN_N1, 0, 0, a2);
  set(d, MOM5GPU_UMASK1, 0, 0, a2);
  /* at rest: zero transports; rho_dzt = 1035 * 100 */
  set(d, MOM5GPU_UHRHO_ET, 0, 0, a3);
  set(d, MOM5GPU_VHRHO_NT, 0, 0, a3);
  set(d, MOM5GPU_WRHO_BT, 0, 0, a3);
  for (size_t p = 0; p < n3; ++p) a3[p] = 1035.0 * 100.0;
  set(d, MOM5GPU_RHO_DZT, 0, 1, a3);
  set(d, MOM5GPU_RHO_DZT, 0, 2, a3);
  for (size_t p = 0; p < n3; ++p) a3[p] = 1.0 / (1035.0 * 100.0);
  set(d, MOM5GPU_RHO_DZTR, 0, 0, a3);
  for (size_t q = 0; q < n2; ++q) a2[q] = 600.0 * tm[q];
  set(d, MOM5GPU_THICKU, 0, 1, a2);
  set(d, MOM5GPU_THICKU, 0, 2, a2);
  for (size_t q = 0; q < n2; ++q) a2[q] = 1035.0 * 9.8;
  set(d, MOM5GPU_RHO_G, 0, 0, a2);
  for (int n = 1; n <= NTR; ++n) {
    for (size_t p = 0; p < n3; ++p) a3[p] = (n == 1 ? 12.5 : 35.0) * tm[p];
    set(d, MOM5GPU_TRACER, n, 1, a3);
  }
  CHECK(mom5gpu_set_vertical_grid(d, dzt, zw, kmt) == MOM5GPU_OK, "set_vertical_grid");
  CHECK(mom5gpu_tracer_advect_init(d) == MOM5GPU_OK, "advect_init: %s", mom5gpu_last_error(d));
  CHECK(mom5gpu_barotropic_init(d, 600.0, 20.0) == MOM5GPU_OK, "barotropic_init: %s", mom5gpu_last_error(d));
  CHECK(mom5gpu_barotropic_nts(d) == 60, "nts %d", mom5gpu_barotropic_nts(d));
  CHECK(mom5gpu_tracer_advection_step(d, 1, 1, 2, 600.0) == MOM5GPU_OK, "step: %s", mom5gpu_last_error(d));
  CHECK(mom5gpu_update_ocean_barotropic(d, 1, 2) == MOM5GPU_OK, "barotropic: %s", mom5gpu_last_error(d));
  /* at rest and uniform: every wet value unchanged (to the rounding of the
   * explicit update's (rho_dzt*T)*(1/rho_dzt)) */
  for (int n = 1; n <= NTR; ++n) {
    CHECK(mom5gpu_get_field(d, MOM5GPU_TRACER, n, 2, a3, 0) == MOM5GPU_OK, "get");
    double want = n == 1 ? 12.5 : 35.0, worst = 0.0;
    for (size_t p = 0; p < n3; ++p)
      if (tm[p] != 0.0) worst = fmax(worst, fabs(a3[p] - want));
    CHECK(worst <= 1e-14 * want, "tracer %d moved by %g at rest", n, worst);
  }
  double content = 0.0;
  CHECK(mom5gpu_global_tracer_content(d, 1, 2, &content) == MOM5GPU_OK, "content");
  CHECK(fabs(content - 12.5 * 1035.0 * 100.0 * 1.0e8 * NI * NJ * NK) <= 1e-12 * content, "content %.17g", content);
  /* the status-code contract: errors are returned, never aborted on */
  CHECK(mom5gpu_horz_advect_tracer(d, NTR + 1, 1, 1, 600.0) == MOM5GPU_EINVAL, "bad tracer accepted");
  CHECK(mom5gpu_last_error(d)[0] != 0, "no message for the last error");
  CHECK(mom5gpu_set_tracer_scheme(d, 1, MOM5GPU_ADVECT_QUICKMOM3, MOM5GPU_ADVECT_QUICKMOM3, -1e10, 1e10) ==
            MOM5GPU_EUNSUPPORTED, "vertical quickmom3 accepted");
  CHECK(mom5gpu_set_itt0(d, -1) == MOM5GPU_EINVAL, "negative itt0 accepted");
  CHECK(mom5gpu_set_field(d, 9999, 0, 0, a3, 0) != MOM5GPU_OK, "unknown field accepted");
  CHECK(mom5gpu_strerror(MOM5GPU_ECFL)[0] != 0, "strerror");
  mom5gpu_destroy(d);
  free(a2);
  free(a3);
  free(tm);
  free(kmt);
  if (fail_count) return 1;
  printf("ok\n");
  return 0;
}
