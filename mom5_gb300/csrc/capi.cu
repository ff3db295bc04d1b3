// Host side of the C ABI declared in include/mom5gpu.h.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

using namespace mom5;

namespace {

thread_local std::string g_create_error;

const FieldInfo kFields[] = {
    {MOM5GPU_DXT, S2D, false, false},         {MOM5GPU_DYT, S2D, false, false},
    {MOM5GPU_DXU, S2D, false, false},         {MOM5GPU_DYU, S2D, false, false},
    {MOM5GPU_DXTE, S2D, false, false},        {MOM5GPU_DYTE, S2D, false, false},
    {MOM5GPU_DXTN, S2D, false, false},        {MOM5GPU_DYTN, S2D, false, false},
    {MOM5GPU_DAT, S2D, false, false},         {MOM5GPU_DATR, S2D, false, false},
    {MOM5GPU_DXUR, S2D, false, false},        {MOM5GPU_DYUR, S2D, false, false},
    {MOM5GPU_DXTER, S2D, false, false},       {MOM5GPU_DYTNR, S2D, false, false},
    {MOM5GPU_DTE, S2D, false, false},         {MOM5GPU_DTW, S2D, false, false},
    {MOM5GPU_DUS, S2D, false, false},         {MOM5GPU_DUN, S2D, false, false},
    {MOM5GPU_DAUR, S2D, false, false},        {MOM5GPU_CORIOLIS_F, S2D, false, false},
    {MOM5GPU_UMASK1, S2D, false, false},      {MOM5GPU_TMASKEN_E1, S2D, false, false},
    {MOM5GPU_TMASKEN_N1, S2D, false, false},  {MOM5GPU_TMASK, S3D, false, false},
    {MOM5GPU_UHRHO_ET, S3D, false, false},    {MOM5GPU_VHRHO_NT, S3D, false, false},
    {MOM5GPU_WRHO_BT, S3DW, false, false},    {MOM5GPU_RHO_DZT, S3D, false, true},
    {MOM5GPU_RHO_DZTR, S3D, false, false},    {MOM5GPU_THICKU, S2D, false, true},
    {MOM5GPU_THICKEN_E, S2D, false, false},   {MOM5GPU_THICKEN_N, S2D, false, false},
    {MOM5GPU_TRACER, S3D, true, true},        {MOM5GPU_TH_TENDENCY, S3D, true, false},
    {MOM5GPU_TMASK_LIMIT, S3D, true, false},  {MOM5GPU_ETA_T, S2D, false, true},
    {MOM5GPU_ETA_T_BAR, S2D, false, true},    {MOM5GPU_ETA_U, S2D, false, true},
    {MOM5GPU_UDRHO_U, S2D, false, true},      {MOM5GPU_UDRHO_V, S2D, false, true},
    {MOM5GPU_CONV_RHO_UD_T, S2D, false, true}, {MOM5GPU_DETA_DT, S2D, false, false},
    {MOM5GPU_FORCING_BT_U, S2D, false, false}, {MOM5GPU_FORCING_BT_V, S2D, false, false},
    {MOM5GPU_SOURCE, S2D, false, false},      {MOM5GPU_ETA_SMOOTH, S2D, false, false},
    {MOM5GPU_PS, S2D, false, false},          {MOM5GPU_GRAD_PS_X, S2D, false, false},
    {MOM5GPU_GRAD_PS_Y, S2D, false, false},   {MOM5GPU_PATM, S2D, false, false},
    {MOM5GPU_PME, S2D, false, false},         {MOM5GPU_RIVER, S2D, false, false},
    {MOM5GPU_RHO_G, S2D, false, false},
    {MOM5GPU_DXT_DXTER, S2D, false, false},   {MOM5GPU_DYT_DYTER, S2D, false, false},
    {MOM5GPU_DXT_DXTNR, S2D, false, false},   {MOM5GPU_DYT_DYTNR, S2D, false, false},
    {MOM5GPU_DIVERGE_T, S3D, false, false},   {MOM5GPU_RHO_DZU, S3D, false, true},
    {MOM5GPU_RHO_DZTEN_E, S3D, false, false}, {MOM5GPU_RHO_DZTEN_N, S3D, false, false},
    {MOM5GPU_RHO_DZT_TENDENCY, S3D, false, false}, {MOM5GPU_MASS_SOURCE, S3D, false, false},
    {MOM5GPU_U_VEL, S3D, false, true},        {MOM5GPU_V_VEL, S3D, false, true},
    {MOM5GPU_TMASKEN_E, S3D, false, false},   {MOM5GPU_TMASKEN_N, S3D, false, false},
    {MOM5GPU_TPME, S2D, true, false},         {MOM5GPU_TRACER_ETA_SMOOTH, S2D, true, false},
    {MOM5GPU_PBOT_SMOOTH, S2D, true, false},  {MOM5GPU_ACCEL_U, S3D, false, false},
    {MOM5GPU_ACCEL_V, S3D, false, false},     {MOM5GPU_SMF_U, S2D, false, false},
    {MOM5GPU_SMF_V, S2D, false, false},       {MOM5GPU_BMF_U, S2D, false, false},
    {MOM5GPU_BMF_V, S2D, false, false},
    {MOM5GPU_PSOM_S0, S3D, true, false},      {MOM5GPU_PSOM_SX, S3D, true, false},
    {MOM5GPU_PSOM_SXX, S3D, true, false},     {MOM5GPU_PSOM_SY, S3D, true, false},
    {MOM5GPU_PSOM_SYY, S3D, true, false},     {MOM5GPU_PSOM_SZ, S3D, true, false},
    {MOM5GPU_PSOM_SZZ, S3D, true, false},     {MOM5GPU_PSOM_SXY, S3D, true, false},
    {MOM5GPU_PSOM_SXZ, S3D, true, false},     {MOM5GPU_PSOM_SYZ, S3D, true, false},
    {MOM5GPU_UMASK, S3D, false, false},       {MOM5GPU_DZT, S3D, false, false},
    {MOM5GPU_DZWT, S3DW, false, false},       {MOM5GPU_DZU, S3D, false, false},
    {MOM5GPU_DZWU, S3DW, false, false},       {MOM5GPU_RHO_DZUR, S3D, false, false},
    {MOM5GPU_DZTEN_E, S3D, false, false},     {MOM5GPU_DZTEN_N, S3D, false, false},
    {MOM5GPU_DEPTH_ZT, S3D, false, false},    {MOM5GPU_DEPTH_ZWT, S3D, false, false},
    {MOM5GPU_DEPTH_ZU, S3D, false, false},    {MOM5GPU_DEPTH_ZWU, S3D, false, false},
    {MOM5GPU_MASS_U, S2D, false, true},       {MOM5GPU_MASS_EN_E, S2D, false, false},
    {MOM5GPU_MASS_EN_N, S2D, false, false},
    {MOM5GPU_DYUE, S2D, false, false},        {MOM5GPU_DXUER, S2D, false, false},
    {MOM5GPU_DXUN, S2D, false, false},        {MOM5GPU_DYUNR, S2D, false, false},
    {MOM5GPU_LAP_VISC_CEU, S2D, false, false}, {MOM5GPU_LAP_VISC_CNU, S2D, false, false},
    {MOM5GPU_BIH_VISC_CEU, S2D, false, false}, {MOM5GPU_BIH_VISC_CNU, S2D, false, false},
    {MOM5GPU_LAP_CEU_BACK, S2D, false, false}, {MOM5GPU_LAP_CNU_BACK, S2D, false, false},
    {MOM5GPU_BIH_CEU_BACK, S2D, false, false}, {MOM5GPU_BIH_CNU_BACK, S2D, false, false},
    {MOM5GPU_LAP_FRICTION_BT_U, S2D, false, false}, {MOM5GPU_LAP_FRICTION_BT_V, S2D, false, false},
    {MOM5GPU_BIH_FRICTION_BT_U, S2D, false, false}, {MOM5GPU_BIH_FRICTION_BT_V, S2D, false, false},
    {MOM5GPU_BIH_DEL2_VEL_U, S2D, false, false}, {MOM5GPU_BIH_DEL2_VEL_V, S2D, false, false},
};

// field storage: one block per (field, level) holding every tracer of that level
int slot_of(int id, int level) { return id * 4 + level; }

}  // namespace

namespace mom5 {

const FieldInfo* field_info(int id) {
  for (const FieldInfo& f : kFields)
    if (f.id == id) return &f;
  return nullptr;
}

size_t field_count(const Geo& g, Shape s) {
  switch (s) {
    case S2D: return (size_t)g.n2;
    case S3D: return (size_t)g.n3;
    case S3DW: return (size_t)g.n2 * (g.nk + 1);
  }
  return 0;
}

int fail(mom5gpu_domain* d, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (d) d->err = buf;
  else g_create_error = buf;
  return code;
}

int cuda_fail(mom5gpu_domain* d, cudaError_t e, const char* where) {
  return fail(d, MOM5GPU_ECUDA, "%s: %s", where, cudaGetErrorString(e));
}

// Device pointer of (field, tracer n, level) if its block was ever allocated.
double* fptr_if_set(mom5gpu_domain* d, int id, int n, int level) {
  const FieldInfo* fi = field_info(id);
  if (!fi) return nullptr;
  int ntr = d->dims.num_prog_tracers;
  if (fi->per_tracer && (n < 1 || n > ntr)) return nullptr;
  if (fi->per_level && (level < 1 || level > 3)) return nullptr;
  int slot = slot_of(id, fi->per_level ? level : 0);
  if ((size_t)slot >= d->field.size() || !d->field[slot]) return nullptr;
  return d->field[slot] + (fi->per_tracer ? (size_t)(n - 1) * field_count(d->geo, fi->shape) : 0);
}

// Device pointer of (field, tracer n, level); the block is allocated (zeroed)
// on first use.  Returns nullptr on a bad index or allocation failure.
double* fptr(mom5gpu_domain* d, int id, int n, int level) {
  const FieldInfo* fi = field_info(id);
  if (!fi) return nullptr;
  int ntr = d->dims.num_prog_tracers;
  if (fi->per_tracer && (n < 1 || n > ntr)) return nullptr;
  if (fi->per_level && (level < 1 || level > 3)) return nullptr;
  int lv = fi->per_level ? level : 0;
  int slot = slot_of(id, lv);
  if ((size_t)slot >= d->field.size()) d->field.resize(slot + 1, nullptr);
  size_t cnt = field_count(d->geo, fi->shape);
  size_t per = fi->per_tracer ? (size_t)ntr : 1;
  if (!d->field[slot]) {
    double* p = nullptr;
    if (cudaMalloc(&p, sizeof(double) * cnt * per) != cudaSuccess) {
      cudaGetLastError();
      fail(d, MOM5GPU_ENOMEM, "allocating field %d (%zu bytes)", id, sizeof(double) * cnt * per);
      return nullptr;
    }
    // The first use of a field may be a copy queued on another stream
    // (mom5gpu_copy_field_async): the zeroing must be complete before this
    // returns, not merely queued behind the domain stream's pending work.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(d->stream, &cs);
    if (cs == cudaStreamCaptureStatusNone) {
      cudaMemset(p, 0, sizeof(double) * cnt * per);
      cudaDeviceSynchronize();
    } else {
      cudaMemsetAsync(p, 0, sizeof(double) * cnt * per, d->stream);
    }
    d->bytes += sizeof(double) * cnt * per;
    d->field[slot] = p;
  }
  return d->field[slot] + (fi->per_tracer ? (size_t)(n - 1) * cnt : 0);
}

static cudaEvent_t take_event(mom5gpu_domain* d) {
  if (!d->event_pool.empty()) {
    cudaEvent_t e = d->event_pool.back();
    d->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ClockScope::ClockScope(mom5gpu_domain* d_, int s) : d(d_), sec(s) {
  if (!d->timing) return;
  a = take_event(d);
  cudaEventRecord(a, d->stream);
}

ClockScope::~ClockScope() {
  if (!d->timing || !a) return;
  cudaEvent_t b = take_event(d);
  cudaEventRecord(b, d->stream);
  d->clocks.push_back({sec, a, b});
}

static void resolve_clocks(mom5gpu_domain* d) {
  for (auto& c : d->clocks) {
    cudaEventSynchronize(c.b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c.a, c.b);
    d->clock_ms[c.section] += ms;
    d->clock_calls[c.section] += 1;
    d->event_pool.push_back(c.a);
    d->event_pool.push_back(c.b);
  }
  d->clocks.clear();
}

// The device words of the bounded waits, in one allocation: the error word
// (bit 0: a TMA-staged copy did not arrive; bit 1: a grid barrier gave up) and
// the arrival counter of the cooperative subcycle kernel's grid barriers.
int ensure_wait_words(mom5gpu_domain* d) {
  if (d->wait_err) return MOM5GPU_OK;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p, 0, 2 * sizeof(int));
  if (e != cudaSuccess) {
    if (p) cudaFree(p);
    return cuda_fail(d, e, "error word");
  }
  d->wait_err = (int*)p;
  d->bt_sync = (unsigned*)p + 1;
  return MOM5GPU_OK;
}

}  // namespace mom5

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

void mom5gpu_default_options(mom5gpu_options* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->advect_sweby_all = 0;
  o->limit_with_upwind = 0;
  o->zero_tracer_advect_horz = 0;
  o->zero_tracer_advect_vert = 0;
  o->barotropic_time_stepping_A = 0;
  o->barotropic_time_stepping_B = 0;
  o->initsum_with_bar = 1;
  o->pred_corr_gamma = 0.2;
  o->rho0 = 1035.0;
  o->grav = 9.80;
  o->precision = MOM5GPU_PRECISION_FP64;
  o->zero_forcing_bt = 0;
  o->zero_nonlinear_forcing_bt = 0;
  o->psom_limit_prather = 0;
  o->udrho_lap = 0;
  o->udrho_bih = 0;
  o->udrho_lap_vel_micom = 0.05;
  o->udrho_bih_vel_micom = 0.01;
}

const char* mom5gpu_strerror(int s) {
  switch (s) {
    case MOM5GPU_OK: return "ok";
    case MOM5GPU_EINVAL: return "invalid argument";
    case MOM5GPU_ENOMEM: return "out of device memory";
    case MOM5GPU_ECUDA: return "CUDA runtime error";
    case MOM5GPU_ESTATE: return "call out of order";
    case MOM5GPU_ECFL: return "barotropic CFL violated";
    case MOM5GPU_ENUMERIC: return "non-finite value";
    case MOM5GPU_ETIMEDOUT: return "bounded wait timed out";
    case MOM5GPU_EUNSUPPORTED: return "unsupported option";
    case MOM5GPU_EFULL: return "no free slot";
  }
  return "unknown status";
}

int mom5gpu_create(const mom5gpu_dims* dims, const mom5gpu_options* opt, mom5gpu_domain** out) {
  if (!dims || !out) return fail(nullptr, MOM5GPU_EINVAL, "mom5gpu_create: null argument");
  *out = nullptr;
  if (dims->ni < 2 || dims->nj < 2 || dims->nk < 1 || dims->num_prog_tracers < 0)
    return fail(nullptr, MOM5GPU_EINVAL, "mom5gpu_create: bad dimensions %d x %d x %d, %d tracers", dims->ni,
                dims->nj, dims->nk, dims->num_prog_tracers);
  if (dims->horz_grid != MOM5GPU_BGRID && dims->horz_grid != MOM5GPU_CGRID)
    return fail(nullptr, MOM5GPU_EINVAL, "mom5gpu_create: horz_grid must be MOM5GPU_BGRID or MOM5GPU_CGRID");
  mom5gpu_domain* d = new (std::nothrow) mom5gpu_domain();
  if (!d) return fail(nullptr, MOM5GPU_ENOMEM, "mom5gpu_create: host allocation");
  d->dims = *dims;
  if (opt) d->opt = *opt;
  else mom5gpu_default_options(&d->opt);
  if (d->opt.precision != MOM5GPU_PRECISION_FP64 && d->opt.precision != MOM5GPU_PRECISION_MIXED) {
    delete d;
    return fail(nullptr, MOM5GPU_EINVAL, "mom5gpu_create: precision must be FP64 or MIXED");
  }
  Geo& g = d->geo;
  g.ni = dims->ni;
  g.nj = dims->nj;
  g.nk = dims->nk;
  g.nxd = g.ni + 2;
  g.nyd = g.nj + 2;
  g.cx = dims->cyclic_x ? 1 : 0;
  g.cy = dims->cyclic_y ? 1 : 0;
  g.n2 = (long)g.nxd * g.nyd;
  g.n3 = g.n2 * g.nk;
  d->scheme.resize(dims->num_prog_tracers);
  for (int n = 1; n <= dims->num_prog_tracers; ++n) {
    d->tracer_name.push_back("tracer" + std::to_string(n));
    d->tracer_file.push_back("ocean_tracer.res.nc");  // default_restart_file, ocean_tpm_util.F90:76
  }
  cudaError_t e = cudaStreamCreateWithFlags(&d->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete d;
    return fail(nullptr, MOM5GPU_ECUDA, "mom5gpu_create: stream: %s", cudaGetErrorString(e));
  }
  d->stream = d->own_stream;
  *out = d;
  return MOM5GPU_OK;
}

void mom5gpu_destroy(mom5gpu_domain* d) {
  if (!d) return;
  if (d->stream) cudaStreamSynchronize(d->stream);
  for (double* p : d->field)
    if (p) cudaFree(p);
  if (d->mask2) cudaFree(d->mask2);
  QuickerWeights& q = d->qw;
  for (double* p : {q.quick_x, q.quick_y, q.curv_xp, q.curv_xn, q.curv_yp, q.curv_yn, q.quick_z, q.curv_zp, q.curv_zn})
    if (p) cudaFree(p);
  for (double* p : {d->cori1, d->cori2, d->mdfl_a, d->mdfl_b, d->bt, d->red, d->ppm_scr, d->psom_scr})
    if (p) cudaFree(p);
  if (d->mixed_scr) cudaFree(d->mixed_scr);
  if (d->flag) cudaFree(d->flag);
  if (d->wait_err) cudaFree(d->wait_err);  // bt_sync shares its allocation
  if (d->hz) cudaFree(d->hz);
  if (d->hx) cudaFree(d->hx);
  if (d->kmt_d) cudaFree(d->kmt_d);
  for (auto& gr : d->bt_graphs)
    if (gr.exec) cudaGraphExecDestroy(gr.exec);
  if (d->red_h) cudaFreeHost(d->red_h);
  for (auto& c : d->clocks) {
    cudaEventDestroy(c.a);
    cudaEventDestroy(c.b);
  }
  for (cudaEvent_t e : d->event_pool) cudaEventDestroy(e);
  if (d->own_stream) cudaStreamDestroy(d->own_stream);
  delete d;
}

const char* mom5gpu_last_error(const mom5gpu_domain* d) { return d ? d->err.c_str() : g_create_error.c_str(); }

int mom5gpu_set_stream(mom5gpu_domain* d, void* stream) {
  if (!d) return MOM5GPU_EINVAL;
  d->stream = stream ? (cudaStream_t)stream : d->own_stream;
  return MOM5GPU_OK;
}

int mom5gpu_synchronize(mom5gpu_domain* d) {
  if (!d) return MOM5GPU_EINVAL;
  cudaError_t e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return cuda_fail(d, e, "synchronize");
  if (d->wait_err) {  // a bounded wait of a kernel gave up
    int v = 0;
    e = cudaMemcpy(&v, d->wait_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(d, e, "synchronize");
    if (v) {
      cudaMemset(d->wait_err, 0, sizeof(int));
      if (v & 2)
        return fail(d, MOM5GPU_ETIMEDOUT, "barotropic subcycles: a grid barrier wait gave up; the step's results are void");
      return fail(d, MOM5GPU_ETIMEDOUT, "precision form: a tile's staged copy did not arrive; its results are void");
    }
  }
  return MOM5GPU_OK;
}

size_t mom5gpu_device_bytes(const mom5gpu_domain* d) { return d ? d->bytes : 0; }

size_t mom5gpu_field_count(const mom5gpu_domain* d, int field) {
  const FieldInfo* fi = field_info(field);
  if (!d || !fi) return 0;
  return field_count(d->geo, fi->shape);
}

static int check_field(mom5gpu_domain* d, int field, int n, int level, double** p, size_t* cnt) {
  const FieldInfo* fi = field_info(field);
  if (!fi) return fail(d, MOM5GPU_EINVAL, "unknown field id %d", field);
  if (fi->per_tracer && (n < 1 || n > d->dims.num_prog_tracers))
    return fail(d, MOM5GPU_EINVAL, "field %d: tracer %d outside 1..%d", field, n, d->dims.num_prog_tracers);
  if (fi->per_level && (level < 1 || level > 3))
    return fail(d, MOM5GPU_EINVAL, "field %d: time level %d outside 1..3", field, level);
  *p = fptr(d, field, n, level);
  if (!*p) return MOM5GPU_ENOMEM;
  *cnt = field_count(d->geo, fi->shape);
  return MOM5GPU_OK;
}

int mom5gpu_set_field(mom5gpu_domain* d, int field, int n, int level, const double* src, int on_device) {
  if (!d || !src) return d ? fail(d, MOM5GPU_EINVAL, "set_field: null source") : MOM5GPU_EINVAL;
  double* p;
  size_t cnt;
  int rc = check_field(d, field, n, level, &p, &cnt);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(p, src, sizeof(double) * cnt, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDefault,
                                  d->stream);
  if (e != cudaSuccess) return cuda_fail(d, e, "set_field copy");
  if (field == MOM5GPU_TMASK) d->advect_ready = false;
  return MOM5GPU_OK;
}

int mom5gpu_set_ppm_limiter(mom5gpu_domain* d, int n, int lim) {
  if (!d) return MOM5GPU_EINVAL;
  if (n < 1 || n > d->dims.num_prog_tracers) return fail(d, MOM5GPU_EINVAL, "set_ppm_limiter: tracer %d", n);
  if (lim < 1 || lim > 3)
    return fail(d, MOM5GPU_EINVAL, "set_ppm_limiter: must choose ppm_hlimiter=1,2 or 3 (got %d)", lim);
  d->scheme[n - 1].ppm_limiter = lim;
  return MOM5GPU_OK;
}

int mom5gpu_set_psom_limit(mom5gpu_domain* d, int n, int on) {
  if (!d) return MOM5GPU_EINVAL;
  if (n < 1 || n > d->dims.num_prog_tracers) return fail(d, MOM5GPU_EINVAL, "set_psom_limit: tracer %d", n);
  d->scheme[n - 1].psom_limit = on ? 1 : 0;
  return MOM5GPU_OK;
}

int mom5gpu_set_itt0(mom5gpu_domain* d, long itt0) {
  if (!d) return MOM5GPU_EINVAL;
  // mod(itt0, 6) of a negative counter matches none of the sweep orders
  if (itt0 < 0) return fail(d, MOM5GPU_EINVAL, "set_itt0: the time-step counter must be >= 0 (got %ld)", itt0);
  d->itt0 = itt0;
  return MOM5GPU_OK;
}

int mom5gpu_get_field(mom5gpu_domain* d, int field, int n, int level, double* dst, int on_device) {
  if (!d || !dst) return d ? fail(d, MOM5GPU_EINVAL, "get_field: null destination") : MOM5GPU_EINVAL;
  double* p;
  size_t cnt;
  int rc = check_field(d, field, n, level, &p, &cnt);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(dst, p, sizeof(double) * cnt, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDefault,
                                  d->stream);
  if (e == cudaSuccess && !on_device) e = cudaStreamSynchronize(d->stream);
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "get_field copy");
}

int mom5gpu_copy_field_async(mom5gpu_domain* d, int field, int n, int level, double* host, int to_device,
                             void* stream) {
  if (!d || !host) return d ? fail(d, MOM5GPU_EINVAL, "copy_field_async: null host buffer") : MOM5GPU_EINVAL;
  double* p;
  size_t cnt;
  int rc = check_field(d, field, n, level, &p, &cnt);
  if (rc) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : d->stream;
  cudaError_t e = to_device ? cudaMemcpyAsync(p, host, sizeof(double) * cnt, cudaMemcpyDefault, s)
                            : cudaMemcpyAsync(host, p, sizeof(double) * cnt, cudaMemcpyDefault, s);
  if (e != cudaSuccess) return cuda_fail(d, e, "copy_field_async");
  if (to_device && field == MOM5GPU_TMASK) d->advect_ready = false;
  return MOM5GPU_OK;
}

int mom5gpu_field_device_ptr(mom5gpu_domain* d, int field, int n, int level, double** dptr) {
  if (!d || !dptr) return MOM5GPU_EINVAL;
  size_t cnt;
  return check_field(d, field, n, level, dptr, &cnt);
}

int mom5gpu_set_vertical_grid(mom5gpu_domain* d, const double* dzt, const double* zw, const int* kmt) {
  if (!d || !dzt || !zw || !kmt) return d ? fail(d, MOM5GPU_EINVAL, "set_vertical_grid: null argument") : MOM5GPU_EINVAL;
  d->dzt_h.assign(dzt, dzt + d->geo.nk);
  d->zw_h.assign(zw, zw + d->geo.nk);
  d->kmt_h.assign(kmt, kmt + d->geo.n2);
  return MOM5GPU_OK;
}

int mom5gpu_set_tracer_scheme(mom5gpu_domain* d, int n, int horz, int vert, double tmin, double tmax) {
  if (!d) return MOM5GPU_EINVAL;
  if (n < 1 || n > d->dims.num_prog_tracers) return fail(d, MOM5GPU_EINVAL, "set_tracer_scheme: tracer %d", n);
  auto ok = [](int s) {
    return s == MOM5GPU_ADVECT_UPWIND || s == MOM5GPU_ADVECT_2ND_ORDER || s == MOM5GPU_ADVECT_4TH_ORDER ||
           s == MOM5GPU_ADVECT_6TH_ORDER || s == MOM5GPU_ADVECT_QUICKER || s == MOM5GPU_ADVECT_MDPPM ||
           s == MOM5GPU_ADVECT_MDFL_SUP_B || s == MOM5GPU_ADVECT_MDFL_SWEBY || s == MOM5GPU_ADVECT_DST_LINEAR ||
           s == MOM5GPU_ADVECT_PSOM;
  };
  if (vert == MOM5GPU_ADVECT_QUICKMOM3)
    return fail(d, MOM5GPU_EUNSUPPORTED, "set_tracer_scheme: vertical quickmom3 reads levels nk+1 and nk+2 at the "
                                          "bottom level and, under tmask_limit, upos/uneg before it sets them "
                                          "(ocean_tracer_advect.F90:3060-3150): its result is undefined there");
  if (!(ok(horz) || horz == MOM5GPU_ADVECT_QUICKMOM3) || !ok(vert))
    return fail(d, MOM5GPU_EUNSUPPORTED, "set_tracer_scheme: scheme %d/%d is outside upwind, 2nd/4th/6th order, "
                                          "quicker, quickmom3 (horizontal), mdfl_sup_b, mdppm, mdfl_sweby, "
                                          "dst_linear, psom", horz, vert);
  // MDPPM reads a halo of 4: at least 4 compute points across a cyclic direction
  if (horz == MOM5GPU_ADVECT_MDPPM && ((d->geo.cx && d->geo.ni < 4) || (d->geo.cy && d->geo.nj < 4)))
    return fail(d, MOM5GPU_EUNSUPPORTED, "set_tracer_scheme: mdppm needs ni, nj >= 4 across cyclic edges");
  // a halo of 3 (6th order) needs at least 3 compute points across a cyclic direction
  if ((horz == MOM5GPU_ADVECT_6TH_ORDER || horz == MOM5GPU_ADVECT_4TH_ORDER) &&
      ((d->geo.cx && d->geo.ni < 3) || (d->geo.cy && d->geo.nj < 3)))
    return fail(d, MOM5GPU_EUNSUPPORTED, "set_tracer_scheme: 4th/6th order needs ni, nj >= 3 across cyclic edges");
  // ocean_tracer.F90:1076-1087: a 3-D scheme must be chosen for both directions
  auto three_d = [](int s) {
    return s == MOM5GPU_ADVECT_MDFL_SWEBY || s == MOM5GPU_ADVECT_DST_LINEAR || s == MOM5GPU_ADVECT_MDPPM ||
           s == MOM5GPU_ADVECT_MDFL_SUP_B || s == MOM5GPU_ADVECT_PSOM;
  };
  bool h3 = three_d(horz), v3 = three_d(vert);
  if (h3 != v3 || (h3 && horz != vert))
    return fail(d, MOM5GPU_EINVAL, "tracer %d: a 3-D scheme (MDFL, Super-B, DST, MDPPM, PSOM) must be used for both horizontal and "
                                   "vertical advection", n);
  d->scheme[n - 1].horz = horz;
  d->scheme[n - 1].vert = vert;
  d->scheme[n - 1].min_limit = tmin;
  d->scheme[n - 1].max_limit = tmax;
  return MOM5GPU_OK;
}

// ---- init ----------------------------------------------------------------

static int download(mom5gpu_domain* d, int field, int level, std::vector<double>& h) {
  const FieldInfo* fi = field_info(field);
  h.resize(field_count(d->geo, fi->shape));
  return mom5gpu_get_field(d, field, 0, level, h.data(), 0);
}

static int upload_new(mom5gpu_domain* d, double** dst, const std::vector<double>& h) {
  if (!*dst) {
    cudaError_t e = cudaMalloc(dst, sizeof(double) * h.size());
    if (e != cudaSuccess) return cuda_fail(d, e, "init allocation");
    d->bytes += sizeof(double) * h.size();
  }
  cudaError_t e = cudaMemcpyAsync(*dst, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, d->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "init upload");
}

// quicker_init (ocean_tracer_advect.F90:1442-1586), host side.
static int quicker_init(mom5gpu_domain* d, const std::vector<double>& dxt, const std::vector<double>& dyt) {
  const Geo& g = d->geo;
  int ni = g.ni, nj = g.nj, nk = g.nk;
  int nx2 = ni + 4, ny2 = nj + 4;
  auto H = [&](int i, int j) { return (size_t)(j + 1) * nx2 + (i + 1); };
  auto D = [&](int i, int j) { return (size_t)j * g.nxd + i; };
  std::vector<double> dxq((size_t)nx2 * ny2, 0.0), dyq((size_t)nx2 * ny2, 0.0);
  for (int j = 1; j <= nj; ++j)
    for (int i = 1; i <= ni; ++i) {
      dxq[H(i, j)] = dxt[D(i, j)];
      dyq[H(i, j)] = dyt[D(i, j)];
    }
  // boundary fill for the non-cyclic case (:1489-1507)
  for (int i = -1; i <= 0; ++i) {
    for (int j = 1; j <= nj; ++j) dxq[H(i, j)] = dxq[H(1, j)];
    for (int j = -1; j <= nj + 2; ++j) dyq[H(i, j)] = dyq[H(1, j)];
  }
  for (int i = ni + 1; i <= ni + 2; ++i) {
    for (int j = 1; j <= nj; ++j) dxq[H(i, j)] = dxq[H(ni, j)];
    for (int j = -1; j <= nj + 2; ++j) dyq[H(i, j)] = dyq[H(ni, j)];
  }
  for (int j = -1; j <= 0; ++j)
    for (int i = -1; i <= ni + 2; ++i) {
      dxq[H(i, j)] = dxq[H(i, 1)];
      dyq[H(i, j)] = dyq[H(i, 1)];
    }
  for (int j = nj + 1; j <= nj + 2; ++j)
    for (int i = -1; i <= ni + 2; ++i) {
      dxq[H(i, j)] = dxq[H(i, nj)];
      dyq[H(i, j)] = dyq[H(i, nj)];
    }
  // halo-2 update of dxt_quick/dyt_quick (:1508-1509)
  for (std::vector<double>* a : {&dxq, &dyq}) {
    std::vector<double>& v = *a;
    if (g.cx)
      for (int j = 1; j <= nj; ++j)
        for (int h = 1; h <= 2; ++h) {
          v[H(1 - h, j)] = v[H(ni + 1 - h, j)];
          v[H(ni + h, j)] = v[H(h, j)];
        }
    if (g.cy)
      for (int i = 1; i <= ni; ++i)
        for (int h = 1; h <= 2; ++h) {
          v[H(i, 1 - h)] = v[H(i, nj + 1 - h)];
          v[H(i, nj + h)] = v[H(i, h)];
        }
    if (g.cx && g.cy)
      for (int hj = 1; hj <= 2; ++hj)
        for (int hi = 1; hi <= 2; ++hi) {
          v[H(1 - hi, 1 - hj)] = v[H(ni + 1 - hi, nj + 1 - hj)];
          v[H(ni + hi, 1 - hj)] = v[H(hi, nj + 1 - hj)];
          v[H(1 - hi, nj + hj)] = v[H(ni + 1 - hi, hj)];
          v[H(ni + hi, nj + hj)] = v[H(hi, hj)];
        }
  }
  size_t n2 = (size_t)g.n2;
  std::vector<double> qx(2 * n2, 0.0), qy(2 * n2, 0.0), cxp(3 * n2, 0.0), cxn(3 * n2, 0.0), cyp(3 * n2, 0.0),
      cyn(3 * n2, 0.0);
  auto X = [&](int i, int j) { return dxq[H(i, j)]; };
  auto Y = [&](int i, int j) { return dyq[H(i, j)]; };
  for (int i = 0; i <= ni; ++i)
    for (int j = 0; j <= nj; ++j) {
      size_t q = D(i, j);
      qx[q] = X(i + 1, j) / (X(i + 1, j) + X(i, j));
      qx[n2 + q] = X(i, j) / (X(i + 1, j) + X(i, j));
      qy[q] = Y(i, j + 1) / (Y(i, j + 1) + Y(i, j));
      qy[n2 + q] = Y(i, j) / (Y(i, j + 1) + Y(i, j));
      cxp[q] = X(i, j) * X(i + 1, j) / ((X(i - 1, j) + 2.0 * X(i, j) + X(i + 1, j)) * (X(i, j) + X(i + 1, j)));
      cxp[n2 + q] = -X(i, j) * X(i + 1, j) / ((X(i, j) + X(i + 1, j)) * (X(i - 1, j) + X(i, j)));
      cxp[2 * n2 + q] = X(i, j) * X(i + 1, j) / ((X(i - 1, j) + 2.0 * X(i, j) + X(i + 1, j)) * (X(i - 1, j) + X(i, j)));
      cxn[q] = X(i, j) * X(i + 1, j) / ((X(i, j) + 2.0 * X(i + 1, j) + X(i + 2, j)) * (X(i + 1, j) + X(i + 2, j)));
      cxn[n2 + q] = -X(i, j) * X(i + 1, j) / ((X(i + 1, j) + X(i + 2, j)) * (X(i, j) + X(i + 1, j)));
      cxn[2 * n2 + q] = X(i, j) * X(i + 1, j) / ((X(i, j) + 2.0 * X(i + 1, j) + X(i + 2, j)) * (X(i, j) + X(i + 1, j)));
      cyp[q] = Y(i, j) * Y(i, j + 1) / ((Y(i, j - 1) + 2.0 * Y(i, j) + Y(i, j + 1)) * (Y(i, j) + Y(i, j + 1)));
      cyp[n2 + q] = -Y(i, j) * Y(i, j + 1) / ((Y(i, j) + Y(i, j + 1)) * (Y(i, j - 1) + Y(i, j)));
      cyp[2 * n2 + q] = Y(i, j) * Y(i, j + 1) / ((Y(i, j - 1) + 2.0 * Y(i, j) + Y(i, j + 1)) * (Y(i, j - 1) + Y(i, j)));
      cyn[q] = Y(i, j) * Y(i, j + 1) / ((Y(i, j) + 2.0 * Y(i, j + 1) + Y(i, j + 2)) * (Y(i, j + 1) + Y(i, j + 2)));
      cyn[n2 + q] = -Y(i, j) * Y(i, j + 1) / ((Y(i, j + 1) + Y(i, j + 2)) * (Y(i, j) + Y(i, j + 1)));
      cyn[2 * n2 + q] = Y(i, j) * Y(i, j + 1) / ((Y(i, j) + 2.0 * Y(i, j + 1) + Y(i, j + 2)) * (Y(i, j) + Y(i, j + 1)));
    }
  std::vector<double> qz(2 * nk, 0.0), czp(3 * nk, 0.0), czn(3 * nk, 0.0);
  const std::vector<double>& dz = d->dzt_h;
  for (int k = 0; k < nk; ++k) {
    int kp2 = k + 2 < nk ? k + 2 : nk - 1;
    int kp1 = k + 1 < nk ? k + 1 : nk - 1;
    int km1 = k > 0 ? k - 1 : 0;
    qz[k] = dz[kp1] / (dz[kp1] + dz[k]);
    qz[nk + k] = dz[k] / (dz[kp1] + dz[k]);
    czp[k] = dz[k] * dz[kp1] / ((dz[km1] + 2.0 * dz[k] + dz[kp1]) * (dz[k] + dz[kp1]));
    czp[nk + k] = -dz[k] * dz[kp1] / ((dz[k] + dz[kp1]) * (dz[km1] + dz[k]));
    czp[2 * nk + k] = dz[k] * dz[kp1] / ((dz[km1] + 2.0 * dz[k] + dz[kp1]) * (dz[km1] + dz[k]));
    czn[k] = dz[k] * dz[kp1] / ((dz[k] + 2.0 * dz[kp1] + dz[kp2]) * (dz[kp1] + dz[kp2]));
    czn[nk + k] = -dz[k] * dz[kp1] / ((dz[kp1] + dz[kp2]) * (dz[k] + dz[kp1]));
    czn[2 * nk + k] = dz[k] * dz[kp1] / ((dz[k] + 2.0 * dz[kp1] + dz[kp2]) * (dz[k] + dz[kp1]));
  }
  QuickerWeights& w = d->qw;
  int rc;
  if ((rc = upload_new(d, &w.quick_x, qx)) || (rc = upload_new(d, &w.quick_y, qy)) ||
      (rc = upload_new(d, &w.curv_xp, cxp)) || (rc = upload_new(d, &w.curv_xn, cxn)) ||
      (rc = upload_new(d, &w.curv_yp, cyp)) || (rc = upload_new(d, &w.curv_yn, cyn)) ||
      (rc = upload_new(d, &w.quick_z, qz)) || (rc = upload_new(d, &w.curv_zp, czp)) ||
      (rc = upload_new(d, &w.curv_zn, czn)))
    return rc;
  return MOM5GPU_OK;
}

int mom5gpu_tracer_advect_init(mom5gpu_domain* d) {
  if (!d) return MOM5GPU_EINVAL;
  const Geo& g = d->geo;
  std::vector<double> tmask, dxt, dyt;
  int rc;
  if ((rc = download(d, MOM5GPU_TMASK, 0, tmask)) || (rc = download(d, MOM5GPU_DXT, 0, dxt)) ||
      (rc = download(d, MOM5GPU_DYT, 0, dyt)))
    return rc;
  // tmask_mdfl / tmask_quick: tmask on the compute domain, halo-2 update (:1660-1669)
  int nx2 = g.ni + 4, ny2 = g.nj + 4;
  std::vector<uint8_t> m2((size_t)nx2 * ny2 * g.nk, 0);
  auto H = [&](int i, int j, int k) { return ((size_t)k * ny2 + (j + 1)) * nx2 + (i + 1); };
  for (int k = 0; k < g.nk; ++k)
    for (int j = 1; j <= g.nj; ++j)
      for (int i = 1; i <= g.ni; ++i) {
        double t = tmask[((size_t)k * g.nyd + j) * g.nxd + i];
        if (t != 0.0 && t != 1.0) return fail(d, MOM5GPU_EINVAL, "tmask must hold 0.0 or 1.0");
        m2[H(i, j, k)] = t != 0.0;
      }
  for (int k = 0; k < g.nk; ++k) {
    if (g.cx)
      for (int j = 1; j <= g.nj; ++j)
        for (int h = 1; h <= 2; ++h) {
          m2[H(1 - h, j, k)] = m2[H(g.ni + 1 - h, j, k)];
          m2[H(g.ni + h, j, k)] = m2[H(h, j, k)];
        }
    if (g.cy)
      for (int i = 1; i <= g.ni; ++i)
        for (int h = 1; h <= 2; ++h) {
          m2[H(i, 1 - h, k)] = m2[H(i, g.nj + 1 - h, k)];
          m2[H(i, g.nj + h, k)] = m2[H(i, h, k)];
        }
    if (g.cx && g.cy)
      for (int hj = 1; hj <= 2; ++hj)
        for (int hi = 1; hi <= 2; ++hi) {
          m2[H(1 - hi, 1 - hj, k)] = m2[H(g.ni + 1 - hi, g.nj + 1 - hj, k)];
          m2[H(g.ni + hi, 1 - hj, k)] = m2[H(hi, g.nj + 1 - hj, k)];
          m2[H(1 - hi, g.nj + hj, k)] = m2[H(g.ni + 1 - hi, hj, k)];
          m2[H(g.ni + hi, g.nj + hj, k)] = m2[H(hi, hj, k)];
        }
  }
  if (!d->mask2) {
    cudaError_t e = cudaMalloc(&d->mask2, m2.size());
    if (e != cudaSuccess) return cuda_fail(d, e, "mask2");
    d->bytes += m2.size();
  }
  cudaError_t e = cudaMemcpy(d->mask2, m2.data(), m2.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(d, e, "mask2 upload");
  if (d->dzt_h.size() == (size_t)g.nk) {
    rc = quicker_init(d, dxt, dyt);
    if (rc) return rc;
  }
  d->advect_ready = true;
  return MOM5GPU_OK;
}

int mom5gpu_barotropic_init(mom5gpu_domain* d, double dtuv, double dtbt) {
  if (!d) return MOM5GPU_EINVAL;
  const mom5gpu_options& o = d->opt;
  // exactly one time-stepping flag (ocean_barotropic.F90:1536-1543)
  if (o.barotropic_time_stepping_A && o.barotropic_time_stepping_B)
    return fail(d, MOM5GPU_EINVAL, "barotropic_time_stepping_A and barotropic_time_stepping_B cannot both be true");
  if (!o.barotropic_time_stepping_A && !o.barotropic_time_stepping_B)
    return fail(d, MOM5GPU_EINVAL, "barotropic_time_stepping_A and barotropic_time_stepping_B cannot both be false");
  // time-step consistency (:1546-1585)
  if (lround(dtuv) <= 0) return fail(d, MOM5GPU_EINVAL, "dtuv must be positive");
  if (lround(dtbt) > lround(dtuv)) return fail(d, MOM5GPU_EINVAL, "dtbt > dtuv is not allowed");
  if (lround(dtbt) == 0) return fail(d, MOM5GPU_EINVAL, "dtbt=0 when dtuv > 0 is not implemented");
  if (lround(dtuv) == lround(dtbt))
    return fail(d, MOM5GPU_EUNSUPPORTED, "unsplit system (dtbt == dtuv) is outside the implemented path");
  int nts = (int)lround((2.0 * dtuv) / dtbt);
  if (fabs((2.0 * dtuv) / nts - dtbt) > 1.e-6)
    return fail(d, MOM5GPU_EINVAL, "splitting requires mod(2*dtuv,dtbt)=0; use dtbt = %.10g", (2.0 * dtuv) / nts);
  const Geo& g = d->geo;
  // gravity-wave CFL check (:1595-1662) when the vertical grid is known
  if (d->zw_h.size() == (size_t)g.nk && d->kmt_h.size() == (size_t)g.n2) {
    std::vector<double> dxt, dyt;
    int rc;
    if ((rc = download(d, MOM5GPU_DXT, 0, dxt)) || (rc = download(d, MOM5GPU_DYT, 0, dyt))) return rc;
    double max_dt = 1.e6, cgmax = 1.0;
    int icg = 1, jcg = 1;
    for (int j = 1; j <= g.nj; ++j)
      for (int i = 1; i <= g.ni; ++i) {
        size_t q = (size_t)j * g.nxd + i;
        int kmt = d->kmt_h[q];
        if (kmt > 0) {
          double cgext = sqrt(o.grav * d->zw_h[kmt - 1]);
          double gridsp = 1.0 / (dxt[q] * dxt[q]) + 1.0 / (dyt[q] * dyt[q]);
          gridsp = sqrt(1.0 / gridsp);
          double dtcg = gridsp / cgext;
          if (dtcg < max_dt) {
            max_dt = dtcg;
            cgmax = cgext;
            icg = i;
            jcg = j;
          }
        }
      }
    max_dt = (double)(long)max_dt;
    if (dtbt > max_dt)
      return fail(d, MOM5GPU_ECFL, "barotropic stability violated at T-cell (%d,%d): dtbt = %g s must be below %g s "
                                   "(gravity wave speed %.1f m/s)", icg, jcg, dtbt, max_dt, cgmax);
  }
  // cori1 = 0.5*dtbt*f, cori2 = 1/(1+cori1**2) (:1283-1288)
  std::vector<double> f;
  int rc = download(d, MOM5GPU_CORIOLIS_F, 0, f);
  if (rc) return rc;
  std::vector<double> c1(f.size()), c2(f.size());
  for (size_t q = 0; q < f.size(); ++q) {
    c1[q] = 0.5 * dtbt * f[q];
    c2[q] = 1.0 / (1.0 + c1[q] * c1[q]);
  }
  if ((rc = upload_new(d, &d->cori1, c1)) || (rc = upload_new(d, &d->cori2, c2))) return rc;
  if (!d->bt) {
    int planes = kBtPlanes + (d->opt.precision == MOM5GPU_PRECISION_MIXED ? kBtFastPlanes : 0);
    size_t bytes = sizeof(double) * planes * (size_t)g.n2;
    cudaError_t e = cudaMalloc(&d->bt, bytes);
    if (e != cudaSuccess) return cuda_fail(d, e, "barotropic scratch");
    cudaMemsetAsync(d->bt, 0, bytes, d->stream);
    d->bytes += bytes;
  }
  d->nts = nts;
  d->dtuv = dtuv;
  d->dtbt = dtbt;
  d->baro_ready = true;
  return MOM5GPU_OK;
}

int mom5gpu_barotropic_nts(const mom5gpu_domain* d) { return d ? d->nts : 0; }

// ---- hot path -------------------------------------------------------------

static int check_levels(mom5gpu_domain* d, int a, int b) {
  if (a < 1 || a > 3 || b < 1 || b > 3) return fail(d, MOM5GPU_EINVAL, "time levels must be in 1..3 (got %d, %d)", a, b);
  return MOM5GPU_OK;
}

int mom5gpu_advect_tracer_sweby_all(mom5gpu_domain* d, int taum1, int tau, double dtime) {
  if (!d) return MOM5GPU_EINVAL;
  int rc = check_levels(d, taum1, tau);
  if (rc) return rc;
  if (!d->advect_ready) return fail(d, MOM5GPU_ESTATE, "advection before mom5gpu_tracer_advect_init");
  if (d->dims.num_prog_tracers < 1) return MOM5GPU_OK;
  return launch_mdfl(d, true, 1, d->dims.num_prog_tracers, taum1, tau, dtime, 1.0);
}

int mom5gpu_horz_advect_tracer(mom5gpu_domain* d, int n, int taum1, int tau, double dtime) {
  if (!d) return MOM5GPU_EINVAL;
  if (d->opt.zero_tracer_advect_horz) return MOM5GPU_OK;
  int rc = check_levels(d, taum1, tau);
  if (rc) return rc;
  if (n < 1 || n > d->dims.num_prog_tracers) return fail(d, MOM5GPU_EINVAL, "horz_advect_tracer: tracer %d", n);
  if (!d->advect_ready) return fail(d, MOM5GPU_ESTATE, "advection before mom5gpu_tracer_advect_init");
  if (d->opt.advect_sweby_all) {
    if (n == 1) return mom5gpu_advect_tracer_sweby_all(d, taum1, tau, dtime);
    return MOM5GPU_OK;
  }
  switch (d->scheme[n - 1].horz) {
    case MOM5GPU_ADVECT_UPWIND: return launch_upwind_horz(d, n, taum1);
    case MOM5GPU_ADVECT_2ND_ORDER: return launch_centred(d, n, tau, 2, true);
    case MOM5GPU_ADVECT_4TH_ORDER: return launch_centred(d, n, tau, 4, true);
    case MOM5GPU_ADVECT_6TH_ORDER: return launch_centred(d, n, tau, 6, true);
    case MOM5GPU_ADVECT_QUICKER:
      if (!d->qw.quick_x) return fail(d, MOM5GPU_ESTATE, "quicker needs mom5gpu_set_vertical_grid before init");
      return launch_quicker_horz(d, n, taum1, tau);
    case MOM5GPU_ADVECT_QUICKMOM3:
      if (!d->qw.quick_x) return fail(d, MOM5GPU_ESTATE, "quickmom3 needs mom5gpu_set_vertical_grid before init");
      return launch_quickmom3_horz(d, n, taum1, tau);
    case MOM5GPU_ADVECT_MDFL_SWEBY:
      if (d->opt.precision == MOM5GPU_PRECISION_MIXED) return launch_mdfl_mixed(d, n, 1, taum1, tau, 0, dtime, false);
      return launch_mdfl(d, false, n, 1, taum1, tau, dtime, 1.0);
    case MOM5GPU_ADVECT_DST_LINEAR: return launch_mdfl(d, false, n, 1, taum1, tau, dtime, 0.0);
    case MOM5GPU_ADVECT_MDPPM: return launch_mdppm(d, n, taum1, tau, dtime);
    case MOM5GPU_ADVECT_MDFL_SUP_B: return launch_mdfl_sup_b(d, n, taum1, tau, dtime);
    case MOM5GPU_ADVECT_PSOM: return launch_psom(d, n, taum1, dtime);
  }
  return fail(d, MOM5GPU_EINVAL, "horz_advect_tracer: invalid horz advection scheme");
}

int mom5gpu_vert_advect_tracer(mom5gpu_domain* d, int n, int taum1, int tau, double dtime) {
  (void)dtime;
  if (!d) return MOM5GPU_EINVAL;
  if (d->opt.zero_tracer_advect_vert) return MOM5GPU_OK;
  int rc = check_levels(d, taum1, tau);
  if (rc) return rc;
  if (n < 1 || n > d->dims.num_prog_tracers) return fail(d, MOM5GPU_EINVAL, "vert_advect_tracer: tracer %d", n);
  if (d->opt.advect_sweby_all) return MOM5GPU_OK;
  switch (d->scheme[n - 1].vert) {
    case MOM5GPU_ADVECT_UPWIND: return launch_upwind_vert(d, n, taum1);
    case MOM5GPU_ADVECT_2ND_ORDER: return launch_centred(d, n, tau, 2, false);
    case MOM5GPU_ADVECT_4TH_ORDER: return launch_centred(d, n, tau, 4, false);
    case MOM5GPU_ADVECT_6TH_ORDER: return launch_centred(d, n, tau, 6, false);
    case MOM5GPU_ADVECT_QUICKER:
      if (!d->qw.quick_z) return fail(d, MOM5GPU_ESTATE, "quicker needs mom5gpu_set_vertical_grid before init");
      return launch_quicker_vert(d, n, taum1, tau);
    case MOM5GPU_ADVECT_MDFL_SWEBY:
    case MOM5GPU_ADVECT_DST_LINEAR:
    case MOM5GPU_ADVECT_MDFL_SUP_B:
    case MOM5GPU_ADVECT_PSOM:
    case MOM5GPU_ADVECT_MDPPM: return MOM5GPU_OK;  // 3-D schemes: done in horz_advect_tracer
  }
  return fail(d, MOM5GPU_EINVAL, "vert_advect_tracer: invalid advection scheme");
}

int mom5gpu_compute_tmask_limit(mom5gpu_domain* d, int tau, int index_temp, int index_salt) {
  if (!d) return MOM5GPU_EINVAL;
  if (tau < 1 || tau > 3) return fail(d, MOM5GPU_EINVAL, "compute_tmask_limit: tau %d", tau);
  for (int n = 1; n <= d->dims.num_prog_tracers; ++n) {
    int rc = launch_tmask_limit(d, n, tau);
    if (rc) return rc;
  }
  if (index_temp > 0 && index_salt > 0 && index_temp <= d->dims.num_prog_tracers &&
      index_salt <= d->dims.num_prog_tracers)
    return launch_tmask_limit_ts_same(d, index_temp, index_salt);
  return MOM5GPU_OK;
}

int mom5gpu_zero_th_tendency(mom5gpu_domain* d, int n) {
  if (!d) return MOM5GPU_EINVAL;
  int ntr = d->dims.num_prog_tracers;
  if (n < 0 || n > ntr) return fail(d, MOM5GPU_EINVAL, "zero_th_tendency: tracer %d", n);
  if (ntr == 0) return MOM5GPU_OK;
  double* p = fptr(d, MOM5GPU_TH_TENDENCY, n == 0 ? 1 : n, 0);
  if (!p) return MOM5GPU_ENOMEM;
  size_t cnt = (size_t)d->geo.n3 * (n == 0 ? ntr : 1);
  cudaError_t e = cudaMemsetAsync(p, 0, sizeof(double) * cnt, d->stream);
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "zero_th_tendency");
}

int mom5gpu_update_tracer(mom5gpu_domain* d, int n, int taum1, int taup1, double dtime) {
  if (!d) return MOM5GPU_EINVAL;
  int rc = check_levels(d, taum1, taup1);
  if (rc) return rc;
  int ntr = d->dims.num_prog_tracers;
  if (n < 0 || n > ntr) return fail(d, MOM5GPU_EINVAL, "update_tracer: tracer %d", n);
  if (ntr == 0) return MOM5GPU_OK;
  return launch_update_tracer(d, n == 0 ? 1 : n, n == 0 ? ntr : 1, taum1, taup1, dtime);
}

int mom5gpu_tracer_advection_step(mom5gpu_domain* d, int taum1, int tau, int taup1, double dtime) {
  if (!d) return MOM5GPU_EINVAL;
  int rc = check_levels(d, taum1, tau);
  if (rc || (rc = check_levels(d, tau, taup1))) return rc;
  if (!d->advect_ready) return fail(d, MOM5GPU_ESTATE, "advection before mom5gpu_tracer_advect_init");
  int ntr = d->dims.num_prog_tracers;
  if (ntr == 0) return MOM5GPU_OK;
  // all-MDFL, FP64: one launch set over every tracer; mixed precision: fused kernel
  bool all_mdfl = true;
  for (int n = 0; n < ntr; ++n)
    if (d->scheme[n].horz != MOM5GPU_ADVECT_MDFL_SWEBY) all_mdfl = false;
  if (all_mdfl && !d->opt.zero_tracer_advect_horz && d->opt.precision == MOM5GPU_PRECISION_MIXED)
    return launch_mdfl_mixed(d, 1, ntr, taum1, tau, taup1, dtime, true);
  if (all_mdfl && !d->opt.zero_tracer_advect_horz) {
    // th_tendency starts at +0: the y pass writes every compute cell, only the
    // halo ring is zeroed here
    double* th = fptr(d, MOM5GPU_TH_TENDENCY, 1, 0);
    if (!th) return MOM5GPU_ENOMEM;
    launch_zero_ring(d->geo, th, (long)ntr * d->geo.nk, d->stream);
    count_launches(d, 1);
    rc = launch_mdfl(d, d->opt.advect_sweby_all != 0, 1, ntr, taum1, tau, dtime, 1.0, true);
    if (rc) return rc;
  } else {
    if ((rc = mom5gpu_zero_th_tendency(d, 0))) return rc;
    for (int n = 1; n <= ntr; ++n) {
      if ((rc = mom5gpu_horz_advect_tracer(d, n, taum1, tau, dtime))) return rc;
      if ((rc = mom5gpu_vert_advect_tracer(d, n, taum1, tau, dtime))) return rc;
    }
  }
  return launch_update_tracer(d, 1, ntr, taum1, taup1, dtime);
}

int mom5gpu_set_barotropic_fusion(mom5gpu_domain* d, int mode) {
  if (!d) return MOM5GPU_EINVAL;
  if (mode < 0 || mode > 2) return fail(d, MOM5GPU_EINVAL, "set_barotropic_fusion: mode 0, 1 or 2");
  if (mode != d->bt_fused) {
    // the cached subcycle graphs hold the other form (their key is the kernel arguments)
    for (auto& gr : d->bt_graphs)
      if (gr.exec) cudaGraphExecDestroy(gr.exec);
    d->bt_graphs.clear();
  }
  d->bt_fused = mode;
  return MOM5GPU_OK;
}

int mom5gpu_grid_barrier_selftest(mom5gpu_domain* d, int rounds, int unreachable) {
  if (!d) return MOM5GPU_EINVAL;
  if (rounds < 1 || rounds > 100000) return fail(d, MOM5GPU_EINVAL, "grid_barrier_selftest: rounds 1..100000");
  return grid_barrier_selftest(d, rounds, unreachable);
}

int mom5gpu_set_tuning(mom5gpu_domain* d, int rows, int prefetch, int tj) {
  if (!d) return MOM5GPU_EINVAL;
  if ((rows != 16 && rows != 24 && rows != 32 && rows != 64) || prefetch < 0 || prefetch > 3 ||
      (prefetch == 1 && rows != 16) || (prefetch == 2 && rows != 16 && rows != 24) || (prefetch == 3 && rows != 16) ||
      !(tj == 0 || tj == 2 || tj == 4 || tj == 8 || tj == 16))
    return fail(d, MOM5GPU_EINVAL,
                "set_tuning: rows 16|24|32|64, prefetch 0, 1 (cp.async, rows 16), 2 (TMA, rows 16|24) or 3 "
                "(TMA, 5 tracers per block, rows 16), "
                "tj 0|2|4|8|16");
  d->tune_mixed_rows = rows;
  d->tune_mixed_pf = prefetch;
  d->tune_y_tj = tj;
  return MOM5GPU_OK;
}

int mom5gpu_get_tuning(const mom5gpu_domain* d, int* rows, int* prefetch, int* tj) {
  if (!d || !rows || !prefetch || !tj) return MOM5GPU_EINVAL;
  *rows = d->tune_mixed_rows;
  *prefetch = d->tune_mixed_pf;
  *tj = d->tune_y_tj;
  return MOM5GPU_OK;
}

int mom5gpu_autotune(mom5gpu_domain* d, double dtime, char* report, size_t report_len) {
  if (!d) return MOM5GPU_EINVAL;
  if (!d->advect_ready) return fail(d, MOM5GPU_ESTATE, "autotune before mom5gpu_tracer_advect_init");
  bool mixed = d->opt.precision == MOM5GPU_PRECISION_MIXED;
  // candidate launch shapes: precision-form tile height (and tracer prefetch); FP64 y-pass rows per thread
  const int kRows[] = {32, 64, 24, 16, 16, 16, 24, 16};
  const int kPf[] = {0, 0, 0, 0, 1, 2, 2, 3};
  const int kTj[] = {2, 4, 8, 16};
  int ncand = mixed ? (d->geo.ni % 2 == 0 ? 8 : 5) : 4;
  cudaEvent_t t0, t1;
  if (cudaEventCreate(&t0) != cudaSuccess) return fail(d, MOM5GPU_ECUDA, "autotune events");
  if (cudaEventCreate(&t1) != cudaSuccess) {
    cudaEventDestroy(t0);
    return fail(d, MOM5GPU_ECUDA, "autotune events");
  }
  std::string rep;
  double best = 1e30;
  int bestc = 0, rc = MOM5GPU_OK;
  for (int c = 0; c < ncand && rc == MOM5GPU_OK; ++c) {
    if (mixed) {
      d->tune_mixed_rows = kRows[c];
      d->tune_mixed_pf = kPf[c];
    } else {
      d->tune_y_tj = kTj[c];
    }
    rc = mom5gpu_tracer_advection_step(d, 1, 1, 2, dtime);  // warm-up
    cudaEventRecord(t0, d->stream);
    for (int r = 0; r < 3 && rc == MOM5GPU_OK; ++r) rc = mom5gpu_tracer_advection_step(d, 1, 1, 2, dtime);
    cudaEventRecord(t1, d->stream);
    if (rc) break;
    cudaError_t e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) {
      rc = cuda_fail(d, e, "autotune");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    ms /= 3.f;
    char line[96];
    if (mixed)
      snprintf(line, sizeof(line), "rows=%d%s: %.3f ms; ", kRows[c], kPf[c] == 3 ? "+tma5" : kPf[c] == 2 ? "+tma" : kPf[c] ? "+prefetch" : "",
               ms);
    else snprintf(line, sizeof(line), "tj=%d: %.3f ms; ", kTj[c], ms);
    rep += line;
    if (ms < best) {
      best = ms;
      bestc = c;
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (mixed) {
    d->tune_mixed_rows = kRows[bestc];
    d->tune_mixed_pf = kPf[bestc];
  } else {
    d->tune_y_tj = kTj[bestc];
  }
  if (rc) return rc;
  char line[64];
  if (mixed)
    snprintf(line, sizeof(line), "chosen rows=%d%s", kRows[bestc],
             kPf[bestc] == 3 ? "+tma5" : kPf[bestc] == 2 ? "+tma" : kPf[bestc] ? "+prefetch" : "");
  else snprintf(line, sizeof(line), "chosen tj=%d", kTj[bestc]);
  rep += line;
  if (report && report_len) {
    strncpy(report, rep.c_str(), report_len - 1);
    report[report_len - 1] = 0;
  }
  return MOM5GPU_OK;
}

int mom5gpu_eta_and_pbot_tendency(mom5gpu_domain* d, int tau) {
  if (!d) return MOM5GPU_EINVAL;
  if (tau < 1 || tau > 3) return fail(d, MOM5GPU_EINVAL, "eta_and_pbot_tendency: tau %d", tau);
  return launch_eta_tendency(d, tau);
}

int mom5gpu_eta_and_pbot_update(mom5gpu_domain* d, int taum1, int taup1, double dtime) {
  if (!d) return MOM5GPU_EINVAL;
  int rc = check_levels(d, taum1, taup1);
  if (rc) return rc;
  return launch_eta_update(d, taum1, taup1, dtime);
}

int mom5gpu_ocean_advection_velocity(mom5gpu_domain* d, int tau) {
  if (!d) return MOM5GPU_EINVAL;
  if (tau < 1 || tau > 3) return fail(d, MOM5GPU_EINVAL, "ocean_advection_velocity: tau %d", tau);
  return launch_advection_velocity(d, tau);
}

int mom5gpu_tracer_boundary_terms(mom5gpu_domain* d, int n) {
  if (!d) return MOM5GPU_EINVAL;
  int ntr = d->dims.num_prog_tracers;
  if (n < 0 || n > ntr) return fail(d, MOM5GPU_EINVAL, "tracer_boundary_terms: tracer %d", n);
  if ((int)d->kmt_h.size() != (int)d->geo.n2)
    return fail(d, MOM5GPU_ESTATE, "tracer_boundary_terms before mom5gpu_set_vertical_grid");
  int rc = MOM5GPU_OK;
  for (int m = (n == 0 ? 1 : n); m <= (n == 0 ? ntr : n) && rc == MOM5GPU_OK; ++m) rc = launch_tracer_boundary(d, m);
  return rc;
}

int mom5gpu_update_ucell_thickness(mom5gpu_domain* d, int taup1, int vert_coordinate, int linear_free_surface,
                                   int update_dzwu_k0) {
  if (!d) return MOM5GPU_EINVAL;
  if (taup1 < 1 || taup1 > 3) return fail(d, MOM5GPU_EINVAL, "update_ucell_thickness: taup1 %d", taup1);
  if (vert_coordinate < MOM5GPU_GEOPOTENTIAL || vert_coordinate > MOM5GPU_PSIGMA)
    return fail(d, MOM5GPU_EINVAL, "update_ucell_thickness: vertical coordinate %d", vert_coordinate);
  return launch_update_ucell_thickness(d, taup1, vert_coordinate, linear_free_surface != 0, update_dzwu_k0 != 0);
}

int mom5gpu_ocean_barotropic_forcing(mom5gpu_domain* d) {
  if (!d) return MOM5GPU_EINVAL;
  if (d->opt.udrho_lap || d->opt.udrho_bih)
    return fail(d, MOM5GPU_EINVAL,
                "ocean_barotropic_forcing: udrho_lap/udrho_bih act on udrho(tau): use "
                "mom5gpu_ocean_barotropic_forcing_tau");
  return launch_barotropic_forcing(d, 0);
}

int mom5gpu_ocean_barotropic_forcing_tau(mom5gpu_domain* d, int tau) {
  if (!d) return MOM5GPU_EINVAL;
  if (tau < 1 || tau > 3) return fail(d, MOM5GPU_EINVAL, "ocean_barotropic_forcing: tau %d (1..3)", tau);
  return launch_barotropic_forcing(d, tau);
}

int mom5gpu_update_ocean_barotropic(mom5gpu_domain* d, int tau, int taup1) {
  if (!d) return MOM5GPU_EINVAL;
  int rc = check_levels(d, tau, taup1);
  if (rc) return rc;
  return launch_barotropic(d, tau, taup1);
}

int mom5gpu_global_tracer_content(mom5gpu_domain* d, int n, int level, double* out) {
  if (!d || !out) return MOM5GPU_EINVAL;
  if (n < 1 || n > d->dims.num_prog_tracers || level < 1 || level > 3)
    return fail(d, MOM5GPU_EINVAL, "global_tracer_content: tracer %d level %d", n, level);
  return launch_content(d, n, level, out);
}

int mom5gpu_tracer_content_fixed(mom5gpu_domain* d, int n, int level, long long* acc) {
  if (!d || !acc) return MOM5GPU_EINVAL;
  if (n < 1 || n > d->dims.num_prog_tracers || level < 1 || level > 3)
    return fail(d, MOM5GPU_EINVAL, "tracer_content_fixed: tracer %d level %d", n, level);
  return launch_content_fixed(d, n, level, acc);
}

// Normalise the chunk accumulators into a two's complement integer of 32-bit
// words (value = X * 2^-100), take its magnitude and round the top bits to 53.
int mom5gpu_fixed_to_double(const long long* acc, double* out) {
  if (!acc || !out) return MOM5GPU_EINVAL;
  constexpr int NC = MOM5GPU_FIXED_CHUNKS, NW = NC + 3;  // words; room for the carries
  uint32_t w[NW];
  long long carry = 0;
  for (int i = 0; i < NW; ++i) {
    // acc[i] + carry fits: |acc| < 2^63 - 2^32 * 2^31 headroom is the caller's (<= 2^31 values)
    long long v = (i < NC ? acc[i] : 0) + carry;
    w[i] = (uint32_t)(v & 0xffffffffLL);
    carry = (v - (long long)w[i]) / 4294967296LL;  // exact: v - low word is a multiple of 2^32
  }
  const bool neg = (w[NW - 1] & 0x80000000u) != 0;
  if (neg) {  // magnitude: two's complement negation
    uint64_t c = 1;
    for (int i = 0; i < NW; ++i) {
      uint64_t t = (uint64_t)(uint32_t)~w[i] + c;
      w[i] = (uint32_t)t;
      c = t >> 32;
    }
  }
  int top = -1;  // highest set bit
  for (int i = NW - 1; i >= 0 && top < 0; --i)
    if (w[i]) top = 32 * i + 31 - __builtin_clz(w[i]);
  if (top < 0) {
    *out = 0.0;
    return MOM5GPU_OK;
  }
  auto bit = [&](int b) -> unsigned { return b < 0 ? 0u : (w[b >> 5] >> (b & 31)) & 1u; };
  // 53 significant bits from `top` down, then round to nearest, ties to even
  uint64_t m = 0;
  for (int b = top; b > top - 53; --b) m = (m << 1) | bit(b);
  const int lsb = top - 52;
  unsigned guard = bit(lsb - 1), sticky = 0;
  for (int b = lsb - 2; b >= 0 && !sticky; --b) sticky |= bit(b);
  if (guard && (sticky || (m & 1u))) ++m;  // a carry to 2^53 stays exact in ldexp
  *out = ldexp((double)m, lsb - 100) * (neg ? -1.0 : 1.0);
  return MOM5GPU_OK;
}

int mom5gpu_global_eta_integral(mom5gpu_domain* d, int field, int level, double* out) {
  if (!d || !out) return MOM5GPU_EINVAL;
  const FieldInfo* fi = field_info(field);
  if (!fi || fi->shape != S2D) return fail(d, MOM5GPU_EINVAL, "global_eta_integral: field %d is not 2-D", field);
  double* p = fptr(d, field, 0, fi->per_level ? level : 0);
  if (!p) return fail(d, MOM5GPU_EINVAL, "global_eta_integral: bad level %d", level);
  return launch_eta_integral(d, p, out);
}

int mom5gpu_check_finite(mom5gpu_domain* d, int n, int level, int* out) {
  if (!d || !out) return MOM5GPU_EINVAL;
  int ntr = d->dims.num_prog_tracers;
  if (n < 0 || n > ntr || level < 1 || level > 3) return fail(d, MOM5GPU_EINVAL, "check_finite: tracer %d", n);
  if (ntr == 0) {
    *out = 0;
    return MOM5GPU_OK;
  }
  const double* p = fptr(d, MOM5GPU_TRACER, n == 0 ? 1 : n, level);
  int bad = 0;
  int rc = launch_check_finite(d, p, (size_t)d->geo.n3 * (n == 0 ? ntr : 1), &bad);
  if (rc) return rc;
  *out = bad ? 1 : 0;
  return MOM5GPU_OK;
}

static const char* kSectionNames[SEC_N] = {"mdfl", "mdfl_mixed", "tracer_update", "barotropic", "upwind",
                                           "quicker", "batch"};

int mom5gpu_enable_timing(mom5gpu_domain* d, int on) {
  if (!d) return MOM5GPU_EINVAL;
  resolve_clocks(d);
  d->timing = on != 0;
  for (int s = 0; s < SEC_N; ++s) {
    d->clock_ms[s] = 0.0;
    d->clock_calls[s] = 0;
  }
  return MOM5GPU_OK;
}

int mom5gpu_timing_query(mom5gpu_domain* d, const char* section, double* total_ms, long* calls) {
  if (!d || !section || !total_ms || !calls) return MOM5GPU_EINVAL;
  resolve_clocks(d);
  for (int s = 0; s < SEC_N; ++s)
    if (strcmp(section, kSectionNames[s]) == 0) {
      *total_ms = d->clock_ms[s];
      *calls = d->clock_calls[s];
      return MOM5GPU_OK;
    }
  return fail(d, MOM5GPU_EINVAL, "unknown timing section '%s'", section);
}

long mom5gpu_launch_count(const mom5gpu_domain* d) { return d ? d->launches : 0; }

}  // extern "C"
