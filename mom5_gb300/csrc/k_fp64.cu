// FP64 kernels of the drop-in path.
//
// Built with --fmad=false: every product and sum is rounded on its own, in the
// order the reference's Fortran evaluates it, so results agree with the
// reference arithmetic value for value (IEEE equality; only the sign of an
// exact zero may differ).  Where the reference multiplies by a 0/1 mask, these
// kernels select instead, and where one of two terms of an upwind pair is an
// exact zero they skip it; both transformations return the identical value for
// finite operands and move work off the FP64 pipe, which on GB300 issues about
// 1.7 instructions per clock per SM against ~119 for FP32.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "internal.h"
#include "fp64_bodies.cuh"
#include "mdppm_body.cuh"

namespace mom5 {

#define DEVI __device__ __forceinline__

using namespace fp64;

// ---------------------------------------------------------------------------
// halo update of a data-domain array (single-PE mpp_update_domains)
// ---------------------------------------------------------------------------
__global__ void k_halo_fill(Geo g, double* a, int nlev, int flags) {
  int k = blockIdx.y;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  double* p = a + (long)k * g.n2;
  if ((flags & 1) && g.cx && t >= 1 && t <= g.nj) {
    p[I2(g, 0, t)] = p[I2(g, g.ni, t)];
    p[I2(g, g.ni + 1, t)] = p[I2(g, 1, t)];
  }
  if ((flags & 2) && g.cy && t >= 1 && t <= g.ni) {
    p[I2(g, t, 0)] = p[I2(g, t, g.nj)];
    p[I2(g, t, g.nj + 1)] = p[I2(g, t, 1)];
  }
  if (flags == 3 && g.cx && g.cy && t == 0) {
    p[I2(g, 0, 0)] = p[I2(g, g.ni, g.nj)];
    p[I2(g, g.ni + 1, 0)] = p[I2(g, 1, g.nj)];
    p[I2(g, 0, g.nj + 1)] = p[I2(g, g.ni, 1)];
    p[I2(g, g.ni + 1, g.nj + 1)] = p[I2(g, 1, 1)];
  }
}

void launch_halo_fill(const Geo& g, double* a, int nlev, int flags, cudaStream_t s) {
  if (!(g.cx || g.cy) || nlev <= 0) return;
  int n = (g.ni > g.nj ? g.ni : g.nj) + 1;
  dim3 grid((n + 255) / 256, nlev);
  k_halo_fill<<<grid, 256, 0, s>>>(g, a, nlev, flags);
}

// zero the halo ring (i in {0, ni+1} or j in {0, nj+1}) of nlev data-domain levels
__global__ void k_zero_ring(Geo g, double* a, long nlev) {
  const long r = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long row = g.ni + 2;
  if (r >= 2 * row + 2L * g.nj) return;
  int i, j;
  if (r < row) {
    i = (int)r;
    j = 0;
  } else if (r < 2 * row) {
    i = (int)(r - row);
    j = g.nj + 1;
  } else {
    const long q = r - 2 * row;
    i = q < g.nj ? 0 : g.ni + 1;
    j = 1 + (int)(q % g.nj);
  }
  for (long k = blockIdx.y; k < nlev; k += gridDim.y) a[k * g.n2 + I2(g, i, j)] = 0.0;
}

void launch_zero_ring(const Geo& g, double* a, long nlev, cudaStream_t s) {
  if (nlev <= 0) return;
  const long nring = 2L * (g.ni + 2) + 2L * g.nj;
  dim3 grid((unsigned)((nring + 255) / 256), (unsigned)(nlev < 1024 ? nlev : 1024));
  k_zero_ring<<<grid, 256, 0, s>>>(g, a, nlev);
}

// ---------------------------------------------------------------------------
// MDFL Sweby / DST-linear: ocean_tracer_advect.F90:3806-4066 (ALL = false) and
// advect_tracer_sweby_all :4104-4511 (ALL = true).  Three passes with the
// intermediate tracer_mdfl in global scratch; the tracer-independent terms of
// each face are computed once and reused for every tracer of the launch.
// ---------------------------------------------------------------------------

template <bool ALL, bool SWEBY, int MAXN>
__global__ void __launch_bounds__(128) k_mdfl_z(MdflArgs a) {
  mdfl_z_body<ALL, SWEBY, MAXN>(a, blockIdx.x, blockIdx.y);
}
// blockIdx.z: the segment of L levels
template <bool ALL, bool SWEBY, int MAXN>
__global__ void __launch_bounds__(128) k_mdfl_z_seg(MdflArgs a, int L) {
  const int k0 = blockIdx.z * L;
  mdfl_z_body<ALL, SWEBY, MAXN, MdflFaceArith, MdflUpdArith, true>(a, blockIdx.x, blockIdx.y, k0, k0 + L);
}

// Levels per z-pass segment.  A domain with few columns gives the column march
// few blocks (120 x 80 columns: 80 blocks on 152 SMs), each a long latency-bound
// chain; cutting the columns into segments of L levels multiplies the blocks by
// nk / L for one extra face per segment.  Aim at about four blocks per SM.
static int z_segment_levels(const Geo& g) {
  const long blocks = (long)((g.ni + 127) / 128) * g.nj;
  const long want = 4L * 152;
  if (blocks >= want || g.nk < 4) return g.nk;
  int nseg = (int)((want + blocks - 1) / blocks);
  if (nseg > g.nk / 2) nseg = g.nk / 2;  // segments of at least two levels
  int L = (g.nk + nseg - 1) / nseg;
  return L < 2 ? 2 : L;
}
template <bool ALL, bool SWEBY, int MAXN>
static void launch_mdfl_z(const MdflArgs& a, cudaStream_t s) {
  const Geo& g = a.g;
  const int L = z_segment_levels(g);
  if (L >= g.nk) {
    k_mdfl_z<ALL, SWEBY, MAXN><<<dim3((g.ni + 127) / 128, g.nj), 128, 0, s>>>(a);
  } else {
    dim3 grid((g.ni + 127) / 128, g.nj, (g.nk + L - 1) / L);
    k_mdfl_z_seg<ALL, SWEBY, MAXN><<<grid, 128, 0, s>>>(a, L);
  }
}

template <bool ALL, bool SWEBY, int MAXN>
__global__ void __launch_bounds__(kTX) k_mdfl_x(MdflArgs a) {
  mdfl_x_body<ALL, SWEBY, MAXN>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <bool ALL, bool SWEBY, int MAXN>
__global__ void __launch_bounds__(128, 6) k_mdfl_y(MdflArgs a, int TJ) {
  mdfl_y_body<ALL, SWEBY, MAXN>(a, TJ, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <bool ALL, bool SWEBY, int MAXN>
static void run_mdfl(const MdflArgs& a, cudaStream_t s) {
  const Geo& g = a.g;
  launch_mdfl_z<ALL, SWEBY, MAXN>(a, s);
  dim3 bx((g.ni + kTX - 1) / kTX, g.nj, g.nk);
  k_mdfl_x<ALL, SWEBY, MAXN><<<bx, kTX, 0, s>>>(a);
  // rows per thread: keep >= ~8 warps per SM of work where the domain allows
  long cols = (long)g.ni * g.nk;
  int TJ = 16;
  while (TJ > 2 && cols * ((g.nj + TJ - 1) / TJ) < 152L * 32 * 16) TJ /= 2;
  if (a.tj > 0) TJ = a.tj;
  dim3 by((g.ni + 127) / 128, (g.nj + TJ - 1) / TJ, g.nk);
  k_mdfl_y<ALL, SWEBY, MAXN><<<by, 128, 0, s>>>(a, TJ);
}

template <bool ALL, bool SWEBY>
static void run_mdfl_n(const MdflArgs& a, cudaStream_t s) {
  if (a.ntr <= 1) run_mdfl<ALL, SWEBY, 1>(a, s);
  else if (a.ntr <= 2) run_mdfl<ALL, SWEBY, 2>(a, s);
  else if (a.ntr <= 4) run_mdfl<ALL, SWEBY, 4>(a, s);
  else run_mdfl<ALL, SWEBY, kMdflChunk>(a, s);
}

// one pass (1 z, 2 x, 3 y) of run_mdfl: a decomposed domain exchanges halos between them
template <bool ALL, bool SWEBY, int MAXN>
static void run_mdfl_one(const MdflArgs& a, int pass, cudaStream_t s) {
  const Geo& g = a.g;
  if (pass == 1) {
    launch_mdfl_z<ALL, SWEBY, MAXN>(a, s);
  } else if (pass == 2) {
    dim3 bx((g.ni + kTX - 1) / kTX, g.nj, g.nk);
    k_mdfl_x<ALL, SWEBY, MAXN><<<bx, kTX, 0, s>>>(a);
  } else {
    long cols = (long)g.ni * g.nk;
    int TJ = 16;
    while (TJ > 2 && cols * ((g.nj + TJ - 1) / TJ) < 152L * 32 * 16) TJ /= 2;
    if (a.tj > 0) TJ = a.tj;
    dim3 by((g.ni + 127) / 128, (g.nj + TJ - 1) / TJ, g.nk);
    k_mdfl_y<ALL, SWEBY, MAXN><<<by, 128, 0, s>>>(a, TJ);
  }
}

template <bool ALL, bool SWEBY>
static void run_mdfl_one_n(const MdflArgs& a, int pass, cudaStream_t s) {
  if (a.ntr <= 1) run_mdfl_one<ALL, SWEBY, 1>(a, pass, s);
  else if (a.ntr <= 2) run_mdfl_one<ALL, SWEBY, 2>(a, pass, s);
  else if (a.ntr <= 4) run_mdfl_one<ALL, SWEBY, 4>(a, pass, s);
  else run_mdfl_one<ALL, SWEBY, kMdflChunk>(a, pass, s);
}

void run_mdfl_pass(const MdflArgs& a, bool all, bool sweby, int pass, cudaStream_t s) {
  if (all) {
    if (sweby) run_mdfl_one_n<true, true>(a, pass, s);
    else run_mdfl_one_n<true, false>(a, pass, s);
  } else {
    if (sweby) run_mdfl_one_n<false, true>(a, pass, s);
    else run_mdfl_one_n<false, false>(a, pass, s);
  }
}

void run_mdfl_kernels(const MdflArgs& a, bool all, bool sweby, cudaStream_t s) {
  if (all) {
    if (sweby) run_mdfl_n<true, true>(a, s);
    else run_mdfl_n<true, false>(a, s);
  } else {
    if (sweby) run_mdfl_n<false, true>(a, s);
    else run_mdfl_n<false, false>(a, s);
  }
}

int ensure_mdfl_scratch(mom5gpu_domain* d, int ntr) {
  if ((int)d->mdfl_cap >= ntr) return MOM5GPU_OK;
  if (d->mdfl_a) cudaFree(d->mdfl_a);
  if (d->mdfl_b) cudaFree(d->mdfl_b);
  d->mdfl_a = d->mdfl_b = nullptr;
  size_t bytes = sizeof(double) * (size_t)d->geo.n3 * ntr;
  cudaError_t e = cudaMalloc(&d->mdfl_a, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&d->mdfl_b, bytes);
  if (e != cudaSuccess) {
    d->mdfl_cap = 0;
    return fail(d, MOM5GPU_ENOMEM, "mdfl scratch of %zu bytes: %s", 2 * bytes, cudaGetErrorString(e));
  }
  d->bytes += 2 * bytes;
  d->mdfl_cap = ntr;
  return MOM5GPU_OK;
}

int make_mdfl_args(mom5gpu_domain* d, int n_first, int ntr, int taum1, int tau, double dtime, MdflArgs* ap) {
  MdflArgs& a = *ap;
  const Geo& g = d->geo;
  int NT = d->dims.num_prog_tracers;
  a.g = g;
  a.ntr = ntr;
  a.dtime = dtime;
  a.mask2 = d->mask2;
  a.dat = fptr(d, MOM5GPU_DAT, 0, 0);
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.dxte = fptr(d, MOM5GPU_DXTE, 0, 0);
  a.dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a.dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a.dytn = fptr(d, MOM5GPU_DYTN, 0, 0);
  a.uh = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a.vh = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a.w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  a.rdz = fptr(d, MOM5GPU_RHO_DZT, 0, tau);
  a.T = fptr(d, MOM5GPU_TRACER, n_first, taum1);
  a.tstride = NT > 1 ? (long)(fptr(d, MOM5GPU_TRACER, 2, 1) - fptr(d, MOM5GPU_TRACER, 1, 1)) : g.n3;
  a.tz = d->mdfl_a;
  a.tx = d->mdfl_b;
  a.th = fptr(d, MOM5GPU_TH_TENDENCY, n_first, 0);
  a.tj = d->tune_y_tj;
  a.nbr = d->nbr;
  a.hz = d->hz ? d->hz + (size_t)(n_first - 1) * g.nk * g.nj * 4 : nullptr;
  a.hx = d->hx ? d->hx + (size_t)(n_first - 1) * g.nk * 4 * g.ni : nullptr;
  long thstride = NT > 1 ? (long)(fptr(d, MOM5GPU_TH_TENDENCY, 2, 0) - fptr(d, MOM5GPU_TH_TENDENCY, 1, 0)) : g.n3;
  if (thstride != g.n3 || a.tstride != g.n3) return fail(d, MOM5GPU_ESTATE, "unexpected tracer layout");
  if (!a.dat || !a.datr || !a.dxte || !a.dyte || !a.dxtn || !a.dytn || !a.uh || !a.vh || !a.w || !a.rdz || !a.T ||
      !a.th || !a.mask2)
    return fail(d, MOM5GPU_ESTATE, "mdfl: a required field was never set");
  return MOM5GPU_OK;
}

int launch_mdfl(mom5gpu_domain* d, bool all, int n_first, int ntr, int taum1, int tau, double dtime,
                double sweby_limiter, bool th_fresh) {
  // tracers per launch set: at most kMdflChunk, in chunks of equal size (the
  // tracer-independent face terms are computed once per chunk)
  int nchunks = (ntr + kMdflChunk - 1) / kMdflChunk;
  int csize = (ntr + nchunks - 1) / nchunks;
  int rc = ensure_mdfl_scratch(d, csize);
  if (rc) return rc;
  ClockScope clk(d, SEC_MDFL);
  for (int c0 = 0; c0 < ntr; c0 += csize) {
    int cn = ntr - c0 < csize ? ntr - c0 : csize;
    MdflArgs a;
    rc = make_mdfl_args(d, n_first + c0, cn, taum1, tau, dtime, &a);
    if (rc) return rc;
    a.th_fresh = th_fresh ? 1 : 0;
    count_launches(d, 3);
    run_mdfl_kernels(a, all, sweby_limiter != 0.0, d->stream);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "mdfl launch");
}

// ---------------------------------------------------------------------------
// Launch shapes shared by the flux-form schemes (upwind, centred, Quicker).
// Horizontal: th += -tmask*(fx(i) - fx(i-1) + fy(j) - fy(j-1))*datr with each
// face flux formed once: a block of HB threads along i covers the cells
// i0 .. i0+HB-2 and the x faces i0-1 .. i0+HB-2 (thread t: face i0-1+t, through
// shared memory) and marches a strip of HR rows carrying the southern y flux.
// Vertical: th += -tmask*(fz(k-1) - fz(k)) with fz(k) the flux through the
// bottom of level k (0 above the first), VS levels per thread and the flux
// above a segment formed again by its thread.
// ---------------------------------------------------------------------------
constexpr int HB = 128, HR = 8, VS = 8;

inline dim3 horz_grid(const Geo& g) { return dim3((g.ni + HB - 2) / (HB - 1), (g.nj + HR - 1) / HR, g.nk); }
inline dim3 vert_grid(const Geo& g) { return dim3((g.ni + 127) / 128, g.nj, (g.nk + VS - 1) / VS); }

template <class FX, class FY>
DEVI void horz_faces_once(const Geo& g, const double* tmask, const double* datr, double* th, FX fx, FY fy) {
  __shared__ double sfx[HB];
  const int t = threadIdx.x;
  const int i0 = blockIdx.x * (HB - 1) + 1, j0 = blockIdx.y * HR + 1, k = blockIdx.z;
  const int iface = i0 - 1 + t, i = i0 + t;
  const bool cell = t <= HB - 2 && i <= g.ni, face_ok = iface <= g.ni;
  double fs = 0.0;  // y flux through the south face of the current row
  if (cell) fs = fy(i, j0 - 1, k);
  for (int r = 0; r < HR; ++r) {
    const int j = j0 + r;
    if (j > g.nj) break;  // the same j for the whole block
    __syncthreads();      // the previous row's x fluxes are read
    sfx[t] = face_ok ? fx(iface, j, k) : 0.0;
    __syncthreads();
    if (cell) {
      double fn = fy(i, j, k);
      long p = I3(g, i, j, k);
      double rr = mask_mul(sfx[t + 1] - sfx[t] + fn - fs, tmask[p]) * datr[I2(g, i, j)];
      th[p] = th[p] + (-rr);
      fs = fn;
    }
  }
}

template <class FZ>
DEVI void vert_segment(const Geo& g, const double* tmask, double* th, FZ fz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
  if (i > g.ni) return;
  const int k0 = blockIdx.z * VS, k1 = k0 + VS < g.nk ? k0 + VS : g.nk;
  double ft1 = k0 > 0 ? fz(i, j, k0 - 1) : 0.0;
  for (int k = k0; k < k1; ++k) {
    double ft2 = fz(i, j, k);
    long p = I3(g, i, j, k);
    double r = mask_mul(ft1 - ft2, tmask[p]);
    th[p] = th[p] + (-r);
    ft1 = ft2;
  }
}

// ---------------------------------------------------------------------------
// Upwind: ocean_tracer_advect.F90:2238-2294 and :2792-2824.
// ---------------------------------------------------------------------------
struct UpwArgs {
  Geo g;
  const double *tmask, *dyte, *dxtn, *datr, *dat, *uh, *vh, *w, *T;
  double* th;
};

// 0.5*u, the mask tests and the products by a mask of 1.0 run on the integer pipe
// (exact: the same values as the FP64 operations).
DEVI double upw_fe(const UpwArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  double velocity = half_exact(a.uh[I3(g, i, j, k)]);
  double upos = velocity + fabs(velocity);
  double uneg = velocity - fabs(velocity);
  double f = a.dyte[I2(g, i, j)] * (upos * a.T[I3(g, i, j, k)] + uneg * a.T[I3(g, i + 1, j, k)]);
  double m0 = a.tmask[I3(g, i, j, k)], m1 = a.tmask[I3(g, i + 1, j, k)];
  return (!is_zero(m0) && !is_zero(m1)) ? mask_mul(mask_mul(f, m0), m1) : 0.0;
}
DEVI double upw_fn(const UpwArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  double velocity = half_exact(a.vh[I3(g, i, j, k)]);
  double upos = velocity + fabs(velocity);
  double uneg = velocity - fabs(velocity);
  double f = a.dxtn[I2(g, i, j)] * (upos * a.T[I3(g, i, j, k)] + uneg * a.T[I3(g, i, j + 1, k)]);
  double m0 = a.tmask[I3(g, i, j, k)], m1 = a.tmask[I3(g, i, j + 1, k)];
  return (!is_zero(m0) && !is_zero(m1)) ? mask_mul(mask_mul(f, m0), m1) : 0.0;
}

__global__ void __launch_bounds__(HB) k_upwind_horz(UpwArgs a) {
  horz_faces_once(
      a.g, a.tmask, a.datr, a.th, [&](int i, int j, int k) { return upw_fe(a, i, j, k); },
      [&](int i, int j, int k) { return upw_fn(a, i, j, k); });
}

// flux through the bottom of level k (:2800-2815)
DEVI double upw_fz(const UpwArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  int kp1 = k + 1 < g.nk ? k + 1 : g.nk - 1;
  long p = I3(g, i, j, k), pp = I3(g, i, j, kp1);
  double velocity = half_exact(a.w[I3(g, i, j, k + 1)]);
  double wpos = velocity + fabs(velocity);
  double wneg = velocity - fabs(velocity);
  double ft2 = (wneg * a.T[p] + wpos * a.T[pp]);
  return (!is_zero(a.tmask[p]) && !is_zero(a.tmask[pp])) ? mask_mul(mask_mul(ft2, a.tmask[p]), a.tmask[pp]) : 0.0;
}

__global__ void k_upwind_vert(UpwArgs a) {
  vert_segment(a.g, a.tmask, a.th, [&](int i, int j, int k) { return upw_fz(a, i, j, k); });
}

static UpwArgs upw_args(mom5gpu_domain* d, int n, int level) {
  UpwArgs a;
  a.g = d->geo;
  a.tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  a.dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a.dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.dat = fptr(d, MOM5GPU_DAT, 0, 0);
  a.uh = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a.vh = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a.w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  a.T = fptr(d, MOM5GPU_TRACER, n, level);
  a.th = fptr(d, MOM5GPU_TH_TENDENCY, n, 0);
  return a;
}

int launch_upwind_horz(mom5gpu_domain* d, int n, int taum1) {
  UpwArgs a = upw_args(d, n, taum1);
  const Geo& g = d->geo;
  if (!a.tmask || !a.dyte || !a.dxtn || !a.datr || !a.uh || !a.vh || !a.T || !a.th)
    return fail(d, MOM5GPU_ESTATE, "upwind: a required field was never set");
  ClockScope clk(d, SEC_UPWIND);
  count_launches(d, 1);
  k_upwind_horz<<<horz_grid(g), HB, 0, d->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "upwind horz");
}

int launch_upwind_vert(mom5gpu_domain* d, int n, int taum1) {
  UpwArgs a = upw_args(d, n, taum1);
  const Geo& g = d->geo;
  if (!a.tmask || !a.w || !a.T || !a.th) return fail(d, MOM5GPU_ESTATE, "upwind: a required field was never set");
  ClockScope clk(d, SEC_UPWIND);
  count_launches(d, 1);
  k_upwind_vert<<<vert_grid(g), 128, 0, d->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "upwind vert");
}

// ---------------------------------------------------------------------------
// Quicker: horz :2538-2653, vert :2981-3031 (weights from quicker_init).
// ---------------------------------------------------------------------------
struct QukArgs {
  Geo g;
  int limit_with_upwind;
  const uint8_t* mask2;  // tmask_quick
  const double *tmask, *tmask_limit, *dyte, *dxtn, *datr, *uh, *vh, *w, *Tm1, *T0;
  QuickerWeights q;
  double* th;
};

// tracer_quick: T(taum1) on the compute domain, halo-2 update (cyclic) or 0.
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

DEVI double quk_fx(const QukArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  long q = I2(g, i, j);
  long n2 = g.n2;
  if (a.limit_with_upwind && is_one(a.tmask_limit[I3(g, i, j, k)])) {
    double vel = a.uh[I3(g, i, j, k)];
    double upos = half_exact(vel + fabs(vel));
    double uneg = half_exact(vel - fabs(vel));
    double f = a.dyte[q] * (upos * a.Tm1[I3(g, i, j, k)] + uneg * a.Tm1[I3(g, i + 1, j, k)]);
    return mask_mul(mask_mul(f, a.tmask[I3(g, i, j, k)]), a.tmask[I3(g, i + 1, j, k)]);
  }
  double vel = a.dyte[q] * a.uh[I3(g, i, j, k)];
  double upos = half_exact(vel + fabs(vel));
  double uneg = half_exact(vel - fabs(vel));
  bool mm = a.mask2[IM(g, i - 1, j, k)], m0 = a.mask2[IM(g, i, j, k)];
  bool m1 = a.mask2[IM(g, i + 1, j, k)], m2 = a.mask2[IM(g, i + 2, j, k)];
  bool eastmsk = m0 && !mm;
  bool westmsk = m1 && !m2;
  double tqm = tq(g, a.Tm1, i - 1, j, k), tq0 = tq(g, a.Tm1, i, j, k);
  double tq1 = tq(g, a.Tm1, i + 1, j, k), tq2 = tq(g, a.Tm1, i + 2, j, k);
  return vel * (a.q.quick_x[q] * a.T0[I3(g, i, j, k)] + a.q.quick_x[n2 + q] * a.T0[I3(g, i + 1, j, k)]) -
         upos * (a.q.curv_xp[q] * tq1 + a.q.curv_xp[n2 + q] * tq0 + a.q.curv_xp[2 * n2 + q] * (eastmsk ? tq0 : tqm)) -
         uneg * (a.q.curv_xn[q] * (westmsk ? tq1 : tq2) + a.q.curv_xn[n2 + q] * tq1 + a.q.curv_xn[2 * n2 + q] * tq0);
}

DEVI double quk_fy(const QukArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  long q = I2(g, i, j);
  long n2 = g.n2;
  if (a.limit_with_upwind && is_one(a.tmask_limit[I3(g, i, j, k)])) {
    double vel = a.vh[I3(g, i, j, k)];
    double upos = half_exact(vel + fabs(vel));
    double uneg = half_exact(vel - fabs(vel));
    double f = a.dxtn[q] * (upos * a.Tm1[I3(g, i, j, k)] + uneg * a.Tm1[I3(g, i, j + 1, k)]);
    return mask_mul(mask_mul(f, a.tmask[I3(g, i, j, k)]), a.tmask[I3(g, i, j + 1, k)]);
  }
  double vel = a.dxtn[q] * a.vh[I3(g, i, j, k)];
  double upos = half_exact(vel + fabs(vel));
  double uneg = half_exact(vel - fabs(vel));
  bool mm = a.mask2[IM(g, i, j - 1, k)], m0 = a.mask2[IM(g, i, j, k)];
  bool m1 = a.mask2[IM(g, i, j + 1, k)], m2 = a.mask2[IM(g, i, j + 2, k)];
  bool rnormsk = m0 && !mm;
  bool soutmsk = m1 && !m2;
  double tqm = tq(g, a.Tm1, i, j - 1, k), tq0 = tq(g, a.Tm1, i, j, k);
  double tq1 = tq(g, a.Tm1, i, j + 1, k), tq2 = tq(g, a.Tm1, i, j + 2, k);
  return vel * (a.q.quick_y[q] * a.T0[I3(g, i, j, k)] + a.q.quick_y[n2 + q] * a.T0[I3(g, i, j + 1, k)]) -
         upos * (a.q.curv_yp[q] * tq1 + a.q.curv_yp[n2 + q] * tq0 + a.q.curv_yp[2 * n2 + q] * (rnormsk ? tq0 : tqm)) -
         uneg * (a.q.curv_yn[q] * (soutmsk ? tq1 : tq2) + a.q.curv_yn[n2 + q] * tq1 + a.q.curv_yn[2 * n2 + q] * tq0);
}

__global__ void __launch_bounds__(HB) k_quicker_horz(QukArgs a) {
  horz_faces_once(
      a.g, a.tmask, a.datr, a.th, [&](int i, int j, int k) { return quk_fx(a, i, j, k); },
      [&](int i, int j, int k) { return quk_fy(a, i, j, k); });
}

// flux through the bottom of level k (:2981-3031)
DEVI double quk_fz(const QukArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  const int nk = g.nk;
  int km1 = k > 0 ? k - 1 : 0;
  int kp1 = k + 1 < nk ? k + 1 : nk - 1;
  int p2 = k + 2 < nk ? k + 2 : nk - 1;
  long p = I3(g, i, j, k);
  double vel = a.w[I3(g, i, j, k + 1)];
  double upos = half_exact(vel + fabs(vel));
  double uneg = half_exact(vel - fabs(vel));
  const double* Tm = a.Tm1;
  if (is_one(a.tmask_limit[p]))
    return mask_mul(mask_mul(uneg * Tm[p] + upos * Tm[I3(g, i, j, kp1)], a.tmask[p]), a.tmask[I3(g, i, j, kp1)]);
  // kp2 = nint(tmask(p2)*p2 + (1-tmask(p2))*kp1): p2 when level p2 is wet, else kp1
  int kp2 = !is_zero(a.tmask[I3(g, i, j, p2)]) ? p2 : kp1;
  bool upmsk = !is_zero(a.tmask[p]) && is_zero(a.tmask[I3(g, i, j, km1)]);
  return vel * (a.q.quick_z[k] * a.T0[p] + a.q.quick_z[nk + k] * a.T0[I3(g, i, j, kp1)]) -
         uneg * (a.q.curv_zp[k] * Tm[I3(g, i, j, kp1)] + a.q.curv_zp[nk + k] * Tm[p] +
                 a.q.curv_zp[2 * nk + k] * Tm[I3(g, i, j, km1)]) -
         upos * (a.q.curv_zn[k] * Tm[I3(g, i, j, kp2)] + a.q.curv_zn[nk + k] * Tm[I3(g, i, j, kp1)] +
                 a.q.curv_zn[2 * nk + k] * (upmsk ? Tm[I3(g, i, j, kp1)] : Tm[p]));
}

__global__ void k_quicker_vert(QukArgs a) {
  vert_segment(a.g, a.tmask, a.th, [&](int i, int j, int k) { return quk_fz(a, i, j, k); });
}

// QuickMOM3, horizontal (:2665-2780): the Quicker weights with mask products in
// place of the coast masks and the northern second neighbour clamped to nj
DEVI double qm3_fx(const QukArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  long q = I2(g, i, j);
  long n2 = g.n2;
  if (a.limit_with_upwind && is_one(a.tmask_limit[I3(g, i, j, k)])) {
    double vel = a.uh[I3(g, i, j, k)];
    double upos = half_exact(vel + fabs(vel));
    double uneg = half_exact(vel - fabs(vel));
    double f = a.dyte[q] * (upos * a.Tm1[I3(g, i, j, k)] + uneg * a.Tm1[I3(g, i + 1, j, k)]);
    return mask_mul(mask_mul(f, a.tmask[I3(g, i, j, k)]), a.tmask[I3(g, i + 1, j, k)]);
  }
  auto mq = [&](int ii) { return a.mask2[IM(g, ii, j, k)] ? 1.0 : 0.0; };
  double vel = a.dyte[q] * a.uh[I3(g, i, j, k)];
  double upos = mask_mul(mask_mul(mask_mul(half_exact(vel + fabs(vel)), mq(i - 1)), mq(i)), mq(i + 1));
  double uneg = mask_mul(mask_mul(mask_mul(half_exact(vel - fabs(vel)), mq(i + 2)), mq(i + 1)), mq(i));
  double tqm = tq(g, a.Tm1, i - 1, j, k), tq0 = tq(g, a.Tm1, i, j, k);
  double tq1 = tq(g, a.Tm1, i + 1, j, k), tq2 = tq(g, a.Tm1, i + 2, j, k);
  return vel * (a.q.quick_x[q] * a.T0[I3(g, i, j, k)] + a.q.quick_x[n2 + q] * a.T0[I3(g, i + 1, j, k)]) -
         upos * (a.q.curv_xp[q] * tq1 + a.q.curv_xp[n2 + q] * tq0 + a.q.curv_xp[2 * n2 + q] * tqm) -
         uneg * (a.q.curv_xn[q] * tq2 + a.q.curv_xn[n2 + q] * tq1 + a.q.curv_xn[2 * n2 + q] * tq0);
}

DEVI double qm3_fy(const QukArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  long q = I2(g, i, j);
  long n2 = g.n2;
  if (a.limit_with_upwind && is_one(a.tmask_limit[I3(g, i, j, k)])) {
    double vel = a.vh[I3(g, i, j, k)];
    double upos = half_exact(vel + fabs(vel));
    double uneg = half_exact(vel - fabs(vel));
    double f = a.dxtn[q] * (upos * a.Tm1[I3(g, i, j, k)] + uneg * a.Tm1[I3(g, i, j + 1, k)]);
    return mask_mul(mask_mul(f, a.tmask[I3(g, i, j, k)]), a.tmask[I3(g, i, j + 1, k)]);
  }
  const int jp2 = j + 2 < g.nj ? j + 2 : g.nj;  // min(j+2, jec)
  auto mq = [&](int jj) { return a.mask2[IM(g, i, jj, k)] ? 1.0 : 0.0; };
  double vel = a.dxtn[q] * a.vh[I3(g, i, j, k)];
  double upos = mask_mul(mask_mul(mask_mul(half_exact(vel + fabs(vel)), mq(j - 1)), mq(j)), mq(j + 1));
  double uneg = mask_mul(mask_mul(mask_mul(half_exact(vel - fabs(vel)), mq(jp2)), mq(j + 1)), mq(j));
  double tqm = tq(g, a.Tm1, i, j - 1, k), tq0 = tq(g, a.Tm1, i, j, k);
  double tq1 = tq(g, a.Tm1, i, j + 1, k), tq2 = tq(g, a.Tm1, i, jp2, k);
  return vel * (a.q.quick_y[q] * a.T0[I3(g, i, j, k)] + a.q.quick_y[n2 + q] * a.T0[I3(g, i, j + 1, k)]) -
         upos * (a.q.curv_yp[q] * tq1 + a.q.curv_yp[n2 + q] * tq0 + a.q.curv_yp[2 * n2 + q] * tqm) -
         uneg * (a.q.curv_yn[q] * tq2 + a.q.curv_yn[n2 + q] * tq1 + a.q.curv_yn[2 * n2 + q] * tq0);
}

__global__ void __launch_bounds__(HB) k_quickmom3_horz(QukArgs a) {
  horz_faces_once(
      a.g, a.tmask, a.datr, a.th, [&](int i, int j, int k) { return qm3_fx(a, i, j, k); },
      [&](int i, int j, int k) { return qm3_fy(a, i, j, k); });
}

static int quk_args(mom5gpu_domain* d, int n, int taum1, int tau, QukArgs* a) {
  a->g = d->geo;
  a->limit_with_upwind = d->opt.limit_with_upwind;
  a->mask2 = d->mask2;
  a->tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  a->tmask_limit = fptr(d, MOM5GPU_TMASK_LIMIT, n, 0);
  a->dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a->dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a->datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a->uh = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a->vh = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a->w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  a->Tm1 = fptr(d, MOM5GPU_TRACER, n, taum1);
  a->T0 = fptr(d, MOM5GPU_TRACER, n, tau);
  a->q = d->qw;
  a->th = fptr(d, MOM5GPU_TH_TENDENCY, n, 0);
  if (!a->tmask || !a->tmask_limit || !a->dyte || !a->dxtn || !a->datr || !a->uh || !a->vh || !a->w || !a->Tm1 ||
      !a->T0 || !a->th || !a->q.quick_x)
    return fail(d, MOM5GPU_ESTATE, "quicker: a required field was never set");
  return MOM5GPU_OK;
}

int launch_quicker_horz(mom5gpu_domain* d, int n, int taum1, int tau) {
  QukArgs a;
  int rc = quk_args(d, n, taum1, tau, &a);
  if (rc) return rc;
  ClockScope clk(d, SEC_QUICKER);
  count_launches(d, 1);
  const Geo& g = d->geo;
  k_quicker_horz<<<horz_grid(g), HB, 0, d->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "quicker horz");
}

int launch_quickmom3_horz(mom5gpu_domain* d, int n, int taum1, int tau) {
  QukArgs a;
  int rc = quk_args(d, n, taum1, tau, &a);
  if (rc) return rc;
  ClockScope clk(d, SEC_QUICKER);
  count_launches(d, 1);
  k_quickmom3_horz<<<horz_grid(d->geo), HB, 0, d->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "quickmom3 horz");
}

int launch_quicker_vert(mom5gpu_domain* d, int n, int taum1, int tau) {
  QukArgs a;
  int rc = quk_args(d, n, taum1, tau, &a);
  if (rc) return rc;
  ClockScope clk(d, SEC_QUICKER);
  count_launches(d, 1);
  const Geo& g = d->geo;
  k_quicker_vert<<<vert_grid(g), 128, 0, d->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "quicker vert");
}

// ---------------------------------------------------------------------------
// Centred schemes: 2nd order (ocean_tracer_advect.F90:2306-2352, :2836-2864),
// 4th order (:2361-2435, :2873-2907), 6th order (:2444-2529, :2916-2972).
// tracer_fourth/sixth and tmask_fourth/sixth are read through tq (the
// compute-domain value after a halo update of width 2/3: periodic image or 0).
// ---------------------------------------------------------------------------
constexpr double kA4 = 7.0 / 12.0, kB4 = -1.0 / 12.0;                    // :349
constexpr double kA6 = 37.0 / 60.0, kB6 = -2.0 / 15.0, kC6 = 1.0 / 60.0;  // :350

struct CenArgs {
  Geo g;
  const double *tmask, *dyte, *dxtn, *datr, *uh, *vh, *w, *T;
  const int* kmt;
  double* th;
};

template <int ORDER>
DEVI double cen_fx(const CenArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  double du = a.dyte[I2(g, i, j)] * a.uh[I3(g, i, j, k)];
  if (ORDER == 2) return half_exact(du) * (a.T[I3(g, i + 1, j, k)] + a.T[I3(g, i, j, k)]);
  // the masks are 0.0 or 1.0: products, == 0 tests and the index selections exactly as integers
  auto TM = [&](int ii) { return !is_zero(tq(g, a.tmask, ii, j, k)); };
  auto TT = [&](int ii) { return tq(g, a.T, ii, j, k); };
  if (ORDER == 4 || !(TM(i - 2) && TM(i - 1)) || !(TM(i + 3) && TM(i + 2))) {
    int im1 = TM(i - 1) ? i - 1 : i;
    int ip2 = TM(i + 2) ? i + 2 : i + 1;
    return du * (kA4 * (TT(i + 1) + TT(i)) + kB4 * (TT(ip2) + TT(im1)));
  }
  return du * (kA6 * (TT(i + 1) + TT(i)) + kB6 * (TT(i + 2) + TT(i - 1)) + kC6 * (TT(i + 3) + TT(i - 2)));
}

template <int ORDER>
DEVI double cen_fy(const CenArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  double dv = a.dxtn[I2(g, i, j)] * a.vh[I3(g, i, j, k)];
  if (ORDER == 2) return half_exact(dv) * (a.T[I3(g, i, j + 1, k)] + a.T[I3(g, i, j, k)]);
  auto TM = [&](int jj) { return !is_zero(tq(g, a.tmask, i, jj, k)); };
  auto TT = [&](int jj) { return tq(g, a.T, i, jj, k); };
  if (ORDER == 4 || !(TM(j - 2) && TM(j - 1)) || !(TM(j + 3) && TM(j + 2))) {
    int jm1 = TM(j - 1) ? j - 1 : j;
    int jp2 = TM(j + 2) ? j + 2 : j + 1;
    return dv * (kA4 * (TT(j + 1) + TT(j)) + kB4 * (TT(jp2) + TT(jm1)));
  }
  return dv * (kA6 * (TT(j + 1) + TT(j)) + kB6 * (TT(j + 2) + TT(j - 1)) + kC6 * (TT(j + 3) + TT(j - 2)));
}

template <int ORDER>
__global__ void __launch_bounds__(HB) k_centred_horz(CenArgs a) {
  horz_faces_once(
      a.g, a.tmask, a.datr, a.th, [&](int i, int j, int k) { return cen_fx<ORDER>(a, i, j, k); },
      [&](int i, int j, int k) { return cen_fy<ORDER>(a, i, j, k); });
}

// flux through the bottom of level k (Fortran level K = k+1)
template <int ORDER>
DEVI double cen_fz(const CenArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  const int nk = g.nk, K = k + 1;
  double w = a.w[I3(g, i, j, K)];
  int p1 = K + 1 < nk ? K + 1 : nk, p2 = K + 2 < nk ? K + 2 : nk, km1 = K - 1 > 1 ? K - 1 : 1;
  auto TV = [&](int L) { return a.T[I3(g, i, j, L - 1)]; };
  if (ORDER == 2) return half_exact(w) * (TV(K) + TV(p1));
  int kp2 = is_zero(a.tmask[I3(g, i, j, p2 - 1)]) ? p1 : p2;  // nint(tp2*p2 + (1-tp2)*p1), tp2 0 or 1
  if (ORDER == 6 && !(K <= 2 || K >= nk - 1) && K < a.kmt[I2(g, i, j)] - 2)
    return w * (kA6 * (TV(K) + TV(p1)) + kB6 * (TV(km1) + TV(kp2)) + kC6 * (TV(K - 2) + TV(K + 3)));
  return w * (kA4 * (TV(K) + TV(p1)) + kB4 * (TV(km1) + TV(kp2)));
}

template <int ORDER>
__global__ void k_centred_vert(CenArgs a) {
  vert_segment(a.g, a.tmask, a.th, [&](int i, int j, int k) { return cen_fz<ORDER>(a, i, j, k); });
}

int ensure_kmt_device(mom5gpu_domain* d) {
  if (d->kmt_d) return MOM5GPU_OK;
  const Geo& g = d->geo;
  if ((long)d->kmt_h.size() != g.n2) return fail(d, MOM5GPU_ESTATE, "kmt needed: call mom5gpu_set_vertical_grid");
  cudaError_t e = cudaMalloc(&d->kmt_d, sizeof(int) * g.n2);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d->kmt_d, d->kmt_h.data(), sizeof(int) * g.n2, cudaMemcpyHostToDevice, d->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return cuda_fail(d, e, "kmt upload");
  d->bytes += sizeof(int) * g.n2;
  return MOM5GPU_OK;
}

int launch_centred(mom5gpu_domain* d, int n, int tau, int order, bool horz) {
  const Geo& g = d->geo;
  CenArgs a;
  a.g = g;
  a.tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  a.dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a.dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.uh = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a.vh = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a.w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  a.T = fptr(d, MOM5GPU_TRACER, n, tau);
  a.th = fptr(d, MOM5GPU_TH_TENDENCY, n, 0);
  a.kmt = nullptr;
  if (!a.tmask || !a.dyte || !a.dxtn || !a.datr || !a.uh || !a.vh || !a.w || !a.T || !a.th)
    return fail(d, MOM5GPU_ESTATE, "centred advection: a required field was never set");
  if (!horz && order == 6) {
    int rc = ensure_kmt_device(d);
    if (rc) return rc;
    a.kmt = d->kmt_d;
  }
  count_launches(d, 1);
  if (horz) {
    dim3 grid = horz_grid(g);
    if (order == 2) k_centred_horz<2><<<grid, HB, 0, d->stream>>>(a);
    else if (order == 4) k_centred_horz<4><<<grid, HB, 0, d->stream>>>(a);
    else k_centred_horz<6><<<grid, HB, 0, d->stream>>>(a);
  } else {
    dim3 grid = vert_grid(g);
    if (order == 2) k_centred_vert<2><<<grid, 128, 0, d->stream>>>(a);
    else if (order == 4) k_centred_vert<4><<<grid, 128, 0, d->stream>>>(a);
    else k_centred_vert<6><<<grid, 128, 0, d->stream>>>(a);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "centred advection");
}

// ---------------------------------------------------------------------------
// MDFL Super-B (advect_tracer_mdfl_sup_b, ocean_tracer_advect.F90:3189-3466):
// level by level z, x, y with the superbee limiter.  Levels are independent
// (the z flux of the level above is recomputed), so each pass is one kernel
// over all cells: z (tracer -> tz), x (tz with its halo image -> tx), y and
// the tendency.  tmask_mdfl is the halo-2 byte mask.
// ---------------------------------------------------------------------------
struct SupbArgs {
  Geo g;
  double dtime;
  const uint8_t* mask2;
  const double *tmask, *dat, *datr, *dxte, *dyte, *dxtn, *dytn, *uh, *vh, *w, *rdz, *T;
  double *tz, *tx, *th;
};

DEVI double m2d(const SupbArgs& a, int i, int j, int k) { return a.mask2[IM(a.g, i, j, k)] ? 1.0 : 0.0; }

// face flux 0.5*(mf*(Ta+Tb) - |mf|*(1 + (cfl-1)*Cr)*Rj)*m0*m1 with the superbee limiter (:3244-3263)
DEVI double supb_flux(double mf, double cfl, double Rjm, double Rj, double Rjp, double Ta, double Tb, double m0,
                      double m1) {
  // the comparisons on the integer pipe (sel::), same selections as the FP ones
  const bool pos = sel::gt0(mf);
  double Cr;
  if ((__double_as_longlong(Rj) << 1) != 0) Cr = div_seeded(pos ? Rjm : Rjp, Rj);
  else Cr = (pos ? Rjm : Rjp) * 1.0e20;
  double c2 = 2.0 * Cr;
  double lo = sel::lt_min(1.0, c2), hi = sel::lt_min(2.0, Cr);
  double mx = sel::gt_max(lo, hi);
  Cr = sel::gt_max(0.0, mx);
  return 0.5 * (mf * (Ta + Tb) - fabs(mf) * (1.0 + (cfl - 1.0) * Cr) * Rj) * m0 * m1;
}

DEVI double supb_zflux(const SupbArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  int kp1 = k + 1 < g.nk ? k + 1 : g.nk - 1, kp2 = k + 2 < g.nk ? k + 2 : g.nk - 1, km1 = k > 0 ? k - 1 : 0;
  double Tk = a.T[I3(g, i, j, k)], Tkp1 = a.T[I3(g, i, j, kp1)];
  double Rjp = (a.T[I3(g, i, j, km1)] - Tk) * m2d(a, i, j, km1) * m2d(a, i, j, k);
  double Rj = (Tk - Tkp1) * m2d(a, i, j, k) * m2d(a, i, j, kp1);
  double Rjm = (Tkp1 - a.T[I3(g, i, j, kp2)]) * m2d(a, i, j, kp1) * m2d(a, i, j, kp2);
  double w = a.w[I3(g, i, j, k + 1)];
  double cfl = fabs(div_seeded(w * a.dtime, a.rdz[I3(g, i, j, k)]));
  return supb_flux(a.dat[I2(g, i, j)] * w, cfl, Rjm, Rj, Rjp, Tk, Tkp1, m2d(a, i, j, kp1), m2d(a, i, j, k));
}

// z step down a segment of VS levels carrying the flux through the top of the level
__global__ void k_supb_z(SupbArgs a) {
  const Geo& g = a.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
  if (i > g.ni) return;
  const int k0 = blockIdx.z * VS, k1 = k0 + VS < g.nk ? k0 + VS : g.nk;
  double ftp = k0 > 0 ? supb_zflux(a, i, j, k0 - 1) : 0.0;
  for (int k = k0; k < k1; ++k) {
    long p = I3(g, i, j, k);
    double fbt = supb_zflux(a, i, j, k);
    double wkm1 = k > 0 ? a.w[I3(g, i, j, k)] : 0.0;
    double Tk = a.T[p];
    a.tz[p] = Tk + div_seeded(a.dtime, a.rdz[p]) * (a.datr[I2(g, i, j)] * (fbt - ftp) + Tk * (wkm1 - a.w[I3(g, i, j, k + 1)]));
    ftp = fbt;
  }
}

DEVI double supb_xflux(const SupbArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  auto t = [&](int ii) { return tq(g, a.tz, ii, j, k); };
  double Rjp = (t(i + 2) - t(i + 1)) * m2d(a, i + 2, j, k) * m2d(a, i + 1, j, k);
  double Rj = (t(i + 1) - t(i)) * m2d(a, i + 1, j, k) * m2d(a, i, j, k);
  double Rjm = (t(i) - t(i - 1)) * m2d(a, i, j, k) * m2d(a, i - 1, j, k);
  double u = a.uh[I3(g, i, j, k)];
  double cfl = fabs(div_seeded(u * a.dtime * 2.0, (a.rdz[I3(g, i, j, k)] + a.rdz[I3(g, i + 1, j, k)]) * a.dxte[I2(g, i, j)]));
  return supb_flux(a.dyte[I2(g, i, j)] * u, cfl, Rjm, Rj, Rjp, t(i + 1), t(i), m2d(a, i, j, k), m2d(a, i + 1, j, k));
}

// x step of one row: thread t forms the flux through face i0-1+t once (shared memory)
__global__ void __launch_bounds__(HB) k_supb_x(SupbArgs a) {
  __shared__ double sfx[HB];
  const Geo& g = a.g;
  const int t = threadIdx.x, i0 = blockIdx.x * (HB - 1) + 1, j = blockIdx.y + 1, k = blockIdx.z;
  const int iface = i0 - 1 + t, i = i0 + t;
  sfx[t] = iface <= g.ni ? supb_xflux(a, iface, j, k) : 0.0;
  __syncthreads();
  if (t > HB - 2 || i > g.ni) return;
  long p = I3(g, i, j, k);
  double div = a.dyte[I2(g, i, j)] * a.uh[p] - a.dyte[I2(g, i - 1, j)] * a.uh[I3(g, i - 1, j, k)];
  a.tx[p] = a.tz[p] + div_seeded(a.dtime * m2d(a, i, j, k) * a.datr[I2(g, i, j)], a.rdz[p]) * (sfx[t] - sfx[t + 1] + a.T[p] * div);
}

DEVI double supb_yflux(const SupbArgs& a, int i, int j, int k) {
  const Geo& g = a.g;
  auto t = [&](int jj) { return tq(g, a.tx, i, jj, k); };
  double Rjp = (t(j + 2) - t(j + 1)) * m2d(a, i, j + 2, k) * m2d(a, i, j + 1, k);
  double Rj = (t(j + 1) - t(j)) * m2d(a, i, j + 1, k) * m2d(a, i, j, k);
  double Rjm = (t(j) - t(j - 1)) * m2d(a, i, j, k) * m2d(a, i, j - 1, k);
  double v = a.vh[I3(g, i, j, k)];
  double cfl = fabs(div_seeded(v * a.dtime * 2.0, (a.rdz[I3(g, i, j, k)] + a.rdz[I3(g, i, j + 1, k)]) * a.dytn[I2(g, i, j)]));
  return supb_flux(a.dxtn[I2(g, i, j)] * v, cfl, Rjm, Rj, Rjp, t(j + 1), t(j), m2d(a, i, j, k), m2d(a, i, j + 1, k));
}

// y step and tendency along a strip of HR rows carrying the flux through the south face
__global__ void k_supb_y(SupbArgs a) {
  const Geo& g = a.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j0 = blockIdx.y * HR + 1, k = blockIdx.z;
  if (i > g.ni) return;
  double fs = supb_yflux(a, i, j0 - 1, k);
  for (int j = j0; j < j0 + HR && j <= g.nj; ++j) {
    long p = I3(g, i, j, k);
    double fn = supb_yflux(a, i, j, k);
    double rdz = a.rdz[p], datr = a.datr[I2(g, i, j)], T = a.T[p];
    double t = a.tx[p] + div_seeded(a.dtime * a.tmask[p] * datr, rdz) * (fs - fn);
    double wkm1 = k > 0 ? a.w[I3(g, i, j, k)] : 0.0;
    t = t + div_seeded(a.dtime * T, rdz) *
                (a.w[I3(g, i, j, k + 1)] - wkm1 +
                 datr * (a.dyte[I2(g, i - 1, j)] * a.uh[I3(g, i - 1, j, k)] - a.dyte[I2(g, i, j)] * a.uh[p]));
    double advect = div_seeded(-rdz * (t - T), a.dtime) * m2d(a, i, j, k);
    a.th[p] = a.th[p] + (-advect);
    fs = fn;
  }
}

int launch_mdfl_sup_b(mom5gpu_domain* d, int n, int taum1, int tau, double dtime) {
  const Geo& g = d->geo;
  int rc = ensure_mdfl_scratch(d, 1);
  if (rc) return rc;
  SupbArgs a;
  a.g = g;
  a.dtime = dtime;
  a.mask2 = d->mask2;
  a.tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  a.dat = fptr(d, MOM5GPU_DAT, 0, 0);
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.dxte = fptr(d, MOM5GPU_DXTE, 0, 0);
  a.dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a.dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a.dytn = fptr(d, MOM5GPU_DYTN, 0, 0);
  a.uh = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a.vh = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a.w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  a.rdz = fptr(d, MOM5GPU_RHO_DZT, 0, tau);
  a.T = fptr(d, MOM5GPU_TRACER, n, taum1);
  a.th = fptr(d, MOM5GPU_TH_TENDENCY, n, 0);
  a.tz = d->mdfl_a;
  a.tx = d->mdfl_b;
  const void* need[] = {a.mask2, a.tmask, a.dat, a.datr, a.dxte, a.dyte, a.dxtn, a.dytn, a.uh, a.vh, a.w, a.rdz,
                        a.T, a.th};
  for (const void* p : need)
    if (!p) return fail(d, MOM5GPU_ESTATE, "mdfl_sup_b: a required field was never set");
  ClockScope clk(d, SEC_MDFL);
  count_launches(d, 3);
  k_supb_z<<<vert_grid(g), 128, 0, d->stream>>>(a);
  k_supb_x<<<dim3((g.ni + HB - 2) / (HB - 1), g.nj, g.nk), HB, 0, d->stream>>>(a);
  k_supb_y<<<dim3((g.ni + 127) / 128, (g.nj + HR - 1) / HR, g.nk), 128, 0, d->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "mdfl_sup_b");
}

// ---------------------------------------------------------------------------
// MDPPM (ocean_tracer_advect.F90:5990-6507): vertical pass in three kernels
// (slopes, fluxes by a march down each column, update), then the x and y
// passes streaming along lines (mdppm_body.cuh).
// ---------------------------------------------------------------------------
struct PpmArgs {
  Geo g;
  int lim;
  double dtime;
  const double *tmask, *dat, *datr, *dxte, *dyte, *dxtn, *dytn, *uh, *vh, *w, *rdz, *T;
  double *dak, *fz, *tz, *tx, *th;
};

// vertical slope dak of every cell with the clamped neighbour levels and their
// collapse factors real(kp1-k) ... (:6064-6099)
__global__ void k_ppm_dak(PpmArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z;
  if (i > g.ni) return;
  const int nk = g.nk, K = k + 1;
  int km2 = K - 2 > 1 ? K - 2 : 1, km1 = K - 1 > 1 ? K - 1 : 1, kp1 = K + 1 < nk ? K + 1 : nk,
      kp2 = K + 2 < nk ? K + 2 : nk;
  auto at = [&](const double* f, int L) { return f[I3(g, i, j, L - 1)]; };
  double S[5] = {at(a.T, km2), at(a.T, km1), at(a.T, K), at(a.T, kp1), at(a.T, kp2)};
  double M[5] = {at(a.tmask, km2) * (double)(km1 - km2), at(a.tmask, km1) * (double)(K - km1), at(a.tmask, K),
                 at(a.tmask, kp1) * (double)(kp1 - K), at(a.tmask, kp2) * (double)(kp2 - kp1)};
  double t0, t1, t2, t3;
  ppm::slope(S, M, a.dak[I3(g, i, j, k)], t0, t1, t2, t3);
}

// edge values, limiter and the fluxes through the bottom (massflux <= 0) and top
// (massflux > 0) faces of a cell (:6101-6170).  The reference's loop over the
// levels carries nothing from one level to the next, and a face is written by
// exactly one of its two cells (the same mask-product massflux, <= 0 from above,
// > 0 from below), so every cell runs in its own thread.
__global__ void k_ppm_zflux(PpmArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
  if (i > g.ni) return;
  const int nk = g.nk;
  const long q = I2(g, i, j);
  auto at = [&](const double* f, int L) { return f[I3(g, i, j, L - 1)]; };
  const double dat = a.dat[q];
  {
    const int K = blockIdx.z + 1;
    int km2 = K - 2 > 1 ? K - 2 : 1, km1 = K - 1 > 1 ? K - 1 : 1, kp1 = K + 1 < nk ? K + 1 : nk,
        kp2 = K + 2 < nk ? K + 2 : nk;
    double mskp2 = at(a.tmask, kp2) * (double)(kp2 - kp1), mskp1 = at(a.tmask, kp1) * (double)(kp1 - K);
    double msk0 = at(a.tmask, K), mskm1 = at(a.tmask, km1) * (double)(K - km1);
    double mskm2 = at(a.tmask, km2) * (double)(km1 - km2);
    double Sip2 = at(a.T, kp2), Sip1 = at(a.T, kp1), Si = at(a.T, K), Sim1 = at(a.T, km1), Sim2 = at(a.T, km2);
    double d1m = (Si - Sim1) * mskm1, d1p = (Sip1 - Si) * mskp1;
    double d1mm = (Sim1 - Sim2) * mskm1 * mskm2, d1pp = (Sip2 - Sip1) * mskp1 * mskp2;
    Sim1 = Si - d1m;
    Sip1 = Si + d1p;
    double dk = at(a.dak, K);
    double al = 0.5 * (Sim1 + Si) + ppm::kSixth * (at(a.dak, km1) - dk);
    double ar = 0.5 * (Si + Sip1) + ppm::kSixth * (dk - at(a.dak, kp1));
    ppm::limit(a.lim, Si, dk, d1m, d1p, d1mm, d1pp, al, ar);
    double c6 = 6. * Si - 3. * (ar + al);
    double wk = a.w[I3(g, i, j, K)];
    double massflux = dat * wk * msk0 * mskp1;
    if (!sel::gt0(massflux)) {
      double cfl = fabs(div_seeded(wk * a.dtime, at(a.rdz, K)));
      a.fz[I3(g, i, j, K - 1)] = massflux * (ar + 0.5 * cfl * ((al - ar) + (1. - ppm::kTwoThirds * cfl) * c6));
    }
    double wkm1 = a.w[I3(g, i, j, km1)];
    massflux = dat * wkm1 * msk0 * mskm1;
    if (sel::gt0(massflux)) {
      double cfl = fabs(div_seeded(wkm1 * a.dtime, at(a.rdz, km1)));
      a.fz[I3(g, i, j, km1 - 1)] = massflux * (al + 0.5 * cfl * ((ar - al) + (1. - ppm::kTwoThirds * cfl) * c6));
    }
  }
}

// vertical update of tracer_mdppm (:6173-6182)
__global__ void k_ppm_zupd(PpmArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z;
  if (i > g.ni) return;
  const int K = k + 1, km1 = K - 1 > 1 ? K - 1 : 1;
  const double mskm1 = (double)(K - km1);
  long p = I3(g, i, j, k), pm = I3(g, i, j, km1 - 1);
  double T = a.T[p];
  a.tz[p] = T + div_seeded(a.dtime, a.rdz[p]) *
                    (a.datr[I2(g, i, j)] * (a.fz[p] - mskm1 * a.fz[pm]) +
                     T * (mskm1 * a.w[I3(g, i, j, km1)] - a.w[I3(g, i, j, K)]));
}

// x pass along the rows (:6193-6325): tracer_mdppm after the x halo update;
// segments of PPM_LX - 8 cells, one thread per position
constexpr int PPM_LX = 128, PPM_BY = 8, PPM_LY = 64;

__global__ void __launch_bounds__(PPM_LX) k_ppm_x(PpmArgs a) {
  __shared__ double sm[7][PPM_LX][1];
  const Geo& g = a.g;
  const int j = blockIdx.y + 1, k = blockIdx.z;
  const double dt = a.dtime;
  auto S = [&](int i) { return tq(g, a.tz, i, j, k); };
  auto M = [&](int i) { return tq(g, a.tmask, i, j, k); };
  auto face = [&](int i, double m0, double m1, double aL0, double aR0, double a60, double aL1, double aR1,
                  double a61) {
    double u = a.uh[I3(g, i, j, k)];
    double massflux = a.dyte[I2(g, i, j)] * u;
    double cfl = div_seeded(u * dt * 2.0, (a.rdz[I3(g, i, j, k)] + a.rdz[I3(g, i + 1, j, k)]) * a.dxte[I2(g, i, j)]);
    return ppm::hflux(massflux, m0, m1, cfl, aL0, aR0, a60, aL1, aR1, a61);
  };
  auto upd = [&](int i, double Sv, double m, double Fw, double Fe) {
    long p = I3(g, i, j, k);
    double div = a.dyte[I2(g, i, j)] * a.uh[p] - a.dyte[I2(g, i - 1, j)] * a.uh[I3(g, i - 1, j, k)];
    a.tx[p] = Sv + div_seeded(dt * m * a.datr[I2(g, i, j)], a.rdz[p]) * (Fw - Fe + a.T[p] * div);
  };
  ppm::tile_line<PPM_LX, 1>(g.ni, a.lim, (int)blockIdx.x * (PPM_LX - 8) - 3, threadIdx.x, 0, true, sm, S, M, face,
                            upd);
}

// y pass along the columns (:6330-6502) and the tendency: th += -advect_tracer_mdppm;
// PPM_BY columns per block, segments of PPM_LY - 8 cells
__global__ void __launch_bounds__(PPM_BY* PPM_LY) k_ppm_y(PpmArgs a) {
  __shared__ double sm[7][PPM_LY][PPM_BY];
  const Geo& g = a.g;
  const int i = blockIdx.x * PPM_BY + threadIdx.x + 1, k = blockIdx.z;
  const double dt = a.dtime;
  auto S = [&](int j) { return tq(g, a.tx, i, j, k); };
  auto M = [&](int j) { return tq(g, a.tmask, i, j, k); };
  auto face = [&](int j, double m0, double m1, double aL0, double aR0, double a60, double aL1, double aR1,
                  double a61) {
    double v = a.vh[I3(g, i, j, k)];
    double massflux = a.dxtn[I2(g, i, j)] * v;
    double cfl = div_seeded(v * dt * 2.0, (a.rdz[I3(g, i, j, k)] + a.rdz[I3(g, i, j + 1, k)]) * a.dytn[I2(g, i, j)]);
    return ppm::hflux(massflux, m0, m1, cfl, aL0, aR0, a60, aL1, aR1, a61);
  };
  auto upd = [&](int j, double Sv, double m, double Fs, double Fn) {
    long p = I3(g, i, j, k);
    double rdz = a.rdz[p], datr = a.datr[I2(g, i, j)], T = a.T[p];
    double t = Sv + div_seeded(dt * a.tmask[p] * datr, rdz) * (Fs - Fn);
    double wkm1 = k > 0 ? a.w[I3(g, i, j, k)] : 0.0;
    t = t + div_seeded(dt * T, rdz) *
                (a.w[I3(g, i, j, k + 1)] - wkm1 +
                 datr * (a.dyte[I2(g, i - 1, j)] * a.uh[I3(g, i - 1, j, k)] - a.dyte[I2(g, i, j)] * a.uh[p]));
    double advect = div_seeded(-rdz * (t - T), dt) * m;
    a.th[p] = a.th[p] + (-advect);
  };
  ppm::tile_line<PPM_LY, PPM_BY>(g.nj, a.lim, (int)blockIdx.y * (PPM_LY - 8) - 3, threadIdx.y, threadIdx.x,
                                 i <= g.ni, sm, S, M, face, upd);
}

int launch_mdppm(mom5gpu_domain* d, int n, int taum1, int tau, double dtime) {
  const Geo& g = d->geo;
  int rc = ensure_mdfl_scratch(d, 1);
  if (rc) return rc;
  if (!d->ppm_scr) {
    cudaError_t e = cudaMalloc(&d->ppm_scr, sizeof(double) * 2 * (size_t)g.n3);
    if (e != cudaSuccess) return fail(d, MOM5GPU_ENOMEM, "mdppm scratch: %s", cudaGetErrorString(e));
    d->bytes += sizeof(double) * 2 * (size_t)g.n3;
    cudaMemsetAsync(d->ppm_scr, 0, sizeof(double) * 2 * (size_t)g.n3, d->stream);
  }
  PpmArgs a;
  a.g = g;
  a.lim = d->scheme[n - 1].ppm_limiter;
  a.dtime = dtime;
  a.tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  a.dat = fptr(d, MOM5GPU_DAT, 0, 0);
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.dxte = fptr(d, MOM5GPU_DXTE, 0, 0);
  a.dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a.dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a.dytn = fptr(d, MOM5GPU_DYTN, 0, 0);
  a.uh = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a.vh = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a.w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  a.rdz = fptr(d, MOM5GPU_RHO_DZT, 0, tau);
  a.T = fptr(d, MOM5GPU_TRACER, n, taum1);
  a.th = fptr(d, MOM5GPU_TH_TENDENCY, n, 0);
  a.dak = d->ppm_scr;
  a.fz = d->ppm_scr + g.n3;
  a.tz = d->mdfl_a;
  a.tx = d->mdfl_b;
  const void* need[] = {a.tmask, a.dat, a.datr, a.dxte, a.dyte, a.dxtn, a.dytn, a.uh, a.vh, a.w, a.rdz, a.T, a.th};
  for (const void* p : need)
    if (!p) return fail(d, MOM5GPU_ESTATE, "mdppm: a required field was never set");
  ClockScope clk(d, SEC_MDFL);
  count_launches(d, 5);
  cudaStream_t s = d->stream;
  dim3 g3((g.ni + 127) / 128, g.nj, g.nk);
  k_ppm_dak<<<g3, 128, 0, s>>>(a);
  k_ppm_zflux<<<g3, 128, 0, s>>>(a);
  k_ppm_zupd<<<g3, 128, 0, s>>>(a);
  k_ppm_x<<<dim3((g.ni + PPM_LX - 9) / (PPM_LX - 8), g.nj, g.nk), PPM_LX, 0, s>>>(a);
  k_ppm_y<<<dim3((g.ni + PPM_BY - 1) / PPM_BY, (g.nj + PPM_LY - 9) / (PPM_LY - 8), g.nk), dim3(PPM_BY, PPM_LY), 0, s>>>(
      a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "mdppm");
}

// ---------------------------------------------------------------------------
// explicit tracer update (ocean_tracer.F90:2341-2350)
// ---------------------------------------------------------------------------
// The time levels and th_tendency are distinct arrays (restrict), so the loads of
// several tracers are issued before their stores.
__global__ void k_update_tracer(UpdArgs u) {
  const Geo& g = u.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int j = blockIdx.y + 1, k = blockIdx.z;
  if (i > g.ni) return;
  long p = I3(g, i, j, k);
  const double* __restrict__ Tm1 = u.Tm1 + p;
  const double* __restrict__ th = u.th + p;
  double* __restrict__ Tp1 = u.Tp1 + p;
  const long ts = u.tstride, hs = g.n3;
  double a = u.rdz_m1[p], r = u.rdzr[p];
#pragma unroll 5
  for (int n = 0; n < u.ntr; ++n) Tp1[n * ts] = (a * Tm1[n * ts] + u.dtime * th[n * hs]) * r;
}

int make_upd_args(mom5gpu_domain* d, int taum1, int taup1, double dtime, UpdArgs* u) {
  const Geo& g = d->geo;
  int NT = d->dims.num_prog_tracers;
  u->g = g;
  u->ntr = NT;
  u->dtime = dtime;
  u->rdz_m1 = fptr(d, MOM5GPU_RHO_DZT, 0, taum1);
  u->rdzr = fptr(d, MOM5GPU_RHO_DZTR, 0, 0);
  u->Tm1 = fptr(d, MOM5GPU_TRACER, 1, taum1);
  u->Tp1 = fptr(d, MOM5GPU_TRACER, 1, taup1);
  u->th = fptr(d, MOM5GPU_TH_TENDENCY, 1, 0);
  u->tstride = g.n3;
  if (!u->rdz_m1 || !u->rdzr || !u->Tm1 || !u->Tp1 || !u->th)
    return fail(d, MOM5GPU_ESTATE, "update_tracer: a required field was never set");
  return MOM5GPU_OK;
}

int launch_update_tracer(mom5gpu_domain* d, int n_first, int ntr, int taum1, int taup1, double dtime) {
  const Geo& g = d->geo;
  UpdArgs u;
  int rc = make_upd_args(d, taum1, taup1, dtime, &u);
  if (rc) return rc;
  u.ntr = ntr;
  u.Tm1 += (long)(n_first - 1) * g.n3;
  u.Tp1 += (long)(n_first - 1) * g.n3;
  u.th += (long)(n_first - 1) * g.n3;
  ClockScope clk(d, SEC_UPDATE);
  const bool contiguous = u.tstride == g.n3;  // the tracers' levels follow one another: one halo fill
  count_launches(d, 1 + ((g.cx || g.cy) ? (contiguous ? 1 : ntr) : 0));
  dim3 grid((g.ni + 127) / 128, g.nj, g.nk);
  k_update_tracer<<<grid, 128, 0, d->stream>>>(u);
  if (contiguous) launch_halo_fill(g, u.Tp1, ntr * g.nk, 3, d->stream);
  else
    for (int n = 0; n < ntr; ++n) launch_halo_fill(g, u.Tp1 + n * u.tstride, g.nk, 3, d->stream);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "update_tracer");
}

// ---------------------------------------------------------------------------
// compute_tmask_limit (ocean_tracer.F90:2804-2867)
// ---------------------------------------------------------------------------
__global__ void k_tmask_limit(Geo g, const double* tmask, const double* T, double tmin, double tmax, double* tl) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;  // 0..ni (isc-1..iec)
  int j = blockIdx.y;                             // 0..nj
  int k = blockIdx.z;
  if (i > g.ni) return;
  long p = I3(g, i, j, k);
  double v = 0.0;
  auto out = [&](long q) { return tmask[q] == 1.0 && (T[q] < tmin || T[q] > tmax); };
  if (out(p)) v = tmask[p];
  if (out(I3(g, i + 1, j, k))) v = tmask[p];
  if (out(I3(g, i, j + 1, k))) v = tmask[p];
  if (k < g.nk - 1 && out(I3(g, i, j, k + 1))) v = tmask[p];
  tl[p] = v;
}

int launch_tmask_limit(mom5gpu_domain* d, int n, int tau) {
  const Geo& g = d->geo;
  const double* tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  const double* T = fptr(d, MOM5GPU_TRACER, n, tau);
  double* tl = fptr(d, MOM5GPU_TMASK_LIMIT, n, 0);
  if (!tmask || !T || !tl) return fail(d, MOM5GPU_ESTATE, "tmask_limit: a required field was never set");
  dim3 grid((g.ni + 1 + 127) / 128, g.nj + 1, g.nk);
  const TracerScheme& s = d->scheme[n - 1];
  k_tmask_limit<<<grid, 128, 0, d->stream>>>(g, tmask, T, s.min_limit, s.max_limit, tl);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "tmask_limit");
}

__global__ void k_ts_same(Geo g, double* a, double* b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y, k = blockIdx.z;
  if (i > g.ni) return;
  long p = I3(g, i, j, k);
  if (a[p] == 1.0 || b[p] == 1.0) {
    a[p] = 1.0;
    b[p] = 1.0;
  }
}

int launch_tmask_limit_ts_same(mom5gpu_domain* d, int nt, int ns) {
  const Geo& g = d->geo;
  dim3 grid((g.ni + 1 + 127) / 128, g.nj + 1, g.nk);
  k_ts_same<<<grid, 128, 0, d->stream>>>(g, fptr(d, MOM5GPU_TMASK_LIMIT, nt, 0), fptr(d, MOM5GPU_TMASK_LIMIT, ns, 0));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "tmask_limit_ts_same");
}

// ---------------------------------------------------------------------------
// eta_and_pbot_tendency / _update (ocean_barotropic.F90:2683-2690, :2314-2330)
// ---------------------------------------------------------------------------
__global__ void k_eta_tend(long n2, double rho0r, const double* tmask1, const double* conv, const double* pme,
                           const double* river, const double* source, double* deta) {
  long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (q >= n2) return;
  deta[q] = tmask1[q] * rho0r * (conv[q] + pme[q] + river[q] + source[q]);
}

int launch_eta_tendency(mom5gpu_domain* d, int tau) {
  const Geo& g = d->geo;
  const double* tm = fptr(d, MOM5GPU_TMASK, 0, 0);
  const double* conv = fptr(d, MOM5GPU_CONV_RHO_UD_T, 0, tau);
  const double *pme = fptr(d, MOM5GPU_PME, 0, 0), *river = fptr(d, MOM5GPU_RIVER, 0, 0);
  const double* src = fptr(d, MOM5GPU_SOURCE, 0, 0);
  double* deta = fptr(d, MOM5GPU_DETA_DT, 0, 0);
  if (!tm || !conv || !pme || !river || !src || !deta) return fail(d, MOM5GPU_ESTATE, "eta tendency: field never set");
  k_eta_tend<<<(unsigned)((g.n2 + 255) / 256), 256, 0, d->stream>>>(g.n2, 1.0 / d->opt.rho0, tm, conv, pme, river, src,
                                                                    deta);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "eta tendency");
}

__global__ void k_eta_update(Geo g, double dtime, const double* em1, const double* deta, double* ep1) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int j = blockIdx.y + 1;
  if (i > g.ni) return;
  long q = I2(g, i, j);
  ep1[q] = em1[q] + dtime * deta[q];
}

int launch_eta_update(mom5gpu_domain* d, int taum1, int taup1, double dtime) {
  const Geo& g = d->geo;
  const double* em1 = fptr(d, MOM5GPU_ETA_T, 0, taum1);
  double* ep1 = fptr(d, MOM5GPU_ETA_T, 0, taup1);
  const double* deta = fptr(d, MOM5GPU_DETA_DT, 0, 0);
  if (!em1 || !ep1 || !deta) return fail(d, MOM5GPU_ESTATE, "eta update: field never set");
  dim3 grid((g.ni + 127) / 128, g.nj);
  k_eta_update<<<grid, 128, 0, d->stream>>>(g, dtime, em1, deta, ep1);
  launch_halo_fill(g, ep1, 1, 3, d->stream);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "eta update");
}

// ---------------------------------------------------------------------------
// Barotropic predictor-corrector subcycle.
// ---------------------------------------------------------------------------
__global__ void k_bt_post1(long n2, double rntsp1, double rnts, double* eb, double* uu, double* vv) {
  long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (q >= n2) return;
  eb[q] = rntsp1 * eb[q];
  uu[q] = rnts * uu[q];
  vv[q] = rnts * vv[q];
}

__global__ void k_bt_init(BtArgs a, const double* eta_bar_tau, const double* eta_tau, const double* ud_tau,
                          const double* vd_tau, const double* pme, const double* river, const double* source,
                          const double* eta_smooth, int initsum_with_bar) { bt_init_body(a, eta_bar_tau, eta_tau, ud_tau, vd_tau, pme, river, source, eta_smooth, initsum_with_bar, blockIdx.x, blockIdx.y); }
__global__ void k_bt_cgrid_init(BtArgs a) { bt_cgrid_init_body(a, blockIdx.x, blockIdx.y); }
// The B-grid subcycle kernels are launched as programmatic dependents (launch_pdl).
__global__ void k_bt_pred(BtArgs a, int so, int sn, int reuse) {
  pdl_wait();
  pdl_trigger();
  bt_pred_body(a, so, sn, reuse, blockIdx.x, blockIdx.y);
}
__global__ void k_bt_mom_b(BtArgs a, int so, int sn) {
  pdl_wait();
  pdl_trigger();
  bt_mom_b_body(a, so, sn, blockIdx.x, blockIdx.y);
}
__global__ void k_bt_mom_c(BtArgs a, int so, int sn, int itime) { bt_mom_c_body(a, so, sn, itime, blockIdx.x, blockIdx.y); }
__global__ void k_bt_corr(BtArgs a, int so, int sn, double wgt) {
  pdl_wait();
  pdl_trigger();
  bt_corr_body(a, so, sn, wgt, blockIdx.x, blockIdx.y);
}
__global__ void k_bt_corr_pred(BtArgs a, int so, int sn, double wgt) {
  pdl_wait();
  pdl_trigger();
  bt_corr_pred_body(a, so, sn, wgt, blockIdx.x, blockIdx.y);
}
// 32 x 8 tiles of 352 threads: one point per thread in each phase (the 34 x 10
// pressure ring is the largest); 64 x 8 tiles of 256 threads, several points
// per thread, took 1.80 ms per step on 360x300 against 1.41 ms
constexpr int kFusedTX = 32, kFusedTY = 8, kFusedThreads = 352;
__global__ void __launch_bounds__(kFusedThreads) k_bt_fused(BtArgs a, int so, int sn, int reuse, double wgt) {
  pdl_wait();
  pdl_trigger();
  bt_fused_body<kFusedTX, kFusedTY>(a, so, sn, reuse, wgt, blockIdx.x, blockIdx.y);
}
// ---- every exact B-grid subcycle of a step in one cooperative launch ----
//
// A persistent grid of 128-thread blocks, all resident (cooperative launch),
// walks the blocks of the predictor, momentum and corrector launches (virtual
// block vb = bx + nbx*by of their (ni+2)/128 x (nj+2) grid) with the same
// bodies, and a grid barrier stands where a launch boundary stood, so the
// results are those of the three launches bit for bit.  A barrier is an
// arrival counter: thread 0 of each block publishes the block's writes (fence),
// adds one and waits until the counter reaches the barrier's target.  The wait
// is bounded (kGridWaitCycles of the SM clock, about a second) and watches the
// error word: a block that gives up sets bit 1 of it and returns, every other
// block gives up at its barrier too, and mom5gpu_synchronize reports
// MOM5GPU_ETIMEDOUT.
constexpr long long kGridWaitCycles = 1LL << 31;

DEVI unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
DEVI int ld_relaxed_s32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// false when this block or another gave up (the caller returns)
DEVI bool grid_barrier(unsigned* ctr, unsigned target, int* err, long long limit) {
  __shared__ int pass;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(ctr, 1u);
    int ok = 1;
    const long long t0 = clock64();
    while (ld_acquire_u32(ctr) < target) {
      if (ld_relaxed_s32(err) & 2) {
        ok = 0;
        break;
      }
      if (clock64() - t0 > limit) {
        atomicOr(err, 2);
        ok = 0;
        break;
      }
    }
    __threadfence();
    pass = ok;
  }
  __syncthreads();
  return pass != 0;
}

__global__ void __launch_bounds__(128) k_bt_coop(BtArgs a, unsigned* ctr, int* err) {
  const Geo& g = a.g;
  const int nbx = (g.ni + 2 + 127) / 128, nvb = nbx * (g.nj + 2);
  const unsigned per = gridDim.x;
  unsigned target = 0;
  for (int itime = 1; itime <= a.nts; ++itime) {
    const int so = itime % 2, sn = (itime + 1) % 2;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) bt_pred_body(a, so, sn, itime > 1, vb % nbx, vb / nbx);
    if (!grid_barrier(ctr, target += per, err, kGridWaitCycles)) return;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) bt_mom_b_body(a, so, sn, vb % nbx, vb / nbx);
    if (!grid_barrier(ctr, target += per, err, kGridWaitCycles)) return;
    const double wgt = (double)(a.nts - itime + 1);
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) bt_corr_body(a, so, sn, wgt, vb % nbx, vb / nbx);
    if (itime < a.nts && !grid_barrier(ctr, target += per, err, kGridWaitCycles)) return;
  }
}

// Barrier self-test: `rounds` barriers over a full resident grid; after each,
// every block checks that every block has written the round's number (or the
// next one's).  With extra > 0 the target counts more arrivals than the grid
// has blocks, so every wait runs out after `limit` cycles.
__global__ void __launch_bounds__(128) k_grid_barrier_check(unsigned* ctr, int* err, int* slots, int rounds,
                                                            unsigned extra, long long limit, int* bad) {
  unsigned target = 0;
  for (int r = 1; r <= rounds; ++r) {
    if (threadIdx.x == 0) slots[blockIdx.x] = r;
    target += gridDim.x + extra;
    if (!grid_barrier(ctr, target, err, limit)) return;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
      const int v = ((volatile int*)slots)[b];
      if (v < r || v > r + 1) atomicOr(bad, 1);
    }
  }
}

// Resident blocks per SM of a cooperative kernel (-1: no cooperative launch).
static int coop_resident(mom5gpu_domain* d, const void* kernel) {
  int dev = 0, coop = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!d->coop_sms) cudaDeviceGetAttribute(&d->coop_sms, cudaDevAttrMultiProcessorCount, dev);
  if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 128, 0) != cudaSuccess) per = 0;
  cudaGetLastError();
  return (coop && per > 0 && d->coop_sms > 0) ? per : -1;
}

// Every SM gets the same number of blocks, no more than the walk has blocks of
// work for and no more than can be resident.
static int launch_bt_coop(mom5gpu_domain* d, const BtArgs& a, cudaStream_t s) {
  int rc = ensure_wait_words(d);
  if (rc) return rc;
  if (!d->coop_blocks) d->coop_blocks = coop_resident(d, (const void*)k_bt_coop);
  if (d->coop_blocks < 0) return MOM5GPU_EUNSUPPORTED;
  const Geo& g = a.g;
  const int nvb = ((g.ni + 2 + 127) / 128) * (g.nj + 2);
  int bps = (nvb + d->coop_sms - 1) / d->coop_sms;
  if (bps > d->coop_blocks) bps = d->coop_blocks;
  cudaMemsetAsync(d->bt_sync, 0, sizeof(unsigned), s);
  BtArgs av = a;
  unsigned* ctr = d->bt_sync;
  int* err = d->wait_err;
  void* args[] = {&av, &ctr, &err};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_bt_coop, dim3(d->coop_sms * bps), dim3(128), args, 0, s);
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "barotropic subcycles (cooperative launch)");
}

// Form of the exact B-grid subcycles: 0 three launches each (replayed from a
// CUDA graph; the default), 1 one launch each (k_bt_fused, the ring
// recomputed), 2 all of a step in one cooperative launch (k_bt_coop).  Measured
// on GB300 both alternatives are slower on every domain tried: the one-launch
// form adds about 11% FP64 work for its ring to a loop bound by the FP64 pipe;
// the cooperative launch holds 7 blocks of 72 registers per SM (28 warps)
// against the three kernels' 16 blocks of 30-32 registers (64 warps), which
// hide the FP64 latency better, and a grid barrier across about a thousand
// blocks costs as much as a launch gap of the graph replay.
static int bt_form(const mom5gpu_domain* d, const BtArgs& a) {
  if (a.cgrid) return 0;
  if (a.btf) return d->bt_fused == 1 ? 1 : 0;  // the precision form has no cooperative form
  return d->bt_fused;
}
static bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return cs != cudaStreamCaptureStatusNone;
}

int grid_barrier_selftest(mom5gpu_domain* d, int rounds, int unreachable) {
  int rc = ensure_wait_words(d);
  if (rc) return rc;
  const int per = coop_resident(d, (const void*)k_grid_barrier_check);
  if (per < 0) return MOM5GPU_EUNSUPPORTED;
  const int nb = per * d->coop_sms;
  int* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, sizeof(int) * (nb + 1));
  if (e != cudaSuccess) return cuda_fail(d, e, "grid barrier self-test");
  cudaStream_t s = d->stream;
  cudaMemsetAsync(buf, 0, sizeof(int) * (nb + 1), s);
  cudaMemsetAsync(d->bt_sync, 0, sizeof(unsigned), s);
  unsigned* ctr = d->bt_sync;
  int* err = d->wait_err;
  int* slots = buf;
  int* bad = buf + nb;
  unsigned extra = unreachable ? 1u : 0u;
  long long limit = unreachable ? (1LL << 24) : kGridWaitCycles;  // about 8 ms when every wait must run out
  void* args[] = {&ctr, &err, &slots, &rounds, &extra, &limit, &bad};
  e = cudaLaunchCooperativeKernel((const void*)k_grid_barrier_check, dim3(nb), dim3(128), args, 0, s);
  int hbad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(d, e, "grid barrier self-test");
  if (hbad) return fail(d, MOM5GPU_ENUMERIC, "grid barrier self-test: a block passed a barrier early");
  return MOM5GPU_OK;
}

__global__ void k_bt_post2(BtArgs a, double* conv, double* eta_u, double* ps_out) { bt_post2_body(a, conv, eta_u, ps_out, blockIdx.x, blockIdx.y); }
__global__ void k_bt_post3(BtArgs a, const double* ps, double* gxo, double* gyo) { bt_post3_body(a, ps, gxo, gyo, blockIdx.x, blockIdx.y); }

int make_bt_args(mom5gpu_domain* d, int tau, int taup1, BtArgs* ap, BtExtra* xp) {
  const Geo& g = d->geo;
  if (!d->baro_ready) return fail(d, MOM5GPU_ESTATE, "update_ocean_barotropic before mom5gpu_barotropic_init");
  BtArgs& a = *ap;
  BtExtra& x = *xp;
  memset(&a, 0, sizeof(BtArgs));  // padding too: the bytes key the subcycle graph
  a.g = g;
  a.cgrid = d->dims.horz_grid == MOM5GPU_CGRID;
  a.nts = d->nts;
  a.stepB = d->opt.barotropic_time_stepping_B;
  a.dtbt = d->dtbt;
  double rho0r = 1.0 / d->opt.rho0;
  a.gamma = d->opt.pred_corr_gamma;
  a.dtbt_gamma_rho0r = d->dtbt * d->opt.pred_corr_gamma * rho0r;
  a.dtbt_rho0r = d->dtbt * rho0r;
  a.tmask1 = fptr(d, MOM5GPU_TMASK, 0, 0);  // level 1 is the first plane
  a.umask1 = fptr(d, MOM5GPU_UMASK1, 0, 0);
  a.f = fptr(d, MOM5GPU_CORIOLIS_F, 0, 0);
  a.dxu = fptr(d, MOM5GPU_DXU, 0, 0);
  a.dyu = fptr(d, MOM5GPU_DYU, 0, 0);
  a.dxur = fptr(d, MOM5GPU_DXUR, 0, 0);
  a.dyur = fptr(d, MOM5GPU_DYUR, 0, 0);
  a.dat = fptr(d, MOM5GPU_DAT, 0, 0);
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.dxter = fptr(d, MOM5GPU_DXTER, 0, 0);
  a.dytnr = fptr(d, MOM5GPU_DYTNR, 0, 0);
  a.tmen_e = fptr(d, MOM5GPU_TMASKEN_E1, 0, 0);
  a.tmen_n = fptr(d, MOM5GPU_TMASKEN_N1, 0, 0);
  a.dte = fptr(d, MOM5GPU_DTE, 0, 0);
  a.dtw = fptr(d, MOM5GPU_DTW, 0, 0);
  a.dus = fptr(d, MOM5GPU_DUS, 0, 0);
  a.dun = fptr(d, MOM5GPU_DUN, 0, 0);
  a.daur = fptr(d, MOM5GPU_DAUR, 0, 0);
  a.patm = fptr(d, MOM5GPU_PATM, 0, 0);
  a.thicku = fptr(d, MOM5GPU_THICKU, 0, tau);
  a.thicken_e = fptr(d, MOM5GPU_THICKEN_E, 0, 0);
  a.thicken_n = fptr(d, MOM5GPU_THICKEN_N, 0, 0);
  a.forcing_u = fptr(d, MOM5GPU_FORCING_BT_U, 0, 0);
  a.forcing_v = fptr(d, MOM5GPU_FORCING_BT_V, 0, 0);
  a.rho_g = fptr(d, MOM5GPU_RHO_G, 0, 0);
  a.cori1 = d->cori1;
  a.cori2 = d->cori2;
  long n2 = g.n2;
  a.eta_bt = d->bt;
  a.ubt = d->bt + 2 * n2;
  a.vbt = d->bt + 4 * n2;
  a.steady = d->bt + 6 * n2;
  a.ps = d->bt + 7 * n2;
  a.cf = d->bt + 8 * n2;
  a.ca = d->bt + 14 * n2;
  a.uhb = a.cgrid ? nullptr : d->bt + 8 * n2;
  a.dvs = d->bt + 16 * n2;
  a.vhb = a.cgrid ? nullptr : d->bt + 10 * n2;
  a.btf = (!a.cgrid && d->opt.precision == MOM5GPU_PRECISION_MIXED) ? d->bt + kBtPlanes * n2 : nullptr;
  a.eta_bar = fptr(d, MOM5GPU_ETA_T_BAR, 0, taup1);
  a.udrho_u = fptr(d, MOM5GPU_UDRHO_U, 0, taup1);
  a.udrho_v = fptr(d, MOM5GPU_UDRHO_V, 0, taup1);
  x.eta_bar_tau = fptr(d, MOM5GPU_ETA_T_BAR, 0, tau);
  x.eta_tau = fptr(d, MOM5GPU_ETA_T, 0, tau);
  x.ud_tau = fptr(d, MOM5GPU_UDRHO_U, 0, tau);
  x.vd_tau = fptr(d, MOM5GPU_UDRHO_V, 0, tau);
  x.pme = fptr(d, MOM5GPU_PME, 0, 0);
  x.river = fptr(d, MOM5GPU_RIVER, 0, 0);
  x.source = fptr(d, MOM5GPU_SOURCE, 0, 0);
  x.eta_smooth = fptr(d, MOM5GPU_ETA_SMOOTH, 0, 0);
  x.conv = fptr(d, MOM5GPU_CONV_RHO_UD_T, 0, taup1);
  x.eta_u = fptr(d, MOM5GPU_ETA_U, 0, taup1);
  x.ps_out = fptr(d, MOM5GPU_PS, 0, 0);
  x.gxo = fptr(d, MOM5GPU_GRAD_PS_X, 0, 0);
  x.gyo = fptr(d, MOM5GPU_GRAD_PS_Y, 0, 0);
  x.initsum_with_bar = d->opt.initsum_with_bar;
  const void* need[] = {a.tmask1, a.umask1, a.f, a.dxu, a.dyu, a.dxur, a.dyur, a.dat, a.datr, a.patm, a.thicku,
                        a.forcing_u, a.forcing_v, a.rho_g, a.eta_bar, a.udrho_u, a.udrho_v, x.eta_bar_tau, x.eta_tau,
                        x.ud_tau, x.vd_tau, x.pme, x.river, x.source, x.eta_smooth, x.conv, x.eta_u, x.ps_out, x.gxo,
                        x.gyo, a.dte, a.dtw, a.dus, a.dun, a.daur};
  for (const void* p : need)
    if (!p) return fail(d, MOM5GPU_ESTATE, "update_ocean_barotropic: a required field was never set");
  if (a.cgrid && (!a.dxter || !a.dytnr || !a.tmen_e || !a.tmen_n || !a.thicken_e || !a.thicken_n))
    return fail(d, MOM5GPU_ESTATE, "C-grid barotropic: a required field was never set");
  return MOM5GPU_OK;
}

// Replays the domain's graph of the subcycle loop captured with the same BtArgs
// bytes, else captures enqueue(stream) into a new graph (kept with the last few:
// the time levels rotate) and launches it.  Returns false (nothing enqueued)
// when the stream cannot be captured; the caller then launches directly.
constexpr size_t kBtGraphs = 6;
template <class F>
bool replay_subcycle_graph(mom5gpu_domain* d, const BtArgs& a, F&& enqueue) {
  // inside a capture the caller runs (its own graph), launch directly
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(d->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return false;
  }
  const unsigned char* key = reinterpret_cast<const unsigned char*>(&a);
  for (auto& gr : d->bt_graphs)
    if (gr.exec && gr.key.size() == sizeof(BtArgs) && memcmp(gr.key.data(), key, sizeof(BtArgs)) == 0)
      return cudaGraphLaunch(gr.exec, d->stream) == cudaSuccess;
  if (cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  enqueue(d->stream);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaStreamEndCapture(d->stream, &graph);
  if (e == cudaSuccess && graph) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess || !exec) {
    cudaGetLastError();
    return false;
  }
  if (d->bt_graphs.size() >= kBtGraphs) {
    cudaGraphExecDestroy(d->bt_graphs.front().exec);
    d->bt_graphs.erase(d->bt_graphs.begin());
  }
  d->bt_graphs.push_back({exec, std::vector<unsigned char>(key, key + sizeof(BtArgs))});
  return cudaGraphLaunch(exec, d->stream) == cudaSuccess;
}

int launch_barotropic(mom5gpu_domain* d, int tau, int taup1) {
  const Geo& g = d->geo;
  BtArgs a;
  BtExtra x;
  int rc = make_bt_args(d, tau, taup1, &a, &x);
  if (rc) return rc;
  long n2 = g.n2;
  const double *eta_bar_tau = x.eta_bar_tau, *eta_tau = x.eta_tau, *ud_tau = x.ud_tau, *vd_tau = x.vd_tau;
  const double *pme = x.pme, *river = x.river, *src = x.source, *esm = x.eta_smooth;
  double *conv = x.conv, *eta_u = x.eta_u, *ps_out = x.ps_out, *gxo = x.gxo, *gyo = x.gyo;
  cudaStream_t s = d->stream;
  ClockScope clk(d, SEC_BAROTROPIC);
  int halo = (g.cx || g.cy) ? 1 : 0;
  const int form = bt_form(d, a);
  const bool coop = form == 2 && !capturing(s);
  const bool fused = form == 1;
  const long sub_launches = coop      ? 1
                            : fused   ? (long)a.nts
                            : a.cgrid ? (long)a.nts * (3 + 2 * halo)
                                      : 1 + 2L * a.nts;
  count_launches(d, 1 + (a.cgrid ? 1 : 0) + (a.btf ? 1 : 0) + sub_launches + 4 + 5 * halo);
  k_bt_init<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(a, eta_bar_tau, eta_tau, ud_tau, vd_tau, pme, river, src,
                                                          esm, d->opt.initsum_with_bar);
  dim3 g2((g.ni + 2 + 127) / 128, g.nj + 2);
  if (a.cgrid) {
    cudaMemsetAsync(a.cf, 0, sizeof(double) * 8 * n2, s);
    dim3 gc((g.ni + 127) / 128, g.nj);
    k_bt_cgrid_init<<<gc, 128, 0, s>>>(a);
  }
  if (a.btf) launch_btf_prep(a, s);
  // the nts subcycles (3 to 5 launches each, all arguments in a): one CUDA graph,
  // captured on first use and replayed while a is unchanged
  const dim3 gf((g.ni + 2 + kFusedTX - 1) / kFusedTX, (g.nj + 2 + kFusedTY - 1) / kFusedTY);
  auto subcycles = [&](cudaStream_t st) {
    for (int itime = 1; itime <= a.nts; ++itime) {
      int so = (itime + 0) % 2, sn = (itime + 1) % 2;
      if (a.btf) {  // precision form: FP32 increments
        launch_btf_subcycle(a, itime, a.nts, fused, st);
        continue;
      }
      if (fused) {  // predictor, momentum and corrector in one launch
        launch_pdl(k_bt_fused, gf, dim3(kFusedThreads), st, a, so, sn, (int)(itime > 1), (double)(a.nts - itime + 1));
        continue;
      }
      if (!a.cgrid) {
        // B grid: the predictor as a launch of its own only in the first
        // subcycle; every corrector but the last forms the next predictor
        const double wgt = (double)(a.nts - itime + 1);
        if (itime == 1) launch_pdl(k_bt_pred, g2, dim3(128), st, a, so, sn, 0);
        launch_pdl(k_bt_mom_b, g2, dim3(128), st, a, so, sn);
        if (itime < a.nts) launch_pdl(k_bt_corr_pred, g2, dim3(128), st, a, so, sn, wgt);
        else launch_pdl(k_bt_corr, g2, dim3(128), st, a, so, sn, wgt);
        continue;
      }
      k_bt_pred<<<g2, 128, 0, st>>>(a, so, sn, itime > 1);
      k_bt_mom_c<<<g2, 128, 0, st>>>(a, so, sn, itime);
      launch_halo_fill(g, a.ubt + sn * n2, 1, 3, st);
      launch_halo_fill(g, a.vbt + sn * n2, 1, 3, st);
      k_bt_corr<<<g2, 128, 0, st>>>(a, so, sn, (double)(a.nts - itime + 1));
    }
  };
  int crc = coop ? launch_bt_coop(d, a, s) : MOM5GPU_EUNSUPPORTED;
  if (crc != MOM5GPU_OK && crc != MOM5GPU_EUNSUPPORTED) return crc;
  if (crc == MOM5GPU_EUNSUPPORTED && !replay_subcycle_graph(d, a, subcycles)) subcycles(s);
  double rntsp1 = 1.0 / ((double)a.nts + 1.0);
  double rnts = a.stepB ? 2.0 / ((double)a.nts * (double)(a.nts + 1)) : 1.0 / (double)a.nts;
  k_bt_post1<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(n2, rntsp1, rnts, a.eta_bar, a.udrho_u, a.udrho_v);
  launch_halo_fill(g, a.eta_bar, 1, 3, s);
  launch_halo_fill(g, a.udrho_u, 1, 3, s);
  launch_halo_fill(g, a.udrho_v, 1, 3, s);
  k_bt_post2<<<g2, 128, 0, s>>>(a, conv, eta_u, ps_out);
  launch_halo_fill(g, conv, 1, 3, s);
  launch_halo_fill(g, eta_u, 1, 3, s);
  k_bt_post3<<<g2, 128, 0, s>>>(a, ps_out, gxo, gyo);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "barotropic");
}

// One phase of launch_barotropic for a decomposed block (B grid, FP64): the
// same kernels in the same order, with the single-PE halo fills left to the
// caller's exchanges (a block is created non-cyclic).
int launch_barotropic_phase(mom5gpu_domain* d, int tau, int taup1, int phase, int itime) {
  const Geo& g = d->geo;
  BtArgs a;
  BtExtra x;
  int rc = make_bt_args(d, tau, taup1, &a, &x);
  if (rc) return rc;
  if (a.cgrid || a.btf) return fail(d, MOM5GPU_EUNSUPPORTED, "decomposed barotropic: B grid, FP64 only");
  if (phase < 0 || phase > 5) return fail(d, MOM5GPU_EINVAL, "barotropic phase %d (0..5)", phase);
  if ((phase == 1 || phase == 2) && (itime < 1 || itime > a.nts))
    return fail(d, MOM5GPU_EINVAL, "barotropic subcycle %d (1..%d)", itime, a.nts);
  long n2 = g.n2;
  cudaStream_t s = d->stream;
  dim3 g2((g.ni + 2 + 127) / 128, g.nj + 2);
  int so = (itime + 0) % 2, sn = (itime + 1) % 2;
  switch (phase) {
    case 0:
      k_bt_init<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(a, x.eta_bar_tau, x.eta_tau, x.ud_tau, x.vd_tau, x.pme,
                                                              x.river, x.source, x.eta_smooth,
                                                              d->opt.initsum_with_bar);
      count_launches(d, 1);
      break;
    case 1:
      k_bt_pred<<<g2, 128, 0, s>>>(a, so, sn, itime > 1);
      count_launches(d, 1);
      break;
    case 2:
      k_bt_mom_b<<<g2, 128, 0, s>>>(a, so, sn);
      k_bt_corr<<<g2, 128, 0, s>>>(a, so, sn, (double)(a.nts - itime + 1));
      count_launches(d, 2);
      break;
    case 3: {
      double rntsp1 = 1.0 / ((double)a.nts + 1.0);
      double rnts = a.stepB ? 2.0 / ((double)a.nts * (double)(a.nts + 1)) : 1.0 / (double)a.nts;
      k_bt_post1<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(n2, rntsp1, rnts, a.eta_bar, a.udrho_u, a.udrho_v);
      count_launches(d, 1);
      break;
    }
    case 4:
      k_bt_post2<<<g2, 128, 0, s>>>(a, x.conv, x.eta_u, x.ps_out);
      count_launches(d, 1);
      break;
    default:
      k_bt_post3<<<g2, 128, 0, s>>>(a, x.ps_out, x.gxo, x.gyo);
      count_launches(d, 1);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "barotropic phase");
}

// ---------------------------------------------------------------------------
// ocean_advection_velocity, T-cell part (ocean_advection_velocity.F90:568-672)
// ---------------------------------------------------------------------------
struct AdvVelArgs {
  Geo g;
  int cgrid;
  const double *u, *v, *rdzu, *rdzten_e, *rdzten_n, *dxu, *dyu, *dyte, *dxtn, *dxt_dxter, *dyt_dyter, *dxt_dxtnr,
      *dyt_dytnr, *datr, *tmask, *tend, *msrc, *pme, *river;
  double *ue, *vn, *div, *w;
};

// face fluxes at every data-domain point: B grid BAY/BAX (ocean_operators.F90:834-902,
// zero on the first row / column) divided by the face length; C grid products (:645-654)
__global__ void k_adv_vel_faces(AdvVelArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j), p = I3(g, i, j, k);
  if (!a.cgrid) {
    double bay = 0.0, bax = 0.0;
    if (j >= 1) {
      long qs = q - g.nxd, ps = p - g.nxd;
      bay = half_exact(a.u[p] * a.dyu[q] * a.rdzu[p] + a.u[ps] * a.dyu[qs] * a.rdzu[ps]);
    }
    if (i >= 1) bax = half_exact(a.v[p] * a.dxu[q] * a.rdzu[p] + a.v[p - 1] * a.dxu[q - 1] * a.rdzu[p - 1]);
    a.ue[p] = div_seeded(bay, a.dyte[q]);
    a.vn[p] = div_seeded(bax, a.dxtn[q]);
  } else {
    a.ue[p] = a.u[p] * a.rdzten_e[p] * a.dxt_dxter[q] * a.dyt_dyter[q];
    a.vn[p] = a.v[p] * a.rdzten_n[p] * a.dxt_dxtnr[q] * a.dyt_dytnr[q];
  }
}

// diverge_t = tmask*(BDX_ET + BDY_NT) (ocean_operators.F90:945-958, :1230-1243) and the
// continuity sum down each column (ocean_advection_velocity.F90:609-625)
__global__ void k_adv_vel_w(AdvVelArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double w = -(a.pme[q] + a.river[q]);
  a.w[q] = w;
  double datr = a.datr[q], dyte = a.dyte[q], dxtn = a.dxtn[q];
  for (int k = 0; k < g.nk; ++k) {
    long p = I3(g, i, j, k);
    double bdx = i >= 1 ? (dyte * a.ue[p] - a.dyte[q - 1] * a.ue[p - 1]) * datr : 0.0;
    double bdy = j >= 1 ? (dxtn * a.vn[p] - a.dxtn[q - g.nxd] * a.vn[p - g.nxd]) * datr : 0.0;
    double tm = a.tmask[p];
    double div = tm * (bdx + bdy);
    a.div[p] = div;
    double tmp = a.tend[p] - a.msrc[p];
    w = (tmp + div + w) * tm;
    a.w[(long)(k + 1) * g.n2 + q] = w;
  }
}

int launch_advection_velocity(mom5gpu_domain* d, int tau) {
  const Geo& g = d->geo;
  AdvVelArgs a;
  a.g = g;
  a.cgrid = d->dims.horz_grid == MOM5GPU_CGRID;
  a.u = fptr(d, MOM5GPU_U_VEL, 0, tau);
  a.v = fptr(d, MOM5GPU_V_VEL, 0, tau);
  a.rdzu = a.cgrid ? nullptr : fptr(d, MOM5GPU_RHO_DZU, 0, tau);
  a.rdzten_e = a.cgrid ? fptr(d, MOM5GPU_RHO_DZTEN_E, 0, 0) : nullptr;
  a.rdzten_n = a.cgrid ? fptr(d, MOM5GPU_RHO_DZTEN_N, 0, 0) : nullptr;
  a.dxu = fptr(d, MOM5GPU_DXU, 0, 0);
  a.dyu = fptr(d, MOM5GPU_DYU, 0, 0);
  a.dyte = fptr(d, MOM5GPU_DYTE, 0, 0);
  a.dxtn = fptr(d, MOM5GPU_DXTN, 0, 0);
  a.dxt_dxter = a.cgrid ? fptr(d, MOM5GPU_DXT_DXTER, 0, 0) : nullptr;
  a.dyt_dyter = a.cgrid ? fptr(d, MOM5GPU_DYT_DYTER, 0, 0) : nullptr;
  a.dxt_dxtnr = a.cgrid ? fptr(d, MOM5GPU_DXT_DXTNR, 0, 0) : nullptr;
  a.dyt_dytnr = a.cgrid ? fptr(d, MOM5GPU_DYT_DYTNR, 0, 0) : nullptr;
  a.datr = fptr(d, MOM5GPU_DATR, 0, 0);
  a.tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  a.tend = fptr(d, MOM5GPU_RHO_DZT_TENDENCY, 0, 0);
  a.msrc = fptr(d, MOM5GPU_MASS_SOURCE, 0, 0);
  a.pme = fptr(d, MOM5GPU_PME, 0, 0);
  a.river = fptr(d, MOM5GPU_RIVER, 0, 0);
  a.ue = fptr(d, MOM5GPU_UHRHO_ET, 0, 0);
  a.vn = fptr(d, MOM5GPU_VHRHO_NT, 0, 0);
  a.div = fptr(d, MOM5GPU_DIVERGE_T, 0, 0);
  a.w = fptr(d, MOM5GPU_WRHO_BT, 0, 0);
  const void* need[] = {a.u, a.v, a.dxu, a.dyu, a.dyte, a.dxtn, a.datr, a.tmask, a.tend, a.msrc, a.pme, a.river,
                        a.ue, a.vn, a.div, a.w};
  for (const void* p : need)
    if (!p) return fail(d, MOM5GPU_ESTATE, "ocean_advection_velocity: a field could not be allocated");
  if (a.cgrid ? !(a.rdzten_e && a.rdzten_n && a.dxt_dxter && a.dyt_dyter && a.dxt_dxtnr && a.dyt_dytnr) : !a.rdzu)
    return fail(d, MOM5GPU_ESTATE, "ocean_advection_velocity: a thickness or metric field could not be allocated");
  count_launches(d, 2);
  dim3 g3((g.ni + 2 + 127) / 128, g.nj + 2, g.nk);
  k_adv_vel_faces<<<g3, 128, 0, d->stream>>>(a);
  dim3 g2((g.ni + 2 + 127) / 128, g.nj + 2);
  k_adv_vel_w<<<g2, 128, 0, d->stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "ocean_advection_velocity");
}

// ---------------------------------------------------------------------------
// surface and bottom source terms of the explicit tracer step (ocean_tracer.F90:2318-2336)
// ---------------------------------------------------------------------------
__global__ void k_tracer_boundary(Geo g, const double* tmask, const int* kmt, const double* pme, const double* tpme,
                                  const double* esm, const double* pbs, double* th) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1;
  if (i > g.ni) return;
  long q = I2(g, i, j);
  th[q] = th[q] + tmask[q] * (pme[q] * tpme[q] + esm[q]);
  int kbot = kmt[q];
  if (kbot > 0) {
    long p = (long)(kbot - 1) * g.n2 + q;
    th[p] = th[p] + tmask[p] * pbs[q];
  }
}

int launch_tracer_boundary(mom5gpu_domain* d, int n) {
  const Geo& g = d->geo;
  int krc = ensure_kmt_device(d);
  if (krc) return krc;
  const double* tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  const double* pme = fptr(d, MOM5GPU_PME, 0, 0);
  const double* tpme = fptr(d, MOM5GPU_TPME, n, 0);
  const double* esm = fptr(d, MOM5GPU_TRACER_ETA_SMOOTH, n, 0);
  const double* pbs = fptr(d, MOM5GPU_PBOT_SMOOTH, n, 0);
  double* th = fptr(d, MOM5GPU_TH_TENDENCY, n, 0);
  if (!tmask || !pme || !tpme || !esm || !pbs || !th)
    return fail(d, MOM5GPU_ESTATE, "tracer_boundary_terms: a field could not be allocated");
  count_launches(d, 1);
  dim3 grid((g.ni + 127) / 128, g.nj);
  k_tracer_boundary<<<grid, 128, 0, d->stream>>>(g, tmask, d->kmt_d, pme, tpme, esm, pbs, th);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "tracer_boundary_terms");
}

// ---------------------------------------------------------------------------
// ocean_barotropic_forcing (ocean_barotropic.F90:3058-3141)
// ---------------------------------------------------------------------------
__global__ void k_baro_forcing(Geo g, const double* tmen, const double* accel, const double* smf, const double* bmf,
                               int nonlinear, double* f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double v = 0.0;  // forcing_bt = 0.0 on the data domain
  if (i >= 1 && i <= g.ni && j >= 1 && j <= g.nj) {
    double w = 0.0;
    if (nonlinear)
      for (int k = 0; k < g.nk; ++k) w = w + tmen[(long)k * g.n2 + q] * accel[(long)k * g.n2 + q];
    v = w + tmen[q] * (smf[q] - bmf[q]);
  }
  f[q] = v;
}

// forcing_bt + friction_lap + friction_bih with both frictions 0.0 (:3109-3117)
__global__ void k_plus_zero_2d(long n2, double* f) {
  long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (q < n2) f[q] = plus_zero(plus_zero(f[q]));
}

// forcing_bt + friction_lap + friction_bih on the data domain (:3114-3120); a
// null friction is the reference's 0.0
__global__ void k_plus_friction_2d(long n2, double* f, const double* lap, const double* bih) {
  long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (q >= n2) return;
  double v = f[q] + (lap ? lap[q] : 0.0);
  f[q] = v + (bih ? bih[q] : 0.0);
}

// Background viscosities of the barotropic friction (ocean_barotropic.F90:1306-1335):
// smooth_lap_udrho = umask*vel_lap*(2*dxu*dyu/(dxu+dyu)) and smooth_bih_udrho =
// umask*vel_bih*(...)**3 (x**3 as (x*x)*x), averaged onto the east and north
// faces on the compute domain; zero on the halo, which the caller then updates.
struct FricBack {
  const double *dxu, *dyu, *umask;
  double vel_lap, vel_bih;
  double *lap_e, *lap_n, *bih_e, *bih_n;
};
DEVI void smooth_udrho(const FricBack& a, long q, double& sl, double& sb) {
  double x = 2.0 * a.dxu[q] * a.dyu[q] / (a.dxu[q] + a.dyu[q]);
  double um = a.umask[q];
  sl = um * a.vel_lap * x;
  sb = um * a.vel_bih * (x * x * x);
}
__global__ void k_bt_fric_back(Geo g, FricBack a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double le = 0.0, ln = 0.0, be = 0.0, bn = 0.0;
  if (i >= 1 && i <= g.ni && j >= 1 && j <= g.nj) {
    double sl, sb, sle, sbe, sln, sbn;
    smooth_udrho(a, q, sl, sb);
    smooth_udrho(a, I2(g, i + 1, j), sle, sbe);
    smooth_udrho(a, I2(g, i, j + 1), sln, sbn);
    le = 0.5 * (sl + sle);
    ln = 0.5 * (sl + sln);
    be = 0.5 * (sb + sbe);
    bn = 0.5 * (sb + sbn);
  }
  a.lap_e[q] = le;
  a.lap_n[q] = ln;
  a.bih_e[q] = be;
  a.bih_n[q] = bn;
}
// bih_ceu_back = sqrt(bih_ceu_back) over the data domain after its halo update (:1340-1341)
__global__ void k_sqrt_2d(long n2, double* a, double* b) {
  long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (q >= n2) return;
  a[q] = sqrt(a[q]);
  b[q] = sqrt(b[q]);
}

// One application of the barotropic friction operator on the compute domain
// (lap_friction_barotropic, ocean_lap_friction.F90:433-440; each iteration of
// bih_friction_barotropic, ocean_bih_friction.F90:428-448):
//   tmp = BDX_EU((ce_back + ce_visc)*FDX_U(a)) + BDY_NU((cn_back + cn_visc)*FDY_U(a))
// with FDX_U(a)(i) = (a(i+1)-a(i))*dxuer(i), BDX_EU(X)(i) = (dyue(i)*X(i) -
// dyue(i-1)*X(i-1))*daur(i), FDY_U, BDY_NU likewise with dyunr and dxun
// (ocean_operators.F90:917-930, :973-986, :1202-1215, :1258-1271); out = tmp*umask,
// or (-tmp)*umask for the second biharmonic iteration.  Zero on the halo, which
// the caller then updates (the reference's arrays start at 0.0 and only their
// compute domain is written).
struct FricOp {
  const double *dyue, *dxuer, *dxun, *dyunr, *daur, *umask;
  const double *ce_back, *ce_visc, *cn_back, *cn_visc;
};
__global__ void k_bt_fric_op(Geo g, FricOp m, const double* a, int negate, double* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double v = 0.0;
  if (i >= 1 && i <= g.ni && j >= 1 && j <= g.nj) {
    const long qw = I2(g, i - 1, j), qe = I2(g, i + 1, j), qs = I2(g, i, j - 1), qn = I2(g, i, j + 1);
    double fx = (a[qe] - a[q]) * m.dxuer[q];
    double fxw = (a[q] - a[qw]) * m.dxuer[qw];
    double xe = (m.ce_back[q] + m.ce_visc[q]) * fx;
    double xw = (m.ce_back[qw] + m.ce_visc[qw]) * fxw;
    double bdx = (m.dyue[q] * xe - m.dyue[qw] * xw) * m.daur[q];
    double fy = (a[qn] - a[q]) * m.dyunr[q];
    double fys = (a[q] - a[qs]) * m.dyunr[qs];
    double yn = (m.cn_back[q] + m.cn_visc[q]) * fy;
    double ys = (m.cn_back[qs] + m.cn_visc[qs]) * fys;
    double bdy = (m.dxun[q] * yn - m.dxun[qs] * ys) * m.daur[q];
    double tmp = bdx + bdy;
    v = (negate ? -tmp : tmp) * m.umask[q];
  }
  out[q] = v;
}

// The barotropic friction of one velocity component a = udrho(:,:,n,tau) into
// lap (udrho_lap) and bih (udrho_bih; del2 is ocean_bih_friction's del2_vel),
// each with its halo update; a friction that is off is zeroed.
static void launch_bt_friction(const mom5gpu_domain* d, const FricOp& lap_op, const FricOp& bih_op, const double* a,
                               double* lap, double* bih, double* del2, cudaStream_t s) {
  const Geo& g = d->geo;
  dim3 g2((g.ni + 2 + 127) / 128, g.nj + 2);
  if (d->opt.udrho_lap) {
    k_bt_fric_op<<<g2, 128, 0, s>>>(g, lap_op, a, 0, lap);
    launch_halo_fill(g, lap, 1, 3, s);
  } else {
    cudaMemsetAsync(lap, 0, sizeof(double) * g.n2, s);
  }
  if (d->opt.udrho_bih) {
    k_bt_fric_op<<<g2, 128, 0, s>>>(g, bih_op, a, 0, del2);
    launch_halo_fill(g, del2, 1, 3, s);
    k_bt_fric_op<<<g2, 128, 0, s>>>(g, bih_op, del2, 1, bih);
    launch_halo_fill(g, bih, 1, 3, s);
  } else {
    cudaMemsetAsync(bih, 0, sizeof(double) * g.n2, s);
  }
}

int launch_barotropic_forcing(mom5gpu_domain* d, int tau) {
  const Geo& g = d->geo;
  double* fu = fptr(d, MOM5GPU_FORCING_BT_U, 0, 0);
  double* fv = fptr(d, MOM5GPU_FORCING_BT_V, 0, 0);
  if (!fu || !fv) return fail(d, MOM5GPU_ESTATE, "ocean_barotropic_forcing: a field could not be allocated");
  cudaStream_t s = d->stream;
  const bool friction = tau > 0;
  const bool halo = g.cx || g.cy;
  dim3 g2((g.ni + 2 + 127) / 128, g.nj + 2);
  unsigned nb = (unsigned)((g.n2 + 255) / 256);
  double *lap_u = nullptr, *lap_v = nullptr, *bih_u = nullptr, *bih_v = nullptr;
  if (friction) {
    // the background viscosities (ocean_barotropic_init), then the friction of
    // udrho(tau) (:3105-3113); the inputs of a switch that is on must be set
    FricBack fb;
    fb.dxu = fptr_if_set(d, MOM5GPU_DXU, 0, 0);
    fb.dyu = fptr_if_set(d, MOM5GPU_DYU, 0, 0);
    fb.umask = fptr_if_set(d, MOM5GPU_UMASK1, 0, 0);
    fb.vel_lap = d->opt.udrho_lap_vel_micom;
    fb.vel_bih = d->opt.udrho_bih_vel_micom;
    fb.lap_e = fptr(d, MOM5GPU_LAP_CEU_BACK, 0, 0);
    fb.lap_n = fptr(d, MOM5GPU_LAP_CNU_BACK, 0, 0);
    fb.bih_e = fptr(d, MOM5GPU_BIH_CEU_BACK, 0, 0);
    fb.bih_n = fptr(d, MOM5GPU_BIH_CNU_BACK, 0, 0);
    FricOp lo;
    lo.dyue = fptr_if_set(d, MOM5GPU_DYUE, 0, 0);
    lo.dxuer = fptr_if_set(d, MOM5GPU_DXUER, 0, 0);
    lo.dxun = fptr_if_set(d, MOM5GPU_DXUN, 0, 0);
    lo.dyunr = fptr_if_set(d, MOM5GPU_DYUNR, 0, 0);
    lo.daur = fptr_if_set(d, MOM5GPU_DAUR, 0, 0);
    lo.umask = fb.umask;
    FricOp bo = lo;
    lo.ce_back = fb.lap_e;
    lo.cn_back = fb.lap_n;
    lo.ce_visc = fptr(d, MOM5GPU_LAP_VISC_CEU, 0, 0);
    lo.cn_visc = fptr(d, MOM5GPU_LAP_VISC_CNU, 0, 0);
    bo.ce_back = fb.bih_e;
    bo.cn_back = fb.bih_n;
    bo.ce_visc = fptr(d, MOM5GPU_BIH_VISC_CEU, 0, 0);
    bo.cn_visc = fptr(d, MOM5GPU_BIH_VISC_CNU, 0, 0);
    const double* uu = fptr_if_set(d, MOM5GPU_UDRHO_U, 0, tau);
    const double* uv = fptr_if_set(d, MOM5GPU_UDRHO_V, 0, tau);
    lap_u = fptr(d, MOM5GPU_LAP_FRICTION_BT_U, 0, 0);
    lap_v = fptr(d, MOM5GPU_LAP_FRICTION_BT_V, 0, 0);
    bih_u = fptr(d, MOM5GPU_BIH_FRICTION_BT_U, 0, 0);
    bih_v = fptr(d, MOM5GPU_BIH_FRICTION_BT_V, 0, 0);
    double* del2_u = fptr(d, MOM5GPU_BIH_DEL2_VEL_U, 0, 0);
    double* del2_v = fptr(d, MOM5GPU_BIH_DEL2_VEL_V, 0, 0);
    const bool on = d->opt.udrho_lap || d->opt.udrho_bih;
    if (!fb.lap_e || !fb.lap_n || !fb.bih_e || !fb.bih_n || !lo.ce_visc || !lo.cn_visc || !bo.ce_visc ||
        !bo.cn_visc || !lap_u || !lap_v || !bih_u || !bih_v || !del2_u || !del2_v)
      return fail(d, MOM5GPU_ESTATE, "ocean_barotropic_forcing: a field could not be allocated");
    if (on && (!fb.dxu || !fb.dyu || !fb.umask || !lo.dyue || !lo.dxuer || !lo.dxun || !lo.dyunr || !lo.daur ||
               !uu || !uv))
      return fail(d, MOM5GPU_ESTATE,
                  "ocean_barotropic_forcing: barotropic friction needs DXU, DYU, UMASK1, DYUE, DXUER, DXUN, DYUNR, "
                  "DAUR and UDRHO_U/V(tau)");
    if (on) {
      k_bt_fric_back<<<g2, 128, 0, s>>>(g, fb);
      launch_halo_fill(g, fb.lap_e, 1, 3, s);
      launch_halo_fill(g, fb.lap_n, 1, 3, s);
      launch_halo_fill(g, fb.bih_e, 1, 3, s);
      launch_halo_fill(g, fb.bih_n, 1, 3, s);
      k_sqrt_2d<<<nb, 256, 0, s>>>(g.n2, fb.bih_e, fb.bih_n);
      launch_bt_friction(d, lo, bo, uu, lap_u, bih_u, del2_u, s);
      launch_bt_friction(d, lo, bo, uv, lap_v, bih_v, del2_v, s);
    } else {
      for (double* z : {lap_u, lap_v, bih_u, bih_v}) cudaMemsetAsync(z, 0, sizeof(double) * g.n2, s);
      lap_u = lap_v = bih_u = bih_v = nullptr;
    }
    const int per = (d->opt.udrho_lap ? 1 + (halo ? 1 : 0) : 0) + (d->opt.udrho_bih ? 2 + (halo ? 2 : 0) : 0);
    count_launches(d, on ? 2 + (halo ? 4 : 0) + 2 * per : 0);
  }
  if (d->opt.zero_forcing_bt) {  // (:3126-3134)
    count_launches(d, 0);
    cudaMemsetAsync(fu, 0, sizeof(double) * g.n2, s);
    cudaMemsetAsync(fv, 0, sizeof(double) * g.n2, s);
  } else {
    const double* te = fptr(d, MOM5GPU_TMASKEN_E, 0, 0);
    const double* tn = fptr(d, MOM5GPU_TMASKEN_N, 0, 0);
    const double* au = fptr(d, MOM5GPU_ACCEL_U, 0, 0);
    const double* av = fptr(d, MOM5GPU_ACCEL_V, 0, 0);
    const double* su = fptr(d, MOM5GPU_SMF_U, 0, 0);
    const double* sv = fptr(d, MOM5GPU_SMF_V, 0, 0);
    const double* bu = fptr(d, MOM5GPU_BMF_U, 0, 0);
    const double* bv = fptr(d, MOM5GPU_BMF_V, 0, 0);
    if (!te || !tn || !au || !av || !su || !sv || !bu || !bv)
      return fail(d, MOM5GPU_ESTATE, "ocean_barotropic_forcing: a field could not be allocated");
    int nl = d->opt.zero_nonlinear_forcing_bt ? 0 : 1;
    count_launches(d, 4 + ((g.cx || g.cy) ? 2 : 0));
    k_baro_forcing<<<g2, 128, 0, s>>>(g, te, au, su, bu, nl, fu);
    k_baro_forcing<<<g2, 128, 0, s>>>(g, tn, av, sv, bv, nl, fv);
    launch_halo_fill(g, fu, 1, 3, s);
    launch_halo_fill(g, fv, 1, 3, s);
    if (lap_u || bih_u) {
      k_plus_friction_2d<<<nb, 256, 0, s>>>(g.n2, fu, lap_u, bih_u);
      k_plus_friction_2d<<<nb, 256, 0, s>>>(g.n2, fv, lap_v, bih_v);
    } else {
      k_plus_zero_2d<<<nb, 256, 0, s>>>(g.n2, fu);
      k_plus_zero_2d<<<nb, 256, 0, s>>>(g.n2, fv);
    }
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "ocean_barotropic_forcing");
}

// ---------------------------------------------------------------------------
// update_ucell_thickness (ocean_thickness.F90:3507-3886), no blobs
// ---------------------------------------------------------------------------
struct UThkArgs {
  Geo g;
  double rho0;
  int linear_fs, dzwu_k0;
  const double *umask, *tme, *tmn, *dzt, *dzwt, *rho_dzt, *depth_zt, *depth_zwt, *eta_u;
  double *dzu, *dzwu, *rho_dzu, *rho_dzur, *dzten_e, *dzten_n, *rho_dzten_e, *rho_dzten_n, *depth_zu, *depth_zwu;
  double *thicku, *thicken_e, *thicken_n, *mass_u, *mass_en_e, *mass_en_n;
};
constexpr double kEpslnThk = 1.0e-20;  // constants_mod epsln
DEVI double min2(double a, double b) { return a < b ? a : b; }  // Fortran min, evaluated left to right

// geopotential (:3617-3635): only the top U cell moves, with eta_u(taup1)
__global__ void k_uthk_geo(UThkArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  double zt = a.depth_zt[q], zwt = a.depth_zwt[q];  // level 1
  a.dzwu[q] = a.linear_fs ? zt : zt + a.eta_u[q];   // dzwu(:,:,0)
  double dzu1 = a.linear_fs ? zwt : zwt + a.eta_u[q];
  a.dzu[q] = dzu1;
  double r = a.rho0 * dzu1;
  a.rho_dzu[q] = r;
  a.rho_dzur[q] = div_seeded(1.0, r + kEpslnThk);
}

// zsigma / psigma (:3663-3683): the T-cell thicknesses
__global__ void k_uthk_sigma(UThkArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  for (int k = 0; k < g.nk; ++k) {
    long p = (long)k * g.n2 + q;
    double t = a.dzt[p];
    a.dzu[p] = t;
    a.dzten_e[p] = t;
    a.dzten_n[p] = t;
    a.dzwu[p + g.n2] = a.dzwt[p + g.n2];
    a.rho_dzu[p] = a.rho_dzt[p];
  }
  a.dzwu[q] = a.dzwt[q];
}

// other coordinates (:3735-3763): minimum of the neighbouring T cells over isd:iec, jsd:jec
__global__ void k_uthk_min(UThkArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni || j > g.nj) return;
  long q = I2(g, i, j), qe = q + 1, qn = q + g.nxd, qne = qn + 1;
  for (int k = 0; k < g.nk; ++k) {
    long o = (long)k * g.n2, w = o + g.n2;  // 3-D level k; level k+1 of the 0..nk arrays
    const double *t = a.dzt + o, *r = a.rho_dzt + o, *zw = a.dzwt + w;
    a.dzu[o + q] = min2(min2(min2(t[q], t[qe]), t[qn]), t[qne]);
    a.dzwu[w + q] = min2(min2(min2(zw[q], zw[qe]), zw[qn]), zw[qne]);
    a.rho_dzu[o + q] = min2(min2(min2(r[q], r[qe]), r[qn]), r[qne]);
    a.dzten_e[o + q] = min2(t[q], t[qe]);
    a.dzten_n[o + q] = min2(t[q], t[qn]);
    a.rho_dzten_e[o + q] = min2(r[q], r[qe]);
    a.rho_dzten_n[o + q] = min2(r[q], r[qn]);
  }
  if (a.dzwu_k0) a.dzwu[q] = min2(min2(min2(a.dzwt[q], a.dzwt[qe]), a.dzwt[qn]), a.dzwt[qne]);
}

// non-geopotential tail (:3771-3827): rho_dzur and the cumulative depths
__global__ void k_uthk_depths(UThkArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  for (int k = 0; k < g.nk; ++k) {
    long p = (long)k * g.n2 + q;
    a.rho_dzur[p] = div_seeded(a.umask[p], a.rho_dzu[p] + kEpslnThk);
  }
  double zu = a.dzwu[q], zwu = a.dzu[q];
  a.depth_zu[q] = zu;
  a.depth_zwu[q] = zwu;
  for (int k = 1; k < g.nk; ++k) {
    long p = (long)k * g.n2 + q;
    zu = zu + a.dzwu[p];  // + dzwu(k-1) of the 0..nk array
    zwu = zwu + a.dzu[p];
    a.depth_zu[p] = zu;
    a.depth_zwu[p] = zwu;
  }
}

// every coordinate (:3817-3858): thicku, thicken, mass_u, mass_en; kmu counted from umask
__global__ void k_uthk_sums(UThkArgs a) {
  const Geo& g = a.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i > g.ni + 1) return;
  long q = I2(g, i, j);
  int kmu = 0;
  double te = 0.0, tn = 0.0, mu = 0.0, me = 0.0, mn = 0.0;
  for (int k = 0; k < g.nk; ++k) {
    long p = (long)k * g.n2 + q;
    kmu += a.umask[p] != 0.0 ? 1 : 0;
    te = te + a.dzten_e[p];
    tn = tn + a.dzten_n[p];
    mu = mu + a.umask[p] * a.rho_dzu[p];
    me = me + a.tme[p] * a.rho_dzten_e[p];
    mn = mn + a.tmn[p] * a.rho_dzten_n[p];
  }
  a.thicku[q] = kmu > 1 ? a.depth_zwu[(long)(kmu - 1) * g.n2 + q] : 0.0;
  a.thicken_e[q] = te;
  a.thicken_n[q] = tn;
  a.mass_u[q] = mu;
  a.mass_en_e[q] = me;
  a.mass_en_n[q] = mn;
}

int launch_update_ucell_thickness(mom5gpu_domain* d, int taup1, int vcoord, bool linear_fs, bool dzwu_k0) {
  const Geo& g = d->geo;
  UThkArgs a;
  a.g = g;
  a.rho0 = d->opt.rho0;
  a.linear_fs = linear_fs;
  a.dzwu_k0 = dzwu_k0;
  const bool geo = vcoord == MOM5GPU_GEOPOTENTIAL, sigma = vcoord == MOM5GPU_ZSIGMA || vcoord == MOM5GPU_PSIGMA;
  a.umask = fptr_if_set(d, MOM5GPU_UMASK, 0, 0);
  a.tme = fptr_if_set(d, MOM5GPU_TMASKEN_E, 0, 0);
  a.tmn = fptr_if_set(d, MOM5GPU_TMASKEN_N, 0, 0);
  a.dzt = geo ? nullptr : fptr_if_set(d, MOM5GPU_DZT, 0, 0);
  a.dzwt = geo ? nullptr : fptr_if_set(d, MOM5GPU_DZWT, 0, 0);
  a.rho_dzt = geo ? nullptr : fptr_if_set(d, MOM5GPU_RHO_DZT, 0, taup1);
  a.depth_zt = geo ? fptr_if_set(d, MOM5GPU_DEPTH_ZT, 0, 0) : nullptr;
  a.depth_zwt = geo ? fptr_if_set(d, MOM5GPU_DEPTH_ZWT, 0, 0) : nullptr;
  a.eta_u = geo && !linear_fs ? fptr_if_set(d, MOM5GPU_ETA_U, 0, taup1) : nullptr;
  if (!a.umask || !a.tme || !a.tmn || (!geo && (!a.dzt || !a.dzwt || !a.rho_dzt)) ||
      (geo && (!a.depth_zt || !a.depth_zwt || (!linear_fs && !a.eta_u))))
    return fail(d, MOM5GPU_ESTATE, "update_ucell_thickness: an input field was never set");
  a.dzu = fptr(d, MOM5GPU_DZU, 0, 0);
  a.dzwu = fptr(d, MOM5GPU_DZWU, 0, 0);
  a.rho_dzu = fptr(d, MOM5GPU_RHO_DZU, 0, taup1);
  a.rho_dzur = fptr(d, MOM5GPU_RHO_DZUR, 0, 0);
  a.dzten_e = fptr(d, MOM5GPU_DZTEN_E, 0, 0);
  a.dzten_n = fptr(d, MOM5GPU_DZTEN_N, 0, 0);
  a.rho_dzten_e = fptr(d, MOM5GPU_RHO_DZTEN_E, 0, 0);
  a.rho_dzten_n = fptr(d, MOM5GPU_RHO_DZTEN_N, 0, 0);
  a.depth_zu = fptr(d, MOM5GPU_DEPTH_ZU, 0, 0);
  a.depth_zwu = fptr(d, MOM5GPU_DEPTH_ZWU, 0, 0);
  a.thicku = fptr(d, MOM5GPU_THICKU, 0, taup1);
  a.thicken_e = fptr(d, MOM5GPU_THICKEN_E, 0, 0);
  a.thicken_n = fptr(d, MOM5GPU_THICKEN_N, 0, 0);
  a.mass_u = fptr(d, MOM5GPU_MASS_U, 0, taup1);
  a.mass_en_e = fptr(d, MOM5GPU_MASS_EN_E, 0, 0);
  a.mass_en_n = fptr(d, MOM5GPU_MASS_EN_N, 0, 0);
  const void* outs[] = {a.dzu, a.dzwu, a.rho_dzu, a.rho_dzur, a.dzten_e, a.dzten_n, a.rho_dzten_e, a.rho_dzten_n,
                        a.depth_zu, a.depth_zwu, a.thicku, a.thicken_e, a.thicken_n, a.mass_u, a.mass_en_e,
                        a.mass_en_n};
  for (const void* p : outs)
    if (!p) return MOM5GPU_ENOMEM;
  cudaStream_t s = d->stream;
  dim3 g2((g.ni + 2 + 127) / 128, g.nj + 2);
  if (geo) {
    k_uthk_geo<<<g2, 128, 0, s>>>(a);
    count_launches(d, 1);
  } else {
    if (sigma) {
      k_uthk_sigma<<<g2, 128, 0, s>>>(a);
      count_launches(d, 1);
    } else {
      k_uthk_min<<<dim3((g.ni + 1 + 127) / 128, g.nj + 1), 128, 0, s>>>(a);
      for (double* p : {a.dzu, a.rho_dzu, a.dzten_e, a.dzten_n, a.rho_dzten_e, a.rho_dzten_n})
        launch_halo_fill(g, p, g.nk, 3, s);
      launch_halo_fill(g, a.dzwu, g.nk + 1, 3, s);
      count_launches(d, 1 + ((g.cx || g.cy) ? 7 : 0));
    }
    k_uthk_depths<<<g2, 128, 0, s>>>(a);
    count_launches(d, 1);
  }
  k_uthk_sums<<<g2, 128, 0, s>>>(a);
  count_launches(d, 1);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "update_ucell_thickness");
}

// ---------------------------------------------------------------------------
// compensated, fixed-order reductions
// ---------------------------------------------------------------------------
DEVI void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// (hi,lo) += (h2,l2)
DEVI void dd_add(double& hi, double& lo, double h2, double l2) {
  double s, e;
  two_sum(hi, h2, s, e);
  e = e + (lo + l2);
  double t = s + e;
  lo = e - (t - s);
  hi = t;
}

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 304;

DEVI void block_dd_reduce(double hi, double lo, double* out) {
  __shared__ double sh[kRedThreads], sl[kRedThreads];
  sh[threadIdx.x] = hi;
  sl[threadIdx.x] = lo;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double h = sh[threadIdx.x], l = sl[threadIdx.x];
      dd_add(h, l, sh[threadIdx.x + s], sl[threadIdx.x + s]);
      sh[threadIdx.x] = h;
      sl[threadIdx.x] = l;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = sh[0];
    out[2 * blockIdx.x + 1] = sl[0];
  }
}

// total_tracer: per column the reference's k-sum, then a double-double tree
__global__ void __launch_bounds__(kRedThreads) k_content(Geo g, const double* tmask, const double* dat,
                                                         const double* rdz, const double* T, double* part) {
  double hi = 0.0, lo = 0.0;
  long ncol = (long)g.ni * g.nj;
  for (long c = blockIdx.x * (long)kRedThreads + threadIdx.x; c < ncol; c += (long)gridDim.x * kRedThreads) {
    int i = (int)(c % g.ni) + 1, j = (int)(c / g.ni) + 1;
    double col = 0.0;
    double da = dat[I2(g, i, j)];
    for (int k = 0; k < g.nk; ++k) {
      long p = I3(g, i, j, k);
      double t = tmask[p] != 0.0 ? 1.0 * tmask[p] * da : 0.0;
      col = col + t * rdz[p] * T[p];
    }
    dd_add(hi, lo, col, 0.0);
  }
  block_dd_reduce(hi, lo, part);
}

__global__ void k_area(Geo g, const double* tmask1, const double* dat, const double* eta, double* part) {
  double hi = 0.0, lo = 0.0;
  long ncol = (long)g.ni * g.nj;
  for (long c = blockIdx.x * (long)kRedThreads + threadIdx.x; c < ncol; c += (long)gridDim.x * kRedThreads) {
    int i = (int)(c % g.ni) + 1, j = (int)(c / g.ni) + 1;
    long q = I2(g, i, j);
    dd_add(hi, lo, tmask1[q] * dat[q] * eta[q], 0.0);
  }
  block_dd_reduce(hi, lo, part);
}

__global__ void k_final(const double* part, int nparts, double* out) {
  double hi = 0.0, lo = 0.0;
  for (int b = threadIdx.x; b < nparts; b += kRedThreads) dd_add(hi, lo, part[2 * b], part[2 * b + 1]);
  __shared__ double sh[kRedThreads], sl[kRedThreads];
  sh[threadIdx.x] = hi;
  sl[threadIdx.x] = lo;
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double h = sh[threadIdx.x], l = sl[threadIdx.x];
      dd_add(h, l, sh[threadIdx.x + s], sl[threadIdx.x + s]);
      sh[threadIdx.x] = h;
      sl[threadIdx.x] = l;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0] + sl[0];
}

static int ensure_red(mom5gpu_domain* d) {
  if (d->red) return MOM5GPU_OK;
  cudaError_t e = cudaMalloc(&d->red, sizeof(double) * (2 * kRedBlocks + 8));
  if (e != cudaSuccess) return cuda_fail(d, e, "reduction scratch");
  e = cudaMallocHost(&d->red_h, sizeof(double) * 8);
  if (e != cudaSuccess) return cuda_fail(d, e, "reduction host buffer");
  return MOM5GPU_OK;
}

int launch_content(mom5gpu_domain* d, int n, int level, double* out_host) {
  int rc = ensure_red(d);
  if (rc) return rc;
  const Geo& g = d->geo;
  const double* tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  const double* dat = fptr(d, MOM5GPU_DAT, 0, 0);
  const double* rdz = fptr(d, MOM5GPU_RHO_DZT, 0, level);
  const double* T = fptr(d, MOM5GPU_TRACER, n, level);
  if (!tmask || !dat || !rdz || !T) return fail(d, MOM5GPU_ESTATE, "content: a required field was never set");
  k_content<<<kRedBlocks, kRedThreads, 0, d->stream>>>(g, tmask, dat, rdz, T, d->red);
  k_final<<<1, kRedThreads, 0, d->stream>>>(d->red, kRedBlocks, d->red + 2 * kRedBlocks);
  cudaMemcpyAsync(d->red_h, d->red + 2 * kRedBlocks, sizeof(double), cudaMemcpyDeviceToHost, d->stream);
  cudaError_t e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return cuda_fail(d, e, "content");
  *out_host = d->red_h[0];
  return MOM5GPU_OK;
}

// ---- exact fixed-point content (decomposition-independent) ----
//
// Each column's content (the same k-sum as k_content) is truncated to a
// multiple of 2^-kFixFrac and added as an integer, split into kFixChunks
// 32-bit chunks (chunk i weighs 2^(32 i - kFixFrac)) each summed in a signed
// 64-bit accumulator.  Integer addition is exact and associative, so any order
// of summation -- threads, blocks, the blocks of a decomposed domain, ranks of
// an allreduce -- gives the same accumulators.  Up to 2^31 values per sum;
// |value| < 2^(32 kFixChunks - kFixFrac) = 2^156, else the overflow flag is set.
constexpr int kFixChunks = MOM5GPU_FIXED_CHUNKS, kFixFrac = 100;

DEVI void fix_add(long long* acc, double x, int* overflow) {
  const long long b = bits_of(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0x7ff) {  // Inf or NaN
    *overflow = 1;
    return;
  }
  const unsigned long long m = (unsigned long long)(b & 0x000fffffffffffffLL) | (ex ? (1ULL << 52) : 0ULL);
  const int p = (ex ? ex : 1) - 1075 + kFixFrac;  // x = m * 2^(p - kFixFrac)
  if (m && p + 53 > 32 * kFixChunks) {
    *overflow = 1;
    return;
  }
  const bool neg = b < 0;
#pragma unroll
  for (int i = 0; i < kFixChunks; ++i) {
    const int sh = 32 * i - p;  // chunk i = bits [sh, sh+32) of m
    unsigned long long c = 0;
    if (sh >= 0) c = sh < 64 ? (m >> sh) & 0xffffffffULL : 0ULL;
    else c = -sh < 32 ? (m << -sh) & 0xffffffffULL : 0ULL;
    acc[i] += neg ? -(long long)c : (long long)c;
  }
}

__global__ void __launch_bounds__(kRedThreads) k_content_fixed(Geo g, const double* tmask, const double* dat,
                                                               const double* rdz, const double* T,
                                                               unsigned long long* out, int* overflow) {
  long long acc[kFixChunks] = {};
  int ovf = 0;
  long ncol = (long)g.ni * g.nj;
  for (long c = blockIdx.x * (long)kRedThreads + threadIdx.x; c < ncol; c += (long)gridDim.x * kRedThreads) {
    int i = (int)(c % g.ni) + 1, j = (int)(c / g.ni) + 1;
    double col = 0.0;
    double da = dat[I2(g, i, j)];
    for (int k = 0; k < g.nk; ++k) {
      long p = I3(g, i, j, k);
      double t = tmask[p] != 0.0 ? 1.0 * tmask[p] * da : 0.0;
      col = col + t * rdz[p] * T[p];
    }
    fix_add(acc, col, &ovf);
  }
  // integer sums: the warp, then one atomic per chunk and warp (two's complement
  // addition modulo 2^64 is exact while the true sum fits)
#pragma unroll
  for (int q = 0; q < kFixChunks; ++q) {
    long long v = acc[q];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&out[q], (unsigned long long)v);
  }
  if (ovf) atomicOr(overflow, 1);
}

int launch_content_fixed(mom5gpu_domain* d, int n, int level, long long* acc_host) {
  int rc = ensure_red(d);
  if (rc) return rc;
  const Geo& g = d->geo;
  const double* tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  const double* dat = fptr(d, MOM5GPU_DAT, 0, 0);
  const double* rdz = fptr(d, MOM5GPU_RHO_DZT, 0, level);
  const double* T = fptr(d, MOM5GPU_TRACER, n, level);
  if (!tmask || !dat || !rdz || !T) return fail(d, MOM5GPU_ESTATE, "content: a required field was never set");
  // accumulators and the overflow flag in the reduction scratch (2*kRedBlocks + 8 doubles)
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(d->red);
  int* ovf = reinterpret_cast<int*>(acc + kFixChunks);
  cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * (kFixChunks + 1), d->stream);
  k_content_fixed<<<kRedBlocks, kRedThreads, 0, d->stream>>>(g, tmask, dat, rdz, T, acc, ovf);
  long long hbuf[kFixChunks + 1];
  cudaMemcpyAsync(hbuf, acc, sizeof(long long) * (kFixChunks + 1), cudaMemcpyDeviceToHost, d->stream);
  cudaError_t e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return cuda_fail(d, e, "fixed-point content");
  if ((int)hbuf[kFixChunks])
    return fail(d, MOM5GPU_ENUMERIC, "fixed-point content: a column value is not finite or exceeds 2^155");
  for (int q = 0; q < kFixChunks; ++q) acc_host[q] = hbuf[q];
  return MOM5GPU_OK;
}

int launch_eta_integral(mom5gpu_domain* d, const double* eta, double* out_host) {
  int rc = ensure_red(d);
  if (rc) return rc;
  const Geo& g = d->geo;
  const double* tmask = fptr(d, MOM5GPU_TMASK, 0, 0);
  const double* dat = fptr(d, MOM5GPU_DAT, 0, 0);
  if (!tmask || !dat) return fail(d, MOM5GPU_ESTATE, "eta integral: grid never set");
  k_area<<<kRedBlocks, kRedThreads, 0, d->stream>>>(g, tmask, dat, eta, d->red);
  k_final<<<1, kRedThreads, 0, d->stream>>>(d->red, kRedBlocks, d->red + 2 * kRedBlocks);
  cudaMemcpyAsync(d->red_h, d->red + 2 * kRedBlocks, sizeof(double), cudaMemcpyDeviceToHost, d->stream);
  cudaError_t e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return cuda_fail(d, e, "eta integral");
  *out_host = d->red_h[0];
  return MOM5GPU_OK;
}

__global__ void k_finite(const double* a, long n, int* flag) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    long long b = __double_as_longlong(a[q]);
    if (((b >> 52) & 0x7ff) == 0x7ff) atomicOr(flag, 1);
  }
}

int launch_check_finite(mom5gpu_domain* d, const double* a, size_t count, int* out_host) {
  if (!d->flag) {
    cudaError_t e = cudaMalloc(&d->flag, sizeof(int) * 4);
    if (e != cudaSuccess) return cuda_fail(d, e, "flag");
  }
  int rc = ensure_red(d);
  if (rc) return rc;
  cudaMemsetAsync(d->flag, 0, sizeof(int), d->stream);
  k_finite<<<kRedBlocks, 256, 0, d->stream>>>(a, (long)count, d->flag);
  cudaMemcpyAsync(d->red_h, d->flag, sizeof(int), cudaMemcpyDeviceToHost, d->stream);
  cudaError_t e = cudaStreamSynchronize(d->stream);
  if (e != cudaSuccess) return cuda_fail(d, e, "check_finite");
  *out_host = *(int*)d->red_h;
  return MOM5GPU_OK;
}

}  // namespace mom5
