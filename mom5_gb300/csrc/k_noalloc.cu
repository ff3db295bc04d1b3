// Allocation-free entry point: the MDFL Sweby / DST-linear tendency of one
// tracer, with every scratch array in a fixed, file-scope device array.
//
// Some callers of this library cannot let it allocate device memory: a model
// whose GPU memory is reserved up front by its own pool or arena, a host that
// runs under a strict per-process device-memory cap, or code that must not call
// cudaMalloc/cudaFree because those calls synchronise the whole device and
// would stall work it has in flight on other streams.  The domain API
// (mom5gpu_create) allocates fields and scratch on the device, so those callers
// use this entry point instead: they pass device pointers to inputs and output,
// and the kernels' scratch (the two intermediate tracer_mdfl fields and the
// 2-cell-halo land mask) lives in g_noalloc_scratch below.
//
// The array is static: every GPU that loads this library holds its 36 MB until
// the process exits.  On the first call on each device the call looks up the
// array's device address with cudaGetSymbolAddress while that device is
// current (in host code the array's name is only a host-side stand-in, not a
// device address) and caches it; that first call should therefore come before
// any stream capture.  The cached address is that of the device's primary
// context (the runtime's): it is not valid in another context made current
// through the driver API, nor after cudaDeviceReset.  All calls on a device share the one array: calls that
// overlap on the GPU (on different streams, or from different host threads)
// race on it and must be serialised by the caller.  Every element a call reads
// is written earlier in the same call, so nothing needs to be cleared between
// calls.
#include <mutex>
#include <stdio.h>

#include "internal.h"

namespace mom5 {
namespace {

constexpr long kMaxCells = 1L << 21;       // (ni+2)*(nj+2)*nk, data-domain cells
constexpr long kMaxMaskBytes = 1L << 22;   // (ni+4)*(nj+4)*nk, 2-cell-halo mask
constexpr long kScratchDoubles = 2 * kMaxCells + kMaxMaskBytes / 8;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_mu;
double* g_addr[kMaxDevices] = {nullptr};

// tmask with a 2-cell halo under the single-domain halo rules: the compute
// value, its periodic image in a cyclic direction (corners only when both
// directions are cyclic), or zero beyond a wall (mdfl_init,
// ocean_tracer_advect.F90:1660-1669).  tmask holds 0.0 or 1.0; any non-zero
// value counts as wet.
__global__ void k_build_mask2(Geo g, const double* tmask, uint8_t* m2) {
  long n = (long)(g.ni + 4) * (g.nj + 4) * g.nk;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
    int i = (int)(q % (g.ni + 4)) - 1;
    long r = q / (g.ni + 4);
    int j = (int)(r % (g.nj + 4)) - 1;
    int k = (int)(r / (g.nj + 4));
    bool hx = i < 1 || i > g.ni, hy = j < 1 || j > g.nj;
    bool ok = (!hx || g.cx) && (!hy || g.cy);
    uint8_t v = 0;
    if (ok) {
      int ii = i < 1 ? i + g.ni : (i > g.ni ? i - g.ni : i);
      int jj = j < 1 ? j + g.nj : (j > g.nj ? j - g.nj : j);
      v = tmask[((long)k * g.nyd + jj) * g.nxd + ii] != 0.0;
    }
    m2[q] = v;
  }
}

int setup_device(double** base) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(nullptr, MOM5GPU_ECUDA, "mdfl_sweby_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, MOM5GPU_EINVAL, "mdfl_sweby_noalloc: device %d", dev);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(nullptr, MOM5GPU_ECUDA, "mdfl_sweby_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *base = g_addr[dev];
  return MOM5GPU_OK;
}

}  // namespace
}  // namespace mom5

using namespace mom5;

extern "C" int mom5gpu_mdfl_sweby_noalloc(const mom5gpu_dims* dims, int scheme, double dtime, const double* tmask,
                                          const double* dat, const double* datr, const double* dxte,
                                          const double* dyte, const double* dxtn, const double* dytn,
                                          const double* uhrho_et, const double* vhrho_nt, const double* wrho_bt,
                                          const double* rho_dzt, const double* T, double* th_tendency, void* stream) {
  if (!dims) return fail(nullptr, MOM5GPU_EINVAL, "mdfl_sweby_noalloc: null dims");
  if (dims->ni < 2 || dims->nj < 2 || dims->nk < 1)
    return fail(nullptr, MOM5GPU_EINVAL, "mdfl_sweby_noalloc: bad dimensions %d x %d x %d", dims->ni, dims->nj, dims->nk);
  if (scheme != MOM5GPU_ADVECT_MDFL_SWEBY && scheme != MOM5GPU_ADVECT_DST_LINEAR)
    return fail(nullptr, MOM5GPU_EINVAL, "mdfl_sweby_noalloc: scheme must be MDFL_SWEBY (9) or DST_LINEAR (10)");
  const void* need[] = {tmask, dat, datr, dxte, dyte, dxtn, dytn, uhrho_et, vhrho_nt, wrho_bt, rho_dzt, T, th_tendency};
  for (const void* p : need)
    if (!p) return fail(nullptr, MOM5GPU_EINVAL, "mdfl_sweby_noalloc: null array argument");
  Geo g;
  g.ni = dims->ni;
  g.nj = dims->nj;
  g.nk = dims->nk;
  g.nxd = g.ni + 2;
  g.nyd = g.nj + 2;
  g.cx = dims->cyclic_x ? 1 : 0;
  g.cy = dims->cyclic_y ? 1 : 0;
  g.n2 = (long)g.nxd * g.nyd;
  g.n3 = g.n2 * g.nk;
  long mask_bytes = (long)(g.ni + 4) * (g.nj + 4) * g.nk;
  if (g.n3 > kMaxCells || mask_bytes > kMaxMaskBytes)
    return fail(nullptr, MOM5GPU_EINVAL,
                "mdfl_sweby_noalloc: a %d x %d x %d domain needs %ld data-domain cells; the allocation-free entry "
                "point holds at most %ld (use the domain API for larger domains)",
                g.ni, g.nj, g.nk, g.n3, kMaxCells);
  double* base = nullptr;
  int rc = setup_device(&base);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  uint8_t* mask2 = reinterpret_cast<uint8_t*>(base + 2 * kMaxCells);
  k_build_mask2<<<304, 256, 0, s>>>(g, tmask, mask2);
  MdflArgs a;
  a.g = g;
  a.ntr = 1;
  a.dtime = dtime;
  a.mask2 = mask2;
  a.dat = dat;
  a.datr = datr;
  a.dxte = dxte;
  a.dyte = dyte;
  a.dxtn = dxtn;
  a.dytn = dytn;
  a.uh = uhrho_et;
  a.vh = vhrho_nt;
  a.w = wrho_bt;
  a.rdz = rho_dzt;
  a.T = T;
  a.tstride = g.n3;
  a.tz = base;
  a.tx = base + kMaxCells;
  a.th = th_tendency;
  run_mdfl_kernels(a, false, scheme == MOM5GPU_ADVECT_MDFL_SWEBY, s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(nullptr, MOM5GPU_ECUDA, "mdfl_sweby_noalloc: launch: %s", cudaGetErrorString(e));
  return MOM5GPU_OK;
}
