// Precision form of MDFL Sweby: fluxes and limiters in FP32, tracer state in FP64.
//
// One fused kernel does the z, x and y passes of advect_tracer_mdfl_sweby
// (ocean_tracer_advect.F90:3806-4066) for a tile of 28 columns by ZR-4 rows
// (ZR = 16, 24 or 32, autotuned), marching down k, with the tile's 2-cell halo
// recomputed instead of exchanged: the z pass runs on the 32 x ZR
// tile-plus-halo, the x pass on ZR rows x 28 columns, the y pass on the
// interior.  Face terms (mass flux, Courant number,
// d0, d1, the limiter slope) are computed once per level and shared by every
// tracer of the launch.
//
// The increment T_mdfl - T is carried as the sum of the three flux-divergence
// increments; the divergence corrections the reference adds per pass and
// removes at the end cancel exactly and are applied only to the intermediate
// values the next pass limits on.  The state update
// T(taup1) = (rho_dzt(taum1)*T + dtime*th)*rho_dztr (ocean_tracer.F90:2341-2350)
// is evaluated as T + [(rho_dzt(taum1)*rho_dztr - 1)*T + rho_dzt(tau)*rho_dztr*dT]
// with one FP64 add per tracer-cell.  FP64<->FP32 conversions are done with
// integer operations: on GB300 a conversion issues at the FP64 rate.
#include <math.h>


#include "mixed_body.cuh"
#include "bt_fast_body.cuh"

namespace mom5 {

using namespace mixed;

namespace {

// shared memory: the tile arrays, then (prefetch variant) the tracer buffers
template <int ZR, bool PF>
constexpr size_t mixed_smem() {
  return ((sizeof(SmemT<ZR>) + 15) & ~(size_t)15) + (PF ? sizeof(PrefetchT<ZR>) : 0);
}

template <int NC, int ZR, bool PF>
__global__ void __launch_bounds__(tile_threads(ZR), PF ? 2 : (ZR == 16 ? 4 : ZR == 24 ? 3 : ZR == 64 ? 1 : 2))
    k_mdfl_mixed(MixArgs a, int n0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemT<ZR>& s = *reinterpret_cast<SmemT<ZR>*>(smem_raw);
  PrefetchT<ZR>* pf =
      PF ? reinterpret_cast<PrefetchT<ZR>*>(smem_raw + ((sizeof(SmemT<ZR>) + 15) & ~(size_t)15)) : nullptr;
  mixed_tile<NC, ZR, PF, tile_threads(ZR)>(a, n0, blockIdx.x, blockIdx.y, s, pf);
}

template <int NC, int ZR, bool PF>
int run_mixed_zr(mom5gpu_domain* d, MixArgs a, int n0) {
  const Geo& g = d->geo;
  constexpr size_t smem = mixed_smem<ZR, PF>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e =
        cudaFuncSetAttribute(k_mdfl_mixed<NC, ZR, PF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(d, e, "mixed kernel attribute");
    configured = true;
  }
  constexpr int TJ = ZR - 4;
  dim3 grid((g.ni + TI - 1) / TI, (g.nj + TJ - 1) / TJ);
  k_mdfl_mixed<NC, ZR, PF><<<grid, tile_threads(ZR), smem, d->stream>>>(a, n0);
  count_launches(d, 1);
  return MOM5GPU_OK;
}

template <int NC>
int run_mixed(mom5gpu_domain* d, MixArgs a, int n0) {
  if (d->tune_mixed_rows == 16 && d->tune_mixed_pf == 1) return run_mixed_zr<NC, 16, true>(d, a, n0);
  if (d->tune_mixed_rows == 16) return run_mixed_zr<NC, 16, false>(d, a, n0);
  if (d->tune_mixed_rows == 24) return run_mixed_zr<NC, 24, false>(d, a, n0);
  if (d->tune_mixed_rows == 64) return run_mixed_zr<NC, 64, false>(d, a, n0);
  return run_mixed_zr<NC, 32, false>(d, a, n0);
}

}  // namespace

__global__ void __launch_bounds__(128) k_btf_prep(BtArgs a) { btfast::prep_body(a, blockIdx.x, blockIdx.y); }
// The subcycle kernels are launched as programmatic dependents (launch_pdl).
__global__ void __launch_bounds__(128) k_btf_pred(BtArgs a, int so, int sn, int reuse) {
  pdl_wait();
  pdl_trigger();
  btfast::pred_body(a, so, sn, reuse, blockIdx.x, blockIdx.y);
}
__global__ void __launch_bounds__(128) k_btf_mom(BtArgs a, int so, int sn, double wgt) {
  pdl_wait();
  pdl_trigger();
  btfast::mom_body(a, so, sn, wgt, blockIdx.x, blockIdx.y);
}
__global__ void __launch_bounds__(128) k_btf_corr(BtArgs a, int so, int sn) {
  pdl_wait();
  pdl_trigger();
  btfast::corr_body(a, so, sn, blockIdx.x, blockIdx.y);
}
__global__ void __launch_bounds__(128) k_btf_corr_pred(BtArgs a, int so, int sn) {
  pdl_wait();
  pdl_trigger();
  btfast::corr_pred_body(a, so, sn, blockIdx.x, blockIdx.y);
}

void launch_btf_prep(const BtArgs& a, cudaStream_t s) {
  dim3 g2((a.g.ni + 2 + 127) / 128, a.g.nj + 2);
  k_btf_prep<<<g2, 128, 0, s>>>(a);
}

// One launch per subcycle (mom5gpu_set_barotropic_fusion mode 1): 32 x 8 tiles of
// 352 threads, one point per thread in each phase (the 34 x 10 surface-pressure
// ring is the largest).  Measured per precision-form step: 0.66 ms against 0.72
// ms for form 0 on 360x300 (80 subcycles), where the launches set the time, but
// 7.2 ms against 4.6 ms on 1440x1080 (60 subcycles), which form 0's streaming
// launches keep near the memory bound.  On 360x300 the 64 x 8 (256 threads,
// several points per thread), 32 x 16, 128 x 4 and 64 x 16 tiles were slower
// than 32 x 8.
constexpr int kBtfTX = 32, kBtfTY = 8, kBtfThreads = 352;
__global__ void __launch_bounds__(kBtfThreads) k_btf_fused(BtArgs a, int so, int sn, int reuse, double wgt) {
  pdl_wait();
  pdl_trigger();
  btfast::fused_body<kBtfTX, kBtfTY>(a, so, sn, reuse, wgt, blockIdx.x, blockIdx.y);
}

// Subcycle itime of nts.  Form 0: the predictor (a launch of its own only in the
// first subcycle), the momentum step, and the corrector, which in every
// subcycle but the last also forms the next subcycle's predictor; 1 + 2*nts
// launches per step.  Form 1: one launch per subcycle.  Returns the launches.
int launch_btf_subcycle(const BtArgs& a, int itime, int nts, bool fused, cudaStream_t s) {
  const int so = itime % 2, sn = (itime + 1) % 2;
  const double wgt = (double)(nts - itime + 1);
  if (fused) {
    dim3 gf((a.g.ni + 2 + kBtfTX - 1) / kBtfTX, (a.g.nj + 2 + kBtfTY - 1) / kBtfTY);
    launch_pdl(k_btf_fused, gf, dim3(kBtfThreads), s, a, so, sn, (int)(itime > 1), wgt);
    return 1;
  }
  dim3 g2((a.g.ni + 2 + 127) / 128, a.g.nj + 2);
  if (itime == 1) launch_pdl(k_btf_pred, g2, dim3(128), s, a, so, sn, 0);
  launch_pdl(k_btf_mom, g2, dim3(128), s, a, so, sn, wgt);
  if (itime < nts) launch_pdl(k_btf_corr_pred, g2, dim3(128), s, a, so, sn);
  else launch_pdl(k_btf_corr, g2, dim3(128), s, a, so, sn);
  return itime == 1 ? 3 : 2;
}

int make_mix_args(mom5gpu_domain* d, int taum1, int tau, int taup1, double dtime, MixArgs* ap) {
  MixArgs& a = *ap;
  a.g = d->geo;
  a.ntr = d->dims.num_prog_tracers;
  a.dtime = (float)dtime;
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
  a.rdz_m1 = fptr(d, MOM5GPU_RHO_DZT, 0, taum1);
  a.rdzr = fptr(d, MOM5GPU_RHO_DZTR, 0, 0);
  a.fused = 1;
  a.T = a.ntr > 0 ? fptr(d, MOM5GPU_TRACER, 1, taum1) : nullptr;
  a.out = a.ntr > 0 ? fptr(d, MOM5GPU_TRACER, 1, taup1) : nullptr;
  if (!a.dat || !a.datr || !a.dxte || !a.dyte || !a.dxtn || !a.dytn || !a.uh || !a.vh || !a.w || !a.rdz || !a.rdz_m1 ||
      !a.rdzr || !d->mask2 || !a.T || !a.out)
    return fail(d, MOM5GPU_ESTATE, "precision form: a required field was never set");
  return MOM5GPU_OK;
}

int launch_mdfl_mixed(mom5gpu_domain* d, int n_first, int ntr, int taum1, int tau, int taup1, double dtime,
                      bool fused_update) {
  ClockScope clk(d, SEC_MDFL_MIXED);
  const Geo& g = d->geo;
  MixArgs a;
  a.g = g;
  a.dtime = (float)dtime;
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
  a.rdz_m1 = fptr(d, MOM5GPU_RHO_DZT, 0, taum1);
  a.rdzr = fptr(d, MOM5GPU_RHO_DZTR, 0, 0);
  a.fused = fused_update ? 1 : 0;
  if (!a.dat || !a.datr || !a.dxte || !a.dyte || !a.dxtn || !a.dytn || !a.uh || !a.vh || !a.w || !a.rdz || !a.rdz_m1 ||
      !a.rdzr || !d->mask2)
    return fail(d, MOM5GPU_ESTATE, "precision form: a required field was never set");
  int rc = MOM5GPU_OK;
  for (int c0 = 0; c0 < ntr && rc == MOM5GPU_OK; c0 += 10) {
    int cn = ntr - c0 < 10 ? ntr - c0 : 10;
    a.ntr = cn;
    a.T = fptr(d, MOM5GPU_TRACER, n_first + c0, taum1);
    if (fused_update) {
      a.out = fptr(d, MOM5GPU_TRACER, 1, taup1);  // indexed with the absolute tracer number
    } else {
      a.out = fptr(d, MOM5GPU_TH_TENDENCY, n_first + c0, 0);
    }
    if (!a.T || !a.out) return fail(d, MOM5GPU_ENOMEM, "precision form: tracer storage");
    int n0 = fused_update ? n_first - 1 + c0 : 0;
    if (d->tune_mixed_pf >= 2) {
      rc = launch_mixed_tma(d, a, n0, fptr(d, MOM5GPU_TRACER, 1, taum1), n_first - 1 + c0,
                            d->dims.num_prog_tracers);
      if (rc != MOM5GPU_EUNSUPPORTED) continue;
    }
    if (cn <= 1) rc = run_mixed<1>(d, a, n0);
    else if (cn <= 2) rc = run_mixed<2>(d, a, n0);
    else if (cn <= 4) rc = run_mixed<4>(d, a, n0);
    else rc = run_mixed<10>(d, a, n0);
  }
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "precision form launch");
}

}  // namespace mom5
