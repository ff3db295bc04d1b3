// Persistent batched kernel of the precision form: a fixed grid of resident
// blocks drains a queue of (domain, tile) items (largest domains first),
// running the same tile body as the one-domain kernel (mixed_body.cuh).
#include "internal.h"
#include "mixed_body.cuh"
#include "bt_fast_body.cuh"

namespace mom5 {

using namespace mixed;

namespace {

DEVI int find_entry_m(const int* prefix, int count, int b) {
  int lo = 0, hi = count;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (prefix[mid] <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <int NC, int ZR>
__global__ void __launch_bounds__(tile_threads(ZR), ZR == 16 ? 4 : 2) kb_mixed(const MixArgs* d, BatchWork w,
                                                                              int* counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemT<ZR>& s = *reinterpret_cast<SmemT<ZR>*>(smem_raw);
  __shared__ int item;
  const int total = w.tm;
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = item;
    __syncthreads();
    if (it >= total) break;
    int e = find_entry_m(w.pm, w.count, it);
    const MixArgs& a = d[w.entries[e]];
    int local = it - w.pm[e];
    int ntx = (a.g.ni + TI - 1) / TI;
    mixed_tile<NC, ZR, false, tile_threads(ZR)>(a, 0, local % ntx, local / ntx, s);
  }
}

// precision-form barotropic subcycle over a work list of (domain, 2-D block) items
#define BTF_ENTRY                                    \
  int e = find_entry_m(w.pb2, w.count, blockIdx.x);  \
  const BtArgs& a = d[w.entries[e]];                 \
  int local = blockIdx.x - w.pb2[e];                 \
  int nb = (a.g.ni + 2 + 127) / 128;                 \
  int bx = local % nb, by = local / nb;

__global__ void __launch_bounds__(128) kb_btf_prep(const BtArgs* d, BatchWork w) {
  BTF_ENTRY
  btfast::prep_body(a, bx, by);
}
__global__ void __launch_bounds__(128) kb_btf_pred(const BtArgs* d, BatchWork w, int so, int sn, int reuse) {
  pdl_wait();
  pdl_trigger();
  BTF_ENTRY
  btfast::pred_body(a, so, sn, reuse, bx, by);
}
__global__ void __launch_bounds__(128) kb_btf_mom(const BtArgs* d, BatchWork w, int so, int sn, double wgt) {
  pdl_wait();
  pdl_trigger();
  BTF_ENTRY
  btfast::mom_body(a, so, sn, wgt, bx, by);
}
__global__ void __launch_bounds__(128) kb_btf_corr(const BtArgs* d, BatchWork w, int so, int sn) {
  pdl_wait();
  pdl_trigger();
  BTF_ENTRY
  btfast::corr_body(a, so, sn, bx, by);
}
__global__ void __launch_bounds__(128) kb_btf_corr_pred(const BtArgs* d, BatchWork w, int so, int sn) {
  pdl_wait();
  pdl_trigger();
  BTF_ENTRY
  btfast::corr_pred_body(a, so, sn, bx, by);
}

template <int NC, int ZR>
int configure() {
  return cudaFuncSetAttribute(kb_mixed<NC, ZR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemT<ZR>)) ==
                 cudaSuccess
             ? MOM5GPU_OK
             : MOM5GPU_ECUDA;
}

template <int NC, int ZR>
int run(const MixArgs* m, const BatchWork& w, int blocks, int* counter, cudaStream_t s) {
  size_t smem = sizeof(SmemT<ZR>);
  cudaMemsetAsync(counter, 0, sizeof(int), s);
  kb_mixed<NC, ZR><<<blocks, tile_threads(ZR), smem, s>>>(m, w, counter);
  return MOM5GPU_OK;
}

template <int ZR>
int run_nc(const MixArgs* m, const BatchWork& w, int ntr, int blocks, int* counter, cudaStream_t s) {
  if (ntr <= 1) return run<1, ZR>(m, w, blocks, counter, s);
  if (ntr <= 2) return run<2, ZR>(m, w, blocks, counter, s);
  if (ntr <= 4) return run<4, ZR>(m, w, blocks, counter, s);
  return run<10, ZR>(m, w, blocks, counter, s);
}

}  // namespace

void launch_batch_btf_prep(const BtArgs* bt, const BatchWork& w, cudaStream_t s) {
  if (w.tb2 > 0) kb_btf_prep<<<w.tb2, 128, 0, s>>>(bt, w);
}

// subcycle itime of nts, as the one-domain form 0: the predictor launched only in
// the first subcycle, the corrector forming the next subcycle's predictor in all
// but the last; returns the launches
int launch_batch_btf_subcycle(const BtArgs* bt, const BatchWork& w, int itime, int nts, cudaStream_t s) {
  if (w.tb2 <= 0) return 0;
  const int so = itime % 2, sn = (itime + 1) % 2;
  const double wgt = (double)(nts - itime + 1);
  const dim3 g2(w.tb2), b(128);
  if (itime == 1) launch_pdl(kb_btf_pred, g2, b, s, bt, w, so, sn, 0);
  launch_pdl(kb_btf_mom, g2, b, s, bt, w, so, sn, wgt);
  if (itime < nts) launch_pdl(kb_btf_corr_pred, g2, b, s, bt, w, so, sn);
  else launch_pdl(kb_btf_corr, g2, b, s, bt, w, so, sn);
  return itime == 1 ? 3 : 2;
}

int prepare_batch_mixed() {
  int rc = 0;
  rc |= configure<1, 32>() | configure<2, 32>() | configure<4, 32>() | configure<10, 32>();
  rc |= configure<1, 16>() | configure<2, 16>() | configure<4, 16>() | configure<10, 16>();
  return rc ? MOM5GPU_ECUDA : MOM5GPU_OK;
}

int launch_batch_mixed(const MixArgs* mix, const void* tma, const BatchWork& w, int ntr, int rows, int blocks,
                       int sms, int* counter, cudaStream_t s) {
  int rc = MOM5GPU_OK;
  if (w.tm > 0)
    rc = rows == 16 ? run_nc<16>(mix, w, ntr, blocks, counter, s) : run_nc<32>(mix, w, ntr, blocks, counter, s);
  if (rc == MOM5GPU_OK && rows == 24 && w.tt > 0) rc = launch_batch_mixed_tma(mix, tma, w, ntr, sms, counter + 1, s);
  return rc;
}

}  // namespace mom5
