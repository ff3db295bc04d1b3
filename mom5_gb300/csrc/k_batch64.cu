// Batched FP64 kernels: the MDFL passes, the explicit update and the barotropic
// phases of many domains in one launch each.  A launch's blocks are a flat
// work list; a block finds its (domain, block) from the per-pass prefix sums
// and runs the same body as the one-domain kernel (fp64_bodies.cuh), so every
// domain's result is identical to stepping it alone.  Built with --fmad=false.
#include "internal.h"
#include "fp64_bodies.cuh"

namespace mom5 {

using namespace fp64;

namespace {

// entry of block b: the largest e with prefix[e] <= b
DEVI int find_entry(const int* prefix, int count, int b) {
  int lo = 0, hi = count;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (prefix[mid] <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <bool SWEBY, int MAXN>
__global__ void __launch_bounds__(128) kb_mdfl_z(const MdflArgs* d, BatchWork w) {
  int e = find_entry(w.pz, w.count, blockIdx.x);
  const MdflArgs& a = d[w.entries[e]];
  int local = blockIdx.x - w.pz[e];
  int nb = (a.g.ni + 127) / 128;
  mdfl_z_body<false, SWEBY, MAXN>(a, local % nb, local / nb);
}

template <bool SWEBY, int MAXN>
__global__ void __launch_bounds__(kTX) kb_mdfl_x(const MdflArgs* d, BatchWork w) {
  int e = find_entry(w.px, w.count, blockIdx.x);
  const MdflArgs& a = d[w.entries[e]];
  int local = blockIdx.x - w.px[e];
  int nb = (a.g.ni + kTX - 1) / kTX;
  mdfl_x_body<false, SWEBY, MAXN>(a, local % nb, (local / nb) % a.g.nj, local / (nb * a.g.nj));
}

template <bool SWEBY, int MAXN>
__global__ void __launch_bounds__(128, 6) kb_mdfl_y(const MdflArgs* d, BatchWork w, int TJ) {
  int e = find_entry(w.py, w.count, blockIdx.x);
  const MdflArgs& a = d[w.entries[e]];
  int local = blockIdx.x - w.py[e];
  int nb = (a.g.ni + 127) / 128;
  int ns = (a.g.nj + TJ - 1) / TJ;
  mdfl_y_body<false, SWEBY, MAXN>(a, TJ, local % nb, (local / nb) % ns, local / (nb * ns));
}

__global__ void __launch_bounds__(128) kb_update(const UpdArgs* d, BatchWork w) {
  int e = find_entry(w.pu, w.count, blockIdx.x);
  const UpdArgs& u = d[w.entries[e]];
  const Geo& g = u.g;
  int local = blockIdx.x - w.pu[e];
  int nb = (g.ni + 127) / 128;
  int i = (local % nb) * 128 + threadIdx.x + 1;
  int j = (local / nb) % g.nj + 1, k = local / (nb * g.nj);
  if (i > g.ni) return;
  long p = I3(g, i, j, k);
  double a = u.rdz_m1[p], r = u.rdzr[p];
  for (int n = 0; n < u.ntr; ++n) u.Tp1[n * u.tstride + p] = (a * u.Tm1[n * u.tstride + p] + u.dtime * u.th[n * g.n3 + p]) * r;
}

__global__ void __launch_bounds__(256) kb_bt_init(const BtArgs* d, const BtExtra* xs, BatchWork w) {
  int e = find_entry(w.pb1, w.count, blockIdx.x);
  const BtArgs& a = d[w.entries[e]];
  const BtExtra& x = xs[w.entries[e]];
  bt_init_body(a, x.eta_bar_tau, x.eta_tau, x.ud_tau, x.vd_tau, x.pme, x.river, x.source, x.eta_smooth,
               x.initsum_with_bar, blockIdx.x - w.pb1[e], 0);
}

#define BT2D_ENTRY                                   \
  int e = find_entry(w.pb2, w.count, blockIdx.x);    \
  const BtArgs& a = d[w.entries[e]];                 \
  int local = blockIdx.x - w.pb2[e];                 \
  int nb = (a.g.ni + 2 + 127) / 128;                 \
  int bx = local % nb, by = local / nb;

__global__ void __launch_bounds__(128) kb_bt_pred(const BtArgs* d, BatchWork w, int so, int sn, int reuse) {
  pdl_wait();
  pdl_trigger();
  BT2D_ENTRY
  bt_pred_body(a, so, sn, reuse, bx, by);
}
__global__ void __launch_bounds__(128) kb_bt_mom_b(const BtArgs* d, BatchWork w, int so, int sn) {
  pdl_wait();
  pdl_trigger();
  BT2D_ENTRY
  bt_mom_b_body(a, so, sn, bx, by);
}
__global__ void __launch_bounds__(128) kb_bt_corr(const BtArgs* d, BatchWork w, int so, int sn, double wgt) {
  pdl_wait();
  pdl_trigger();
  BT2D_ENTRY
  bt_corr_body(a, so, sn, wgt, bx, by);
}
__global__ void __launch_bounds__(128) kb_bt_corr_pred(const BtArgs* d, BatchWork w, int so, int sn, double wgt) {
  pdl_wait();
  pdl_trigger();
  BT2D_ENTRY
  bt_corr_pred_body(a, so, sn, wgt, bx, by);
}
__global__ void __launch_bounds__(256) kb_bt_post1(const BtArgs* d, BatchWork w, double rntsp1, double rnts) {
  int e = find_entry(w.pb1, w.count, blockIdx.x);
  const BtArgs& a = d[w.entries[e]];
  long q = (long)(blockIdx.x - w.pb1[e]) * 256 + threadIdx.x;
  if (q >= a.g.n2) return;
  a.eta_bar[q] = rntsp1 * a.eta_bar[q];
  a.udrho_u[q] = rnts * a.udrho_u[q];
  a.udrho_v[q] = rnts * a.udrho_v[q];
}
__global__ void __launch_bounds__(128) kb_bt_post2(const BtArgs* d, const BtExtra* xs, BatchWork w) {
  BT2D_ENTRY
  const BtExtra& x = xs[w.entries[e]];
  bt_post2_body(a, x.conv, x.eta_u, x.ps_out, bx, by);
}
__global__ void __launch_bounds__(128) kb_bt_post3(const BtArgs* d, const BtExtra* xs, BatchWork w) {
  BT2D_ENTRY
  const BtExtra& x = xs[w.entries[e]];
  bt_post3_body(a, x.ps_out, x.gxo, x.gyo, bx, by);
}

template <bool SWEBY, int MAXN>
void adv(const MdflArgs* m, const UpdArgs* u, const BatchWork& w, int TJ, cudaStream_t s) {
  if (w.tz > 0) kb_mdfl_z<SWEBY, MAXN><<<w.tz, 128, 0, s>>>(m, w);
  if (w.tx > 0) kb_mdfl_x<SWEBY, MAXN><<<w.tx, kTX, 0, s>>>(m, w);
  if (w.ty > 0) kb_mdfl_y<SWEBY, MAXN><<<w.ty, 128, 0, s>>>(m, w, TJ);
  if (w.tu > 0) kb_update<<<w.tu, 128, 0, s>>>(u, w);
}

}  // namespace

BatchBlocks batch_blocks(const Geo& g, int TJ, int mixed_rows, bool tma, int ntr) {
  BatchBlocks b;
  int nb = (g.ni + 127) / 128;
  b.z = nb * g.nj;
  b.x = ((g.ni + kTX - 1) / kTX) * g.nj * g.nk;
  b.y = nb * ((g.nj + TJ - 1) / TJ) * g.nk;
  b.u = nb * g.nj * g.nk;
  b.b2 = ((g.ni + 2 + 127) / 128) * (g.nj + 2);
  b.b1 = (int)((g.n2 + 255) / 256);
  // rows 24: TMA-staged 24-row tiles where the domain allows them, else the plain 32-row tiles
  const bool staged = mixed_rows == 24 && tma;
  int tj = (mixed_rows == 24 ? 32 : mixed_rows) - 4;
  b.m = staged ? 0 : ((g.ni + 27) / 28) * ((g.nj + tj - 1) / tj);
  const int ttj = staged ? batch_tma_rows(ntr) - 4 : 1;
  b.t = staged ? ((g.ni + 27) / 28) * ((g.nj + ttj - 1) / ttj) : 0;
  return b;
}

void launch_batch_fp64_advection(const MdflArgs* m, const UpdArgs* u, const BatchWork& w, int ntr, bool sweby, int TJ,
                                 cudaStream_t s) {
  if (sweby) {
    if (ntr <= 1) adv<true, 1>(m, u, w, TJ, s);
    else if (ntr <= 2) adv<true, 2>(m, u, w, TJ, s);
    else if (ntr <= 4) adv<true, 4>(m, u, w, TJ, s);
    else adv<true, kMdflChunk>(m, u, w, TJ, s);
  } else {
    if (ntr <= 1) adv<false, 1>(m, u, w, TJ, s);
    else if (ntr <= 2) adv<false, 2>(m, u, w, TJ, s);
    else if (ntr <= 4) adv<false, 4>(m, u, w, TJ, s);
    else adv<false, kMdflChunk>(m, u, w, TJ, s);
  }
}

void launch_batch_barotropic_loop(const BtArgs* bt, const BtExtra* x, const BatchWork& w, int nts, int stepB,
                                  bool fast, cudaStream_t s) {
  kb_bt_init<<<w.tb1, 256, 0, s>>>(bt, x, w);
  if (fast) launch_batch_btf_prep(bt, w, s);
  for (int itime = 1; itime <= nts; ++itime) {
    int so = (itime + 0) % 2, sn = (itime + 1) % 2;
    if (fast) {  // precision form: folded FP64 subcycle
      launch_batch_btf_subcycle(bt, w, itime, nts, s);
      continue;
    }
    // as the one-domain form: the predictor launched only in the first subcycle
    // programmatic dependents (launch_pdl), as the one-domain subcycle kernels
    const dim3 g2(w.tb2), b(128);
    const double wgt = (double)(nts - itime + 1);
    if (itime == 1) launch_pdl(kb_bt_pred, g2, b, s, bt, w, so, sn, 0);
    launch_pdl(kb_bt_mom_b, g2, b, s, bt, w, so, sn);
    if (itime < nts) launch_pdl(kb_bt_corr_pred, g2, b, s, bt, w, so, sn, wgt);
    else launch_pdl(kb_bt_corr, g2, b, s, bt, w, so, sn, wgt);
  }
  (void)stepB;
}

void launch_batch_barotropic_post(const BtArgs* bt, const BtExtra* x, const BatchWork& w, int nts, int stepB, int phase,
                                  cudaStream_t s) {
  if (phase == 1) {
    double rntsp1 = 1.0 / ((double)nts + 1.0);
    double rnts = stepB ? 2.0 / ((double)nts * (double)(nts + 1)) : 1.0 / (double)nts;
    kb_bt_post1<<<w.tb1, 256, 0, s>>>(bt, w, rntsp1, rnts);
  } else if (phase == 2) {
    kb_bt_post2<<<w.tb2, 128, 0, s>>>(bt, x, w);
  } else {
    kb_bt_post3<<<w.tb2, 128, 0, s>>>(bt, x, w);
  }
}

}  // namespace mom5
