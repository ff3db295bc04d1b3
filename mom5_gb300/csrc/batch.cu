// Host side of batches (include/mom5gpu.h, "batching"): per-domain descriptor
// tables on the device, work lists, CUDA-graph capture of whole steps, and the
// autotuner of launch shapes.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "internal.h"

using namespace mom5;

struct mom5gpu_batch {
  std::vector<mom5gpu_domain*> doms;
  int prec = 0, ntr = 0, nts = 0, stepB = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  std::string err;
  // descriptor tables, entry 2*d + parity (parity 0: tau 1 -> 2, parity 1: 2 -> 1)
  MdflArgs* d_mdfl = nullptr;
  UpdArgs* d_upd = nullptr;
  BtArgs* d_bt = nullptr;
  BtExtra* d_btx = nullptr;
  MixArgs* d_mix = nullptr;
  double desc_dtime = -1.0;
  // per-step work list
  int* d_work = nullptr;
  size_t work_cap = 0;  // ints
  // fixed all-domain work lists and their graphs
  int* d_work_all[2] = {nullptr, nullptr};
  BatchWork w_all[2];
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  int g_key[2] = {-1, -1};
  long g_launches[2] = {0, 0};  // kernels per replay of each graph
  int* d_counter = nullptr;  // [0] plain precision tiles, [1] TMA-staged tiles
  // precision form: a table of tensor maps per (domain, parity) for the
  // TMA-staged tiles, and which domains have one (even ni)
  unsigned char* d_tma = nullptr;
  std::vector<char> tma_ok;
  // tuning
  int rows = 32, tj = 0, blocks_per_sm = 2, sms = 152;
  bool any_cyclic = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double last_ms = 0.0;
  long launches = 0;
  // ordering against the domains' own streams
  std::vector<cudaEvent_t> dom_ev;
  cudaEvent_t done_ev = nullptr;
};

namespace {

int bfail(mom5gpu_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  else fail(nullptr, code, "%s", buf);
  return code;
}

int default_tj(const mom5gpu_batch* b) {
  long cols = 0;
  for (auto* d : b->doms) cols += (long)d->geo.ni * d->geo.nk;
  long nj = 0;
  for (auto* d : b->doms) nj = std::max<long>(nj, d->geo.nj);
  int TJ = 16;
  while (TJ > 2 && cols * ((nj + TJ - 1) / TJ) < 152L * 32 * 16) TJ /= 2;
  return TJ;
}

int tj_of(const mom5gpu_batch* b) { return b->tj > 0 ? b->tj : default_tj(b); }

int build_descriptors(mom5gpu_batch* b, double dtime) {
  int n = (int)b->doms.size();
  std::vector<MdflArgs> m(2 * n);
  std::vector<UpdArgs> u(2 * n);
  std::vector<BtArgs> bt(2 * n);
  std::vector<BtExtra> bx(2 * n);
  std::vector<MixArgs> mx(2 * n);
  // tensor maps of the TMA-staged precision tiles, (domain, parity) entries
  const size_t tb = batch_tma_bytes();
  std::vector<unsigned char> tma(b->prec == MOM5GPU_PRECISION_FP64 ? 0 : tb * 2 * n, 0);
  b->tma_ok.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    mom5gpu_domain* d = b->doms[i];
    for (int p = 0; p < 2; ++p) {
      int tau = 1 + p, taup1 = 2 - p, taum1 = tau;
      int rc = MOM5GPU_OK;
      if (b->prec == MOM5GPU_PRECISION_FP64) {
        if ((rc = make_mdfl_args(d, 1, b->ntr, taum1, tau, dtime, &m[2 * i + p])) ||
            (rc = make_upd_args(d, taum1, taup1, dtime, &u[2 * i + p])))
          return bfail(b, rc, "domain %d: %s", i, d->err.c_str());
        m[2 * i + p].th_fresh = 1;  // the step zeroes only the halo ring of th_tendency
      } else if ((rc = make_mix_args(d, taum1, tau, taup1, dtime, &mx[2 * i + p]))) {
        return bfail(b, rc, "domain %d: %s", i, d->err.c_str());
      } else {
        // both parities or neither: a domain's tiles are all staged or all plain
        int tr = fill_batch_tma(d, mx[2 * i + p], tma.data() + tb * (2 * i + p));
        if (tr != MOM5GPU_OK && tr != MOM5GPU_EUNSUPPORTED) return bfail(b, tr, "domain %d: %s", i, d->err.c_str());
        b->tma_ok[i] = (p == 0 ? tr == MOM5GPU_OK : b->tma_ok[i] && tr == MOM5GPU_OK) ? 1 : 0;
      }
      if ((rc = make_bt_args(d, tau, taup1, &bt[2 * i + p], &bx[2 * i + p])))
        return bfail(b, rc, "domain %d: %s", i, d->err.c_str());
    }
  }
  cudaError_t e = cudaSuccess;
  if (b->prec == MOM5GPU_PRECISION_FP64) {
    e = cudaMemcpyAsync(b->d_mdfl, m.data(), sizeof(MdflArgs) * 2 * n, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_upd, u.data(), sizeof(UpdArgs) * 2 * n, cudaMemcpyHostToDevice, b->stream);
  } else {
    e = cudaMemcpyAsync(b->d_mix, mx.data(), sizeof(MixArgs) * 2 * n, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_tma, tma.data(), tma.size(), cudaMemcpyHostToDevice, b->stream);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_bt, bt.data(), sizeof(BtArgs) * 2 * n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_btx, bx.data(), sizeof(BtExtra) * 2 * n, cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bfail(b, MOM5GPU_ECUDA, "descriptor upload: %s", cudaGetErrorString(e));
  b->desc_dtime = dtime;
  for (int p = 0; p < 2; ++p) b->g_key[p] = -1;  // graphs hold the old descriptors' dtime
  return MOM5GPU_OK;
}

// Work list of (domain, parity) entries as ints: entries, then the prefix sums of
// the passes z, x, y, update, 2-D barotropic, 1-D barotropic, precision form
// (plain tiles), precision form (TMA-staged tiles).
void fill_work(const mom5gpu_batch* b, const std::vector<std::pair<int, int>>& list, std::vector<int>& h, BatchWork& w) {
  int c = (int)list.size();
  int TJ = tj_of(b);
  std::vector<std::pair<int, int>> order(list);
  // largest domains first: the persistent kernel then ends with small items
  std::stable_sort(order.begin(), order.end(), [&](const std::pair<int, int>& a, const std::pair<int, int>& z) {
    return b->doms[a.first]->geo.n3 > b->doms[z.first]->geo.n3;
  });
  h.assign((size_t)c + 8 * (size_t)(c + 1), 0);
  int* ent = h.data();
  int* pr[8];
  for (int k = 0; k < 8; ++k) pr[k] = ent + c + k * (c + 1);
  for (int e = 0; e < c; ++e) {
    const int dom = order[e].first;
    ent[e] = 2 * dom + order[e].second;
    BatchBlocks bb =
        batch_blocks(b->doms[dom]->geo, TJ, b->rows, dom < (int)b->tma_ok.size() && b->tma_ok[dom], b->ntr);
    int v[8] = {bb.z, bb.x, bb.y, bb.u, bb.b2, bb.b1, bb.m, bb.t};
    for (int k = 0; k < 8; ++k) pr[k][e + 1] = pr[k][e] + v[k];
  }
  w.count = c;
  w.tz = pr[0][c];
  w.tx = pr[1][c];
  w.ty = pr[2][c];
  w.tu = pr[3][c];
  w.tb2 = pr[4][c];
  w.tb1 = pr[5][c];
  w.tm = pr[6][c];
  w.tt = pr[7][c];
}

void bind_work(BatchWork& w, const int* d) {
  int c = w.count;
  w.entries = d;
  const int* p = d + c;
  w.pz = p;
  w.px = p + (c + 1);
  w.py = p + 2 * (c + 1);
  w.pu = p + 3 * (c + 1);
  w.pb2 = p + 4 * (c + 1);
  w.pb1 = p + 5 * (c + 1);
  w.pm = p + 6 * (c + 1);
  w.pt = p + 7 * (c + 1);
}

// every kernel of one batched step, in stream order
int enqueue_step(mom5gpu_batch* b, const BatchWork& w, const std::vector<std::pair<int, int>>& list) {
  cudaStream_t s = b->stream;
  int rc = MOM5GPU_OK;
  long launches = 0;
  if (b->ntr > 0) {
    if (b->prec == MOM5GPU_PRECISION_FP64) {
      for (auto& it : list) {
        mom5gpu_domain* d = b->doms[it.first];
        double* th = fptr(d, MOM5GPU_TH_TENDENCY, 1, 0);
        launch_zero_ring(d->geo, th, (long)b->ntr * d->geo.nk, s);
        ++launches;
      }
      launch_batch_fp64_advection(b->d_mdfl, b->d_upd, w, b->ntr, true, tj_of(b), s);
      launches += 4;
      for (auto& it : list) {
        mom5gpu_domain* d = b->doms[it.first];
        if (!(d->geo.cx || d->geo.cy)) continue;
        double* tp1 = fptr(d, MOM5GPU_TRACER, 1, 2 - it.second);
        launch_halo_fill(d->geo, tp1, b->ntr * d->geo.nk, 3, s);  // every tracer's levels, one after another
        launches += 1;
      }
    } else {
      rc = launch_batch_mixed(b->d_mix, b->d_tma, w, b->ntr, b->rows, b->blocks_per_sm * b->sms, b->sms, b->d_counter,
                              s);
      if (rc) return bfail(b, rc, "precision-form batch launch");
      launches += (w.tm > 0 ? 1 : 0) + (b->rows == 24 && w.tt > 0 ? 1 : 0);
    }
  }
  launch_batch_barotropic_loop(b->d_bt, b->d_btx, w, b->nts, b->stepB, b->prec == MOM5GPU_PRECISION_MIXED, s);
  launch_batch_barotropic_post(b->d_bt, b->d_btx, w, b->nts, b->stepB, 1, s);
  launches += 2 + (b->prec == MOM5GPU_PRECISION_MIXED ? 2 + 2L * b->nts : 1 + 2L * b->nts);
  auto fill = [&](int field) {
    for (auto& it : list) {
      mom5gpu_domain* d = b->doms[it.first];
      if (!(d->geo.cx || d->geo.cy)) continue;
      launch_halo_fill(d->geo, fptr(d, field, 0, 2 - it.second), 1, 3, s);
      ++launches;
    }
  };
  if (b->any_cyclic) {
    fill(MOM5GPU_ETA_T_BAR);
    fill(MOM5GPU_UDRHO_U);
    fill(MOM5GPU_UDRHO_V);
  }
  launch_batch_barotropic_post(b->d_bt, b->d_btx, w, b->nts, b->stepB, 2, s);
  if (b->any_cyclic) {
    fill(MOM5GPU_CONV_RHO_UD_T);
    fill(MOM5GPU_ETA_U);
  }
  launch_batch_barotropic_post(b->d_bt, b->d_btx, w, b->nts, b->stepB, 3, s);
  launches += 2;
  b->launches += launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : bfail(b, MOM5GPU_ECUDA, "batch step launch: %s", cudaGetErrorString(e));
}

// The batch runs on its own stream: first wait for work already queued on each
// stepped domain's stream, afterwards make those streams wait for the batch.
void order_before(mom5gpu_batch* b, const std::vector<int>& doms) {
  for (int i : doms) {
    mom5gpu_domain* d = b->doms[i];
    if (d->stream == b->stream) continue;
    cudaEventRecord(b->dom_ev[i], d->stream);
    cudaStreamWaitEvent(b->stream, b->dom_ev[i], 0);
  }
}

void order_after(mom5gpu_batch* b, const std::vector<int>& doms) {
  cudaEventRecord(b->done_ev, b->stream);
  for (int i : doms) {
    mom5gpu_domain* d = b->doms[i];
    if (d->stream != b->stream) cudaStreamWaitEvent(d->stream, b->done_ev, 0);
  }
}

int tuning_key(const mom5gpu_batch* b) { return (b->rows * 131 + tj_of(b)) * 131 + b->blocks_per_sm; }

int ensure_work(mom5gpu_batch* b, size_t ints) {
  if (ints <= b->work_cap) return MOM5GPU_OK;
  if (b->d_work) {
    cudaStreamSynchronize(b->stream);
    cudaFree(b->d_work);
  }
  b->d_work = nullptr;
  cudaError_t e = cudaMalloc(&b->d_work, ints * sizeof(int));
  if (e != cudaSuccess) return bfail(b, MOM5GPU_ENOMEM, "batch work list: %s", cudaGetErrorString(e));
  b->work_cap = ints;
  return MOM5GPU_OK;
}

int step_all_graph(mom5gpu_batch* b, int p) {
  int key = tuning_key(b);
  if (!b->gexec[p] || b->g_key[p] != key) {
    if (b->gexec[p]) cudaGraphExecDestroy(b->gexec[p]);
    b->gexec[p] = nullptr;
    std::vector<std::pair<int, int>> list;
    for (int i = 0; i < (int)b->doms.size(); ++i) list.push_back({i, p});
    std::vector<int> h;
    BatchWork w;
    fill_work(b, list, h, w);
    if (b->d_work_all[p]) cudaFree(b->d_work_all[p]);
    b->d_work_all[p] = nullptr;
    cudaError_t e = cudaMalloc(&b->d_work_all[p], h.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_work_all[p], h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bfail(b, MOM5GPU_ECUDA, "graph work list: %s", cudaGetErrorString(e));
    bind_work(w, b->d_work_all[p]);
    b->w_all[p] = w;
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bfail(b, MOM5GPU_ECUDA, "begin capture: %s", cudaGetErrorString(e));
    long l0 = b->launches;
    int rc = enqueue_step(b, w, list);
    long per_step = b->launches - l0;
    b->launches = l0;
    e = cudaStreamEndCapture(b->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return bfail(b, MOM5GPU_ECUDA, "end capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->gexec[p], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return bfail(b, MOM5GPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    b->g_key[p] = key;
    b->g_launches[p] = per_step;
  }
  cudaError_t e = cudaGraphLaunch(b->gexec[p], b->stream);
  if (e != cudaSuccess) return bfail(b, MOM5GPU_ECUDA, "graph launch: %s", cudaGetErrorString(e));
  b->launches += b->g_launches[p];
  return MOM5GPU_OK;
}

}  // namespace

extern "C" {

int mom5gpu_batch_create(mom5gpu_domain* const* domains, int n, mom5gpu_batch** out) {
  if (!domains || n <= 0 || !out) return fail(nullptr, MOM5GPU_EINVAL, "batch_create: no domains");
  *out = nullptr;
  mom5gpu_domain* d0 = domains[0];
  for (int i = 0; i < n; ++i) {
    mom5gpu_domain* d = domains[i];
    if (!d) return fail(nullptr, MOM5GPU_EINVAL, "batch_create: domain %d is NULL", i);
    if (d->opt.precision != d0->opt.precision)
      return fail(nullptr, MOM5GPU_EINVAL, "batch_create: domains mix FP64 and precision form");
    if (d->dims.num_prog_tracers != d0->dims.num_prog_tracers)
      return fail(nullptr, MOM5GPU_EINVAL, "batch_create: domains have different tracer counts");
    if (d->dims.horz_grid != MOM5GPU_BGRID)
      return fail(nullptr, MOM5GPU_EUNSUPPORTED, "batch_create: domain %d is a C grid; batches step B-grid domains", i);
    if (!d->baro_ready || d->nts != d0->nts || d->opt.barotropic_time_stepping_B != d0->opt.barotropic_time_stepping_B)
      return fail(nullptr, MOM5GPU_EINVAL, "batch_create: domain %d: barotropic set-up missing or different nts", i);
    if (d->dims.num_prog_tracers > 0 && !d->advect_ready)
      return fail(nullptr, MOM5GPU_ESTATE, "batch_create: domain %d before mom5gpu_tracer_advect_init", i);
    for (int n2 = 0; n2 < d->dims.num_prog_tracers; ++n2)
      if (d->scheme[n2].horz != MOM5GPU_ADVECT_MDFL_SWEBY)
        return fail(nullptr, MOM5GPU_EUNSUPPORTED, "batch_create: domain %d tracer %d is not MDFL Sweby", i, n2 + 1);
    for (int j = 0; j < i; ++j)
      if (domains[j] == d) return fail(nullptr, MOM5GPU_EINVAL, "batch_create: domain %d listed twice", i);
  }
  int ntr = d0->dims.num_prog_tracers;
  if (d0->opt.precision == MOM5GPU_PRECISION_FP64 && ntr > kMdflChunk)
    return fail(nullptr, MOM5GPU_EUNSUPPORTED, "batch_create: FP64 batches take at most %d tracers", kMdflChunk);
  if (d0->opt.precision == MOM5GPU_PRECISION_MIXED && ntr > 10)
    return fail(nullptr, MOM5GPU_EUNSUPPORTED, "batch_create: precision-form batches take at most 10 tracers");
  mom5gpu_batch* b = new (std::nothrow) mom5gpu_batch();
  if (!b) return fail(nullptr, MOM5GPU_ENOMEM, "batch_create: host allocation");
  b->doms.assign(domains, domains + n);
  b->prec = d0->opt.precision;
  b->ntr = ntr;
  b->nts = d0->nts;
  b->stepB = d0->opt.barotropic_time_stepping_B;
  for (auto* d : b->doms) b->any_cyclic |= (d->geo.cx || d->geo.cy);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
  b->stream = b->own;
  if (e == cudaSuccess) e = cudaEventCreate(&b->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->e1);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done_ev, cudaEventDisableTiming);
  b->dom_ev.assign(n, nullptr);
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->dom_ev[i], cudaEventDisableTiming);
  size_t nd = 2 * (size_t)n;
  if (e == cudaSuccess) e = cudaMalloc(&b->d_bt, sizeof(BtArgs) * nd);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_btx, sizeof(BtExtra) * nd);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counter, 2 * sizeof(int));
  if (e == cudaSuccess && b->prec == MOM5GPU_PRECISION_FP64) {
    e = cudaMalloc(&b->d_mdfl, sizeof(MdflArgs) * nd);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_upd, sizeof(UpdArgs) * nd);
  } else if (e == cudaSuccess) {
    e = cudaMalloc(&b->d_mix, sizeof(MixArgs) * nd);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tma, batch_tma_bytes() * nd);
  }
  if (e != cudaSuccess) {
    mom5gpu_batch_destroy(b);
    return fail(nullptr, MOM5GPU_ENOMEM, "batch_create: %s", cudaGetErrorString(e));
  }
  if (b->prec == MOM5GPU_PRECISION_FP64) {
    for (auto* d : b->doms) {
      int rc = ensure_mdfl_scratch(d, ntr);
      if (rc) {
        std::string msg = d->err;
        mom5gpu_batch_destroy(b);
        return fail(nullptr, rc, "batch_create: %s", msg.c_str());
      }
    }
  } else {
    int rc = prepare_batch_mixed();
    if (!rc) rc = prepare_batch_mixed_tma();
    if (rc) {
      mom5gpu_batch_destroy(b);
      return fail(nullptr, rc, "batch_create: kernel attributes");
    }
  }
  *out = b;
  return MOM5GPU_OK;
}

void mom5gpu_batch_destroy(mom5gpu_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (int p = 0; p < 2; ++p) {
    if (b->gexec[p]) cudaGraphExecDestroy(b->gexec[p]);
    if (b->d_work_all[p]) cudaFree(b->d_work_all[p]);
  }
  for (void* p : {(void*)b->d_mdfl, (void*)b->d_upd, (void*)b->d_bt, (void*)b->d_btx, (void*)b->d_mix, (void*)b->d_work,
                  (void*)b->d_counter, (void*)b->d_tma})
    if (p) cudaFree(p);
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  if (b->done_ev) cudaEventDestroy(b->done_ev);
  for (cudaEvent_t ev : b->dom_ev)
    if (ev) cudaEventDestroy(ev);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
}

const char* mom5gpu_batch_last_error(const mom5gpu_batch* b) { return b ? b->err.c_str() : ""; }

int mom5gpu_batch_set_stream(mom5gpu_batch* b, void* stream) {
  if (!b) return MOM5GPU_EINVAL;
  b->stream = stream ? (cudaStream_t)stream : b->own;
  return MOM5GPU_OK;
}

int mom5gpu_batch_step(mom5gpu_batch* b, const int* index, const int* parity, int count, double dtime) {
  if (!b) return MOM5GPU_EINVAL;
  if (count == 0) return MOM5GPU_OK;
  if (count < -1) return bfail(b, MOM5GPU_EINVAL, "batch_step: count %d", count);
  if (dtime != b->desc_dtime) {
    int rc = build_descriptors(b, dtime);
    if (rc) return rc;
  }
  std::vector<int> stepped;
  int rc;
  if (count == -1) {
    int p = parity ? parity[0] : 0;
    if (p != 0 && p != 1) return bfail(b, MOM5GPU_EINVAL, "batch_step: parity %d", p);
    for (int i = 0; i < (int)b->doms.size(); ++i) stepped.push_back(i);
    order_before(b, stepped);
    cudaEventRecord(b->e0, b->stream);
    rc = step_all_graph(b, p);
  } else {
    if (!index || !parity) return bfail(b, MOM5GPU_EINVAL, "batch_step: null index or parity");
    std::vector<std::pair<int, int>> list;
    std::vector<char> seen(b->doms.size(), 0);
    for (int i = 0; i < count; ++i) {
      if (index[i] < 0 || index[i] >= (int)b->doms.size() || (parity[i] != 0 && parity[i] != 1))
        return bfail(b, MOM5GPU_EINVAL, "batch_step: entry %d (domain %d, parity %d)", i, index[i], parity[i]);
      if (seen[index[i]]) return bfail(b, MOM5GPU_EINVAL, "batch_step: domain %d listed twice", index[i]);
      seen[index[i]] = 1;
      list.push_back({index[i], parity[i]});
    }
    for (auto& it : list) stepped.push_back(it.first);
    std::vector<int> h;
    BatchWork w;
    fill_work(b, list, h, w);
    if ((rc = ensure_work(b, h.size()))) return rc;
    order_before(b, stepped);
    cudaEventRecord(b->e0, b->stream);
    // pageable source: the call returns once the list is staged, so h may go out of scope
    cudaError_t e = cudaMemcpyAsync(b->d_work, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return bfail(b, MOM5GPU_ECUDA, "work list upload: %s", cudaGetErrorString(e));
    bind_work(w, b->d_work);
    rc = enqueue_step(b, w, list);
  }
  cudaEventRecord(b->e1, b->stream);
  order_after(b, stepped);
  return rc;
}

double mom5gpu_batch_last_ms(mom5gpu_batch* b) {
  if (!b) return -1.0;
  float ms = 0.f;
  if (cudaEventSynchronize(b->e1) != cudaSuccess) return -1.0;
  cudaEventElapsedTime(&ms, b->e0, b->e1);
  b->last_ms = ms;
  return ms;
}

long mom5gpu_batch_launch_count(const mom5gpu_batch* b) { return b ? b->launches : 0; }

int mom5gpu_batch_get_tuning(const mom5gpu_batch* b, int* rows, int* tj, int* blocks_per_sm) {
  if (!b || !rows || !tj || !blocks_per_sm) return MOM5GPU_EINVAL;
  *rows = b->rows;
  *tj = b->tj;
  *blocks_per_sm = b->blocks_per_sm;
  return MOM5GPU_OK;
}

int mom5gpu_batch_set_tuning(mom5gpu_batch* b, int rows, int tj, int blocks_per_sm) {
  if (!b) return MOM5GPU_EINVAL;
  if (rows != 16 && rows != 24 && rows != 32) return bfail(b, MOM5GPU_EINVAL, "set_tuning: rows %d (16, 24 or 32)", rows);
  if (tj != 0 && tj != 2 && tj != 4 && tj != 8 && tj != 16)
    return bfail(b, MOM5GPU_EINVAL, "set_tuning: tj %d (0, 2, 4, 8 or 16)", tj);
  if (blocks_per_sm < 1 || blocks_per_sm > 4)
    return bfail(b, MOM5GPU_EINVAL, "set_tuning: blocks_per_sm %d (1..4)", blocks_per_sm);
  b->rows = rows;
  b->tj = tj;
  b->blocks_per_sm = blocks_per_sm;
  return MOM5GPU_OK;
}

int mom5gpu_batch_autotune(mom5gpu_batch* b, double dtime, char* report, size_t report_len) {
  if (!b) return MOM5GPU_EINVAL;
  struct Cand {
    int rows, tj, bps;
  };
  static const Cand kMixed[] = {{32, 0, 1}, {32, 0, 2}, {16, 0, 2}, {16, 0, 3}, {16, 0, 4}, {24, 0, 2}};
  static const Cand kFp64[] = {{32, 2, 2}, {32, 4, 2}, {32, 8, 2}, {32, 16, 2}};
  std::vector<Cand> cands = b->prec == MOM5GPU_PRECISION_MIXED ? std::vector<Cand>(kMixed, kMixed + 6)
                                                                 : std::vector<Cand>(kFp64, kFp64 + 4);
  std::vector<int> idx(b->doms.size()), par(b->doms.size(), 0);
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
  std::string rep;
  double best = 1e30;
  Cand bestc = cands[0];
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  for (const Cand& c : cands) {
    b->rows = c.rows;
    b->tj = c.tj;
    b->blocks_per_sm = c.bps;
    int rc = mom5gpu_batch_step(b, idx.data(), par.data(), (int)idx.size(), dtime);  // warm-up
    if (rc) {
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
      return rc;
    }
    cudaEventRecord(t0, b->stream);
    for (int r = 0; r < 3; ++r) {
      rc = mom5gpu_batch_step(b, idx.data(), par.data(), (int)idx.size(), dtime);
      if (rc) break;
    }
    cudaEventRecord(t1, b->stream);
    cudaError_t e = cudaEventSynchronize(t1);
    if (rc || e != cudaSuccess) {
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
      return rc ? rc : bfail(b, MOM5GPU_ECUDA, "autotune: %s", cudaGetErrorString(e));
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    ms /= 3.f;
    char line[128];
    snprintf(line, sizeof(line), "rows=%d tj=%d blocks/SM=%d: %.3f ms; ", c.rows, c.tj, c.bps, ms);
    rep += line;
    if (ms < best) {
      best = ms;
      bestc = c;
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  b->rows = bestc.rows;
  b->tj = bestc.tj;
  b->blocks_per_sm = bestc.bps;
  char line[128];
  snprintf(line, sizeof(line), "chosen rows=%d tj=%d blocks/SM=%d", bestc.rows, bestc.tj, bestc.bps);
  rep += line;
  if (report && report_len) {
    strncpy(report, rep.c_str(), report_len - 1);
    report[report_len - 1] = 0;
  }
  return MOM5GPU_OK;
}

}  // extern "C"
