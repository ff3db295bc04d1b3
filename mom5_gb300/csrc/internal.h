// Internal declarations shared by the C-ABI layer and the kernel files.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mom5gpu.h"

namespace mom5 {

// Geometry passed by value to every kernel.
struct Geo {
  int ni, nj, nk;   // compute domain
  int nxd, nyd;     // data domain (halo 1)
  int cx, cy;       // cyclic flags
  long n2;          // nxd*nyd
  long n3;          // n2*nk
};

// Field shape classes.
enum Shape { S2D = 0, S3D = 1, S3DW = 2 };

struct FieldInfo {
  int id;
  Shape shape;
  bool per_tracer;
  bool per_level;
};

const FieldInfo* field_info(int id);

// Per-tracer scheme selection (field_table).
struct TracerScheme {
  int horz = MOM5GPU_ADVECT_MDFL_SWEBY;
  int vert = MOM5GPU_ADVECT_MDFL_SWEBY;
  double min_limit = -1.0e10;
  double max_limit = 1.0e10;
  int ppm_limiter = 2;  // ppm_hlimiter (ocean_tpm_util.F90:87): 1 cw84, 2 ifc, 3 sh
  int psom_limit = 0;   // psom_limit (ocean_tpm_util.F90:86)
};

// Quicker weights on the device (quicker_init, ocean_tracer_advect.F90:1442-1586).
struct QuickerWeights {
  double* quick_x = nullptr;  // 2 * n2
  double* quick_y = nullptr;  // 2 * n2
  double* curv_xp = nullptr;  // 3 * n2
  double* curv_xn = nullptr;
  double* curv_yp = nullptr;
  double* curv_yn = nullptr;
  double* quick_z = nullptr;  // 2 * nk
  double* curv_zp = nullptr;  // 3 * nk
  double* curv_zn = nullptr;
};

}  // namespace mom5

struct mom5gpu_domain {
  mom5gpu_dims dims;
  mom5gpu_options opt;
  mom5::Geo geo;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  size_t bytes = 0;
  // one allocation per field id; nullptr until first set/used
  std::vector<double*> field;  // indexed by field id
  std::vector<mom5::TracerScheme> scheme;
  std::vector<std::string> tracer_name, tracer_file;  // T_prog(n)%name, %restart_file
  // host copies needed at init time
  std::vector<double> dzt_h, zw_h;
  std::vector<int> kmt_h;
  // derived device data
  uint8_t* mask2 = nullptr;  // tmask with a 2-cell halo (tmask_mdfl / tmask_quick), (ni+4)(nj+4)nk
  mom5::QuickerWeights qw;
  double* cori1 = nullptr;
  double* cori2 = nullptr;
  bool advect_ready = false;
  bool baro_ready = false;
  int nts = 0;
  double dtuv = 0.0, dtbt = 0.0;
  // scratch
  double* mdfl_a = nullptr;  // tracer_mdfl after the z pass, ntr * n3
  double* mdfl_b = nullptr;  // after the x pass, ntr * n3
  size_t mdfl_cap = 0;       // tracers that fit
  float* mixed_scr = nullptr;  // precision-form scratch
  size_t mixed_cap = 0;
  double* bt = nullptr;        // barotropic scratch
  int* kmt_d = nullptr;        // device copy of kmt (uploaded on first use)
  double* ppm_scr = nullptr;   // MDPPM slope and vertical-flux scratch, 2 x n3
  double* psom_scr = nullptr;  // PSOM mass and x/y/z face fluxes, 4 x n3
  long itt0 = 0;               // Time%itt0 (orders the PSOM sweeps)
  double* red = nullptr;       // reduction scratch (device)
  double* red_h = nullptr;     // pinned host result
  int* flag = nullptr;         // device flag word
  // profiling
  bool timing = false;
  struct Clock {
    int section;
    cudaEvent_t a, b;
  };
  std::vector<Clock> clocks;           // recorded, not yet resolved
  std::vector<cudaEvent_t> event_pool;
  double clock_ms[8] = {0};
  long clock_calls[8] = {0};
  long launches = 0;
  // autotuned launch shapes (0 = built-in heuristic)
  int tune_mixed_rows = 32;  // precision-form tile height incl. halo: 16, 24, 32 or 64
  int tune_mixed_pf = 0;     // precision form: 1 tracer levels prefetched by cp.async (height 16), 2 TMA-staged tiles
  int* wait_err = nullptr;   // set when a bounded device wait gave up: bit 0 a TMA-staged copy, bit 1 a grid barrier
  unsigned* bt_sync = nullptr;  // arrival counter of the cooperative barotropic subcycle's grid barriers
  int tune_y_tj = 0;         // FP64 y-pass rows per thread
  int bt_fused = 0;          // exact B-grid subcycles: 0 three launches each, 1 one launch each,
                             // 2 all in one cooperative launch
  int coop_blocks = 0;       // resident blocks per SM of the cooperative subcycle kernel (0: not queried, -1: none)
  int coop_sms = 0;          // SMs of the device
  // CUDA graphs of the barotropic subcycle loop, one per set of kernel arguments
  // (the bytes of the BtArgs it was captured with: time levels rotate), at most
  // kBtGraphs, the oldest replaced first
  struct BtGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> key;
  };
  std::vector<BtGraph> bt_graphs;
  // domain decomposition (decomp.cu): sides facing a neighbouring subdomain
  // (bits 1 west, 2 east, 4 south, 8 north) and the MDFL halo strips
  int nbr = 0;
  double* hz = nullptr;  // tracer_mdfl after z, columns -1, 0, ni+1, ni+2: ntr*nk*nj*4
  double* hx = nullptr;  // after x, rows -1, 0, nj+1, nj+2: ntr*nk*4*ni
};

namespace mom5 {

// error helpers (capi.cu)
int fail(mom5gpu_domain* d, int code, const char* fmt, ...);
int cuda_fail(mom5gpu_domain* d, cudaError_t e, const char* where);
double* fptr(mom5gpu_domain* d, int id, int n, int level);  // nullptr if absent
double* fptr_if_set(mom5gpu_domain* d, int id, int n, int level);  // nullptr if never allocated
size_t field_count(const Geo& g, Shape s);

// profiling sections
enum Section { SEC_MDFL = 0, SEC_MDFL_MIXED, SEC_UPDATE, SEC_BAROTROPIC, SEC_UPWIND, SEC_QUICKER, SEC_BATCH, SEC_N };
// RAII: events around a section when timing is on
struct ClockScope {
  mom5gpu_domain* d;
  int sec;
  cudaEvent_t a = nullptr;
  ClockScope(mom5gpu_domain* d_, int s);
  ~ClockScope();
};
inline void count_launches(mom5gpu_domain* d, long n) { d->launches += n; }

// Arguments of the FP64 MDFL passes (k_fp64.cu).
struct MdflArgs {
  Geo g;
  int ntr;
  double dtime;
  const uint8_t* mask2;  // tmask_mdfl
  const double *dat, *datr, *dxte, *dyte, *dxtn, *dytn;
  const double *uh, *vh, *w;  // uhrho_et, vhrho_nt, wrho_bt (0:nk)
  const double* rdz;          // rho_dzt(tau)
  const double* T;            // tracer 0 at taum1; tracer n at T + n*tstride
  long tstride;
  double* tz;                 // after z, tracer n at tz + n*g.n3
  double* tx;                 // after x
  double* th;                 // th_tendency of tracer 0, tracer n at th + n*g.n3
  int tj = 0;                 // y-pass rows per thread (0 = choose from the domain size)
  int th_fresh = 0;           // th is +0 at every compute cell: the y pass writes out + 0.0 instead of th + out
  // decomposed domains: sides whose halo comes from a neighbouring subdomain
  // (bits 1 west, 2 east, 4 south, 8 north) and the strips its exchange filled:
  // tracer_mdfl after the z pass at i = -1, 0, ni+1, ni+2 (hz[((n*nk + k)*nj + j-1)*4 + slot])
  // and after the x pass at j = -1, 0, nj+1, nj+2 (hx[((n*nk + k)*4 + slot)*ni + i-1])
  int nbr = 0;
  const double* hz = nullptr;
  const double* hx = nullptr;
};


// Arguments of the barotropic kernels (fp64_bodies.cuh) for one domain and one
// (tau, taup1) pair, and the step's other inputs and outputs.
// Largest number of tracers the FP64 MDFL kernels advect per launch set.
constexpr int kMdflChunk = 10;

struct BtArgs {
  Geo g;
  int cgrid, nts, stepB;
  double dtbt, dtbt_gamma_rho0r, dtbt_rho0r, gamma;
  const double *tmask1, *umask1, *f, *dxu, *dyu, *dxur, *dyur, *dat, *datr, *dxter, *dytnr, *tmen_e, *tmen_n;
  const double *dte, *dtw, *dus, *dun, *daur;
  const double *patm, *thicku, *thicken_e, *thicken_n, *forcing_u, *forcing_v, *rho_g, *cori1, *cori2;
  double* eta_bt;  // 2 levels
  double* ubt;     // 2 levels
  double* vbt;     // 2 levels
  double* steady;
  double* ps;
  double* cf;  // coriolis_force_bt, 6 planes (component-major within AB level)
  double* ca;  // coriolis_accel_bt, 2 planes
  double *eta_bar, *udrho_u, *udrho_v;  // taup1 accumulators
  double *uhb, *vhb;  // B grid: ubt*dyu and vbt*dxu, 2 levels like ubt (reuse the C-grid Coriolis planes)
  double* btf;        // precision form, B grid: folded step coefficients (bt_fast_body.cuh), else nullptr
  double* dvs;        // divergence of the corrector's transports, reused by the next subcycle's predictor
};
// planes of barotropic scratch: 18 for the exact path (the reused divergence in
// two planes for the one-launch subcycle), 9 more for the precision form
constexpr int kBtPlanes = 18, kBtFastPlanes = 10;
struct BtExtra {
  const double *eta_bar_tau, *eta_tau, *ud_tau, *vd_tau, *pme, *river, *source, *eta_smooth;
  double *conv, *eta_u, *ps_out, *gxo, *gyo;
  int initsum_with_bar;
};

// Arguments of the precision-form kernel (mixed_body.cuh).
struct MixArgs {
  Geo g;
  int ntr;
  float dtime;
  const uint8_t* mask2;
  const double *dat, *datr, *dxte, *dyte, *dxtn, *dytn, *uh, *vh, *w;
  const double *rdz, *rdz_m1, *rdzr;  // rho_dzt(tau), rho_dzt(taum1), rho_dztr
  const double* T;                    // tracer 0 at taum1 (tracer n at + n*g.n3)
  double* out;                        // fused: T(taup1); else th_tendency (tracer n at + n*g.n3)
  int fused;
};

// Arguments of the FP64 explicit update.
struct UpdArgs {
  Geo g;
  int ntr;
  long tstride;
  const double *rdz_m1, *rdzr, *Tm1, *th;
  double* Tp1;
  double dtime;
};

// argument builders (k_fp64.cu, k_mixed.cu); status codes as the C ABI
int make_mdfl_args(mom5gpu_domain* d, int n_first, int ntr, int taum1, int tau, double dtime, MdflArgs* a);
int make_upd_args(mom5gpu_domain* d, int taum1, int taup1, double dtime, UpdArgs* u);
int make_bt_args(mom5gpu_domain* d, int tau, int taup1, BtArgs* a, BtExtra* x);
int make_mix_args(mom5gpu_domain* d, int taum1, int tau, int taup1, double dtime, MixArgs* a);

// ---- FP64 kernels (k_fp64.cu) ----
// the three MDFL passes on the stream, for the tracers described by a
// (at most 8 per call); scratch a.tz/a.tx and a.mask2 are the caller's.
void run_mdfl_kernels(const MdflArgs& a, bool all, bool sweby, cudaStream_t s);
void run_mdfl_pass(const MdflArgs& a, bool all, bool sweby, int pass, cudaStream_t s);
int launch_barotropic_phase(mom5gpu_domain* d, int tau, int taup1, int phase, int itime);
void launch_halo_fill(const Geo& g, double* a, int nlev, int flags, cudaStream_t s);
void launch_zero_ring(const Geo& g, double* a, long nlev, cudaStream_t s);
int launch_mdfl(mom5gpu_domain* d, bool all, int n_first, int ntr, int taum1, int tau, double dtime,
                double sweby_limiter, bool th_fresh = false);
int launch_upwind_horz(mom5gpu_domain* d, int n, int taum1);
int launch_upwind_vert(mom5gpu_domain* d, int n, int taum1);
int launch_quicker_horz(mom5gpu_domain* d, int n, int taum1, int tau);
int launch_quicker_vert(mom5gpu_domain* d, int n, int taum1, int tau);
int launch_update_tracer(mom5gpu_domain* d, int n_first, int ntr, int taum1, int taup1, double dtime);
int launch_tmask_limit(mom5gpu_domain* d, int n, int tau);
int launch_tmask_limit_ts_same(mom5gpu_domain* d, int nt, int ns);
int launch_eta_tendency(mom5gpu_domain* d, int tau);
int launch_eta_update(mom5gpu_domain* d, int taum1, int taup1, double dtime);
// Programmatic dependent launch of the barotropic subcycle kernels.  A kernel
// launched by launch_pdl may be scheduled while the kernel before it in the
// stream runs its last blocks; its blocks first wait in pdl_wait()
// (griddepcontrol.wait) until that kernel has completed and its writes are
// visible, then allow the next kernel to be scheduled (pdl_trigger), so every
// kernel still reads only completed results.  Launched the ordinary way, the
// two instructions do nothing.
#ifdef __CUDACC__
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
#endif
template <typename... P, typename... A>
cudaError_t launch_pdl(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t s, A... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// precision-form barotropic subcycle (k_mixed.cu, k_batch.cu)
void launch_btf_prep(const BtArgs& a, cudaStream_t s);
int launch_btf_subcycle(const BtArgs& a, int itime, int nts, bool fused, cudaStream_t s);
int launch_centred(mom5gpu_domain* d, int n, int tau, int order, bool horz);
int ensure_kmt_device(mom5gpu_domain* d);
int launch_mdfl_sup_b(mom5gpu_domain* d, int n, int taum1, int tau, double dtime);
int launch_mdppm(mom5gpu_domain* d, int n, int taum1, int tau, double dtime);
int launch_psom(mom5gpu_domain* d, int n, int taum1, double dtime);
int launch_quickmom3_horz(mom5gpu_domain* d, int n, int taum1, int tau);
int launch_tracer_boundary(mom5gpu_domain* d, int n);
int launch_barotropic_forcing(mom5gpu_domain* d, int tau);  // tau 0: no friction
int launch_update_ucell_thickness(mom5gpu_domain* d, int taup1, int vcoord, bool linear_fs, bool dzwu_k0);
int launch_advection_velocity(mom5gpu_domain* d, int tau);
int launch_barotropic(mom5gpu_domain* d, int tau, int taup1);
int grid_barrier_selftest(mom5gpu_domain* d, int rounds, int unreachable);
int launch_content(mom5gpu_domain* d, int n, int level, double* out_host);
int launch_content_fixed(mom5gpu_domain* d, int n, int level, long long* acc_host);
int launch_eta_integral(mom5gpu_domain* d, const double* eta, double* out_host);
int launch_check_finite(mom5gpu_domain* d, const double* a, size_t count, int* out_host);

// FP64 MDFL scratch of a domain, for ntr tracers at a time (k_fp64.cu)
int ensure_mdfl_scratch(mom5gpu_domain* d, int ntr);

// ---- batched launches (k_batch64.cu, k_batch.cu) ----
// One work list in device memory: entries[e] is the descriptor index of entry
// e; p*[e] is the first block of entry e in each pass (p*[count] = total).
struct BatchWork {
  const int* entries;
  const int *pz, *px, *py, *pu, *pb2, *pb1, *pm, *pt;
  int count;
  int tz, tx, ty, tu, tb2, tb1, tm, tt;  // total blocks of each pass
};
// blocks of one domain in each pass, for the work-list prefix sums; t: the
// TMA-staged precision tiles (mixed_rows 24 on a domain that allows them)
struct BatchBlocks {
  int z, x, y, u, b2, b1, m, t;
};
BatchBlocks batch_blocks(const Geo& g, int TJ, int mixed_rows, bool tma, int ntr);
// FP64: z/x/y MDFL passes and the explicit update for every entry
void launch_batch_fp64_advection(const MdflArgs* mdfl, const UpdArgs* upd, const BatchWork& w, int ntr, bool sweby,
                                 int TJ, cudaStream_t s);
// the barotropic step (init, nts x (pred, mom, corr), post) for every entry; halo fills of
// cyclic domains are issued by the caller between the post phases
void launch_batch_barotropic_loop(const BtArgs* bt, const BtExtra* x, const BatchWork& w, int nts, int stepB, bool fast,
                                  cudaStream_t s);
// precision form: folded subcycle over the work list (k_batch.cu)
// precision form, TMA-staged 24-row tiles over a batch's work list (k_mixed_tma.cu):
// the bytes of one (domain, parity) entry of the device table, filling an entry
// (MOM5GPU_EUNSUPPORTED when the domain cannot be described to TMA), the launch
size_t batch_tma_bytes();
int batch_tma_rows(int ntr);
int fill_batch_tma(mom5gpu_domain* d, const MixArgs& a, void* host_entry);
int launch_batch_mixed_tma(const MixArgs* mix, const void* tma, const BatchWork& w, int ntr, int blocks, int* counter,
                           cudaStream_t s);
void launch_batch_btf_prep(const BtArgs* bt, const BatchWork& w, cudaStream_t s);
int launch_batch_btf_subcycle(const BtArgs* bt, const BatchWork& w, int itime, int nts, cudaStream_t s);
void launch_batch_barotropic_post(const BtArgs* bt, const BtExtra* x, const BatchWork& w, int nts, int stepB, int phase,
                                  cudaStream_t s);
// precision form: persistent kernel over (entry, tile) items
// rows 16 or 32: the plain persistent tile kernel; rows 24: the TMA-staged tiles
// (table tma, counter[1]) and the plain 32-row tiles for the other domains
int launch_batch_mixed(const MixArgs* mix, const void* tma, const BatchWork& w, int ntr, int rows, int blocks,
                       int sms, int* counter, cudaStream_t s);
// sets the shared-memory attribute of every instantiation (before any graph capture)
int prepare_batch_mixed();
int prepare_batch_mixed_tma();

// ---- precision form (k_mixed.cu) ----
int launch_mdfl_mixed(mom5gpu_domain* d, int n_first, int ntr, int taum1, int tau, int taup1, double dtime,
                      bool fused_update);
// TMA-staged variant of one launch (k_mixed_tma.cu); MOM5GPU_EUNSUPPORTED: use the plain kernel
int ensure_wait_words(mom5gpu_domain* d);
int launch_mixed_tma(mom5gpu_domain* d, const MixArgs& a, int n0, const double* Tall, int zt0, int ntr_all);

}  // namespace mom5
