// Precision form of MDFL Sweby with its tiles staged into shared memory by TMA.
//
// The same method and the same FP32 arithmetic, operation for operation (the
// helpers of mixed_body.cuh, every product and sum rounded on its own), as the
// plain tile kernel, so every result is bit-identical to it: a tile of 28
// columns by ZR-4 rows with its 2-cell halo recomputed, marching down k, the
// face terms of a level shared by every tracer of the launch.  What changes is
// where the operands come from and how often the block synchronises:
//   * one tile position per thread (a warp per tile row), the tracers' levels
//     k-1, k, k+1 carried down the column (in a shared-memory ring or in
//     registers), so each level of each tracer is brought on chip once instead
//     of four times;
//   * two block barriers per level (after the z and x passes of every tracer
//     and after the y fluxes of every tracer), the per-tracer intermediates in
//     shared memory, instead of two barriers per tracer;
//   * the level that enters the window (k+2) arrives by TMA
//     (cp.async.bulk.tensor, completion on an mbarrier) into one shared-memory
//     slot per tracer, requested as soon as the slot is free -- one level and
//     the rest of the tracers ahead of its use;
//   * the level's fields (uhrho_et, vhrho_nt, wrho_bt, rho_dzt(tau),
//     rho_dztr, rho_dzt(taum1)) arrive by TMA one level ahead, with the
//     neighbours the face terms need in the same box;
//   * the 2-D metrics are read once per tile into registers.
// A TMA box is 34 columns wide starting at an even column (16-byte aligned for
// FP64), covering the tile's 32 columns and the +-1 neighbours.  Box cells
// outside the data domain read as zero; tile positions outside the compute
// domain (halo columns and rows, periodic images) take their values from
// global memory at their image, exactly as the plain kernel does, so the seam
// of a periodic domain needs no special box.  Requires an even ni (row stride
// a multiple of 16 bytes); the launcher falls back to the plain kernel
// otherwise.
//
// Every wait on an mbarrier is bounded; a wait that gives up sets *err, the
// block stops at its next barrier (after waiting, again bounded, for the
// copies it issued) and mom5gpu_synchronize reports MOM5GPU_ETIMEDOUT.
// Tile heights 16 and 24 (the per-tracer intermediates of 10 tracers at 32 rows
// would not fit in shared memory); at height 16 also with at most 5 tracers per
// block and two blocks per SM.
#include <cuda.h>
#include <math.h>
#include <string.h>

#include "mixed_body.cuh"

namespace mom5 {

using namespace mixed;

namespace {

constexpr int BX = 34;  // box width: tile columns i0-3 .. i0+30

struct TmaMaps {
  CUtensorMap T, f[6];  // tracers (every tracer of the time level), then the fields below
};
enum { F_UH = 0, F_VH, F_W, F_RDZ, F_RDZR, F_RDZM1 };

DEVI unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
DEVI void mbar_init(uint64_t* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(b)) : "memory");
}
DEVI void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
DEVI void mbar_inval(uint64_t* b) { asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(su32(b)) : "memory"); }
DEVI void mbar_expect(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
DEVI void tma3(void* dst, const CUtensorMap* m, int x, int y, int z, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(su32(dst)),
      "l"(reinterpret_cast<unsigned long long>(m)), "r"(x), "r"(y), "r"(z), "r"(su32(b))
      : "memory");
}
DEVI bool mbar_test(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of an mbarrier: false after kSpin polls (each
// poll itself waits a hardware-chosen while before it reports not ready).
constexpr unsigned kSpin = 1u << 22;
DEVI bool mbar_wait(uint64_t* b, unsigned parity) {
  for (unsigned it = 0; it < kSpin; ++it)
    if (mbar_test(b, parity)) return true;
  return false;
}

// Where the window of each tracer (levels k-1, k, k+1 in FP32 and the flux
// through the top face) lives (WM): 0 all in registers; 1 the top-face flux in
// shared memory, the levels in registers; 2 all in shared memory, the levels as
// a ring of three (level L in slot L mod 3).  Moving state to shared memory
// frees registers for the kernel's own scheduling: 35 in the 10-tracer 16-row
// kernel (WM 2, measured 1.8% faster), 10 in the 24-row kernel (WM 1), whose
// shared memory has room for no more.
template <int NC, int ZR, int WM>
struct WindowStore {};
template <int NC, int ZR>
struct WindowStore<NC, ZR, 1> {
  float ftp[NC][ZR * 32];
};
template <int NC, int ZR>
struct WindowStore<NC, ZR, 2> {
  float win[3][NC][ZR * 32];
  float ftp[NC][ZR * 32];
};

template <int NC, int ZR, int WM>
struct TmaSmem {
  static constexpr int SLOT = ZR * BX;  // doubles per box (a multiple of 16: 128-byte aligned slots)
  double t[NC][SLOT];                   // level k+2 of each tracer
  double f[6][SLOT];                    // the level's fields
  float tx[NC][ZR * 32];                // each tracer after the x pass
  float fzx[NC][ZR * 32];               // its z + x increment
  float fy[NC][ZR * 32];                // its y fluxes
  uint8_t wet[ZR * 32];                 // tmask at level k
  alignas(8) uint64_t bar[NC + 1];      // one per tracer slot, one for the fields
  int pending[NC + 1];                  // 1 + parity of a phase in flight, 0 = none (thread 0's bookkeeping)
  WindowStore<NC, ZR, WM> ws;
};
// as much of the window in shared memory as fits beside one block per SM
template <int NC, int ZR, int MINB>
constexpr int kWindowMode = MINB != 1 ? 0 : ZR == 16 ? 2 : 1;

// The FP64 T(k) that the state update of each tracer adds to is read from global
// memory (the FP32 window cannot supply it).  The compiler cannot tell T from
// T(taup1), so it keeps every load after the stores that precede it in the code;
// loaded one tracer at a time, each load would wait a full L2 round trip with
// nothing else to do.  Instead a ring of kOutRing loads is kept in flight: the
// first kOutRing are requested before the y fluxes, and tracer n+kOutRing's as
// soon as tracer n's value is used (measured on the C2 grid: 12.7 ms per step
// against 14.3 ms loading one at a time; rings of 2 and 3, and groups loaded
// together before their stores, were slower).
constexpr int kOutRing = 4;

// One level is three phases: (1) the level's face terms, (2) the z and x passes
// of every tracer, (3) the y fluxes of every tracer, then the outputs, with a
// block barrier after phases 2 and 3 -- two barriers per level whatever the
// tracer count.  Phase 1 reads only the field boxes and its own registers, so it
// runs into phase 2 without one; the next level's field boxes are fetched after
// the phase 2 barrier, which every thread reaches only once its phase 1 is done.
// One tile (tile_x, tile_y) of the domain a, with the block's whole shared memory;
// false when a bounded wait gave up (*err set; the block must stop).  The
// barriers are initialised at the start and invalidated at the end, so a
// persistent block can run tile after tile.
template <int NC, int ZR, int MINB>
DEVI bool tma_tile(const MixArgs& a, int n0, int zt0, const TmaMaps& maps, int* err, int tile_x, int tile_y) {
  constexpr int WM = kWindowMode<NC, ZR, MINB>;
  using S = TmaSmem<NC, ZR, WM>;
  constexpr int SLOT = S::SLOT;
  constexpr int TJ = ZR - 4;
  constexpr int kRing = NC < kOutRing ? NC : kOutRing;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);
  const Geo& g = a.g;
  const int zi = threadIdx.x & 31, zj = threadIdx.x >> 5, c = zj * 32 + zi;
  const int i0 = 1 + tile_x * TI, j0 = 1 + tile_y * TJ;
  const int bx0 = i0 - 3, by0 = j0 - 2;  // box origin (bx0 even)
  const int sc = zj * BX + zi + 1;       // this position in a box
  const float dt = a.dtime;
  const int ntr = a.ntr < NC ? a.ntr : NC;
  // this position: raw data-domain coordinates, its image, whether the boxes hold it
  const int pi = i0 - 2 + zi, pj = j0 - 2 + zj;
  int i = pi, j = pj;
  const bool in = image(g, i, j);
  const bool direct = pi >= 1 && pi <= g.ni && pj >= 1 && pj <= g.nj;
  const long o = in ? I2(g, i, j) : 0;
  const bool interior = zj >= 2 && zj <= ZR - 3 && zi >= 2 && zi <= 29 && pi <= g.ni && pj <= g.nj;
  const bool xin = in && zi >= 2 && zi <= 29;
  bool bad = false;

  if (threadIdx.x == 0) {
    for (int q = 0; q <= NC; ++q) {
      mbar_init(&s.bar[q]);
      s.pending[q] = 0;
    }
    mbar_fence_init();
  }
  __syncthreads();
  // first loads: the fields of level 0 and level min(2, nk-1) of every tracer
  if (threadIdx.x == 0) {
    mbar_expect(&s.bar[NC], 6u * SLOT * 8u);
    for (int f = 0; f < 6; ++f) tma3(s.f[f], &maps.f[f], bx0, by0, f == F_W ? 1 : 0, &s.bar[NC]);
    s.pending[NC] = 1;  // phase 0 in flight
    const int l2 = g.nk > 2 ? 2 : g.nk - 1;
    for (int n = 0; n < ntr; ++n) {
      mbar_expect(&s.bar[n], SLOT * 8u);
      tma3(s.t[n], &maps.T, bx0, by0, (zt0 + n) * g.nk + l2, &s.bar[n]);
      s.pending[n] = 1;
    }
  }
  // 2-D metrics of this position, once per tile
  float m_dat = 0.f, m_datr = 0.f, m_dyte = 0.f, m_dyte_w = 0.f, m_dxte = 0.f, m_dxtn = 0.f, m_dytn = 0.f;
  if (in) {
    m_dat = d2f(a.dat[o]);
    m_datr = d2f(a.datr[o]);
    m_dyte = d2f(a.dyte[o]);
    m_dyte_w = d2f(a.dyte[I2(g, i - 1, j)]);
    m_dxte = d2f(a.dxte[o]);
    m_dxtn = d2f(a.dxtn[o]);
    m_dytn = d2f(a.dytn[o]);
  }
  // the window of each tracer: levels km1, k, kp1 (at k = 0: 0, 0, min(1, nk-1)),
  // and the flux through the top face
  constexpr int NW = WM == 2 ? 1 : NC, NF = WM == 0 ? NC : 1;
  float w0[NW], w1[NW], w2[NW], ftp[NF];
  {
    const int l1 = g.nk > 1 ? 1 : 0;
#pragma unroll
    for (int n = 0; n < NC; ++n) {
      float t0 = 0.f, t1 = 0.f;
      if (n < ntr && in) {
        const double* T = a.T + (long)n * g.n3;
        t0 = d2f(T[o]);
        t1 = d2f(T[(long)l1 * g.n2 + o]);
      }
      if constexpr (WM == 2) {  // the level above level 0 is level 0 itself (ring slot 2)
        s.ws.win[2][n][c] = t0;
        s.ws.win[0][n][c] = t0;
        s.ws.win[1][n][c] = t1;
      } else {
        w0[n] = w1[n] = t0;
        w2[n] = t1;
      }
      if constexpr (WM == 0) ftp[n] = 0.f;
      else s.ws.ftp[n][c] = 0.f;
    }
  }
  // wet bits of levels km1, k, kp1, kp2 (mask2 at the raw position)
  unsigned mb = 0;
  {
    const int l1 = g.nk > 1 ? 1 : 0, l2 = g.nk > 2 ? 2 : g.nk - 1;
    mb = (mask_at(g, a.mask2, pi, pj, 0) ? 3u : 0u) | (mask_at(g, a.mask2, pi, pj, l1) ? 4u : 0u) |
         (mask_at(g, a.mask2, pi, pj, l2) ? 8u : 0u);
  }
  float wk_prev = 0.f;  // w at the top face of the level (0 at the surface)

  for (int k = 0; k < g.nk; ++k) {
    const int kp2 = k + 2 < g.nk ? k + 2 : g.nk - 1;
    const int kp3 = k + 3 < g.nk ? k + 3 : g.nk - 1;
    // the wet bit that enters the window at the next level, loaded a level ahead
    const bool m_next = (k + 1 < g.nk) && mask_at(g, a.mask2, pi, pj, kp3);
    // ---- phase 1: face terms of this position ----
    if (!mbar_wait(&s.bar[NC], (unsigned)(k & 1))) bad = true;
    const bool wet = (mb & 2u) != 0;
    float zmf = 0.f, zd0 = 0.f, zd1 = 0.f, zc = 0.f, zdtr = 0.f, zwd = 0.f;
    float xmf = 0.f, xd0 = 0.f, xd1 = 0.f, xc = 0.f, xcoef = 0.f, xdiv = 0.f;
    float ymf = 0.f, yd0 = 0.f, yd1 = 0.f, yc = 0.f, uq = 0.f, ur = 0.f;
    if (in) {
      // own values and the neighbours' (i+1, i-1, j+1): from the boxes for a
      // compute-domain position, else from global memory at the image
      const long p = I3(g, i, j, k);
      const double rdz_c = direct ? s.f[F_RDZ][sc] : a.rdz[p];
      const double uh_c = direct ? s.f[F_UH][sc] : a.uh[p];
      const float wk = d2f(direct ? s.f[F_W][sc] : a.w[I3(g, i, j, k + 1)]);
      z_terms(wk, wk_prev, d2f(rdz_c), m_dat, dt, zmf, zd0, zd1, zc, zdtr, zwd);
      wk_prev = wk;
      if (zi >= 1 && zi <= 29) {
        const double rdz_e = direct ? s.f[F_RDZ][sc + 1] : a.rdz[I3(g, i + 1, j, k)];
        h_terms(d2f(uh_c), m_dyte, d2f(rdz_c), d2f(rdz_e), m_dxte, dt, xmf, xd0, xd1, xc);
      }
      if (xin) {
        const double uh_w = direct ? s.f[F_UH][sc - 1] : a.uh[I3(g, i - 1, j, k)];
        xcoef = x_coef(wet, dt, m_datr, d2f(rdz_c));
        xdiv = x_div(m_dyte, d2f(uh_c), m_dyte_w, d2f(uh_w));
      }
      if (zj >= 1 && zj <= ZR - 3 && zi >= 2 && zi <= 29) {
        const double rdz_n = direct ? s.f[F_RDZ][sc + BX] : a.rdz[I3(g, i, j + 1, k)];
        const double vh_c = direct ? s.f[F_VH][sc] : a.vh[p];
        h_terms(d2f(vh_c), m_dxtn, d2f(rdz_c), d2f(rdz_n), m_dytn, dt, ymf, yd0, yd1, yc);
      }
      if (zj >= 2 && zj <= ZR - 3 && zi >= 2 && zi <= 29) {
        if (a.fused) {
          const double r = direct ? s.f[F_RDZR][sc] : a.rdzr[p];
          const double m1 = direct ? s.f[F_RDZM1][sc] : a.rdz_m1[p];
          uq = d2f(fma(m1, r, -1.0));
          ur = wet ? d2f(rdz_c * r) : 0.0f;
        } else {
          ur = wet ? d2f(rdz_c) / dt : 0.0f;
        }
      }
    }
    // read by the neighbouring rows in phase 3, after the next barrier
    s.wet[c] = in && wet;

    const int r_km1 = (k + 2) % 3, r_k = k % 3, r_kp1 = (k + 1) % 3;  // ring slots of levels k-1, k, k+1
    // ---- phase 2: z and x passes of every tracer ----
    const unsigned full = 0xffffffffu;
    const unsigned wt = (in && wet) ? 1u : 0u;
    const unsigned wA = __shfl_up_sync(full, wt, 1), wC = __shfl_down_sync(full, wt, 1);
    const unsigned wD = __shfl_down_sync(full, wt, 2);
    // every tracer's level k+2 first (issued a level ago), so that no wait -- a
    // memory fence to the compiler -- separates the tracers' work below and
    // their instructions can interleave
    for (int n = 0; n < ntr; ++n)
      if (!mbar_wait(&s.bar[n], (unsigned)(k & 1))) bad = true;
#pragma unroll
    for (int n = 0; n < NC; ++n) {
      if (n >= ntr) break;
      // Every position computes and the values of those outside the domain, of
      // dry faces and of halo cells are discarded by selects: no branch, so no
      // divergent paths, in the tracer loop.  A position outside a wall reads its
      // level at the offset o = 0 (in the array; its value is never kept).
      const float tkp2 = d2f(direct ? s.t[n][sc] : a.T[(long)n * g.n3 + (long)kp2 * g.n2 + o]);
      float tkm1, tk, tkp1, ftn, fzv;
      if constexpr (WM == 2) {
        tkm1 = s.ws.win[r_km1][n][c];
        tk = s.ws.win[r_k][n][c];
        tkp1 = s.ws.win[r_kp1][n][c];
      } else {
        tkm1 = w0[n];
        tk = w1[n];
        tkp1 = w2[n];
      }
      if constexpr (WM == 0) ftn = ftp[n];
      else ftn = s.ws.ftp[n][c];
      const float tzc = z_cell(tkm1, tk, tkp1, tkp2, mb, zmf, zd0, zd1, zc, m_datr, zdtr, zwd, ftn, fzv);
      const float tzv = in ? tzc : 0.f;
      if constexpr (WM == 2) {
        s.ws.win[r_km1][n][c] = tkp2;  // level k+2 takes the slot of level k-1
      } else if (in) {
        w0[n] = tk;
        w1[n] = w2[n];
        w2[n] = tkp2;
      }
      if constexpr (WM == 0) {
        if (in) ftp[n] = ftn;
      } else {
        s.ws.ftp[n][c] = in ? ftn : 0.f;
      }
      // x flux of face zi (between zi and zi+1) by warp shuffles
      const float tA = __shfl_up_sync(full, tzv, 1), tC = __shfl_down_sync(full, tzv, 1);
      const float tD = __shfl_down_sync(full, tzv, 2);
      const float hf = h_flux(tA, tzv, tC, tD, wA, wD, xmf, xd0, xd1, xc);
      const float f = (zi >= 1 && zi <= 29 && wt && wC) ? hf : 0.f;
      const float fw = __shfl_up_sync(full, f, 1);
      float fic;
      const float tc = x_cell(tzv, tk, fw, f, xcoef, xdiv, fic);
      s.tx[n][c] = xin ? tc : 0.f;
      s.fzx[n][c] = fa(in ? fzv : 0.f, xin ? fic : 0.f);
    }
    // every thread is done with the level's field boxes and every tracer's slot:
    // the fields of the next level and level k+3 of each tracer are fetched
    if (__syncthreads_or(bad)) goto abort;
    if (threadIdx.x == 0) {
      if (k + 1 < g.nk) {
        mbar_expect(&s.bar[NC], 6u * SLOT * 8u);
        for (int f = 0; f < 6; ++f) tma3(s.f[f], &maps.f[f], bx0, by0, f == F_W ? k + 2 : k + 1, &s.bar[NC]);
        s.pending[NC] = 1 + ((k + 1) & 1);
      } else {
        s.pending[NC] = 0;
      }
      for (int n = 0; n < ntr; ++n) {
        if (k + 1 < g.nk) {
          mbar_expect(&s.bar[n], SLOT * 8u);
          tma3(s.t[n], &maps.T, bx0, by0, (zt0 + n) * g.nk + kp3, &s.bar[n]);
          s.pending[n] = 1 + ((k + 1) & 1);
        } else {
          s.pending[n] = 0;
        }
      }
    }

    // the first ring of T(k) loads of the outputs, issued before the y fluxes
    double t64[kRing];
    {
      const long pp = I3(g, pi, pj, k);
#pragma unroll
      for (int q = 0; q < kRing; ++q) t64[q] = (a.fused && interior && q < ntr) ? a.T[(long)q * g.n3 + pp] : 0.0;
    }
    // ---- phase 3: y fluxes of every tracer (face zj, between rows zj and zj+1) ----
    const bool yface = zj >= 1 && zj <= ZR - 3 && zi >= 2 && zi <= 29;
    const bool m0 = yface && s.wet[c - 32], m1 = yface && s.wet[c];
    const bool m2 = yface && s.wet[c + 32], m3 = yface && s.wet[c + 64];
    // rows either side of face zj; a position without a y face reads its own row
    const int cA = yface ? c - 32 : c, cC = yface ? c + 32 : c, cD = yface ? c + 64 : c;
#pragma unroll
    for (int n = 0; n < NC; ++n) {
      if (n >= ntr) break;
      const float hf = h_flux(s.tx[n][cA], s.tx[n][c], s.tx[n][cC], s.tx[n][cD], m1 && m0, m3 && m2, ymf, yd0, yd1, yc);
      s.fy[n][c] = (m1 && m2) ? hf : 0.f;
    }
    if (__syncthreads_or(bad)) goto abort;
    // ---- outputs of the interior cells ----
    if (interior && (wet || a.fused)) {
      const long p = I3(g, pi, pj, k);
      if (a.fused) {
        // T(taup1) = T + (rho_dzt(taum1)*rho_dztr - 1)*T + rho_dzt(tau)*rho_dztr*dT, the FP64 T(k)
        // from the ring of loads in flight (kOutRing)
        const int hi = (g.cx && pi == g.ni) ? 0 : (g.cx && pi == 1) ? g.ni + 1 : -1;
        const int hj = (g.cy && pj == g.nj) ? 0 : (g.cy && pj == 1) ? g.nj + 1 : -1;
#pragma unroll
        for (int n = 0; n < NC; ++n) {
          if (n >= ntr) break;
          const float dT = total_inc(s.fzx[n][c], xcoef, s.fy[n][c - 32], s.fy[n][c]);
          // T(k) in FP32 is ring slot k mod 3, or w0 after the shift
          float tkk;
          if constexpr (WM == 2) tkk = s.ws.win[k % 3][n][c];
          else tkk = w0[n];
          const double tn = t64[n % kRing] + f2d(update_inc(uq, tkk, ur, dT));
          double* out = a.out + (long)(n0 + n) * g.n3;
          out[p] = tn;
          // halo update of T(taup1) in cyclic directions (ocean_model.F90:1903-1911)
          if (hi >= 0) out[I3(g, hi, pj, k)] = tn;
          if (hj >= 0) out[I3(g, pi, hj, k)] = tn;
          if (hi >= 0 && hj >= 0) out[I3(g, hi, hj, k)] = tn;
          if (n + kRing < NC && n + kRing < ntr) t64[n % kRing] = a.T[(long)(n + kRing) * g.n3 + p];
        }
      } else {
#pragma unroll
        for (int n = 0; n < NC; ++n) {
          if (n >= ntr) break;
          const float dT = total_inc(s.fzx[n][c], xcoef, s.fy[n][c - 32], s.fy[n][c]);
          double* out = a.out + (long)n * g.n3;
          out[p] = out[p] + f2d(fm(ur, dT));
        }
      }
    }
    // the window of wet bits moves down one level
    mb = (mb >> 1) | (m_next ? 8u : 0u);
  }
  // every copy of this tile has been waited for (the last level issues none)
  __syncthreads();
  if (threadIdx.x == 0)
    for (int q = 0; q <= NC; ++q) mbar_inval(&s.bar[q]);
  return true;

abort:
  if (threadIdx.x == 0) {
    atomicOr(err, 1);
    // wait, bounded, for the copies this block still has in flight
    for (int q = 0; q <= NC; ++q)
      if (s.pending[q]) mbar_wait(&s.bar[q], (unsigned)(s.pending[q] - 1));
  }
  __syncthreads();
  return false;
}

template <int NC, int ZR, int MINB>
__global__ void __launch_bounds__(32 * ZR, MINB)
    k_mdfl_mixed_tma(MixArgs a, int n0, int zt0, const __grid_constant__ TmaMaps maps, int* err) {
  tma_tile<NC, ZR, MINB>(a, n0, zt0, maps, err, blockIdx.x, blockIdx.y);
}

// ---- host side ----
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

// a 3-D FP64 tensor [nz][nyd][nxd] at base, boxes of 34 x rows x 1
bool encode(CUtensorMap* m, const double* base, const Geo& g, long nz, int rows) {
  EncodeTiled fn = encoder();
  if (!fn || !base) return false;
  cuuint64_t dim[3] = {(cuuint64_t)g.nxd, (cuuint64_t)g.nyd, (cuuint64_t)nz};
  cuuint64_t stride[2] = {(cuuint64_t)g.nxd * 8, (cuuint64_t)g.n2 * 8};
  cuuint32_t box[3] = {(cuuint32_t)BX, (cuuint32_t)rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(base), dim, stride, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NC, int ZR, int MINB>
int run_tma_zr(mom5gpu_domain* d, const MixArgs& a, int n0, const double* Tall, int zt0, int ntr_all) {
  const Geo& g = d->geo;
  constexpr size_t smem = sizeof(TmaSmem<NC, ZR, kWindowMode<NC, ZR, MINB>>);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_mdfl_mixed_tma<NC, ZR, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return cuda_fail(d, e, "TMA precision kernel attribute");
    configured = true;
  }
  TmaMaps maps;
  bool ok = encode(&maps.T, Tall, g, (long)ntr_all * g.nk, ZR) && encode(&maps.f[F_UH], a.uh, g, g.nk, ZR) &&
            encode(&maps.f[F_VH], a.vh, g, g.nk, ZR) && encode(&maps.f[F_W], a.w, g, g.nk + 1, ZR) &&
            encode(&maps.f[F_RDZ], a.rdz, g, g.nk, ZR) && encode(&maps.f[F_RDZR], a.rdzr, g, g.nk, ZR) &&
            encode(&maps.f[F_RDZM1], a.rdz_m1, g, g.nk, ZR);
  if (!ok) return fail(d, MOM5GPU_ECUDA, "TMA precision kernel: tensor-map encoding failed");
  constexpr int TJ = ZR - 4;
  dim3 grid((g.ni + TI - 1) / TI, (g.nj + TJ - 1) / TJ);
  k_mdfl_mixed_tma<NC, ZR, MINB><<<grid, 32 * ZR, smem, d->stream>>>(a, n0, zt0, maps, d->wait_err);
  count_launches(d, 1);
  return MOM5GPU_OK;
}

template <int NC>
int run_tma(mom5gpu_domain* d, const MixArgs& a, int n0, const double* Tall, int zt0, int ntr_all) {
  if (d->tune_mixed_rows == 24) return run_tma_zr<NC, 24, 1>(d, a, n0, Tall, zt0, ntr_all);
  return run_tma_zr<NC, 16, 1>(d, a, n0, Tall, zt0, ntr_all);
}

// Two resident blocks per SM (16-row tiles, at most 5 tracers per block, 64
// registers): the tracers of the launch go in sub-launches of up to 5, each
// recomputing the level's face terms.
int run_tma_pairs(mom5gpu_domain* d, const MixArgs& a, int n0, const double* Tall, int zt0, int ntr_all) {
  for (int q = 0; q < a.ntr; q += 5) {
    MixArgs b = a;
    b.ntr = a.ntr - q < 5 ? a.ntr - q : 5;
    b.T = a.T + (long)q * a.g.n3;
    if (!a.fused) b.out = a.out + (long)q * a.g.n3;
    const int m0 = a.fused ? n0 + q : 0;
    int rc = b.ntr <= 2 ? run_tma_zr<2, 16, 2>(d, b, m0, Tall, zt0 + q, ntr_all)
                        : run_tma_zr<5, 16, 2>(d, b, m0, Tall, zt0 + q, ntr_all);
    if (rc) return rc;
  }
  return MOM5GPU_OK;
}

// ---- batches: TMA-staged tiles over a work list ----

// tile height of the batched TMA kernel for a tracer count: 32 rows (1024 threads)
// where the shared memory holds them, at most 4 tracers (C3, 4 tracers: 19.27 ms
// per step against 19.37 with 24 rows), else 24
template <int NC>
constexpr int kBatchRows = NC <= 4 ? 32 : 24;

// one (domain, parity) entry of a batch's device table: the tensor maps of its
// tracer level and fields, and its domain's error word
struct BatchTma {
  TmaMaps m;
  int* err;
};

DEVI int find_tile_entry(const int* prefix, int count, int b) {
  int lo = 0, hi = count;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (prefix[mid] <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Persistent: one block (768 or 1024 threads) per SM takes tiles from an atomic counter
// (largest domains first) and runs each as the one-domain kernel does.  A block
// whose bounded wait gave up stops; the others go on, and the domain's
// mom5gpu_synchronize reports MOM5GPU_ETIMEDOUT.
template <int NC>
__global__ void __launch_bounds__(32 * kBatchRows<NC>, 1)
    kb_mixed_tma(const MixArgs* __restrict__ d, const BatchTma* __restrict__ tm, BatchWork w, int* counter) {
  constexpr int ZR = kBatchRows<NC>;
  __shared__ int item;
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = item;
    __syncthreads();
    if (it >= w.tt) return;
    const int e = find_tile_entry(w.pt, w.count, it);
    const int ent = w.entries[e];
    const MixArgs& a = d[ent];
    const int local = it - w.pt[e];
    const int ntx = (a.g.ni + TI - 1) / TI;
    if (!tma_tile<NC, ZR, 1>(a, 0, 0, tm[ent].m, tm[ent].err, local % ntx, local / ntx)) return;
  }
}

template <int NC>
int configure_batch_tma() {
  constexpr int ZR = kBatchRows<NC>;
  return cudaFuncSetAttribute(kb_mixed_tma<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(TmaSmem<NC, ZR, kWindowMode<NC, ZR, 1>>)) == cudaSuccess
             ? MOM5GPU_OK
             : MOM5GPU_ECUDA;
}

template <int NC>
void run_batch_tma(const MixArgs* mix, const BatchTma* tm, const BatchWork& w, int blocks, int* counter,
                   cudaStream_t s) {
  constexpr int ZR = kBatchRows<NC>;
  cudaMemsetAsync(counter, 0, sizeof(int), s);
  kb_mixed_tma<NC><<<blocks, 32 * ZR, sizeof(TmaSmem<NC, ZR, kWindowMode<NC, ZR, 1>>), s>>>(mix, tm, w, counter);
}

}  // namespace

size_t batch_tma_bytes() { return sizeof(BatchTma); }

// the tile height for ntr tracers (the kernel instantiation launch_batch_mixed_tma picks)
int batch_tma_rows(int ntr) {
  return ntr <= 1 ? kBatchRows<1> : ntr <= 2 ? kBatchRows<2> : ntr <= 4 ? kBatchRows<4> : kBatchRows<10>;
}

int fill_batch_tma(mom5gpu_domain* d, const MixArgs& a, void* host_entry) {
  const Geo& g = d->geo;
  if (g.ni % 2 != 0 || !a.T || a.ntr < 1) return MOM5GPU_EUNSUPPORTED;
  int rc = ensure_wait_words(d);
  if (rc) return rc;
  BatchTma t;
  memset(&t, 0, sizeof(t));
  const int zr = batch_tma_rows(a.ntr);
  bool ok = encode(&t.m.T, a.T, g, (long)a.ntr * g.nk, zr) && encode(&t.m.f[F_UH], a.uh, g, g.nk, zr) &&
            encode(&t.m.f[F_VH], a.vh, g, g.nk, zr) && encode(&t.m.f[F_W], a.w, g, g.nk + 1, zr) &&
            encode(&t.m.f[F_RDZ], a.rdz, g, g.nk, zr) && encode(&t.m.f[F_RDZR], a.rdzr, g, g.nk, zr) &&
            encode(&t.m.f[F_RDZM1], a.rdz_m1, g, g.nk, zr);
  if (!ok) return MOM5GPU_EUNSUPPORTED;
  t.err = d->wait_err;
  memcpy(host_entry, &t, sizeof(t));
  return MOM5GPU_OK;
}

int prepare_batch_mixed_tma() {
  int rc = configure_batch_tma<1>() | configure_batch_tma<2>() | configure_batch_tma<4>() | configure_batch_tma<10>();
  return rc ? MOM5GPU_ECUDA : MOM5GPU_OK;
}

int launch_batch_mixed_tma(const MixArgs* mix, const void* tma, const BatchWork& w, int ntr, int blocks, int* counter,
                           cudaStream_t s) {
  if (w.tt <= 0) return MOM5GPU_OK;
  const BatchTma* tm = static_cast<const BatchTma*>(tma);
  if (ntr <= 1) run_batch_tma<1>(mix, tm, w, blocks, counter, s);
  else if (ntr <= 2) run_batch_tma<2>(mix, tm, w, blocks, counter, s);
  else if (ntr <= 4) run_batch_tma<4>(mix, tm, w, blocks, counter, s);
  else run_batch_tma<10>(mix, tm, w, blocks, counter, s);
  return MOM5GPU_OK;
}

// The TMA variant of one launch of launch_mdfl_mixed (a = the launch's
// arguments, tracers zt0 .. zt0+a.ntr-1 of the level whose first tracer is
// Tall, ntr_all tracers in all).  MOM5GPU_EUNSUPPORTED when the domain cannot
// be described to TMA (odd ni: the row stride is not a multiple of 16 bytes):
// the caller then launches the plain kernel.
int launch_mixed_tma(mom5gpu_domain* d, const MixArgs& a, int n0, const double* Tall, int zt0, int ntr_all) {
  if (d->geo.ni % 2 != 0) return MOM5GPU_EUNSUPPORTED;
  int rc = ensure_wait_words(d);
  if (rc) return rc;
  if (d->tune_mixed_pf == 3) return run_tma_pairs(d, a, n0, Tall, zt0, ntr_all);
  if (a.ntr <= 1) return run_tma<1>(d, a, n0, Tall, zt0, ntr_all);
  if (a.ntr <= 2) return run_tma<2>(d, a, n0, Tall, zt0, ntr_all);
  if (a.ntr <= 4) return run_tma<4>(d, a, n0, Tall, zt0, ntr_all);
  return run_tma<10>(d, a, n0, Tall, zt0, ntr_all);
}

}  // namespace mom5
