// Body of the precision-form MDFL kernel (FP32 fluxes and limiters, FP64
// state), shared by the one-domain kernel (k_mixed.cu) and the persistent
// batched kernel (k_batch.cu).  See k_mixed.cu for the method.
#pragma once
#include <math.h>

#include "internal.h"

namespace mom5 {
namespace mixed {

#define DEVI __device__ __forceinline__


constexpr int ZW = 32;       // tile width incl. the 2-cell halo on each side (one warp)
constexpr int TI = ZW - 4;   // interior width
constexpr int NT = 256;      // threads of the 16- and 24-row tiles
// ZR (template): tile height incl. halo; interior height ZR - 4
// Threads per block of a tile height: 8 warps, 16 for the 32-row tile and 32
// for the 64-row tile, so that the 16-, 32- and 64-row tiles hold two tile rows
// per thread (the 24-row tile three) and the tall tiles still give 32 warps per
// SM (two blocks of 32 rows, one of 64).
__host__ __device__ constexpr int tile_threads(int ZR) { return ZR == 64 ? 1024 : ZR == 32 ? 512 : NT; }

DEVI long I2(const Geo& g, int i, int j) { return (long)j * g.nxd + i; }
DEVI long I3(const Geo& g, int i, int j, int k) { return (long)k * g.n2 + (long)j * g.nxd + i; }
DEVI long IM(const Geo& g, int i, int j, int k) { return ((long)k * (g.nj + 4) + (j + 1)) * (g.ni + 4) + (i + 1); }

// FP64 -> FP32 by truncation of the significand, with integer operations.
DEVI float d2f(double x) {
  unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
  if (mag < (897u << 20)) return __uint_as_float(sign);
  if (mag >= (1151u << 20)) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((mag - (896u << 20)) << 3) | (lo >> 29));
}
// FP64 -> FP32 rounded to nearest (ties away from zero): half an FP32 ulp added
// to the bit pattern, then truncated.
DEVI float d2f_rn(double x) { return d2f(__longlong_as_double(__double_as_longlong(x) + (1LL << 28))); }
// FP32 -> FP64, exact, with integer operations (subnormal floats read as zero).
DEVI double f2d(float f) {
  unsigned b = __float_as_uint(f);
  unsigned sign = b & 0x80000000u, mag = b & 0x7fffffffu;
  if (mag < 0x00800000u) return __hiloint2double((int)sign, 0);
  return __hiloint2double((int)(sign | ((mag >> 3) + (896u << 20))), (int)(mag << 29));
}

// The FP32 arithmetic of the precision form.  Every product and sum is rounded
// on its own (__fmul_rn / __fadd_rn / __fsub_rn are never contracted into a
// multiply-add), so the result of a formula does not depend on how the
// compiler schedules the kernel around it: every tile kernel built on these
// helpers (plain, prefetching, TMA-staged, batched) gives the same bits.
DEVI float fm(float a, float b) { return __fmul_rn(a, b); }
DEVI float fa(float a, float b) { return __fadd_rn(a, b); }
DEVI float fs(float a, float b) { return __fsub_rn(a, b); }

DEVI float limiter(float theta, float d0, float d1, float c) {
  float lin = fa(d0, fm(d1, theta));
  return fmaxf(0.0f, fminf(fminf(1.0f, lin), fm(c, theta)));
}

// One division and one limiter for either sign of mf (operands selected first);
// Tm - p is evaluated as Tm + (-p), the same IEEE operation.
DEVI float face_flux(float mf, float Rjm, float Rj, float Rjp, float Tp, float Tm, float d0, float d1, float c) {
  bool pos = mf > 0.0f;
  float theta = __fdividef(pos ? Rjm : Rjp, fa(1.0e-30f, Rj));
  float p = fm(limiter(theta, d0, d1, c), Rj);
  float r = fm(mf, fa(pos ? Tp : Tm, pos ? p : -p));
  return (pos || mf < 0.0f) ? r : 0.0f;
}

// d0, d1 and the limiter slope (1-cfl)/(1e-30+cfl) of a Courant number
DEVI void cfl_terms(float cfl, float& d0, float& d1, float& c) {
  const float sixth = 1.0f / 6.0f;
  d0 = fm(fm(fs(2.0f, cfl), fs(1.0f, cfl)), sixth);
  d1 = fm(fs(1.0f, fm(cfl, cfl)), sixth);
  c = __fdividef(fs(1.0f, cfl), fa(1.0e-30f, cfl));
}
// vertical face terms of a column: mass flux dat*w, cfl = |w*dt/rho_dzt|
DEVI void z_terms(float wk, float wkm1, float rdz, float dat, float dt, float& mf, float& d0, float& d1, float& c,
                  float& dtr, float& wd) {
  float rr = 1.0f / rdz;
  mf = fm(dat, wk);
  cfl_terms(fabsf(fm(fm(wk, dt), rr)), d0, d1, c);
  dtr = fm(dt, rr);
  wd = fs(wkm1, wk);
}
// horizontal face terms: mass flux len*u, cfl = |u*dt*2/((rdz + rdz_nb)*dist)|
DEVI void h_terms(float u, float len, float rdz, float rdz_nb, float dist, float dt, float& mf, float& d0, float& d1,
                  float& c) {
  mf = fm(len, u);
  float den = fm(fa(rdz, rdz_nb), dist);
  cfl_terms(fabsf(__fdividef(fm(fm(u, dt), 2.0f), den)), d0, d1, c);
}
// x-cell terms: dtime*datr/rho_dzt where wet, and the x divergence dyte*uh - dyte(i-1)*uh(i-1)
DEVI float x_coef(bool wet, float dt, float datr, float rdz) { return wet ? fm(dt, datr) / rdz : 0.0f; }
DEVI float x_div(float dyte, float uh, float dyte_w, float uh_w) { return fs(fm(dyte, uh), fm(dyte_w, uh_w)); }
// z pass of one column cell: returns tracer_mdfl after z; fz the z increment
DEVI float z_cell(float tkm1, float tk, float tkp1, float tkp2, unsigned mb, float mf, float d0, float d1, float c,
                  float datr, float dtr, float wd, float& ftp, float& fz) {
  const bool mkm1 = mb & 1u, mk = mb & 2u, mkp1 = mb & 4u, mkp2 = mb & 8u;
  float Rjp = (mkm1 && mk) ? fs(tkm1, tk) : 0.f;
  float Rj = (mk && mkp1) ? fs(tk, tkp1) : 0.f;
  float Rjm = (mkp1 && mkp2) ? fs(tkp1, tkp2) : 0.f;
  // the flux of every face is formed and a dry face's discarded: a select, not a
  // branch around the division and the limiter
  const float ff = face_flux(mf, Rjm, Rj, Rjp, tkp1, tk, d0, d1, c);
  float fbt = (mkp1 && mk) ? ff : 0.f;
  float adiv = fm(datr, fs(fbt, ftp));
  fz = fm(dtr, adiv);
  ftp = fbt;
  return fa(tk, fm(dtr, fa(adiv, fm(tk, wd))));
}
// flux of a face between cells B and C given A (upstream of B) and D (beyond C)
// and their wet flags
DEVI float h_flux(float tA, float tB, float tC, float tD, bool wA, bool wD, float mf, float d0, float d1, float c) {
  float Rjp = wD ? fs(tD, tC) : 0.f;
  float Rj = fs(tC, tB);
  float Rjm = wA ? fs(tB, tA) : 0.f;
  return face_flux(mf, Rjm, Rj, Rjp, tB, tC, d0, d1, c);
}
// x update of a cell: returns tracer_mdfl after x; fi the x increment
DEVI float x_cell(float tz, float tk, float fw, float f, float coef, float div, float& fi) {
  fi = fm(coef, fs(fw, f));
  return fa(tz, fa(fi, fm(coef, fm(tk, div))));
}
// the total increment of a cell from its z + x part and the y fluxes either side
DEVI float total_inc(float fzx, float coef, float fy_s, float fy_n) { return fa(fzx, fm(coef, fs(fy_s, fy_n))); }
// state update increment (rho_dzt(taum1)*rho_dztr - 1)*T + rho_dzt(tau)*rho_dztr*dT
DEVI float update_inc(float uq, float tk, float ur, float dT) { return fa(fm(uq, tk), fm(ur, dT)); }



// image of a tile position under the single-domain halo rules; false when it lies
// outside a non-cyclic boundary (the reference's halo holds zero there)
DEVI bool image(const Geo& g, int& i, int& j) {
  if (i < 1 || i > g.ni) {
    if (!g.cx) return false;
    i = ((i - 1) % g.ni + g.ni) % g.ni + 1;
  }
  if (j < 1 || j > g.nj) {
    if (!g.cy) return false;
    j = ((j - 1) % g.nj + g.nj) % g.nj + 1;
  }
  return true;
}

DEVI bool mask_at(const Geo& g, const uint8_t* m2, int i, int j, int k) {
  if (i < -1 || i > g.ni + 2 || j < -1 || j > g.nj + 2) return false;
  return m2[IM(g, i, j, k)] != 0;
}

template <int ZR>
struct SmemT {
  // z pass, per z-column (32x32)
  float zmf[ZR * ZW], zd0[ZR * ZW], zd1[ZR * ZW], zc[ZR * ZW], zdtr[ZR * ZW], zwd[ZR * ZW], zdatr[ZR * ZW];
  uint8_t zmask[ZR * ZW];  // bit0..3 = wet at k-1, k, k+1, k+2
  // x pass: faces between columns zi and zi+1 (index zj*ZW+zi), cells
  float xmf[ZR * ZW], xd0[ZR * ZW], xd1[ZR * ZW], xc[ZR * ZW];
  float xcoef[ZR * ZW], xdiv[ZR * ZW];
  float tx[ZR * ZW];  // tracer after x
  // y pass: faces between rows zj and zj+1
  float ymf[ZR * ZW], yd0[ZR * ZW], yd1[ZR * ZW], yc[ZR * ZW];
  float fy[ZR * ZW];
  // state-update factors: rho_dzt(taum1)*rho_dztr - 1 and rho_dzt(tau)*rho_dztr*tmask (or rho_dzt/dtime*tmask)
  float uq[ZR * ZW], ur[ZR * ZW];
  uint8_t xin[ZR * ZW];  // x-cell position inside the domain (or a cyclic image)
  int off[ZR * ZW];      // 2-D offset j*nxd+i of the position's image; -1 outside a wall
};

// Stream-ordered 8-byte copy global -> shared (cp.async, L1-allocating); src_size 0
// fills the destination with zeros and reads nothing.
DEVI void cp_async8(void* dst, const void* src, int src_size) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_size) : "memory");
}
DEVI void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
DEVI void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Shared memory of the tracer prefetch: two buffers of the four levels
// km1, k, kp1, kp2 of one tracer over the tile (FP64, as stored).
template <int ZR>
struct PrefetchT {
  double tb[2][4][ZR * ZW];
};

template <int NC, int ZR, bool PF = false, int NTH = NT>
DEVI void mixed_tile(const MixArgs& a, int n0, int tile_x, int tile_y, SmemT<ZR>& s, PrefetchT<ZR>* pf = nullptr) {
  constexpr int TJ = ZR - 4;
  constexpr int NWT = NTH / 32;  // warps of the block; tile row zj belongs to warp zj % NWT
  static_assert(ZR % NWT == 0, "tile height must be a multiple of the warps per block");
  constexpr int ROWS_PER_WARP = ZR / NWT;
  const Geo& g = a.g;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i0 = 1 + tile_x * TI, j0 = 1 + tile_y * TJ;
  const float dt = a.dtime;
  // image offsets of this thread's tile positions (the same at every level)
  int offr[ROWS_PER_WARP];
#pragma unroll
  for (int m = 0; m < ROWS_PER_WARP; ++m) {
    int i = i0 - 2 + lane, j = j0 - 2 + warp + NWT * m;
    offr[m] = image(g, i, j) ? (int)I2(g, i, j) : -1;
  }
  // queue the four levels of tracer n into prefetch buffer b (zeros outside a wall)
  auto prefetch = [&](int n, int b, int km1, int k, int kp1, int kp2) {
    const double* T = a.T + (long)n * g.n3;
    const int lev[4] = {km1, k, kp1, kp2};
#pragma unroll
    for (int m = 0; m < ROWS_PER_WARP; ++m) {
      const int c = (warp + NWT * m) * ZW + lane, o = offr[m];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double* src = o >= 0 ? T + (long)lev[q] * g.n2 + o : T;
        cp_async8(&pf->tb[b][q][c], src, o >= 0 ? 8 : 0);
      }
    }
    cp_async_commit();
  };

  // per-thread z columns: zi = lane, zj = warp + NWT*m
  float ftp[NC][ROWS_PER_WARP];
#pragma unroll
  for (int n = 0; n < NC; ++n)
#pragma unroll
    for (int m = 0; m < ROWS_PER_WARP; ++m) ftp[n][m] = 0.0f;

  for (int k = 0; k < g.nk; ++k) {
    const int kp1 = k + 1 < g.nk ? k + 1 : g.nk - 1;
    const int kp2 = k + 2 < g.nk ? k + 2 : g.nk - 1;
    const int km1 = k > 0 ? k - 1 : 0;
    __syncthreads();  // previous level done with every tile array
    if (PF && a.ntr > 0) prefetch(0, 0, km1, k, kp1, kp2);  // overlaps the level terms
    // ---- level terms: z columns, x faces/cells, y faces ----
#pragma unroll
    for (int m = 0; m < ROWS_PER_WARP; ++m) {
      const int zj = warp + NWT * m, zi = lane, c = zj * ZW + zi;
      int i = i0 - 2 + zi, j = j0 - 2 + zj;
      const int pi = i, pj = j;
      bool in = image(g, i, j);
      uint8_t mbits = 0;
      float mf = 0.f, d0 = 0.f, d1 = 0.f, cc = 0.f, dtr = 0.f, wd = 0.f, datr = 0.f;
      if (in) {
        mbits = (mask_at(g, a.mask2, pi, pj, km1) ? 1 : 0) | (mask_at(g, a.mask2, pi, pj, k) ? 2 : 0) |
                (mask_at(g, a.mask2, pi, pj, kp1) ? 4 : 0) | (mask_at(g, a.mask2, pi, pj, kp2) ? 8 : 0);
        float wk = d2f(a.w[I3(g, i, j, k + 1)]);
        float wkm1 = k > 0 ? d2f(a.w[I3(g, i, j, k)]) : 0.0f;
        datr = d2f(a.datr[I2(g, i, j)]);
        z_terms(wk, wkm1, d2f(a.rdz[I3(g, i, j, k)]), d2f(a.dat[I2(g, i, j)]), dt, mf, d0, d1, cc, dtr, wd);
      }
      s.zmask[c] = mbits;
      s.off[c] = in ? (int)I2(g, i, j) : -1;
      s.zmf[c] = mf;
      s.zd0[c] = d0;
      s.zd1[c] = d1;
      s.zc[c] = cc;
      s.zdtr[c] = dtr;
      s.zwd[c] = wd;
      s.zdatr[c] = datr;
      // x face between zi and zi+1 of row zj (needed for zi = 1..29)
      float xmf = 0.f, xd0 = 0.f, xd1 = 0.f, xc = 0.f;
      if (in && zi >= 1 && zi <= ZW - 3)
        h_terms(d2f(a.uh[I3(g, i, j, k)]), d2f(a.dyte[I2(g, i, j)]), d2f(a.rdz[I3(g, i, j, k)]),
                d2f(a.rdz[I3(g, i + 1, j, k)]), d2f(a.dxte[I2(g, i, j)]), dt, xmf, xd0, xd1, xc);
      s.xmf[c] = xmf;
      s.xd0[c] = xd0;
      s.xd1[c] = xd1;
      s.xc[c] = xc;
      // x cell terms (cells zi = 2..29): dtime*tmask*datr/rho_dzt and the x divergence
      float coef = 0.f, div = 0.f;
      bool xin = in && zi >= 2 && zi <= ZW - 3;
      if (xin) {
        bool wet = (mbits & 2) != 0;
        coef = x_coef(wet, dt, datr, d2f(a.rdz[I3(g, i, j, k)]));
        div = x_div(d2f(a.dyte[I2(g, i, j)]), d2f(a.uh[I3(g, i, j, k)]), d2f(a.dyte[I2(g, i - 1, j)]),
                    d2f(a.uh[I3(g, i - 1, j, k)]));
      }
      s.xcoef[c] = coef;
      s.xdiv[c] = div;
      s.xin[c] = xin;
      // y face between rows zj and zj+1 (needed for zj = 1..29, zi = 2..29)
      float ymf = 0.f, yd0 = 0.f, yd1 = 0.f, yc = 0.f;
      if (in && zj >= 1 && zj <= ZR - 3 && zi >= 2 && zi <= ZW - 3)
        h_terms(d2f(a.vh[I3(g, i, j, k)]), d2f(a.dxtn[I2(g, i, j)]), d2f(a.rdz[I3(g, i, j, k)]),
                d2f(a.rdz[I3(g, i, j + 1, k)]), d2f(a.dytn[I2(g, i, j)]), dt, ymf, yd0, yd1, yc);
      s.ymf[c] = ymf;
      s.yd0[c] = yd0;
      s.yd1[c] = yd1;
      s.yc[c] = yc;
      // state-update factors of interior cells
      float uq = 0.f, ur = 0.f;
      if (in && zj >= 2 && zj <= ZR - 3 && zi >= 2 && zi <= ZW - 3) {
        long p = I3(g, i, j, k);
        bool wet = (mbits & 2) != 0;
        if (a.fused) {
          double r = a.rdzr[p];
          uq = d2f(fma(a.rdz_m1[p], r, -1.0));
          ur = wet ? d2f(a.rdz[p] * r) : 0.0f;
        } else {
          ur = wet ? d2f(a.rdz[p]) / dt : 0.0f;
        }
      }
      s.uq[c] = uq;
      s.ur[c] = ur;
    }
    if (PF) cp_async_wait_all();
    __syncthreads();

#pragma unroll
    for (int n = 0; n < NC; ++n) {
      if (n >= a.ntr) break;
      const double* T = a.T + (long)n * g.n3;
      if (PF) {
        if (n > 0) {  // tracer n has arrived and every thread is done with tracer n-1
          cp_async_wait_all();
          __syncthreads();
        }
        if (n + 1 < a.ntr && n + 1 < NC) prefetch(n + 1, (n + 1) & 1, km1, k, kp1, kp2);
      }
      // A tile row (32 columns) is one warp: the z pass, the x fluxes and the x
      // update of a row exchange neighbours with warp shuffles; only the y pass
      // reads other rows (shared memory, two barriers per tracer).
      float tkr[ROWS_PER_WARP], fzr[ROWS_PER_WARP], fir[ROWS_PER_WARP];
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NWT * m, zi = lane, c = zj * ZW + zi;
        // ---- z pass ----
        const int o = s.off[c];
        const uint8_t mb = s.zmask[c];
        float tzv = 0.f, tk = 0.f, fzv = 0.f;
        if (o >= 0) {
          float tkm1, tkp1, tkp2;
          if (PF) {
            const int b = n & 1;
            tkm1 = d2f(pf->tb[b][0][c]);
            tk = d2f(pf->tb[b][1][c]);
            tkp1 = d2f(pf->tb[b][2][c]);
            tkp2 = d2f(pf->tb[b][3][c]);
          } else {
            tk = d2f(T[(long)k * g.n2 + o]);
            tkm1 = d2f(T[(long)km1 * g.n2 + o]);
            tkp1 = d2f(T[(long)kp1 * g.n2 + o]);
            tkp2 = d2f(T[(long)kp2 * g.n2 + o]);
          }
          tzv = z_cell(tkm1, tk, tkp1, tkp2, mb, s.zmf[c], s.zd0[c], s.zd1[c], s.zc[c], s.zdatr[c], s.zdtr[c],
                       s.zwd[c], ftp[n][m], fzv);
        }
        // ---- x fluxes: face zi (between zi and zi+1), zi = 1..29 ----
        const unsigned full = 0xffffffffu;
        float tA = __shfl_up_sync(full, tzv, 1), tC = __shfl_down_sync(full, tzv, 1);
        float tD = __shfl_down_sync(full, tzv, 2);
        unsigned wet = (mb >> 1) & 1u;
        unsigned wA = __shfl_up_sync(full, wet, 1), wC = __shfl_down_sync(full, wet, 1);
        unsigned wD = __shfl_down_sync(full, wet, 2);
        float f = 0.f;
        if (zi >= 1 && zi <= ZW - 3 && wet && wC)
          f = h_flux(tA, tzv, tC, tD, wA, wD, s.xmf[c], s.xd0[c], s.xd1[c], s.xc[c]);
        // ---- x update: cells zi = 2..29 ----
        float fw = __shfl_up_sync(full, f, 1);
        float t = 0.f, fi = 0.f;
        if (s.xin[c]) t = x_cell(tzv, tk, fw, f, s.xcoef[c], s.xdiv[c], fi);
        s.tx[c] = t;
        tkr[m] = tk;
        fzr[m] = fzv;
        fir[m] = fi;
      }
      __syncthreads();
      // ---- y fluxes: face zj (between rows zj and zj+1), zj = 1..29, zi = 2..29 ----
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NWT * m, zi = lane, c = zj * ZW + zi;
        float f = 0.f;
        if (zj >= 1 && zj <= ZR - 3 && zi >= 2 && zi <= ZW - 3) {
          bool m0 = s.zmask[c - ZW] & 2, m1 = s.zmask[c] & 2, m2 = s.zmask[c + ZW] & 2, m3 = s.zmask[c + 2 * ZW] & 2;
          if (m1 && m2)
            f = h_flux(s.tx[c - ZW], s.tx[c], s.tx[c + ZW], s.tx[c + 2 * ZW], m1 && m0, m3 && m2, s.ymf[c], s.yd0[c],
                       s.yd1[c], s.yc[c]);
        }
        s.fy[c] = f;
      }
      __syncthreads();
      // ---- interior: total increment and output ----
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NWT * m, zi = lane, c = zj * ZW + zi;
        if (zj < 2 || zj > ZR - 3 || zi < 2 || zi > ZW - 3) continue;
        const int i = i0 - 2 + zi, j = j0 - 2 + zj;
        if (i > g.ni || j > g.nj) continue;
        bool wet = s.zmask[c] & 2;
        if (!wet && !a.fused) continue;
        float dT = total_inc(fa(fzr[m], fir[m]), s.xcoef[c], s.fy[c - ZW], s.fy[c]);
        long p = I3(g, i, j, k);
        if (a.fused) {
          // T(taup1) = T + (rho_dzt(taum1)*rho_dztr - 1)*T + rho_dzt(tau)*rho_dztr*dT
          float inc = update_inc(s.uq[c], tkr[m], s.ur[c], dT);
          double tn = (PF ? pf->tb[n & 1][1][c] : T[p]) + f2d(inc);
          double* o = a.out + (long)(n0 + n) * g.n3;
          o[p] = tn;
          // halo update of T(taup1) in cyclic directions (ocean_model.F90:1903-1911)
          int hi = (g.cx && i == g.ni) ? 0 : (g.cx && i == 1) ? g.ni + 1 : -1;
          int hj = (g.cy && j == g.nj) ? 0 : (g.cy && j == 1) ? g.nj + 1 : -1;
          if (hi >= 0) o[I3(g, hi, j, k)] = tn;
          if (hj >= 0) o[I3(g, i, hj, k)] = tn;
          if (hi >= 0 && hj >= 0) o[I3(g, hi, hj, k)] = tn;
        } else if (wet) {
          double* o = a.out + (long)n * g.n3;
          o[p] = o[p] + f2d(fm(s.ur[c], dT));
        }
      }
      // the next tracer writes tx only after this tracer's y fluxes were read
      // (second barrier above) and fy only after its own first barrier
    }
  }
}


}  // namespace mixed
}  // namespace mom5
