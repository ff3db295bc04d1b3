// Precision form of MDFL Sweby: fluxes and limiters in FP32, tracer state in FP64.
//
// One fused kernel does the z, x and y passes of advect_tracer_mdfl_sweby
// (ocean_tracer_advect.F90:3806-4066) for a 28x28 tile of columns, marching
// down k, with the tile's 2-cell halo recomputed instead of exchanged: the
// z pass runs on the 32x32 tile-plus-halo, the x pass on 32 rows x 28 columns,
// the y pass on the 28x28 interior.  Face terms (mass flux, Courant number,
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

#include "internal.h"

namespace mom5 {

#define DEVI __device__ __forceinline__

namespace {

constexpr int ZW = 32;       // z tile width (interior + 2 halo each side)
constexpr int TI = ZW - 4;   // interior width
constexpr int TJ = ZW - 4;   // interior height
constexpr int NT = 256;      // threads
constexpr int NW = NT / 32;  // warps
constexpr int ROWS_PER_WARP = ZW / NW;

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
// FP32 -> FP64, exact, with integer operations (subnormal floats read as zero).
DEVI double f2d(float f) {
  unsigned b = __float_as_uint(f);
  unsigned sign = b & 0x80000000u, mag = b & 0x7fffffffu;
  if (mag < 0x00800000u) return __hiloint2double((int)sign, 0);
  return __hiloint2double((int)(sign | ((mag >> 3) + (896u << 20))), (int)(mag << 29));
}

DEVI float limiter(float theta, float d0, float d1, float c) {
  float lin = d0 + d1 * theta;
  return fmaxf(0.0f, fminf(fminf(1.0f, lin), c * theta));
}

DEVI float face_flux(float mf, float Rjm, float Rj, float Rjp, float Tp, float Tm, float d0, float d1, float c) {
  if (mf > 0.0f) {
    float theta = __fdividef(Rjm, 1.0e-30f + Rj);
    return mf * (Tp + limiter(theta, d0, d1, c) * Rj);
  } else if (mf < 0.0f) {
    float theta = __fdividef(Rjp, 1.0e-30f + Rj);
    return mf * (Tm - limiter(theta, d0, d1, c) * Rj);
  }
  return 0.0f;
}

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

struct Smem {
  // z pass, per z-column (32x32)
  float zmf[ZW * ZW], zd0[ZW * ZW], zd1[ZW * ZW], zc[ZW * ZW], zdtr[ZW * ZW], zwd[ZW * ZW], zdatr[ZW * ZW];
  uint8_t zmask[ZW * ZW];  // bit0..3 = wet at k-1, k, k+1, k+2
  float tz[ZW * ZW];       // tracer after z
  float tf[ZW * ZW];       // tracer at taum1 (FP32)
  float fz[ZW * ZW];       // z flux-divergence increment
  // x pass: faces between columns zi and zi+1 (index zj*ZW+zi), cells
  float xmf[ZW * ZW], xd0[ZW * ZW], xd1[ZW * ZW], xc[ZW * ZW];
  float xcoef[ZW * ZW], xdiv[ZW * ZW];
  float fx[ZW * ZW], tx[ZW * ZW], fxi[ZW * ZW];
  // y pass: faces between rows zj and zj+1
  float ymf[ZW * ZW], yd0[ZW * ZW], yd1[ZW * ZW], yc[ZW * ZW];
  float fy[ZW * ZW];
  // state-update factors: rho_dzt(taum1)*rho_dztr - 1 and rho_dzt(tau)*rho_dztr*tmask (or rho_dzt/dtime*tmask)
  float uq[ZW * ZW], ur[ZW * ZW];
  uint8_t xin[ZW * ZW];  // x-cell position inside the domain (or a cyclic image)
};

template <int NC>
__global__ void __launch_bounds__(NT, 2) k_mdfl_mixed(MixArgs a, int n0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& s = *reinterpret_cast<Smem*>(smem_raw);
  const Geo& g = a.g;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i0 = 1 + blockIdx.x * TI, j0 = 1 + blockIdx.y * TJ;
  const float dt = a.dtime;
  const float sixth = 1.0f / 6.0f;

  // per-thread z columns: zi = lane, zj = warp + NW*m
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
    // ---- level terms: z columns, x faces/cells, y faces ----
#pragma unroll
    for (int m = 0; m < ROWS_PER_WARP; ++m) {
      const int zj = warp + NW * m, zi = lane, c = zj * ZW + zi;
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
        float rr = 1.0f / d2f(a.rdz[I3(g, i, j, k)]);
        datr = d2f(a.datr[I2(g, i, j)]);
        mf = d2f(a.dat[I2(g, i, j)]) * wk;
        float cfl = fabsf(wk * dt * rr);
        d0 = (2.0f - cfl) * (1.0f - cfl) * sixth;
        d1 = (1.0f - cfl * cfl) * sixth;
        cc = __fdividef(1.0f - cfl, 1.0e-30f + cfl);
        dtr = dt * rr;
        wd = wkm1 - wk;
      }
      s.zmask[c] = mbits;
      s.zmf[c] = mf;
      s.zd0[c] = d0;
      s.zd1[c] = d1;
      s.zc[c] = cc;
      s.zdtr[c] = dtr;
      s.zwd[c] = wd;
      s.zdatr[c] = datr;
      // x face between zi and zi+1 of row zj (needed for zi = 1..29)
      float xmf = 0.f, xd0 = 0.f, xd1 = 0.f, xc = 0.f;
      if (in && zi >= 1 && zi <= ZW - 3) {
        float u = d2f(a.uh[I3(g, i, j, k)]);
        xmf = d2f(a.dyte[I2(g, i, j)]) * u;
        float den = (d2f(a.rdz[I3(g, i, j, k)]) + d2f(a.rdz[I3(g, i + 1, j, k)])) * d2f(a.dxte[I2(g, i, j)]);
        float cfl = fabsf(__fdividef(u * dt * 2.0f, den));
        xd0 = (2.0f - cfl) * (1.0f - cfl) * sixth;
        xd1 = (1.0f - cfl * cfl) * sixth;
        xc = __fdividef(1.0f - cfl, 1.0e-30f + cfl);
      }
      s.xmf[c] = xmf;
      s.xd0[c] = xd0;
      s.xd1[c] = xd1;
      s.xc[c] = xc;
      // x cell terms (cells zi = 2..29): dtime*tmask*datr/rho_dzt and the x divergence
      float coef = 0.f, div = 0.f;
      bool xin = in && zi >= 2 && zi <= ZW - 3;
      if (xin) {
        bool wet = (mbits & 2) != 0;
        coef = wet ? dt * datr / d2f(a.rdz[I3(g, i, j, k)]) : 0.0f;
        div = d2f(a.dyte[I2(g, i, j)]) * d2f(a.uh[I3(g, i, j, k)]) -
              d2f(a.dyte[I2(g, i - 1, j)]) * d2f(a.uh[I3(g, i - 1, j, k)]);
      }
      s.xcoef[c] = coef;
      s.xdiv[c] = div;
      s.xin[c] = xin;
      // y face between rows zj and zj+1 (needed for zj = 1..29, zi = 2..29)
      float ymf = 0.f, yd0 = 0.f, yd1 = 0.f, yc = 0.f;
      if (in && zj >= 1 && zj <= ZW - 3 && zi >= 2 && zi <= ZW - 3) {
        float v = d2f(a.vh[I3(g, i, j, k)]);
        ymf = d2f(a.dxtn[I2(g, i, j)]) * v;
        float den = (d2f(a.rdz[I3(g, i, j, k)]) + d2f(a.rdz[I3(g, i, j + 1, k)])) * d2f(a.dytn[I2(g, i, j)]);
        float cfl = fabsf(__fdividef(v * dt * 2.0f, den));
        yd0 = (2.0f - cfl) * (1.0f - cfl) * sixth;
        yd1 = (1.0f - cfl * cfl) * sixth;
        yc = __fdividef(1.0f - cfl, 1.0e-30f + cfl);
      }
      s.ymf[c] = ymf;
      s.yd0[c] = yd0;
      s.yd1[c] = yd1;
      s.yc[c] = yc;
      // state-update factors of interior cells
      float uq = 0.f, ur = 0.f;
      if (in && zj >= 2 && zj <= ZW - 3 && zi >= 2 && zi <= ZW - 3) {
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
    __syncthreads();

#pragma unroll
    for (int n = 0; n < NC; ++n) {
      if (n >= a.ntr) break;
      const double* T = a.T + (long)n * g.n3;
      // ---- z pass ----
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NW * m, zi = lane, c = zj * ZW + zi;
        int i = i0 - 2 + zi, j = j0 - 2 + zj;
        uint8_t mb = s.zmask[c];
        float tzv = 0.f, tk = 0.f, fzv = 0.f;
        if (image(g, i, j)) {
          tk = d2f(T[I3(g, i, j, k)]);
          float tkm1 = d2f(T[I3(g, i, j, km1)]);
          float tkp1 = d2f(T[I3(g, i, j, kp1)]);
          float tkp2 = d2f(T[I3(g, i, j, kp2)]);
          bool mkm1 = mb & 1, mk = mb & 2, mkp1 = mb & 4, mkp2 = mb & 8;
          float Rjp = (mkm1 && mk) ? tkm1 - tk : 0.f;
          float Rj = (mk && mkp1) ? tk - tkp1 : 0.f;
          float Rjm = (mkp1 && mkp2) ? tkp1 - tkp2 : 0.f;
          float fbt = (mkp1 && mk) ? face_flux(s.zmf[c], Rjm, Rj, Rjp, tkp1, tk, s.zd0[c], s.zd1[c], s.zc[c]) : 0.f;
          float dtr = s.zdtr[c];
          float adiv = s.zdatr[c] * (fbt - ftp[n][m]);
          fzv = dtr * adiv;
          tzv = tk + dtr * (adiv + tk * s.zwd[c]);
          ftp[n][m] = fbt;
        }
        s.tz[c] = tzv;
        s.tf[c] = tk;
        s.fz[c] = fzv;
      }
      __syncthreads();
      // ---- x fluxes: face zi (between zi and zi+1), zi = 1..29 ----
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NW * m, zi = lane, c = zj * ZW + zi;
        float f = 0.f;
        if (zi >= 1 && zi <= ZW - 3) {
          bool m0 = s.zmask[c - 1] & 2, m1 = s.zmask[c] & 2, m2 = s.zmask[c + 1] & 2, m3 = s.zmask[c + 2] & 2;
          if (m1 && m2) {
            float tA = s.tz[c - 1], tB = s.tz[c], tC = s.tz[c + 1], tD = s.tz[c + 2];
            float Rjp = (m3 && m2) ? tD - tC : 0.f;
            float Rj = tC - tB;
            float Rjm = (m1 && m0) ? tB - tA : 0.f;
            f = face_flux(s.xmf[c], Rjm, Rj, Rjp, tB, tC, s.xd0[c], s.xd1[c], s.xc[c]);
          }
        }
        s.fx[c] = f;
      }
      __syncthreads();
      // ---- x update: cells zi = 2..29 of every row ----
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NW * m, zi = lane, c = zj * ZW + zi;
        float t = 0.f, fi = 0.f;
        if (s.xin[c]) {
          float coef = s.xcoef[c];
          fi = coef * (s.fx[c - 1] - s.fx[c]);
          t = s.tz[c] + (fi + coef * (s.tf[c] * s.xdiv[c]));
        }
        s.tx[c] = t;
        s.fxi[c] = fi;
      }
      __syncthreads();
      // ---- y fluxes: face zj (between rows zj and zj+1), zj = 1..29, zi = 2..29 ----
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NW * m, zi = lane, c = zj * ZW + zi;
        float f = 0.f;
        if (zj >= 1 && zj <= ZW - 3 && zi >= 2 && zi <= ZW - 3) {
          bool m0 = s.zmask[c - ZW] & 2, m1 = s.zmask[c] & 2, m2 = s.zmask[c + ZW] & 2, m3 = s.zmask[c + 2 * ZW] & 2;
          if (m1 && m2) {
            float tA = s.tx[c - ZW], tB = s.tx[c], tC = s.tx[c + ZW], tD = s.tx[c + 2 * ZW];
            float Rjp = (m3 && m2) ? tD - tC : 0.f;
            float Rj = tC - tB;
            float Rjm = (m1 && m0) ? tB - tA : 0.f;
            f = face_flux(s.ymf[c], Rjm, Rj, Rjp, tB, tC, s.yd0[c], s.yd1[c], s.yc[c]);
          }
        }
        s.fy[c] = f;
      }
      __syncthreads();
      // ---- interior: total increment and output ----
#pragma unroll
      for (int m = 0; m < ROWS_PER_WARP; ++m) {
        const int zj = warp + NW * m, zi = lane, c = zj * ZW + zi;
        if (zj < 2 || zj > ZW - 3 || zi < 2 || zi > ZW - 3) continue;
        const int i = i0 - 2 + zi, j = j0 - 2 + zj;
        if (i > g.ni || j > g.nj) continue;
        bool wet = s.zmask[c] & 2;
        if (!wet && !a.fused) continue;
        float fy = s.xcoef[c] * (s.fy[c - ZW] - s.fy[c]);
        float dT = s.fz[c] + s.fxi[c] + fy;
        long p = I3(g, i, j, k);
        if (a.fused) {
          // T(taup1) = T + (rho_dzt(taum1)*rho_dztr - 1)*T + rho_dzt(tau)*rho_dztr*dT
          float inc = s.uq[c] * s.tf[c] + s.ur[c] * dT;
          double tn = T[p] + f2d(inc);
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
          o[p] = o[p] + f2d(s.ur[c] * dT);
        }
      }
      __syncthreads();
    }
  }
}

template <int NC>
int run_mixed(mom5gpu_domain* d, MixArgs a, int n0) {
  const Geo& g = d->geo;
  size_t smem = sizeof(Smem);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_mdfl_mixed<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(d, e, "mixed kernel attribute");
    configured = true;
  }
  dim3 grid((g.ni + TI - 1) / TI, (g.nj + TJ - 1) / TJ);
  k_mdfl_mixed<NC><<<grid, NT, smem, d->stream>>>(a, n0);
  count_launches(d, 1);
  return MOM5GPU_OK;
}

}  // namespace

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
