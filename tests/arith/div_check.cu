// Exactness check of the FP64 division and 1e-30 + x shortcuts of the exact
// schemes (mom5_gb300/csrc/fp64_div.cuh): for every case the bit pattern of
// each shortcut (the seeded division, the division by a two-term reciprocal,
// 1e-30 + x) must equal the FP64 division / addition instruction's, and the
// host's IEEE division (NaN payloads aside).  Cases: uniformly random bit patterns
// (every exponent, subnormals, Inf, NaN), random operands of moderate exponent,
// limiter-like ratios of tracer differences, exact quotients, quotients next
// to rounding midpoints, and the binade edges of the 1e-30 + x shortcut.
// Prints "ok <cases>" and exits 0, else lists the first mismatches and exits 1.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "fp64_div.cuh"

__global__ void k_div(const double* a, const double* b, double* qf, double* qp, double* qr, double* sf, double* sr,
                      long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  qf[i] = mom5::fp64::div_seeded(a[i], b[i]);
  double yh, yl;
  mom5::fp64::recip_pair(b[i], yh, yl);
  qp[i] = mom5::fp64::div_pair(a[i], b[i], yh, yl);
  qr[i] = a[i] / b[i];
  sf[i] = mom5::fp64::add_1em30(b[i]);
  sr[i] = 1.0e-30 + b[i];
}

static uint64_t s_state = 0x9e3779b97f4a7c15ULL;
static uint64_t next_u64() {  // splitmix64
  uint64_t z = (s_state += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
static double uni() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
static double from_bits(uint64_t u) {
  double d;
  memcpy(&d, &u, 8);
  return d;
}
static uint64_t bits(double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
}

int main() {
  std::vector<double> A, B;
  auto add = [&](double a, double b) {
    A.push_back(a);
    B.push_back(b);
  };
  // uniformly random bit patterns
  for (int i = 0; i < 1 << 20; ++i) add(from_bits(next_u64()), from_bits(next_u64()));
  // moderate exponents, random signs
  for (int i = 0; i < 1 << 20; ++i) {
    double a = ldexp(1.0 + uni(), (int)(next_u64() % 121) - 60) * ((next_u64() & 1) ? -1 : 1);
    double b = ldexp(1.0 + uni(), (int)(next_u64() % 121) - 60) * ((next_u64() & 1) ? -1 : 1);
    add(a, b);
  }
  // limiter-like: differences of tracer values, divisor 1e-30 + R
  for (int i = 0; i < 1 << 20; ++i) {
    double t0 = 25.0 * uni(), t1 = t0 + 0.2 * (uni() - 0.5), t2 = t1 + 0.2 * (uni() - 0.5);
    double rj = t1 - t2, rjm = t0 - t1;
    if ((i & 7) == 0) rj = 0.0;
    if ((i & 15) == 1) rjm = rj;  // theta = 1
    add(rjm, 1.0e-30 + rj);
  }
  // exact quotients (powers of two and small integers) and next-to-midpoint quotients
  for (int i = 0; i < 1 << 18; ++i) {
    double b = ldexp(1.0 + uni(), (int)(next_u64() % 41) - 20);
    double q = (double)(1 + next_u64() % 64) * ldexp(1.0, (int)(next_u64() % 21) - 10);
    add(q * b, b);  // may round: then a near-exact quotient
    double qm = ldexp(1.0 + uni(), (int)(next_u64() % 21) - 10);
    double half_ulp = ldexp(1.0, ilogb(qm) - 53);
    add(fma(b, qm, b * half_ulp), b);  // about qm + ulp/2
    add(b, b);
    add(-b, b);
    add(0.0, b);
    add(-0.0, b);
  }
  // binade edges of the 1e-30 + x shortcut and special divisors
  const int kEdges[] = {-48, -47, -46, -45, -44, -43};
  for (int e : kEdges)
    for (int s = -1; s <= 1; s += 2) {
      double x = s * ldexp(1.0, e);
      add(1.0, x);
      add(1.0, nextafter(x, 0.0));
      add(1.0, nextafter(x, s * 1.0));
      add(1.0, x * 1.5);
    }
  const double kSpecial[] = {0.0, -0.0, 1.0e-30, -1.0e-30, INFINITY, -INFINITY, NAN, 1e-310, -1e-310, 1e300, 3.4e38,
                             1.1e-38, 1.0};
  for (double a : kSpecial)
    for (double b : kSpecial) add(a, b);

  long n = (long)A.size();
  size_t bytes = sizeof(double) * n;
  double *dA, *dB, *qf, *qp, *qr, *sf, *sr;
  if (cudaMalloc(&dA, bytes) || cudaMalloc(&dB, bytes) || cudaMalloc(&qf, bytes) || cudaMalloc(&qp, bytes) ||
      cudaMalloc(&qr, bytes) || cudaMalloc(&sf, bytes) || cudaMalloc(&sr, bytes)) {
    printf("cudaMalloc failed\n");
    return 2;
  }
  cudaMemcpy(dA, A.data(), bytes, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B.data(), bytes, cudaMemcpyHostToDevice);
  k_div<<<(unsigned)((n + 255) / 256), 256>>>(dA, dB, qf, qp, qr, sf, sr, n);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    printf("kernel: %s\n", cudaGetErrorString(e));
    return 2;
  }
  std::vector<double> QF(n), QP(n), QR(n), SF(n), SR(n);
  cudaMemcpy(QF.data(), qf, bytes, cudaMemcpyDeviceToHost);
  cudaMemcpy(QP.data(), qp, bytes, cudaMemcpyDeviceToHost);
  cudaMemcpy(QR.data(), qr, bytes, cudaMemcpyDeviceToHost);
  cudaMemcpy(SF.data(), sf, bytes, cudaMemcpyDeviceToHost);
  cudaMemcpy(SR.data(), sr, bytes, cudaMemcpyDeviceToHost);
  long bad = 0;
  for (long i = 0; i < n; ++i) {
    double host = A[i] / B[i];
    bool host_ok = isnan(host) ? isnan(QF[i]) : bits(host) == bits(QF[i]);
    if (bits(QF[i]) != bits(QR[i]) || bits(QP[i]) != bits(QR[i]) || !host_ok || bits(SF[i]) != bits(SR[i])) {
      if (bad < 20)
        printf("case %ld: a=%a b=%a  div %a pair %a (instr %a, host %a)  add %a (instr %a)\n", i, A[i], B[i], QF[i],
               QP[i], QR[i], host, SF[i], SR[i]);
      ++bad;
    }
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(qf);
  cudaFree(qp);
  cudaFree(qr);
  cudaFree(sf);
  cudaFree(sr);
  if (bad) {
    printf("%ld of %ld cases differ\n", bad, n);
    return 1;
  }
  printf("ok %ld\n", n);
  return 0;
}
