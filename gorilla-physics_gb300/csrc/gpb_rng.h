// Counter-based random numbers shared bit for bit by host and device code:
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11) and a natural log built from the atanh series, used by the
// Marsaglia polar normal draw.  Every multiply-add is an explicit fma() and no
// other expression can be contracted, so nvcc's device code and a host
// compiler (x86 or Arm, any -ffp-contract) produce identical results.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace gpb {
__host__ __device__ inline void philox4x32_10(uint32_t k0, uint32_t k1, uint32_t c[4]) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c[0] = n0;
    c[1] = n1;
    c[2] = n2;
    c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// log(x), x > 0 normal: x = m 2^e with m ∈ [√½, √2), atanh series in f=(m−1)/(m+1).
__host__ __device__ inline double det_log(double x) {
  uint64_t bits;
  memcpy(&bits, &x, 8);
  int e = (int)((bits >> 52) & 0x7FF) - 1022;
  bits = (bits & 0x800FFFFFFFFFFFFFull) | (0x3FEull << 52);  // m ∈ [0.5, 1)
  double m;
  memcpy(&m, &bits, 8);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e -= 1;
  }
  double f = (m - 1.0) / (m + 1.0);
  double f2 = f * f;
  double s = 0.0;
  for (int k = 12; k >= 0; --k) s = fma(s, f2, 1.0 / (2.0 * k + 1.0));
  return fma((double)e, 0.69314718055994530942, (2.0 * f) * s);
}

// Uniform in (0, 1) with 53 random bits from the words (w0, w1).
__host__ __device__ inline double u53(uint32_t w0, uint32_t w1) {
  double a = (double)((((uint64_t)w0) << 21) ^ (w1 >> 11)) + 0.5;
  return a * (1.0 / 9007199254740992.0);
}

// One standard normal keyed by (key0, key1) at counter (c0, c1, ·, tag):
// Marsaglia's polar method, attempts use the third counter word.
__host__ __device__ inline double polar_normal(uint32_t key0, uint32_t key1, uint32_t c0,
                                               uint32_t c1, uint32_t tag) {
  const double scale = 2.0 / 9007199254740992.0;
  for (uint32_t attempt = 0; attempt < 64; ++attempt) {
    uint32_t c[4] = {c0, c1, attempt, tag};
    philox4x32_10(key0, key1, c);
    double a = (double)((((uint64_t)c[0]) << 21) ^ (c[1] >> 11)) + 0.5;
    double b = (double)((((uint64_t)c[2]) << 21) ^ (c[3] >> 11)) + 0.5;
    double u1 = fma(a, scale, -1.0);
    double u2 = fma(b, scale, -1.0);
    double s = fma(u1, u1, u2 * u2);
    if (s >= 1.0 || s == 0.0) continue;
    return u1 * ::sqrt((-2.0 * det_log(s)) / s);
  }
  return 0.0;
}

// One uniform in (0, 1) keyed like polar_normal (third counter word 0xFFFF).
__host__ __device__ inline double philox_uniform(uint32_t key0, uint32_t key1, uint32_t c0,
                                                 uint32_t c1, uint32_t tag) {
  uint32_t c[4] = {c0, c1, 0xFFFFu, tag};
  philox4x32_10(key0, key1, c);
  return u53(c[0], c[1]);
}

constexpr uint32_t RNG_TAG_TAU = 0x7A17u;

}  // namespace gpb
