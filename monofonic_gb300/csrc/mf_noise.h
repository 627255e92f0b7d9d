// White-noise generator of the project RNG plugin, one definition for the
// host and the device so that both produce the same bits.
//
// Cell c of an n^3 grid (c = (i*n + j)*n + k) takes draw c of a stream in which
// pair p = c / 2 is one Philox4x32-10 block (Salmon, Moraes, Dror & Shaw 2011)
// at counter (p_lo, p_hi, 0, 0) with key (seed_lo, seed_hi).  The first two
// words give a 53-bit integer b1, the last two b2; Box-Muller turns
// u1 = (b1 + 1/2) 2^-53 and the angle t = 2 pi (b2 + 1/2) 2^-53 into
// r cos t (cell 2p) and r sin t (cell 2p+1), r = sqrt(-2 ln u1).
//
// ln and sin/cos are written here from IEEE basic operations only (each
// multiply, add, fused multiply-add, divide and square root is one correctly
// rounded operation on both sides; the host side is compiled without
// floating-point contraction), so the result does not depend on the libm or
// the device math library:
//   ln u:   u = m 2^e with m in [sqrt(1/2), sqrt(2)], s = (m-1)/(m+1),
//           ln m = 2 atanh s = sum_k 2 s^(2k+1)/(2k+1) (k <= 11, |s| <= 0.172),
//           ln u = e ln2 + ln m.
//   sin/cos of a turn: the quarter-turn index q and the remainder f in
//           [-1/2, 1/2] are split off exactly in integers, then the Taylor
//           series of sin(pi f/2) and cos(pi f/2) (to f^19 / f^18, truncation
//           below 2^-60) and a quadrant rotation.
// The Taylor coefficients are (pi/2)^j / j! and 2/(2k+1), rounded to the
// nearest double.  Accuracy: a few ulp.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define MF_NZ_HD __host__ __device__ __forceinline__
#else
#define MF_NZ_HD inline
#endif

namespace mf {
namespace noise {

MF_NZ_HD double mul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
MF_NZ_HD double add(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
MF_NZ_HD double sub(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
MF_NZ_HD double fma_(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
MF_NZ_HD double div_(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
MF_NZ_HD double sqrt_(double a) {
#if defined(__CUDA_ARCH__)
  return __dsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
MF_NZ_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}
MF_NZ_HD double from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// Philox4x32-10: 10 rounds of the 4x32 S-box with the Weyl key schedule
MF_NZ_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// natural logarithm of a positive normal double
MF_NZ_HD double log_pos(double u) {
  const uint64_t b = bits(u);
  int e = (int)((b >> 52) & 0x7ff) - 1023;
  double m = from_bits((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);  // [1, 2)
  if (m > 0x1.6a09e667f3bcdp+0) {  // > sqrt(2): halve (exact)
    m = mul(m, 0.5);
    e += 1;
  }
  const double s = div_(sub(m, 1.0), add(m, 1.0));
  const double z = mul(s, s);
  double p = 0x1.642c8590b2164p-4;  // 2/23
  p = fma_(p, z, 0x1.8618618618618p-4);  // 2/21
  p = fma_(p, z, 0x1.af286bca1af28p-4);  // 2/19
  p = fma_(p, z, 0x1.e1e1e1e1e1e1ep-4);  // 2/17
  p = fma_(p, z, 0x1.1111111111111p-3);  // 2/15
  p = fma_(p, z, 0x1.3b13b13b13b14p-3);  // 2/13
  p = fma_(p, z, 0x1.745d1745d1746p-3);  // 2/11
  p = fma_(p, z, 0x1.c71c71c71c71cp-3);  // 2/9
  p = fma_(p, z, 0x1.2492492492492p-2);  // 2/7
  p = fma_(p, z, 0x1.999999999999ap-2);  // 2/5
  p = fma_(p, z, 0x1.5555555555555p-1);  // 2/3
  p = fma_(p, z, 2.0);
  return fma_((double)e, 0x1.62e42fefa39efp-1 /* ln 2 */, mul(s, p));
}

// sin and cos of the angle 2 pi (b + 1/2) 2^-53 for a 53-bit integer b
MF_NZ_HD void sincos_turn53(uint64_t b, double* sn, double* cs) {
  // x = 4 t = (2b+1) 2^-52 quarter turns; q = nearest integer, f = x - q
  const uint64_t q = (b + (1ull << 50)) >> 51;  // 0..4
  const int64_t num = (int64_t)(2 * b + 1) - (int64_t)(q << 52);  // |num| <= 2^51
  const double f = mul((double)num, 0x1p-52);
  const double w = mul(f, f);
  double ps = -0x1.8a404211f9547p-45;  // sin(pi f / 2) / f in w = f^2
  ps = fma_(ps, w, 0x1.aaec32af93359p-38);
  ps = fma_(ps, w, -0x1.6fadb9f155744p-31);
  ps = fma_(ps, w, 0x1.e8f434d018d63p-25);
  ps = fma_(ps, w, -0x1.e3074fde8871fp-19);
  ps = fma_(ps, w, 0x1.50783487ee782p-13);
  ps = fma_(ps, w, -0x1.32d2cce62bd86p-8);
  ps = fma_(ps, w, 0x1.466bc6775aae2p-4);
  ps = fma_(ps, w, -0x1.4abbce625be53p-1);
  ps = fma_(ps, w, 0x1.921fb54442d18p+0);
  double pc = -0x1.2a0c591af8314p-41;  // cos(pi f / 2) in w
  pc = fma_(pc, w, 0x1.20c62c2f2d7f5p-34);
  pc = fma_(pc, w, -0x1.b6e24f44b128fp-28);
  pc = fma_(pc, w, 0x1.f9d38a3763cc3p-22);
  pc = fma_(pc, w, -0x1.a6d1f2a204a8cp-16);
  pc = fma_(pc, w, 0x1.e1f506891babbp-11);
  pc = fma_(pc, w, -0x1.55d3c7e3cbffap-6);
  pc = fma_(pc, w, 0x1.03c1f081b5ac4p-2);
  pc = fma_(pc, w, -0x1.3bd3cc9be45dep+0);
  pc = fma_(pc, w, 1.0);
  const double s = mul(f, ps), c = pc;
  switch ((int)(q & 3)) {
    case 0: *sn = s; *cs = c; break;
    case 1: *sn = c; *cs = -s; break;
    case 2: *sn = -s; *cs = -c; break;
    default: *sn = -c; *cs = s; break;
  }
}

// the two N(0,1) draws of pair p (cells 2p and 2p+1)
MF_NZ_HD void normal_pair(uint64_t p, uint64_t seed, double* z0, double* z1) {
  uint32_t c[4] = {(uint32_t)(p & 0xFFFFFFFFu), (uint32_t)(p >> 32), 0u, 0u};
  philox4x32_10(c, (uint32_t)(seed & 0xFFFFFFFFu), (uint32_t)(seed >> 32));
  const uint64_t b1 = ((((uint64_t)c[1]) << 32) | c[0]) >> 11;
  const uint64_t b2 = ((((uint64_t)c[3]) << 32) | c[2]) >> 11;
  const double u1 = mul(add((double)b1, 0.5), 0x1p-53);
  const double r = sqrt_(mul(-2.0, log_pos(u1)));
  double sn, cs;
  sincos_turn53(b2, &sn, &cs);
  *z0 = mul(r, cs);
  *z1 = mul(r, sn);
}

}  // namespace noise
}  // namespace mf
