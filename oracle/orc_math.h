// ORACLE — test infrastructure only. Nothing in the product links this file.
//
// Element-wise arithmetic of the DSM kMC step, restated for the CPU so that the
// oracle reproduces the GPU path bit for bit.  Every function uses only IEEE-754
// single-precision +, -, *, fmaf, correctly rounded division and square root, and
// integer operations, so that a host compiler (with -ffp-contract=off) and nvcc
// (with -fmad=false and explicit fmaf) evaluate exactly the same operations.
//
//  * Philox4x32-10: Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
//    as 1, 2, 3", SC'11.  Replaces the cuRAND XORWOW streams of the reference
//    (common/gpu_random.cu:107-124,201-317).
//  * exp: Cody-Waite reduction by ln2 (hi/lo split) and a degree-7 Taylor
//    polynomial of e^r on |r| <= ln2/2.
//  * log: exponent/mantissa split with the mantissa in (sqrt(1/2), sqrt(2)],
//    log(1+f) = 2 atanh(f/(2+f)) by its odd series to s^9.
//  * sin/cos(2 pi u) for u = j/2^24: exact octant reduction of j, Taylor
//    polynomials of sin and cos on [0, pi/4].
//  * Box-Muller (basic form) for normal deviates.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

static inline float f_as(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline uint32_t as_u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// ---------------------------------------------------------------- Philox4x32-10
struct U4 { uint32_t x, y, z, w; };

static inline U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                        uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return U4{c0, c1, c2, c3};
}

// Counter purposes (high byte of counter word 1).
enum : uint32_t {
  P_EVENT = 0u,   // per kMC event: w0,w1 pick, w2 lifetime uniform, w3 partner
  P_CREATE = 1u,  // per creation event: three normal deviates
  P_BONDS = 2u,   // initialiser: 4 bonds per block
  P_QINIT = 3u,   // initialiser: normals of strand i
  P_TAUINIT = 4u  // initialiser: lifetime of entanglement k
};

// (0,1] uniform with 2^24 levels (same role as curand_uniform in the reference).
static inline float u01(uint32_t w) {
  return (float)((w >> 8) + 1u) * 5.9604644775390625e-08f;
}

// ---------------------------------------------------------------- exp / log
// exp(x); the argument is clamped to [-87.3365, 88.7228] (results between
// ~FLT_MIN and ~FLT_MAX), NaN propagates.  Scaling by 2^k uses two exact
// power-of-two factors 2^(k>>1) * 2^(k-(k>>1)).
static inline float m_exp(float x) {
  const float xc = std::fmin(std::fmax(x, -87.3365448f), 88.7228390f);
  const float MAGIC = 12582912.0f;  // 1.5 * 2^23
  const float t = std::fmaf(xc, 1.44269504088896341f, MAGIC);
  const float kf = t - MAGIC;
  const int32_t k = (int32_t)as_u(t) - (int32_t)as_u(MAGIC);
  float r = std::fmaf(kf, -0.693145751953125f, xc);
  r = std::fmaf(kf, -1.428606765330187e-06f, r);
  float p = 1.98412698e-4f;
  p = std::fmaf(p, r, 1.38888889e-3f);
  p = std::fmaf(p, r, 8.33333333e-3f);
  p = std::fmaf(p, r, 4.16666667e-2f);
  p = std::fmaf(p, r, 1.66666667e-1f);
  p = std::fmaf(p, r, 0.5f);
  p = std::fmaf(p, r, 1.0f);
  p = std::fmaf(p, r, 1.0f);
  const int32_t k1 = k >> 1, k2 = k - k1;
  const float res = (p * f_as((uint32_t)(k1 + 127) << 23)) * f_as((uint32_t)(k2 + 127) << 23);
  return (x != x) ? x : res;
}

// natural log for finite x > 0
static inline float m_log(float x) {
  uint32_t b = as_u(x);
  int32_t e = 0;
  if (b < 0x00800000u) { x = x * 8388608.0f; b = as_u(x); e = -23; }
  e += (int32_t)(b >> 23) - 127;
  uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
  if (mb > 0x3fb504f3u) { mb -= 0x00800000u; e += 1; }
  const float f = f_as(mb) - 1.0f;
  const float s = f / (2.0f + f);
  const float z = s * s;
  float p = 0.222222222f;
  p = std::fmaf(p, z, 0.285714286f);
  p = std::fmaf(p, z, 0.4f);
  p = std::fmaf(p, z, 0.666666667f);
  const float lg = std::fmaf(s * z, p, 2.0f * s);
  const float ef = (float)e;
  return std::fmaf(ef, 0.693145751953125f, std::fmaf(ef, 1.428606765330187e-06f, lg));
}

// x^y for x > 0
static inline float m_pow(float x, float y) { return m_exp(y * m_log(x)); }

// sin and cos of 2*pi*j/2^24, j in [0, 2^24)
static inline void m_sincos2pi(uint32_t j, float* sn, float* cs) {
  const uint32_t oct = (j >> 21) & 7u;
  uint32_t rem = j & 0x1fffffu;
  if (oct & 1u) rem = 0x200000u - rem;
  const float f = (float)rem * 4.76837158203125e-07f;
  const float a = f * 0.785398163397448310f;
  const float z = a * a;
  float ps = 2.75573192e-6f;
  ps = std::fmaf(ps, z, -1.98412698e-4f);
  ps = std::fmaf(ps, z, 8.33333333e-3f);
  ps = std::fmaf(ps, z, -1.66666667e-1f);
  const float sa = std::fmaf(a * z, ps, a);
  float pc = -2.75573192e-7f;
  pc = std::fmaf(pc, z, 2.48015873e-5f);
  pc = std::fmaf(pc, z, -1.38888889e-3f);
  pc = std::fmaf(pc, z, 4.16666667e-2f);
  pc = std::fmaf(pc, z, -0.5f);
  const float ca = std::fmaf(pc, z, 1.0f);
  float s, c;
  switch (oct) {
    case 0: s = sa; c = ca; break;
    case 1: s = ca; c = sa; break;
    case 2: s = ca; c = -sa; break;
    case 3: s = sa; c = -ca; break;
    case 4: s = -sa; c = -ca; break;
    case 5: s = -ca; c = -sa; break;
    case 6: s = -ca; c = sa; break;
    default: s = -sa; c = ca; break;
  }
  *sn = s; *cs = c;
}

// Box-Muller: two normal deviates from two Philox words.
static inline void m_gauss2(uint32_t w0, uint32_t w1, float* g0, float* g1) {
  const float u1 = u01(w0);
  const float r = std::sqrt(-2.0f * m_log(u1));
  float s, c;
  m_sincos2pi(w1 >> 8, &s, &c);
  *g0 = r * c;
  *g1 = r * s;
}

// Q^2 of a strand connector
static inline float m_q2(float x, float y, float z) {
  return std::fmaf(z, z, std::fmaf(y, y, x * x));
}

}  // namespace orc
