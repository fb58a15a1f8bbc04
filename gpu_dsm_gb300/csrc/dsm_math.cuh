// Element-wise arithmetic of the DSM kMC step on sm_103a.
//
// Every function is built from IEEE-754 single-precision operations with
// explicit rounding (__fmaf_rn, __fmul_rn, __fadd_rn, __fdiv_rn, __fsqrt_rn)
// and integer operations only, so the results are reproducible bit for bit by a
// host implementation of the same sequence.  No MUFU approximation and no CUDA
// math-library routine is used on the decision path.
//
//  * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter-based RNG keyed
//    by the run seed; counter = (event index, purpose, chain, ensemble).  It
//    replaces the per-chain cuRAND XORWOW buffers of the reference
//    (common/gpu_random.cu:107-124,201-317).
//  * exp: Cody-Waite reduction by ln2 (16-bit hi / lo split), degree-7 Taylor
//    polynomial of e^r on |r| <= ln2/2, exponent scaling by bit assembly.
//  * log: exponent/mantissa split with mantissa in (sqrt(1/2), sqrt(2)],
//    log(1+f) = 2 atanh(s), s = f/(2+f), odd series to s^9.
//  * sin/cos(2 pi j / 2^24): exact octant reduction on the integer j, Taylor
//    polynomials on [0, pi/4].
//  * Box-Muller (basic, non-rejecting) normal deviates.
#pragma once
#include <cstdint>

namespace dsm {

struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                     uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return U4{c0, c1, c2, c3};
}

enum : uint32_t { P_EVENT = 0u, P_CREATE = 1u, P_BONDS = 2u, P_QINIT = 3u, P_TAUINIT = 4u };

// (0,1] uniform, 2^24 levels
__device__ __forceinline__ float u01(uint32_t w) {
  return __fmul_rn((float)((w >> 8) + 1u), 5.9604644775390625e-08f);
}

// exp(x); argument clamped to [-87.3365, 88.7228], NaN propagates; 2^k applied
// as two exact power-of-two factors.
__device__ __forceinline__ float m_exp(float x) {
  const float xc = fminf(fmaxf(x, -87.3365448f), 88.7228390f);
  const float MAGIC = 12582912.0f;
  const float t = __fmaf_rn(xc, 1.44269504088896341f, MAGIC);
  const float kf = __fsub_rn(t, MAGIC);
  const int k = __float_as_int(t) - __float_as_int(MAGIC);
  float r = __fmaf_rn(kf, -0.693145751953125f, xc);
  r = __fmaf_rn(kf, -1.428606765330187e-06f, r);
  float p = 1.98412698e-4f;
  p = __fmaf_rn(p, r, 1.38888889e-3f);
  p = __fmaf_rn(p, r, 8.33333333e-3f);
  p = __fmaf_rn(p, r, 4.16666667e-2f);
  p = __fmaf_rn(p, r, 1.66666667e-1f);
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  const int k1 = k >> 1, k2 = k - k1;
  const float res = __fmul_rn(__fmul_rn(p, __int_as_float((k1 + 127) << 23)), __int_as_float((k2 + 127) << 23));
  return (x != x) ? x : res;
}

__device__ __forceinline__ float m_log(float x) {
  uint32_t b = __float_as_uint(x);
  int e = 0;
  if (b < 0x00800000u) { x = __fmul_rn(x, 8388608.0f); b = __float_as_uint(x); e = -23; }
  e += (int)(b >> 23) - 127;
  uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
  if (mb > 0x3fb504f3u) { mb -= 0x00800000u; e += 1; }
  const float f = __fsub_rn(__uint_as_float(mb), 1.0f);
  const float s = __fdiv_rn(f, __fadd_rn(2.0f, f));
  const float z = __fmul_rn(s, s);
  float p = 0.222222222f;
  p = __fmaf_rn(p, z, 0.285714286f);
  p = __fmaf_rn(p, z, 0.4f);
  p = __fmaf_rn(p, z, 0.666666667f);
  const float lg = __fmaf_rn(__fmul_rn(s, z), p, __fmul_rn(2.0f, s));
  const float ef = (float)e;
  return __fmaf_rn(ef, 0.693145751953125f, __fmaf_rn(ef, 1.428606765330187e-06f, lg));
}

__device__ __forceinline__ float m_pow(float x, float y) { return m_exp(__fmul_rn(y, m_log(x))); }

__device__ __forceinline__ void m_sincos2pi(uint32_t j, float* sn, float* cs) {
  const uint32_t oct = (j >> 21) & 7u;
  uint32_t rem = j & 0x1fffffu;
  if (oct & 1u) rem = 0x200000u - rem;
  const float f = __fmul_rn((float)rem, 4.76837158203125e-07f);
  const float a = __fmul_rn(f, 0.785398163397448310f);
  const float z = __fmul_rn(a, a);
  float ps = 2.75573192e-6f;
  ps = __fmaf_rn(ps, z, -1.98412698e-4f);
  ps = __fmaf_rn(ps, z, 8.33333333e-3f);
  ps = __fmaf_rn(ps, z, -1.66666667e-1f);
  const float sa = __fmaf_rn(__fmul_rn(a, z), ps, a);
  float pc = -2.75573192e-7f;
  pc = __fmaf_rn(pc, z, 2.48015873e-5f);
  pc = __fmaf_rn(pc, z, -1.38888889e-3f);
  pc = __fmaf_rn(pc, z, 4.16666667e-2f);
  pc = __fmaf_rn(pc, z, -0.5f);
  const float ca = __fmaf_rn(pc, z, 1.0f);
  // octant map: (sin, cos) of oct*pi/4 + angle
  const bool swap = ((oct + 1u) & 2u) != 0u;     // octants 1,2,5,6
  const float s0 = swap ? ca : sa, c0 = swap ? sa : ca;
  const bool sneg = oct >= 4u;                   // octants 4..7
  const bool cneg = (oct >= 2u) && (oct <= 5u);  // octants 2..5
  *sn = sneg ? -s0 : s0;
  *cs = cneg ? -c0 : c0;
}

__device__ __forceinline__ void m_gauss2(uint32_t w0, uint32_t w1, float* g0, float* g1) {
  const float u1 = u01(w0);
  const float r = __fsqrt_rn(__fmul_rn(-2.0f, m_log(u1)));
  float s, c;
  m_sincos2pi(w1 >> 8, &s, &c);
  *g0 = __fmul_rn(r, c);
  *g1 = __fmul_rn(r, s);
}

__device__ __forceinline__ float m_q2(float x, float y, float z) {
  return __fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x)));
}

// floor(log2 x) of a normal positive float, -200 for zero/subnormal
__device__ __forceinline__ int fexp(float x) {
  const int e = (int)((__float_as_uint(x) >> 23) & 0xffu);
  return e == 0 ? -200 : e - 127;
}
__device__ __forceinline__ float pow2f(int s) { return __int_as_float((s + 127) << 23); }

}  // namespace dsm
