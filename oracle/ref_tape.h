// ORACLE — test infrastructure only.  Nothing in the product includes this file.
//
// The random numbers of the reference's three random textures, as both the
// compiled reference kernels (ref_step.cpp) and the oracle's
// reference-arithmetic mode (dsm_oracle.cpp, mode 2) consume them.  The
// reference fills its textures from cuRAND XORWOW (common/gpu_random.cu:107-118,
// 201-317), a stream that cannot be reproduced off the GPU; here every value is
// derived from the Philox4x32-10 words that the oracle's other modes and the
// GPU kernel draw for the same chain and event, so that all modes share one
// random stream:
//   * t_uniformrand (one uniform per kMC step, ensemble_kernel.cu:274):
//     the event words' (w1:w0) as a 64-bit fraction rounded to float, in [0,1];
//   * t_taucd_gauss_rand_CD / _SD (float4 {3 normals, lifetime rate 1/tau_CD}
//     per creation, gpu_random.cu:201-257): the normals by Box-Muller in double
//     from the event's creation words (as the oracle's FP64 mode draws them),
//     the rate from the FP64 lifetime laws of common/pcd_tau.h:67-82
//     (f_d(t) for CD-created, f(t) for SD-created entanglements) at the
//     uniform of event word w2, each rounded to float.
#pragma once
#include <cmath>
#include <cstdint>

#include "orc_math.h"

namespace reftape {

// p_cd constants (common/pcd_tau.h:32-66) that the lifetime laws need
struct Law {
  double c1, At, tau0, alpha, normdt, Adt, Bdt, tau_d, g;
};

struct Key {
  uint64_t seed;
  uint32_t stream, chain_offset;
};

// Philox words of (purpose, event ev, chain) keyed like the oracle's rng_step
inline orc::U4 words(const Key& k, uint32_t purpose, uint64_t ev, uint32_t chain) {
  return orc::philox((uint32_t)ev, (purpose << 24) | ((uint32_t)(ev >> 32) & 0xffffffu), chain + k.chain_offset,
                     k.stream, (uint32_t)k.seed, (uint32_t)(k.seed >> 32));
}

inline float uniform(const Key& k, uint64_t ev, uint32_t chain) {
  const orc::U4 r = words(k, orc::P_EVENT, ev, chain);
  const uint64_t u64 = ((uint64_t)r.y << 32) | r.x;
  return (float)((double)u64 * 5.42101086242752217e-20);  // 2^-64
}

// lifetime rates 1/tau (pcd_tau.h:67-82 in double)
inline double rate_f_t(const Law& p, double u) {
  if (u < 1.0 - p.g) return 1.0 / std::pow(u * p.c1 / p.At + std::pow(p.tau0, p.alpha), 1.0 / p.alpha);
  return 1.0 / p.tau_d;
}
inline double rate_f_dt(const Law& p, double u) {
  const double q = u * p.normdt;
  if (q < p.Bdt) return 1.0 / std::pow(q * p.c1 / p.Adt + std::pow(p.tau0, p.alpha - 1.0), 1.0 / (p.alpha - 1.0));
  return 1.0 / p.tau_d;
}

// {normal, normal, normal, rate} of a new entanglement made at event ev;
// cd_created selects the CD-created lifetime law.
inline void creation(const Key& k, const Law& law, uint64_t ev, uint32_t chain, bool cd_created, float out[4]) {
  const orc::U4 r = words(k, orc::P_EVENT, ev, chain);
  const orc::U4 g = words(k, orc::P_CREATE, ev, chain);
  const double s24 = 1.0 / 16777216.0;
  const double u1a = ((g.x >> 8) + 1u) * s24, u2a = (g.y >> 8) * s24;
  const double u1b = ((g.z >> 8) + 1u) * s24, u2b = (g.w >> 8) * s24;
  const double ra = std::sqrt(-2.0 * std::log(u1a)), rb = std::sqrt(-2.0 * std::log(u1b));
  const double tp = 6.283185307179586;
  out[0] = (float)(ra * std::cos(tp * u2a));
  out[1] = (float)(ra * std::sin(tp * u2a));
  out[2] = (float)(rb * std::cos(tp * u2b));
  const double u = ((r.z >> 8) + 1u) * s24;
  out[3] = (float)(cd_created ? rate_f_dt(law, u) : rate_f_t(law, u));
}

}  // namespace reftape
