// sm_103a kernels of the DSM kinetic Monte Carlo path.
//
// Design (one GB300, one process):
//   * Each chain is simulated by a TILE of W lanes (W = 16 by default, two
//     independent chains per warp; W = 32 for one chain per warp) that keeps
//     the whole chain in shared memory (slot: {Qx,Qy,Qz,Q^2} float4, N int,
//     tau rate float, quantised rate uint64 per strand, correlator level 0)
//     inside a persistent loop.  Tiles pull chains from an atomic work
//     counter, load them with coalesced float4 loads, run them to the end of
//     the launch window (or of a group of flow output windows) and write them
//     back: HBM is touched only at window boundaries and by the long-lag
//     correlator levels.
//   * The event pick is exact integer arithmetic: every rate component is
//     quantised to int64 fixed point (scale 2^S per chain).  The quantised pair
//     totals and the five chain-end rates form one array of Z-1+5 elements in
//     the reference's pick order; each lane sums a contiguous odd-width chunk
//     (bank-conflict free), one tile inclusive scan + ballot finds the lane,
//     the lane walks its chunk.  Integer sums do not depend on order, so a CPU
//     restatement reproduces the pick bit for bit.
//   * Equilibrium: only the <=3 pair rates touched by an event are recomputed
//     (two lanes per pair), and the prefix sums are patched with their deltas;
//     the chain-end rates only when a strand next to an end changes.  The
//     reference recomputes every pair every step (ensemble_kernel.cu
//     strent_kernel).  Flow: all strands are deformed and all rates recomputed
//     every step, as in the reference.
//   * Insert/remove of strands is a tile-cooperative memmove in shared memory
//     (the reference defers it to the next step, ensemble_kernel.cu:64-102).
//   * Randomness: Philox4x32-10 keyed by (seed, event counter, purpose, global
//     chain id, ensemble); lane l computes the words of event base+l, so one
//     Philox evaluation serves W consecutive events.
//   * The hot paths (strand insertion/removal, correlator sampling and level
//     pushes) are inlined into the event loop: calls would save and restore
//     the loop's live registers and spread its code (instruction-fetch stalls).
//   * No tensor cores: nothing on this path is a dense contraction.
#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "dsm_internal.h"
#include "dsm_math.cuh"

namespace dsm {

#define FULL_MASK 0xffffffffu
#define NEND 5
// minimum resident blocks of 4 warps per SM the step kernel is compiled for:
// DSM_MINB (register budget 128) and DSM_MINB_HI (budget 80) for every kind;
// the second build gains from more resident warps when small slots leave the
// shared memory for them (shear at N_K = 100: 6 blocks per SM instead of 4)
#ifndef DSM_MINB
#define DSM_MINB 4
#endif
#ifndef DSM_MINB_HI
#define DSM_MINB_HI 6
#endif
// strand insertion / removal handlers: inlined (0) or out of line (1)
#ifndef DSM_APPLY_NOINLINE
#define DSM_APPLY_NOINLINE 0
#endif
#if DSM_APPLY_NOINLINE
#define DSM_APPLY_ATTR __noinline__
#else
#define DSM_APPLY_ATTR __forceinline__
#endif
// full rate pass of the equilibrium step: out of line (1) or inlined (0)
#ifndef DSM_RATES_NOINLINE
#define DSM_RATES_NOINLINE 1
#endif
#if DSM_RATES_NOINLINE
#define DSM_RATES_ATTR __noinline__
#else
#define DSM_RATES_ATTR __forceinline__
#endif

// ------------------------------------------------------------------ tiles
// A chain is simulated by a tile of W lanes (W = 32: one chain per warp; W = 16:
// two chains per warp).  All collectives of a chain run inside its tile.
template <int W>
struct Tile {
  unsigned mask;  // lanes of this tile within the warp
  int base;       // first warp lane of the tile
  int lane;       // lane within the tile
  __device__ __forceinline__ Tile() {
    const int l = threadIdx.x & 31;
    base = l & ~(W - 1);
    lane = l & (W - 1);
    mask = (W == 32) ? 0xffffffffu : (((1u << W) - 1u) << base);
  }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  template <class T>
  __device__ __forceinline__ T shfl(T v, int src) const { return __shfl_sync(mask, v, src, W); }
  template <class T>
  __device__ __forceinline__ T shfl_up(T v, int d) const { return __shfl_up_sync(mask, v, d, W); }
  template <class T>
  __device__ __forceinline__ T shfl_xor(T v, int d) const { return __shfl_xor_sync(mask, v, d, W); }
  // predicate bits of the tile's lanes, bit i = lane i of the tile
  __device__ __forceinline__ unsigned ballot(bool p) const { return (__ballot_sync(mask, p) & mask) >> base; }
  __device__ __forceinline__ bool any(bool p) const { return (__ballot_sync(mask, p) & mask) != 0u; }
  __device__ __forceinline__ int or_(int v) const {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) v |= shfl_xor(v, o);
    return v;
  }
  __device__ __forceinline__ float sum(float v) const {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) v = __fadd_rn(v, shfl_xor(v, o));
    return v;
  }
  // Sums over the strands of a chain that come out the same for both tile
  // widths: strand i is accumulated into partial i mod 16 in index order and
  // the 16 partials meet in a 16-lane xor tree.  A 32-lane tile does this on
  // its lanes 0..15 and hands lane 0's result to every lane; the callers loop
  // over strands with stride 16 on those lanes only.
  __device__ __forceinline__ bool strand_sum_lane() const { return W == 16 || lane < 16; }
  __device__ __forceinline__ float strand_sum(float v) const {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v = __fadd_rn(v, shfl_xor(v, o));
    return W == 16 ? v : shfl(v, 0);
  }
  __device__ __forceinline__ int maxi(int v) const {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) v = max(v, shfl_xor(v, o));
    return v;
  }
};

template <int W>
__device__ __forceinline__ unsigned long long tile_scan(const Tile<W>& t, unsigned long long v) {
#pragma unroll
  for (int o = 1; o < W; o <<= 1) {
    const unsigned long long u = t.shfl_up(v, o);
    if (t.lane >= o) v += u;
  }
  return v;
}

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ unsigned long long warp_incl_scan_u64(unsigned long long v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(FULL_MASK, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(FULL_MASK, v, o));
  return v;
}

__device__ __forceinline__ int warp_max_i(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULL_MASK, v, o));
  return v;
}

// Quantisation of a rate component to 64-bit fixed point: llrint(x * sf).
__device__ __forceinline__ unsigned long long quant(float x, float sf) {
  return (unsigned long long)__float2ll_rn(__fmul_rn(x, sf));
}

// The same rounding built from 32-bit operations, for update_pairs.  sm_103a
// runs the 64-bit conversion instruction on its narrow FP64 pipe: about 100
// cycles of latency and as many cycles of pipe occupancy per warp instruction
// (about 31 cycles of latency for this form).  update_pairs converts the
// components of every recomputed pair on the critical path of each event.
// Where one or two conversions stand alone (event classification, dt), or in
// the flow pass that converts every pair of the chain each event, the extra
// instructions of this form cost more than they save at full occupancy, and
// the instruction stays (each measured on the N_K = 200 melt and shear).
//
// f2u64_rn: y in [0, 2^63) (or -0.0), the value llrint(y) takes.  Below 2^23
// adding 2^23 rounds y to an integer (the sum's ulp is 1) and the sum's bit
// pattern minus that of 2^23 is the integer, also across the carry into 2^24;
// from 2^23 up y is an integer and its significand shifted by the exponent is
// it.  NaN, infinity and y >= 2^63 give an unspecified value; update_pairs
// flags those inputs and never uses the result.  Both forms are computed and
// one is selected, so no branch splits the caller.
__device__ __forceinline__ unsigned long long f2u64_rn(float y) {
  const unsigned b = __float_as_uint(y) & 0x7fffffffu;
  const int e = (int)(b >> 23) - 150;
  const unsigned small = __float_as_uint(__fadd_rn(__uint_as_float(b), 8388608.0f)) - 0x4B000000u;
  const unsigned long long big = (unsigned long long)((b & 0x7fffffu) | 0x800000u) << (e & 63);
  return e < 0 ? (unsigned long long)small : big;
}

// Philox words (counter layout shared with the oracle)
__device__ __forceinline__ U4 rng_at(const EnsDev& E, uint32_t purpose, uint64_t ctr, uint32_t hi24,
                                     uint32_t chain) {
  // keyed by the global chain id: a chain's stream does not depend on how the
  // chains are sharded over GPUs
  return philox((uint32_t)ctr, (purpose << 24) | (hi24 & 0xffffffu), chain + E.chain_offset, E.stream, E.seed_lo,
                E.seed_hi);
}

// Lifetime samplers returning rates (gpu_random.cu:143-148, pcd_tau.h:67-82)
__device__ __forceinline__ float rate_f_t(const PcdDev& p, float u) {
  return (u < p.one_minus_g) ? m_pow(__fmaf_rn(u, p.At_, p.Dt_), p.Ct_) : p.tau_d_inv;
}
__device__ __forceinline__ float rate_f_dt(const PcdDev& p, float u) {
  return (u < p.Bdt_) ? m_pow(__fmaf_rn(u, p.Adt_, p.Ddt_), p.Cdt_) : p.tau_d_inv;
}
// p_cd fit constants (common/pcd_tau.h:32-66) evaluated in float for a
// partner of N_K = nk Kuhn steps (GEX background, gpu_random.cu:212-228);
// the oracle restates the same float operations
__device__ __noinline__ PcdDev pcd_from_nk(float be, float nk) {
  const float z = (nk + be) / (be + 1.0f);
  const float g = 0.667f;
  float alpha, tau0, tau_max, tau_d;
  if (be != 1.0f) {
    const float lb = m_log(be);
    alpha = (0.053f * lb + 0.31f) * m_pow(z, -0.012f * lb - 0.024f);
    tau0 = 0.285f * m_pow(be + 2.0f, 0.515f);
    tau_max = (nk < 2.0f) ? tau0 : 0.025f * m_pow(be + 2.0f, 2.6f) * m_pow(z, 2.83f);
    tau_d = (nk < 2.0f) ? tau0 : 0.036f * m_pow(be + 2.0f, 3.07f) * m_pow(z - 1.0f, 3.02f);
  } else {
    alpha = 0.267096f - 0.375571f * m_exp(-0.0838237f * nk);
    tau0 = 0.460277f + 0.298913f * m_exp(-0.0705314f * nk);
    tau_max = (nk < 4.0f) ? tau0 : 0.0156137f * m_pow(nk, 3.18849f);
    tau_d = (nk < 4.0f) ? tau0 : 0.0740131f * m_pow(nk, 3.18363f);
  }
  const float pa = m_pow(tau_max, alpha), p0 = m_pow(tau0, alpha);
  const float pam1 = m_pow(tau_max, alpha - 1.0f), p0m1 = m_pow(tau0, alpha - 1.0f);
  const float c1 = pa - p0, cm1 = pam1 - p0m1;
  const float rcm1c1 = (c1 == 0.0f) ? (alpha - 1.0f) / alpha / tau0 : cm1 / c1;
  const float At = 1.0f - g;
  const float Adt = At * alpha / (alpha - 1.0f);
  const float Bdt = Adt * rcm1c1;
  const float normdt = Bdt + g / tau_d;
  PcdDev d;
  d.At_ = c1 / At; d.Dt_ = p0; d.Ct_ = -1.0f / alpha;
  d.Adt_ = normdt * c1 / Adt; d.Bdt_ = Bdt / normdt; d.Cdt_ = -1.0f / (alpha - 1.0f); d.Ddt_ = p0m1;
  d.tau_d_inv = 1.0f / tau_d; d.one_minus_g = 1.0f - g; d.normdt = normdt;
  d.pad_[0] = d.pad_[1] = 0.f;
  return d;
}

// Partner law of a new entanglement.  Monodisperse: the ensemble's p_cd.
// Per-chain N_K: p_cd of a partner chain drawn uniformly from the ensemble.
// GEX background: partner mass from the inverse table (linear interpolation
// at u / step), the CD-weighted table for CD-created entanglements.
__device__ __forceinline__ PcdDev partner_pcd(const EnsDev& E, uint32_t w, bool cd_created) {
  if (E.gex) {
    const float* T = cd_created ? E.gex_Md : E.gex_M;
    const int n = cd_created ? E.gex_nd : E.gex_n;
    const float x = __fdiv_rn(u01(w), cd_created ? E.gex_step_d : E.gex_step);
    int i = (int)floorf(x);
    float di = __fsub_rn(x, (float)i);
    if (i > n - 2) { i = n - 2; di = 1.0f; }
    const float mw = __fadd_rn(__fmul_rn(__ldg(&T[i]), __fsub_rn(1.0f, di)), __fmul_rn(__ldg(&T[i + 1]), di));
    return pcd_from_nk(E.beta, __fmul_rn(mw, E.gex_scale));
  }
  if (!E.poly) return E.pcd;
  const uint32_t idx = __umulhi(w, (uint32_t)E.n_chains);
  return E.pcd_by_nk[__ldg(&E.nk_chain[idx])];
}

// Shift components of the pair (strand j, strand j+1), ensemble_kernel.cu:149-179:
// wp moves a Kuhn step from strand j+1 into strand j, wm the reverse.
// a = NT[N1], b = NT[N2].
__device__ __forceinline__ float shift_plus(const EnsDev& E, int N1, float q1, int N2, float q2, const float4& a,
                                            const float4& b) {
  const bool z1 = (q1 == 0.0f), z2 = (q2 == 0.0f);
  const int i = (z1 ? 4 * N1 + 1 : 2 * N1) + (z2 ? 4 * N2 - 1 : 2 * N2);
  const float t2 = __fmul_rn(q2, b.y);
  const float arg = __fmaf_rn(q1, a.x, -t2);
  const float pw = __fmul_rn(z1 ? 1.0f : a.z, z2 ? 1.0f : b.w);
  const float w = __fmul_rn(__fmul_rn(__ldg(&E.FRIC[i]), pw), m_exp(arg));
  return (N2 > 1) ? w : 0.0f;
}
__device__ __forceinline__ float shift_minus(const EnsDev& E, int N1, float q1, int N2, float q2, const float4& a,
                                             const float4& b) {
  const bool z1 = (q1 == 0.0f), z2 = (q2 == 0.0f);
  const int i = (z1 ? 4 * N1 - 1 : 2 * N1) + (z2 ? 4 * N2 + 1 : 2 * N2);
  const float t1 = __fmul_rn(q1, a.y);
  const float arg = __fmaf_rn(q2, b.x, -t1);
  const float pw = __fmul_rn(z1 ? 1.0f : a.w, z2 ? 1.0f : b.z);
  const float w = __fmul_rn(__fmul_rn(__ldg(&E.FRIC[i]), pw), m_exp(arg));
  return (N1 > 1) ? w : 0.0f;
}

// One of the two shift components, chosen per lane without divergence:
// minus = false gives shift_plus, minus = true shift_minus, with the same
// operations in the same order on selected operands (one exponential per lane).
__device__ __forceinline__ float shift_comp(const EnsDev& E, bool minus, int N1, float q1, int N2, float q2,
                                            const float4& a, const float4& b) {
  const bool z1 = (q1 == 0.0f), z2 = (q2 == 0.0f);
  const int i = (z1 ? 4 * N1 + (minus ? -1 : 1) : 2 * N1) + (z2 ? 4 * N2 + (minus ? 1 : -1) : 2 * N2);
  const float u = minus ? q2 : q1, ux = minus ? b.x : a.x;
  const float v = minus ? q1 : q2, vy = minus ? a.y : b.y;
  const float arg = __fmaf_rn(u, ux, -__fmul_rn(v, vy));
  const float pw = __fmul_rn(z1 ? 1.0f : (minus ? a.w : a.z), z2 ? 1.0f : (minus ? b.z : b.w));
  const float w = __fmul_rn(__fmul_rn(__ldg(&E.FRIC[i]), pw), m_exp(arg));
  return ((minus ? N1 : N2) > 1) ? w : 0.0f;
}

// status flags of a component: bit0 NaN, bit1 inf
__device__ __forceinline__ int comp_bad(float x) {
  return (x != x) ? 1 : ((__float_as_uint(x) == 0x7f800000u) ? 2 : 0);
}

// ------------------------------------------------------------------ SMEM slot
// Per-chain value that the event loop updates off its critical path: lane 0
// keeps it in shared memory, so it holds no registers of the tile.
struct ChainHdr {
  uint64_t hash;  // FNV-1a hash of the event codes
  long long pad_;
};

struct Corr0 {  // correlator level-0 counters of the resident chain
  int ins, navg;
  long long nins;
  float a0, a1, a2;  // block sum (stress) or first value of the block (MSD)
  float r1x;         // MSD mode: first entanglement in the lab frame
  float r1y, r1z;
  long long k_next, t_next;
};

struct Slot {
  float4* Q;                // {Qx, Qy, Qz, Q^2} per strand
  unsigned long long* R;    // quantised pair totals, then the 5 chain-end rates
  unsigned long long* P;    // quantised shift +1 component per pair
  int* N;                   // Kuhn steps per strand
  float* T;                 // CD lifetime rates per entanglement
  ChainHdr* h;              // event hash of the resident chain
  Corr0* k0;                // correlator level-0 counters
  float* Csh;               // correlator level-0 shift register [p][3]
  float2* Cacc;             // correlator level-0 compensated sums [p]
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

__host__ __device__ size_t step_slot_bytes(int slot_cap, int pmax) {
  const size_t n = (size_t)slot_cap + 1, nr = (size_t)slot_cap + NEND + 1;
  size_t b = n * 16 + nr * 8 + n * 8 + n * 4 + n * 4;
  b = align_up(b, 16) + sizeof(ChainHdr) + sizeof(Corr0);
  b = align_up(b, 8) + (size_t)pmax * 12;
  b = align_up(b, 8) + (size_t)pmax * 8;
  return align_up(b, 16);
}

__device__ __forceinline__ Slot make_slot(unsigned char* base, int slot_cap, int pmax) {
  Slot s;
  const size_t n = (size_t)slot_cap + 1, nr = (size_t)slot_cap + NEND + 1;
  s.Q = (float4*)base;
  s.R = (unsigned long long*)(base + n * 16);
  s.P = (unsigned long long*)(base + n * 16 + nr * 8);
  s.N = (int*)(base + n * 24 + nr * 8);
  s.T = (float*)(base + n * 28 + nr * 8);
  size_t off = align_up(n * 32 + nr * 8, 16);
  s.h = (ChainHdr*)(base + off);
  s.k0 = (Corr0*)(base + off + sizeof(ChainHdr));
  off = align_up(off + sizeof(ChainHdr) + sizeof(Corr0), 8);
  s.Csh = (float*)(base + off);
  off = align_up(off + (size_t)pmax * 12, 8);
  s.Cacc = (float2*)(base + off);
  return s;
}

// Whole-strand moves: Q and N over [lo, hi), the pair arrays T, R and P over
// [lo_p, hi - 1), one place up or down.  All arrays of a lane's strand are
// loaded before the tile synchronises and stored after it; a round's stores
// never touch what the next round loads, and a store into a slot that the
// previous round loaded comes after this round's synchronisation, so one
// synchronisation per round and one at the end suffice.
template <int W>
__device__ __forceinline__ void move_strands_up(Slot& sl, int lo, int hi, const Tile<W>& t) {  // -> +1
  for (int top = hi - 1; top >= lo; top -= W) {
    const int s = top - t.lane;
    const bool act = s >= lo, pr = act && s < hi - 1;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    int n = 0;
    float ta = 0.f;
    unsigned long long r = 0, p = 0;
    if (act) { q = sl.Q[s]; n = sl.N[s]; }
    if (pr) { ta = sl.T[s]; r = sl.R[s]; p = sl.P[s]; }
    t.sync();
    if (act) { sl.Q[s + 1] = q; sl.N[s + 1] = n; }
    if (pr) { sl.T[s + 1] = ta; sl.R[s + 1] = r; sl.P[s + 1] = p; }
  }
  t.sync();
}
template <int W>
__device__ __forceinline__ void move_strands_down(Slot& sl, int lo, int lo_p, int hi, const Tile<W>& t) {  // -> -1
  for (int bot = min(lo, lo_p); bot < hi; bot += W) {
    const int s = bot + t.lane;
    const bool act = s >= lo && s < hi, pr = s >= lo_p && s < hi - 1;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    int n = 0;
    float ta = 0.f;
    unsigned long long r = 0, p = 0;
    if (act) { q = sl.Q[s]; n = sl.N[s]; }
    if (pr) { ta = sl.T[s]; r = sl.R[s]; p = sl.P[s]; }
    t.sync();
    if (act) { sl.Q[s - 1] = q; sl.N[s - 1] = n; }
    if (pr) { sl.T[s - 1] = ta; sl.R[s - 1] = r; sl.P[s - 1] = p; }
  }
  t.sync();
}

// float components {CD destruction, shift +1, shift -1, CD creation} of pair p
// (ensemble_kernel.cu:149-181,304-414)
__device__ __forceinline__ void pair_floats(const EnsDev& E, const Slot& sl, int p, float o[4]) {
  const int N1 = sl.N[p], N2 = sl.N[p + 1];
  const float q1 = sl.Q[p].w, q2 = sl.Q[p + 1].w;
  const float4 a = __ldg(&E.NT[N1]), b = __ldg(&E.NT[N2]);
  o[0] = E.cd_flag ? sl.T[p] : 0.0f;
  o[1] = shift_plus(E, N1, q1, N2, q2, a, b);
  o[2] = shift_minus(E, N1, q1, N2, q2, a, b);
  o[3] = E.cd_flag ? __ldg(&E.NE[N1]).w : 0.0f;
}

// Chain-end component q (0 CD creation at the tail, 1 SD creation head, 2 SD
// creation tail, 3 SD destruction head, 4 SD destruction tail),
// ensemble_kernel.cu:219-260; branch-free over the five lanes.
__device__ __forceinline__ float end_comp(const EnsDev& E, int q, int Z, const int* sN, float wz1) {
  const bool tail = (q == 0) || (q == 2) || (q == 4);
  const int Ne = tail ? sN[Z - 1] : sN[0];
  const int Nn = (Z >= 2) ? (tail ? sN[Z - 2] : sN[1]) : 1;
  const float4 e1 = __ldg(&E.NE[Ne]);
  const float4 e2 = __ldg(&E.NE[Nn]);
  const float cdc = E.cd_flag ? e1.w : 0.0f;
  const float sdc = (Z == 1) ? wz1 : ((Ne == 1) ? 0.0f : e1.x);
  const float sdd = (Z == 1 || Ne != 1) ? 0.0f : ((Z == 2) ? e2.y : e2.z);
  return (q == 0) ? cdc : ((q <= 2) ? sdc : sdd);
}

// Recompute quantised totals of pairs [p0, p0+cnt) (cnt <= 3; every caller
// touches at most three pairs) with four lanes per pair, one rate component
// each: k = lane & 3 is 0 CD destruction, 1 shift +1, 2 shift -1, 3 CD
// creation.  All four lanes run the shift-rate arithmetic (the two CD lanes
// discard it) so that the group takes one path; each lane quantises its own
// component, and two xor shuffles form the pair total (an integer sum, so its
// order does not matter).  Returns 4 when a component is NaN, inf or beyond
// the fixed-point range (the caller then runs the full pass, which decides
// between a stall and a lower scale, as the oracle does); *delta gets new - old
// of the pair total on the group's first lane (lanes 0, 4, 8), 0 elsewhere.
template <int W>
__device__ __forceinline__ int update_pairs(const EnsDev& E, Slot& sl, int Z, int S, int p0, int cnt, const Tile<W>& t,
                                            unsigned long long* delta) {
  const int lane = t.lane;
  const int k = lane & 3;
  const int p = p0 + (lane >> 2);
  const bool act = (lane < 4 * cnt) && p >= 0 && p < Z - 1;
  float o = 0.0f;
  if (act) {
    const int N1 = sl.N[p];
    const int N2 = sl.N[p + 1];
    const float q1 = sl.Q[p].w, q2 = sl.Q[p + 1].w;
    const float4 a = __ldg(&E.NT[N1]), b = __ldg(&E.NT[N2]);
    const float w = shift_comp(E, k == 2, N1, q1, N2, q2, a, b);
    // the CD components, loaded by the whole group (same addresses) and selected
    const float tp = sl.T[p], ne = __ldg(&E.NE[N1]).w;
    const float cd = (k == 0) ? tp : ne;
    o = (k == 1 || k == 2) ? w : (E.cd_flag ? cd : 0.0f);
  }
  const float y = __fmul_rn(o, pow2f(S));
  const bool bad = !(y < 281474976710656.0f);  // 2^(LIMIT_E+1); NaN too
  const unsigned long long v = f2u64_rn(y);
  unsigned long long tot = v + t.shfl_xor(v, 1);
  tot += t.shfl_xor(tot, 2);
  unsigned long long d = 0;
  if (act && k == 0) {
    d = tot - sl.R[p];
    sl.R[p] = tot;
  }
  if (act && k == 1) sl.P[p] = v;
  *delta = d;
  t.sync();
  return t.any(bad) ? 4 : 0;
}

// Full pass over all pairs and the chain ends: quantise with the current scale,
// track the max exponent; apply the scale rule shared with the oracle (lower on
// overflow; flow raises again once 2^16 of headroom is free) and requantise if S
// changes.  Returns the new S; *flags_out gets NaN/inf bits (S kept then).
template <bool FLOW, int W>
__device__ __forceinline__ int full_rates_body(const EnsDev& E, Slot& sl, int Z, int S, float wz1, const Tile<W>& t,
                                               int* flags_out) {
  const int lane = t.lane;
  const int np = Z - 1;
  int emax = -200, flags = 0;
  const float sf = pow2f(S);
  // per component: NaN -> bit0, +inf -> bit1, else its exponent counts
  // towards emax; bad components need not be excluded from the exponent
  // maximum (any flag keeps the scale), so the largest |bits| gives it, and
  // a NaN is exactly an |bits| above the infinity pattern
  unsigned mx = 0u;
  for (int p = lane; p < np; p += W) {
    float o[4];
    pair_floats(E, sl, p, o);
    unsigned long long tot = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const unsigned b = __float_as_uint(o[q]);
      mx = max(mx, b & 0x7fffffffu);
      if (b == 0x7f800000u) flags |= 2;
      tot += quant(o[q], sf);
    }
    sl.R[p] = tot;
    sl.P[p] = quant(o[1], sf);
  }
  if (mx > 0x7f800000u) flags |= 1;
  if (mx >= 0x00800000u) emax = max(emax, (int)(mx >> 23) - 127);
  float ev = 0.0f;
  if (lane < NEND) {
    ev = end_comp(E, lane, Z, sl.N, wz1);
    emax = max(emax, fexp(ev));
    sl.R[np + lane] = quant(ev, sf);
  }
  emax = t.maxi(emax);
  flags = t.or_(flags);
  int Snew = S;
  if (flags == 0) {
    if (emax + S > LIMIT_E) Snew = LIMIT_E - emax;
    else if (FLOW && S < E.s0 && emax + S < LIMIT_E - S_HYST) Snew = min(E.s0, LIMIT_E - emax);
  }
  if (Snew != S) {
    const float sf2 = pow2f(Snew);
    for (int p = lane; p < np; p += W) {
      float o[4];
      pair_floats(E, sl, p, o);
      const unsigned long long qp = quant(o[1], sf2);
      sl.R[p] = quant(o[0], sf2) + qp + quant(o[2], sf2) + quant(o[3], sf2);
      sl.P[p] = qp;
    }
    if (lane < NEND) sl.R[np + lane] = quant(ev, sf2);
  }
  t.sync();
  *flags_out = flags;
  return Snew;
}

// Equilibrium ensembles run the full pass only at window starts and after
// scale changes: out of line by default.  Flow runs the body every event,
// inlined (no call, no register save and restore around it).
template <bool FLOW, int W>
__device__ DSM_RATES_ATTR int full_rates(const EnsDev& E, Slot& sl, int Z, int S, float wz1, const Tile<W> t,
                                       int* flags_out) {
  return full_rates_body<FLOW, W>(E, sl, Z, S, wz1, t, flags_out);
}

// Deformation of every strand by the pending dt: Q += dt kappa Q
// (ensemble_kernel.cu:105-110,135-146)
template <int W>
__device__ __forceinline__ void flow_deform(const EnsDev& E, Slot& sl, int Z, float dt_prev, const Tile<W>& t) {
  float a[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) a[q] = __fmul_rn(dt_prev, E.kap[q]);
  for (int s = t.lane; s < Z; s += W) {
    const float4 q = sl.Q[s];
    const float nx = __fmaf_rn(a[2], q.z, __fmaf_rn(a[1], q.y, __fmaf_rn(a[0], q.x, q.x)));
    const float ny = __fmaf_rn(a[5], q.z, __fmaf_rn(a[4], q.y, __fmaf_rn(a[3], q.x, q.y)));
    const float nz = __fmaf_rn(a[8], q.z, __fmaf_rn(a[7], q.y, __fmaf_rn(a[6], q.x, q.z)));
    sl.Q[s] = make_float4(nx, ny, nz, m_q2(nx, ny, nz));
  }
  t.sync();
}

// Stress of the resident chain, sigma_ab = -sum 3 Q_a Q_b / N, Lpp = sum |Q|,
// and Z (ensemble_kernel.cu:504-538); lane 0 writes the 8 floats to o
template <int W>
__device__ __forceinline__ void flow_stress(const EnsDev& E, const Slot& sl, int Z, const Tile<W>& t, float* o) {
  float s[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int i = t.lane; t.strand_sum_lane() && i < Z; i += 16) {
    const float4 q = sl.Q[i];
    const float w = __ldg(&E.INV3N[sl.N[i]]);
    s[0] = __fmaf_rn(-__fmul_rn(q.x, q.x), w, s[0]);
    s[1] = __fmaf_rn(-__fmul_rn(q.y, q.y), w, s[1]);
    s[2] = __fmaf_rn(-__fmul_rn(q.z, q.z), w, s[2]);
    s[3] = __fmaf_rn(-__fmul_rn(q.x, q.y), w, s[3]);
    s[4] = __fmaf_rn(-__fmul_rn(q.y, q.z), w, s[4]);
    s[5] = __fmaf_rn(-__fmul_rn(q.x, q.z), w, s[5]);
    s[6] = __fadd_rn(s[6], __fsqrt_rn(q.w));
  }
#pragma unroll
  for (int q = 0; q < 7; ++q) s[q] = t.strand_sum(s[q]);
  if (t.lane == 0) {
#pragma unroll
    for (int q = 0; q < 7; ++q) o[q] = s[q];
    o[7] = (float)Z;
  }
}

// ------------------------------------------------------------------ correlator
// Levels >= 1 of the multi-tau correlator in HBM (eq_ensemble_kernel.cu:133-227):
// push w into level 1 and cascade while blocks complete.  Stress (type 0):
// the next level gets the block average, lag terms are products.  MSD (type
// 1, :181-189,203,218): the next level gets the first value of each block (a
// position is sampled, not averaged), lag terms are squared differences.
template <int W, bool MSD>
__device__ __forceinline__ void corr_push_levels(const EnsDev& E, int c, float w0, float w1, float w2, const Tile<W> t) {
  const int lane = t.lane;
  const int L = E.corr_levels, p = E.corr_p, m = E.corr_m, dmin = p / m;
  constexpr bool msd = MSD;
  for (int k = 1; k < L; ++k) {
    const size_t lk = (size_t)c * L + k;
    int4* cntp = &E.corr_cnt[lk];
    const int4 cnt = *cntp;
    float* sh = &E.corr_shift[lk * p * 3];
    float* av = &E.corr_avg[lk * 3];
    double* acc = &E.corr_acc[lk * p];
    const int ins = cnt.x;
    const long long nins = (((long long)(unsigned)cnt.w) << 32 | (unsigned)cnt.z) + 1;
    float a0, a1, a2;
    if (!msd) {
      a0 = __fadd_rn(av[0], w0); a1 = __fadd_rn(av[1], w1); a2 = __fadd_rn(av[2], w2);
    } else if (cnt.y == 0) {
      a0 = w0; a1 = w1; a2 = w2;
    } else {
      a0 = av[0]; a1 = av[1]; a2 = av[2];
    }
    t.sync();
    if (lane == 0) { sh[ins * 3 + 0] = w0; sh[ins * 3 + 1] = w1; sh[ins * 3 + 2] = w2; }
    t.sync();
    for (int j = dmin + lane; j < p; j += W) {
      if ((long long)j >= nins) break;
      int i2 = ins - j;
      if (i2 < 0) i2 += p;
      float pv;
      if (msd) {
        const float d0 = __fsub_rn(w0, sh[i2 * 3 + 0]), d1 = __fsub_rn(w1, sh[i2 * 3 + 1]), d2 = __fsub_rn(w2, sh[i2 * 3 + 2]);
        pv = __fmaf_rn(d2, d2, __fmaf_rn(d1, d1, __fmul_rn(d0, d0)));
      } else {
        pv = __fmaf_rn(w2, sh[i2 * 3 + 2], __fmaf_rn(w1, sh[i2 * 3 + 1], __fmul_rn(w0, sh[i2 * 3 + 0])));
      }
      acc[j] += (double)pv;
    }
    const int navg = cnt.y + 1;
    const bool up = (navg == m);
    t.sync();
    if (lane == 0) {
      if (up) { av[0] = 0.f; av[1] = 0.f; av[2] = 0.f; }
      else { av[0] = a0; av[1] = a1; av[2] = a2; }
      *cntp = make_int4(ins + 1 == p ? 0 : ins + 1, up ? 0 : navg, (int)(unsigned)(nins & 0xffffffffll),
                        (int)(unsigned)(nins >> 32));
    }
    t.sync();
    if (!up) break;
    if (msd) {
      w0 = a0; w1 = a1; w2 = a2;
    } else {
      const float rm = (float)m;
      w0 = __fdiv_rn(a0, rm); w1 = __fdiv_rn(a1, rm); w2 = __fdiv_rn(a2, rm);
    }
  }
}

// Centre of mass of the resident chain (eq_ensemble_kernel.cu:297-321): strand
// s contributes N_s/N_K times its midpoint R1 + sum_{i<s} Q_i + Q_s/2.  The
// prefix sums over strands run as tile scans, W strands at a time.
template <int W>
__device__ __forceinline__ void chain_com(const EnsDev& E, const Slot& sl, int Z, int c, const Tile<W>& t, float* v) {
  const int lane = t.lane;
  float cx = 0.f, cy = 0.f, cz = 0.f, px = 0.f, py = 0.f, pz = 0.f;
  for (int base = 0; base < Z; base += W) {
    const int s = base + lane;
    const bool in = s < Z;
    const float4 q = in ? sl.Q[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float n = in ? (float)sl.N[s] : 0.f;
    float ix = q.x, iy = q.y, iz = q.z;
#pragma unroll
    for (int o = 1; o < W; o <<= 1) {
      const float ux = t.shfl_up(ix, o), uy = t.shfl_up(iy, o), uz = t.shfl_up(iz, o);
      if (lane >= o) { ix = __fadd_rn(ix, ux); iy = __fadd_rn(iy, uy); iz = __fadd_rn(iz, uz); }
    }
    float ex = t.shfl_up(ix, 1), ey = t.shfl_up(iy, 1), ez = t.shfl_up(iz, 1);
    if (lane == 0) { ex = 0.f; ey = 0.f; ez = 0.f; }
    cx = __fmaf_rn(__fadd_rn(__fadd_rn(px, ex), __fmul_rn(0.5f, q.x)), n, cx);
    cy = __fmaf_rn(__fadd_rn(__fadd_rn(py, ey), __fmul_rn(0.5f, q.y)), n, cy);
    cz = __fmaf_rn(__fadd_rn(__fadd_rn(pz, ez), __fmul_rn(0.5f, q.z)), n, cz);
    px = __fadd_rn(px, t.shfl(ix, W - 1)); py = __fadd_rn(py, t.shfl(iy, W - 1)); pz = __fadd_rn(pz, t.shfl(iz, W - 1));
  }
  const float nk = (float)(E.poly ? __ldg(&E.nk_chain[c]) : E.nk);
  const Corr0& k0 = *sl.k0;
  v[0] = __fadd_rn(__fdiv_rn(t.sum(cx), nk), k0.r1x);
  v[1] = __fadd_rn(__fdiv_rn(t.sum(cy), nk), k0.r1y);
  v[2] = __fadd_rn(__fdiv_rn(t.sum(cz), nk), k0.r1z);
}

// Take every sample due at chain time T (eq_ensemble_kernel.cu:281-331): the
// shear stresses (xy, yz, xz) or the centre of mass into correlator level 0.
// Inlined into the event loop together with the level pushes: a call would
// save and restore the loop's live registers around every sample (measured
// +5.8 % events/s at N_K = 200, p = 64, m = 8; +15 % at N_K = 50, p = 16, m = 2).
template <int W, bool MSD>
__device__ __forceinline__ void corr_samples(const EnsDev& E, Slot& sl, int Z, int c, long long T, const Tile<W> t) {
  const int lane = t.lane;
  Corr0& k0 = *sl.k0;
  const int p = E.corr_p, m = E.corr_m;
  constexpr bool msd = MSD;
  while (k0.k_next < E.nsamples && T > k0.t_next) {
    float v[3];
    if (msd) {
      chain_com<W>(E, sl, Z, c, t, v);
    } else {
      float sxy = 0.f, syz = 0.f, sxz = 0.f;
      for (int s = lane; t.strand_sum_lane() && s < Z; s += 16) {
        const float4 q = sl.Q[s];
        const float w = __ldg(&E.INV3N[sl.N[s]]);
        sxy = __fmaf_rn(-__fmul_rn(q.x, q.y), w, sxy);
        syz = __fmaf_rn(-__fmul_rn(q.y, q.z), w, syz);
        sxz = __fmaf_rn(-__fmul_rn(q.x, q.z), w, sxz);
      }
      v[0] = t.strand_sum(sxy); v[1] = t.strand_sum(syz); v[2] = t.strand_sum(sxz);
    }
    const int ins = k0.ins;
    const long long n0 = k0.nins + 1;
    t.sync();
    if (lane == 0) { sl.Csh[ins * 3 + 0] = v[0]; sl.Csh[ins * 3 + 1] = v[1]; sl.Csh[ins * 3 + 2] = v[2]; }
    t.sync();
    for (int j = lane; j < p; j += W) {
      if ((long long)j >= n0) break;
      int i2 = ins - j;
      if (i2 < 0) i2 += p;
      float pv;
      if (msd) {
        const float d0 = __fsub_rn(v[0], sl.Csh[i2 * 3 + 0]), d1 = __fsub_rn(v[1], sl.Csh[i2 * 3 + 1]);
        const float d2 = __fsub_rn(v[2], sl.Csh[i2 * 3 + 2]);
        pv = __fmaf_rn(d2, d2, __fmaf_rn(d1, d1, __fmul_rn(d0, d0)));
      } else {
        pv = __fmaf_rn(v[2], sl.Csh[i2 * 3 + 2], __fmaf_rn(v[1], sl.Csh[i2 * 3 + 1], __fmul_rn(v[0], sl.Csh[i2 * 3 + 0])));
      }
      // Kahan-compensated FP32 accumulation
      float2 a = sl.Cacc[j];
      const float y = __fsub_rn(pv, a.y);
      const float tt = __fadd_rn(a.x, y);
      a.y = __fsub_rn(__fsub_rn(tt, a.x), y);
      a.x = tt;
      sl.Cacc[j] = a;
    }
    float a0, a1, a2;
    if (!msd) {
      a0 = __fadd_rn(k0.a0, v[0]); a1 = __fadd_rn(k0.a1, v[1]); a2 = __fadd_rn(k0.a2, v[2]);
    } else if (k0.navg == 0) {
      a0 = v[0]; a1 = v[1]; a2 = v[2];
    } else {
      a0 = k0.a0; a1 = k0.a1; a2 = k0.a2;
    }
    const int navg = k0.navg + 1;
    t.sync();
    if (lane == 0) {
      k0.ins = (ins + 1 == p) ? 0 : ins + 1;
      k0.nins = n0;
      if (navg == m) { k0.a0 = k0.a1 = k0.a2 = 0.f; k0.navg = 0; }
      else { k0.a0 = a0; k0.a1 = a1; k0.a2 = a2; k0.navg = navg; }
      k0.k_next += 1;
      k0.t_next += E.dt_sample_ticks;
    }
    t.sync();
    if (navg == m && E.corr_levels > 1) {
      if (msd) {
        corr_push_levels<W, MSD>(E, c, a0, a1, a2, t);
      } else {
        const float rm = (float)m;
        corr_push_levels<W, MSD>(E, c, __fdiv_rn(a0, rm), __fdiv_rn(a1, rm), __fdiv_rn(a2, rm), t);
      }
    }
  }
}

// ------------------------------------------------------------------ creation events
// Position of a CD creation inside a strand of N1 Kuhn steps
// (ensemble_kernel.cu:386: newn = floor(0.5 + pr (N1 - 2) / w) + 1) on the
// quantised values r < w: x = floor((2 r (N1 - 2) + w) / (2 w)), exactly.  An
// FP32 estimate from the leading 24 bits of r and w (32-bit conversions only)
// is corrected with 128-bit integer products, so no FP64 operation is needed
// (sm_103a's FP64 divide costs about 430 cycles).  x stays in [0, N1 - 2]; the
// estimate is within one of it, and each correction loop moves x towards it.
__device__ __forceinline__ int split_pos(unsigned long long r, unsigned long long w, int N1) {
  const unsigned m = (unsigned)max(N1 - 2, 0);
  if (m == 0u || w == 0ull) return 0;
  // numerator 2 r m + w as nh:nl
  unsigned long long nl = r * m, nh = __umul64hi(r, (unsigned long long)m);
  nh = (nh << 1) | (nl >> 63);
  nl <<= 1;
  nl += w;
  nh += (nl < w) ? 1ull : 0ull;
  const unsigned long long d = w << 1;  // w < 2^62
  const int sh = max(0, 40 - __clzll((long long)w));  // w >> sh < 2^24, r >> sh <= w >> sh
  const float ratio = __fdiv_rn((float)(unsigned)(r >> sh), (float)(unsigned)(w >> sh));
  int q = (int)__fmaf_rn(ratio, (float)m, 0.5f);
  q = min(max(q, 0), (int)m);
  // q d as ph:pl; step q down while q d > num, then up while (q + 1) d <= num
  unsigned long long pl = (unsigned long long)q * d, ph = __umul64hi((unsigned long long)q, d);
  while (ph > nh || (ph == nh && pl > nl)) {
    ph -= (pl < d) ? 1ull : 0ull;
    pl -= d;
    --q;
  }
  for (;;) {
    const unsigned long long l2 = pl + d, h2 = ph + ((l2 < pl) ? 1ull : 0ull);
    if (h2 > nh || (h2 == nh && l2 > nl)) break;
    pl = l2;
    ph = h2;
    ++q;
  }
  return q;
}

// Apply a creation (CD inside strand j / CD at the tail / SD at head or tail):
// returns newn and the pairs to recompute (up0, upn).
template <int W>
__device__ DSM_APPLY_ATTR int apply_create(const EnsDev& E, Slot& sl, int evn, int j, int Z, int c, uint64_t step,
                                         unsigned long long rem, unsigned long long wsel, uint32_t w2, uint32_t w3,
                                         const Tile<W> t, int* up0_out, int* upn_out) {
  const int lane = t.lane;
  int newn = 0;
  if (evn == CDC_MID || evn == CDC_TAIL) {
    const int N1 = (evn == CDC_MID) ? sl.N[j] : sl.N[Z - 1];
    newn = split_pos(rem, wsel, N1) + 1;
    newn = max(1, min(N1 - 1, newn));
  }
  const U4 gr = rng_at(E, P_CREATE, step, (uint32_t)(step >> 32), (uint32_t)c);
  float g0, g1, g2, g3;
  m_gauss2(gr.x, gr.y, &g0, &g1);
  m_gauss2(gr.z, gr.w, &g2, &g3);
  const PcdDev pp = partner_pcd(E, w3, evn == CDC_MID || evn == CDC_TAIL);
  const float u = u01(w2);
  const float trate = E.cd_flag ? ((evn == CDC_MID || evn == CDC_TAIL) ? rate_f_dt(pp, u) : rate_f_t(pp, u)) : 0.0f;
  // The new strands are computed by every lane before the strands move (their
  // latency overlaps the move), and lane 0 stores them after it.
  if (evn == CDC_MID && j > 0) {
    const int N1 = sl.N[j];
    const float4 q1 = sl.Q[j];
    const float sg = __fsqrt_rn(__fdiv_rn((float)(newn * (N1 - newn)), (float)(3 * N1)));
    const float ra = __fdiv_rn((float)newn, (float)N1);
    const float x = __fmaf_rn(q1.x, ra, __fmul_rn(g0, sg));
    const float y = __fmaf_rn(q1.y, ra, __fmul_rn(g1, sg));
    const float z = __fmaf_rn(q1.z, ra, __fmul_rn(g2, sg));
    const float x2 = __fsub_rn(q1.x, x), y2 = __fsub_rn(q1.y, y), z2 = __fsub_rn(q1.z, z);
    const float4 qa = make_float4(x, y, z, m_q2(x, y, z)), qb = make_float4(x2, y2, z2, m_q2(x2, y2, z2));
    t.sync();
    move_strands_up(sl, j, Z, t);
    if (lane == 0) {
      sl.N[j] = newn; sl.Q[j] = qa;
      sl.N[j + 1] = N1 - newn; sl.Q[j + 1] = qb;
      sl.T[j] = trate;
    }
    *up0_out = j - 1; *upn_out = 3;
  } else if ((evn == CDC_MID && j == 0) || evn == SDC_HEAD) {
    const int N0 = sl.N[0];
    const int nn = (evn == SDC_HEAD) ? N0 - 1 : N0 - newn;
    const int nd = (evn == SDC_HEAD) ? 1 : newn;
    const float sg = (evn == SDC_HEAD && Z == 1) ? 0.0f : __fsqrt_rn(__fdiv_rn((float)nn, 3.0f));
    const float x = __fmul_rn(g0, sg), y = __fmul_rn(g1, sg), z = __fmul_rn(g2, sg);
    const float4 qn = make_float4(x, y, z, m_q2(x, y, z));
    t.sync();
    move_strands_up(sl, 0, Z, t);
    if (lane == 0) {
      sl.N[0] = nd; sl.Q[0] = make_float4(0.f, 0.f, 0.f, 0.f);
      sl.N[1] = nn; sl.Q[1] = qn;
      sl.T[0] = trate;
      if (E.corr_type == 1) {  // MSD: the new first entanglement (eq_ensemble_kernel.cu:531-539,606-614)
        Corr0& k0 = *sl.k0;
        k0.r1x = __fsub_rn(k0.r1x, x); k0.r1y = __fsub_rn(k0.r1y, y); k0.r1z = __fsub_rn(k0.r1z, z);
      }
    }
    *up0_out = 0; *upn_out = 2;
  } else {  // CDC_TAIL, SDC_TAIL
    const int Nt = sl.N[Z - 1];
    const int nn = (evn == SDC_TAIL) ? Nt - 1 : newn;
    const int nd = (evn == SDC_TAIL) ? 1 : Nt - newn;
    const float sg = (Z == 1) ? 0.0f : __fsqrt_rn(__fdiv_rn((float)nn, 3.0f));
    const float x = __fmul_rn(g0, sg), y = __fmul_rn(g1, sg), z = __fmul_rn(g2, sg);
    const float4 qn = make_float4(x, y, z, m_q2(x, y, z));
    t.sync();
    if (lane == 0) {
      sl.N[Z] = nd; sl.Q[Z] = make_float4(0.f, 0.f, 0.f, 0.f);
      sl.N[Z - 1] = nn; sl.Q[Z - 1] = qn;
      sl.T[Z - 1] = trate;
    }
    *up0_out = Z - 2; *upn_out = 2;
  }
  t.sync();
  return newn;
}

// Apply a destruction (CD of pair j, SD at head or tail): sets the pairs to
// recompute (up0, upn).
template <int W, bool MSD>
__device__ DSM_APPLY_ATTR void apply_destroy(Slot& sl, int evn, int j, int Z, const Tile<W> t, int* up0_out,
                                          int* upn_out) {
  constexpr bool msd = MSD;
  const int lane = t.lane;
  if (evn == CDD) {  // ensemble_kernel.cu:312-323
    const int n = sl.N[j] + sl.N[j + 1];
    const float4 a = sl.Q[j], b = sl.Q[j + 1];
    const bool endp = (j == Z - 2) || (j == 0);
    // the merged strand, computed by every lane before the move, stored by lane 0 after it
    const float x = endp ? 0.f : __fadd_rn(a.x, b.x);
    const float y = endp ? 0.f : __fadd_rn(a.y, b.y);
    const float z = endp ? 0.f : __fadd_rn(a.z, b.z);
    const float4 qm = make_float4(x, y, z, m_q2(x, y, z));
    t.sync();
    move_strands_down(sl, j + 2, j + 1, Z, t);
    if (lane == 0) {
      sl.N[j] = n; sl.Q[j] = qm;
      if (msd && j == 0) {  // the first entanglement is now the old second one (eq_ensemble_kernel.cu:447-455)
        Corr0& k0 = *sl.k0;
        k0.r1x = __fadd_rn(k0.r1x, b.x); k0.r1y = __fadd_rn(k0.r1y, b.y); k0.r1z = __fadd_rn(k0.r1z, b.z);
      }
    }
    *up0_out = j - 1; *upn_out = 2;
  } else if (evn == SDD_HEAD) {  // ensemble_kernel.cu:492-494
    const int n = sl.N[1] + 1;
    const float4 b = sl.Q[1];
    t.sync();
    move_strands_down(sl, 1, 1, Z, t);
    if (lane == 0) {
      sl.N[0] = n; sl.Q[0] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (msd) {  // eq_ensemble_kernel.cu:645-653
        Corr0& k0 = *sl.k0;
        k0.r1x = __fadd_rn(k0.r1x, b.x); k0.r1y = __fadd_rn(k0.r1y, b.y); k0.r1z = __fadd_rn(k0.r1z, b.z);
      }
    }
    *up0_out = 0; *upn_out = 1;
  } else {  // SDD_TAIL, ensemble_kernel.cu:495-498
    t.sync();
    if (lane == 0) { sl.N[Z - 2] += 1; sl.Q[Z - 2] = make_float4(0.f, 0.f, 0.f, 0.f); }
    *up0_out = Z - 3; *upn_out = 1;
  }
  t.sync();
}

// ------------------------------------------------------------------ phase clocks
// Debug build (-DDSM_PHASE_CLOCKS, library libgpudsm_phases.so, driven by
// gpu_dsm_gb300/phases.py): SM clock cycles of the event loop per phase,
// summed over chains.  Lane k of a tile accumulates phase k (so the counters
// cost one register), lanes 12..14 count sliding, destroying and creating
// events; each chain adds its sums to g_phase at the end of its launch
// (g_phase[20]: its events).  The per-launch sums of one chain must stay below
// 2^32 cycles (about 2 s).  The normal build compiles none of it.
#ifdef DSM_PHASE_CLOCKS
__device__ unsigned long long g_phase[32];
#define DSM_PHASE_BEGIN unsigned ph_acc = 0, ph_cnt = 0, ph_prev = (unsigned)clock()
#define DSM_PHASE(k)                          \
  do {                                        \
    const unsigned n_ = (unsigned)clock();    \
    if (lane == (k)) ph_acc += n_ - ph_prev;  \
    ph_prev = n_;                             \
  } while (0)
#define DSM_PHASE_COUNT(k) \
  do {                     \
    if (lane == (k)) ++ph_cnt; \
  } while (0)
#define DSM_PHASE_FLUSH()                                                                   \
  do {                                                                                      \
    if (lane < 12) atomicAdd(&g_phase[lane], (unsigned long long)ph_acc);                   \
    if (lane >= 12 && lane < 15) atomicAdd(&g_phase[lane + 4], (unsigned long long)ph_cnt); \
  } while (0)
#else
#define DSM_PHASE_BEGIN
#define DSM_PHASE(k)
#define DSM_PHASE_COUNT(k)
#define DSM_PHASE_FLUSH()
#endif

// ------------------------------------------------------------------ step kernel
// CK: correlator kind, 0 none, 1 stress G(t), 2 centre-of-mass MSD (compile
// time, so that the stress kernel carries no MSD code)
// Step kernel: persistent tiles of W lanes pull items (chains) order[0 ..
// n_items) from *work and run each in a slot of slot_cap strands; chains that
// outgrow it are appended to lst.defer (count *lst.n_defer).
// CARVED: several size classes in one launch (StepList::carve_*).  The block
// finds its class among the block ranges and carves its shared memory into
// that class's slots; tiles beyond the class's slot count leave at once (the
// chain loop has no block-wide barrier).  The class fields are read with
// static indices only, so they stay in the parameter space.
template <bool FLOW, int CK, int W, int MB, bool CARVED>
__global__ void __launch_bounds__(128, MB) k_step(const EnsDev* __restrict__ ens, int n_ens,
                                                 const long long* __restrict__ prefix, long long total,
                                                 unsigned int* work, int slot_cap, int pmax,
                                                 const volatile int* abort_flag, int* status, StepList lst) {
  constexpr bool CORR = CK != 0, MSD = CK == 2;
  extern __shared__ __align__(16) unsigned char smem[];
  const Tile<W> t;
  const int lane = t.lane;
  const int tib = threadIdx.x / W;
  long long n_items = lst.dyn_total != nullptr ? (long long)*lst.dyn_total : total;
  const int* order = lst.order;
  if constexpr (CARVED) {
    int k = 0;
#pragma unroll
    for (int i = 1; i < kCarveMax; ++i)
      if (i < lst.carve_n && (int)blockIdx.x >= lst.carve_blk[i]) k = i;
    int tiles = 0, first = 0;
#pragma unroll
    for (int i = 0; i < kCarveMax; ++i)
      if (i == k) {
        slot_cap = lst.carve_slot[i];
        tiles = lst.carve_tiles[i];
        first = lst.carve_first[i];
        n_items = lst.carve_count[i];
      }
    if (tib >= tiles) return;
    order += first;
    work = lst.carve_work + k;
  }
  Slot sl = make_slot(smem + (size_t)tib * step_slot_bytes(slot_cap, pmax), slot_cap, pmax);

  for (;;) {
    unsigned int item = 0;
    if (lane == 0) item = atomicAdd(work, 1u);
    item = t.shfl(item, 0);
    if ((long long)item >= n_items) break;
    if (abort_flag != nullptr && *abort_flag != 0) {
      if (lane == 0) atomicOr(status, 1);
      break;
    }
    const long long gid = order != nullptr ? (long long)order[item] : (long long)item;
    int e = 0;
    while (e + 1 < n_ens && prefix[e + 1] <= gid) ++e;
    const EnsDev& E = ens[e];
    const int c = (int)(gid - prefix[e]);
    const int cap = E.cap;
    // slot smaller than the ensemble's capacity: the chain may outgrow it
    const int zlim = cap > slot_cap ? slot_cap : 0x7fffffff;

    // ---- load chain into the slot
    const ChainState st = E.cs[c];
    if (st.Z > slot_cap) {  // does not fit at all: hand it to a larger slot
      if (lane == 0) {
        lst.defer[atomicAdd(lst.n_defer, 1u)] = (int)gid;
        atomicAdd(&E.counters[2], 1ull);
      }
      continue;
    }
    DSM_PHASE_BEGIN;
    int Z = st.Z, S = st.S, stall = st.stall;
    long long T = st.T;
    uint64_t step = st.step;
    if (lane == 0) sl.h->hash = st.hash;
    float dt_prev = st.dt_prev;
    // stop at step_lim; if the watchdog cap is the tighter one, stopping there
    // is a stall (step_lim then differs from E.step_limit)
    long long t_end = E.t_end_ticks;
    long long wd = E.watchdog_events;
    // flow output series: the chain's next window of this launch
    int win = 0;
    const bool series = FLOW && E.n_win > 0;
    if (series) {
      win = (int)st.k_next;
      t_end = win < E.n_win ? E.win[win] : INT64_MIN;
      wd = win < E.n_win ? E.win[E.win_stride + win] : 0;
    }
    long long step_lim = (wd < E.step_limit - (long long)step) ? (long long)step + wd : E.step_limit;
    bool aborted = false;
    const float4* gq = E.QN + (size_t)c * cap;
    const float* gt = E.tau + (size_t)c * cap;
    for (int s = lane; s < Z; s += W) {
      const float4 q = gq[s];
      sl.Q[s] = make_float4(q.x, q.y, q.z, m_q2(q.x, q.y, q.z));
      sl.N[s] = (int)q.w;
      sl.T[s] = gt[s];
    }
    const float wz1 = __double2float_rn(__ddiv_rn(1.0, __dmul_rn(E.beta_d, (double)st.nk)));
    if (CORR && lane == 0) {
      const size_t l0 = (size_t)c * E.corr_levels;
      const int4 cn = E.corr_cnt[l0];
      Corr0& k0 = *sl.k0;
      k0.ins = cn.x; k0.navg = cn.y;
      k0.nins = ((long long)(unsigned)cn.w) << 32 | (unsigned)cn.z;
      k0.a0 = E.corr_avg[l0 * 3 + 0]; k0.a1 = E.corr_avg[l0 * 3 + 1]; k0.a2 = E.corr_avg[l0 * 3 + 2];
      k0.k_next = st.k_next;
      k0.t_next = st.k_next * E.dt_sample_ticks;
      if (MSD) { k0.r1x = st.r1[0]; k0.r1y = st.r1[1]; k0.r1z = st.r1[2]; }
    }
    if (CORR) {
      const int p = E.corr_p;
      const size_t l0 = (size_t)c * E.corr_levels;
      for (int j = lane; j < p; j += W) {
        sl.Csh[j * 3 + 0] = E.corr_shift[l0 * p * 3 + j * 3 + 0];
        sl.Csh[j * 3 + 1] = E.corr_shift[l0 * p * 3 + j * 3 + 1];
        sl.Csh[j * 3 + 2] = E.corr_shift[l0 * p * 3 + j * 3 + 2];
        sl.Cacc[j] = make_float2(0.f, 0.f);
      }
    }
    t.sync();

    // NaN (bit 0) and inf (bit 1) from a full rate pass
    int pend = 0;
    // rate work due before the next event: bit 0 the chain-end rates, bit 1 the
    // prefix rebuild, bit 2 a full pass (scale overflow of an incremental update)
    int dirty = 0;
    if (!FLOW) {
      // equilibrium keeps quantised rates in the slot; the overflow rule can
      // only lower the scale, and is kept only if an event follows (the oracle
      // applies it inside a step)
      S = full_rates<false, W>(E, sl, Z, S, wz1, t, &pend);
      // a NaN or inf found here stalls the chain at its first step, after that
      // step's checks: the pending pass repeats the rates and sets them again
      if (pend & 3) dirty = 4;
      dirty |= 2;
    }
    // (5) per-lane exclusive/inclusive prefix of the element array (contiguous
    // odd-width chunks over pairs + ends) and its total;
    // rebuilt by a chunk sum + warp scan every event in flow, and in
    // equilibrium inside the rate-pass dispatch, after structural events, end
    // or scale changes; sliding events patch them with the deltas of the <=3
    // recomputed pairs
    unsigned long long incl = 0, excl = 0, tot = 0;
    int cw = 1, j0 = 0;
    auto rebuild = [&](int ne) {
      cw = ((ne + W - 1) / W) | 1;
      j0 = lane * cw;
      const int j1 = min(j0 + cw, ne);
      unsigned long long part = 0;
      for (int jj = j0; jj < j1; ++jj) part += sl.R[jj];
      incl = tile_scan(t, part);
      excl = incl - part;
      tot = t.shfl(incl, W - 1);
    };

    uint32_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
    // equilibrium: the Philox words of the current batch of W events are
    // loaded here; flow loads them at its first event
    bool words = !FLOW;
    if (!FLOW) {
      const uint64_t ctr = (step & ~(uint64_t)(W - 1)) + (uint64_t)lane;
      const U4 q = rng_at(E, P_EVENT, ctr, (uint32_t)(ctr >> 32), (uint32_t)c);
      r0 = q.x; r1 = q.y; r2 = q.z; r3 = q.w;
    }
    DSM_PHASE(10);  // chain load and first rate pass

    // a chain that stalled in an earlier launch stays put (inside the loop a
    // stall always ends it at once, so the loop tests no stall code)
    if (stall != 0) dt_prev = 0.0f;
    else for (;;) {
      // (1) flow: deformation by the previous dt (ensemble_kernel.cu:135-146)
      if (FLOW && dt_prev != 0.0f) flow_deform<W>(E, sl, Z, dt_prev, t);
      // (2) equilibrium stress samples due (eq_ensemble_kernel.cu:281-331)
      if (CORR && T > sl.k0->t_next && sl.k0->k_next < E.nsamples) corr_samples<W, MSD>(E, sl, Z, c, T, t);
      // (3) reach / stall / window checks (ensemble_kernel.cu:199-207); a full
      // slot (a creation could need strand Z+1) ends the launch for this chain
      // at this step boundary, exactly like a window end
      if (T >= t_end || (long long)step >= step_lim || Z >= zlim) {
        if (stall == 0 && T < t_end && (long long)step >= step_lim && step_lim != E.step_limit) stall = ST_WATCHDOG;
        dt_prev = 0.0f;
        // a window of a flow series ends: record the stress and go on with
        // the next window, exactly as a new launch would (no deformation by
        // the last dt, event cap counted from here)
        if (series && stall == 0 && T >= t_end && win < E.n_win) {
          flow_stress<W>(E, sl, Z, t, E.win_stress + ((size_t)win * E.n_chains + c) * 8);
          if (++win < E.n_win) {
            t_end = E.win[win];
            wd = E.win[E.win_stride + win];
            step_lim = (wd < E.step_limit - (long long)step) ? (long long)step + wd : E.step_limit;
            continue;
          }
        }
        break;
      }
      DSM_PHASE(0);  // checks and correlator samples
      const int np = Z - 1;
      // (4) rates: flow recomputes everything; equilibrium refreshes the chain
      // ends when a strand next to an end changed
      if (FLOW) {
        S = full_rates_body<true, W>(E, sl, Z, S, wz1, t, &pend);
        if (pend & 3) {
          stall = (pend & 1) ? ST_NAN : ST_INF;
          dt_prev = 0.0f;
          break;
        }
        rebuild(np + NEND);
      } else if (dirty != 0) {
        // one branch in the common case (nothing due): the chain-end refresh
        // (bit 0), the full pass that a scale overflow asks for (bit 2), then
        // the prefix rebuild that these and structural events (bit 1) need
        if (dirty & 1) {
          int over = 0;
          if (lane < NEND) {
            const float ev = end_comp(E, lane, Z, sl.N, wz1);
            over = (fexp(ev) + S > LIMIT_E) ? 4 : 0;
            sl.R[np + lane] = quant(ev, pow2f(S));
          }
          dirty |= t.or_(over);
          if (dirty & 4) S = full_rates<false, W>(E, sl, Z, S, wz1, t, &pend);
          t.sync();
        } else if (dirty & 4) {
          S = full_rates<false, W>(E, sl, Z, S, wz1, t, &pend);
        }
        dirty = 0;
        // NaN and inf come only from a full pass
        if (pend & 3) {
          stall = (pend & 1) ? ST_NAN : ST_INF;
          dt_prev = 0.0f;
          break;
        }
        rebuild(np + NEND);
      }
      DSM_PHASE(1);  // chain-end rates, rate passes, prefix rebuild
      const float sf = pow2f(S);
      // (6) dt = 1/sum W (ensemble_kernel.cu:262-272)
      const float sumw = __fmul_rn(__ll2float_rn((long long)tot), pow2f(-S));
      const float dt = __fdiv_rn(1.0f, sumw);
      if (dt == 0.0f) { stall = ST_DT_ZERO; dt_prev = 0.0f; break; }
      if (!(dt < 2.0e9f)) { stall = ST_INF; dt_prev = 0.0f; break; }
      const long long dtt = __float2ll_rn(__fmul_rn(dt, 4294967296.0f));
      DSM_PHASE(2);  // dt
      // (7) Philox words of this event (one evaluation per W events)
      if ((step & (uint64_t)(W - 1)) == 0 || (FLOW && !words)) {
        // the run flag, polled every 4096 events (nothing of the event is applied yet)
        if (abort_flag != nullptr && (step & 4095) == 0 && *abort_flag != 0) {
          if (lane == 0) atomicOr(status, 1);
          dt_prev = 0.0f;
          aborted = true;
          break;
        }
        const uint64_t ctr = (step & ~(uint64_t)(W - 1)) + (uint64_t)lane;
        const U4 q = rng_at(E, P_EVENT, ctr, (uint32_t)(ctr >> 32), (uint32_t)c);
        r0 = q.x; r1 = q.y; r2 = q.z; r3 = q.w;
        words = true;
      }
      const int src = (int)(step & (uint64_t)(W - 1));
      const uint32_t w0 = t.shfl(r0, src);
      const uint32_t w1 = t.shfl(r1, src);
      // (8) pick (ensemble_kernel.cu:274-501): pr uniform in [0, tot)
      const unsigned long long pr = __umul64hi(tot, ((unsigned long long)w1 << 32) | w0);
      const int L = __ffs(t.ballot(incl > pr)) - 1;
      int jj = 0;
      unsigned long long r = 0;
      if (lane == L) {
        r = pr - excl;
        jj = j0;
        // three loads in flight per round; jj stays below ne = Z + 4, so
        // jj + 2 <= slot_cap + 5 is inside the R array (slot_cap + NEND + 1)
        for (;;) {
          const unsigned long long a = sl.R[jj], b = sl.R[jj + 1], d = sl.R[jj + 2];
          if (r < a) break;
          r -= a; ++jj;
          if (r < b) break;
          r -= b; ++jj;
          if (r < d) break;
          r -= d; ++jj;
        }
      }
      jj = t.shfl(jj, L);
      r = t.shfl(r, L);
      DSM_PHASE(3);  // Philox, pick, chunk walk
      int evn, j = -1;
      unsigned long long rem = 0, wsel = 0;
      if (jj < np) {
        // inside pair j: CD destruction, shift +1, shift -1, CD creation
        j = jj;
        // the CD components selected as floats (0 without CD) and always quantised
        const bool cd = E.cd_flag != 0;
        const float tq = sl.T[j], eq = __ldg(&E.NE[sl.N[j]]).w;
        const unsigned long long q0 = quant(cd ? tq : 0.0f, sf);
        const unsigned long long q3 = quant(cd ? eq : 0.0f, sf);
        const unsigned long long lim = sl.R[j] - q3;
        if (r < q0) evn = CDD;
        else if (r >= lim) { evn = CDC_MID; rem = r - lim; wsel = q3; }
        else evn = (r - q0 < sl.P[j]) ? SDP : SDM;
      } else {
        const int q = jj - np;
        rem = r;
        wsel = sl.R[jj];
        evn = (q == 0) ? CDC_TAIL : (q == 1) ? SDC_HEAD : (q == 2) ? SDC_TAIL : (q == 3) ? SDD_HEAD : SDD_TAIL;
      }
      DSM_PHASE(4);  // classification
      T += dtt;
      // (9) apply
      uint32_t code = ((uint32_t)evn << 24) | (uint32_t)(j < 0 ? 0 : j);
      int up0 = 0, upn = 0;
      bool slide = false;
      if (evn == SDP || evn == SDM) {
        t.sync();
        {
          // every lane computes (broadcast loads), lane 0 stores
          const int d = (evn == SDP) ? 1 : -1;
          const int na = sl.N[j] + d, nb = sl.N[j + 1] - d;
          if (lane == 0) { sl.N[j] = na; sl.N[j + 1] = nb; }
        }
        up0 = j - 1; upn = 3;
        slide = !((j <= 1) || (j + 1 >= Z - 2));
        dirty = slide ? 0 : 1;
      } else if (evn == CDD || evn == SDD_HEAD || evn == SDD_TAIL) {
        // away from both chain ends (pair 2 <= j < Z - 3) a destruction keeps
        // what the end rates depend on (Z >= 3, the two strands at each end):
        // their quantised values move down with the pairs, not recomputed
        const bool mid = !FLOW && j >= 2 && j + 3 < Z;
        unsigned long long ev = 0;
        if (mid && lane < NEND) ev = sl.R[np + lane];
        apply_destroy<W, MSD>(sl, evn, j, Z, t, &up0, &upn);
        if (mid && lane < NEND) sl.R[np - 1 + lane] = ev;
        Z -= 1;
        dirty = mid ? 0 : 1;
      } else if (Z >= cap) {
        code |= (uint32_t)NULL_FLAG << 24;  // creation refused at capacity (ensemble_kernel.cu:380,423,451)
      } else {
        const uint32_t w2 = t.shfl(r2, src);
        const uint32_t w3 = t.shfl(r3, src);
        // the same for a creation inside a strand away from both ends
        const bool mid = !FLOW && j >= 2 && j + 3 < Z;
        unsigned long long ev = 0;
        if (mid && lane < NEND) ev = sl.R[np + lane];
        const int newn = apply_create<W>(E, sl, evn, j, Z, c, step, rem, wsel, w2, w3, t, &up0, &upn);
        if (mid && lane < NEND) sl.R[np + 1 + lane] = ev;
        Z += 1;
        dirty = mid ? 0 : 1;
        code |= (uint32_t)newn << 8;
      }
      t.sync();
#ifdef DSM_PHASE_CLOCKS
      {
        const int k_ = (evn == SDP || evn == SDM) ? 0 : (evn == CDD || evn == SDD_HEAD || evn == SDD_TAIL) ? 1 : 2;
        DSM_PHASE(5 + k_);  // apply: slide, destruction, creation
        DSM_PHASE_COUNT(12 + k_);
      }
#endif
      if (!FLOW && upn > 0) {
        unsigned long long dl;
        dirty |= update_pairs<W>(E, sl, Z, S, up0, upn, t, &dl);
        if (slide) {
          // patch the prefix sums with the deltas of pairs j-1, j, j+1 (lanes
          // 0, 4, 8); pair j lies in lane L's chunk, its neighbours in L's
          // or the adjacent chunk (out-of-range pairs carry d == 0)
          const int jL = L * cw;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const unsigned long long d = t.shfl(dl, 4 * k);
            const int own = (k == 0) ? ((j == jL) ? L - 1 : L) : (k == 1) ? L : ((j + 1 == jL + cw) ? L + 1 : L);
            if (lane >= own) incl += d;
            if (lane > own) excl += d;
            tot += d;
          }
        } else {
          dirty |= 2;
        }
      }
      DSM_PHASE(8);  // pair-rate update, prefix patch
      if (lane == 0) sl.h->hash = (sl.h->hash ^ (uint64_t)code) * 0x100000001B3ull;
      ++step;
      dt_prev = dt;
      DSM_PHASE(9);  // event hash, counters
    }
    DSM_PHASE(0);

    // stopped early because the slot is full (an abort ends the launch anyway)
    const bool deferred = E.cap > slot_cap && Z >= slot_cap && stall == 0 && T < t_end && (long long)step < step_lim;
    // ---- flow: stress at the end of the window (ensemble_kernel.cu:504-538)
    if (FLOW && !deferred && !series) flow_stress<W>(E, sl, Z, t, E.out_stress + (size_t)c * 8);
    // a chain that stalled stands still for the remaining windows of a series
    // and is left out of their sums (NaN marker, as a stalled chain is left
    // out at the end of a launch)
    if (series && !deferred && !aborted && lane == 0)
      for (int w = win; w < E.n_win; ++w) E.win_stress[((size_t)w * E.n_chains + c) * 8] = __int_as_float(0x7fc00000);
    // ---- correlator level 0 back to HBM (compensated FP32 sums -> FP64)
    long long k_next = -1;  // -1: unchanged (no correlator)
    if (CORR) {
      const int p = E.corr_p;
      const size_t l0 = (size_t)c * E.corr_levels;
      for (int j = lane; j < p; j += W) {
        E.corr_shift[l0 * p * 3 + j * 3 + 0] = sl.Csh[j * 3 + 0];
        E.corr_shift[l0 * p * 3 + j * 3 + 1] = sl.Csh[j * 3 + 1];
        E.corr_shift[l0 * p * 3 + j * 3 + 2] = sl.Csh[j * 3 + 2];
        const float2 a = sl.Cacc[j];
        E.corr_acc[l0 * p + j] += (double)a.x - (double)a.y;
      }
      const Corr0& k0 = *sl.k0;
      k_next = k0.k_next;
      if (lane == 0) {
        E.corr_cnt[l0] = make_int4(k0.ins, k0.navg, (int)(unsigned)(k0.nins & 0xffffffffll),
                                   (int)(unsigned)(k0.nins >> 32));
        E.corr_avg[l0 * 3 + 0] = k0.a0; E.corr_avg[l0 * 3 + 1] = k0.a1; E.corr_avg[l0 * 3 + 2] = k0.a2;
      }
    }
    // ---- chain back to HBM
    float4* wq = E.QN + (size_t)c * cap;
    float* wt = E.tau + (size_t)c * cap;
    for (int s = lane; s < Z; s += W) {
      const float4 q = sl.Q[s];
      wq[s] = make_float4(q.x, q.y, q.z, (float)sl.N[s]);
      wt[s] = (s < Z - 1) ? sl.T[s] : 0.0f;
    }
    if (lane == 0) {
      // the launch's start values are still in HBM: events done, stored scale
      ChainState* cs = &E.cs[c];
      const unsigned long long done = step - cs->step;
      // a rescale at load is kept only if an event followed (as in the oracle)
      if (done > 0) cs->S = S;
      cs->Z = Z; cs->stall = stall; cs->dt_prev = dt_prev;
      cs->T = T; cs->step = step; cs->hash = sl.h->hash;
      if (k_next >= 0) cs->k_next = k_next;
      if (series) cs->k_next = win;
      if (MSD) {
        const Corr0& q = *sl.k0;
        cs->r1[0] = q.r1x; cs->r1[1] = q.r1y; cs->r1[2] = q.r1z;
      }
      atomicAdd(&E.counters[0], done);
#ifdef DSM_PHASE_CLOCKS
      atomicAdd(&g_phase[20], done);
#endif
      if (deferred) {
        lst.defer[atomicAdd(lst.n_defer, 1u)] = (int)(prefix[e] + c);
        atomicAdd(&E.counters[2], 1ull);
      } else {
        atomicAdd(&E.counters[1], 1ull);
      }
    }
    DSM_PHASE(11);  // chain store
    DSM_PHASE_FLUSH();
    t.sync();
  }
}

// ------------------------------------------------------------------ initialiser
// Equilibrium chains (role of chain.cu:199-283): each of the NK-1 bonds between
// Kuhn steps carries an entanglement with probability 1/(1+beta), which gives
// Z-1 ~ Binomial(NK-1, 1/(1+beta)) with N uniform over compositions; Q ~ N(0,
// N/3) for internal strands, 0 for dangling ends; tau rates from f_t.
__global__ void __launch_bounds__(128) k_init(const EnsDev* __restrict__ ensp, int slot_cap) {
  extern __shared__ __align__(16) unsigned char smem[];
  const EnsDev& E = *ensp;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int c = blockIdx.x * (blockDim.x >> 5) + wib;
  if (c >= E.n_chains) return;
  int* pos = (int*)(smem + (size_t)wib * (size_t)(slot_cap + 1) * 8);
  int* sN = pos + (slot_cap + 1);
  const int nk = E.poly ? __ldg(&E.nk_chain[c]) : E.nk;
  const int cap = E.cap;
  const double pe = 1.0 / (1.0 + (double)E.beta);
  double thr_d = floor(pe * 4294967296.0);
  if (thr_d > 4294967295.0) thr_d = 4294967295.0;
  const uint32_t thr = (uint32_t)thr_d;
  const int nb = nk - 1;                  // bonds
  const int nblk = (nb + 3) >> 2;         // Philox blocks of 4 bonds
  int Zm1 = 0;
  for (uint32_t att = 0; att < 64; ++att) {
    int count = 0;
    for (int b = lane; b < nblk; b += 32) {
      const U4 r = rng_at(E, P_BONDS, (uint64_t)b, att, (uint32_t)c);
      const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) count += (4 * b + q < nb && w[q] < thr) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) count += __shfl_xor_sync(FULL_MASK, count, o);
    Zm1 = count;
    if (Zm1 + 1 <= cap || att == 63) {
      // ordered positions: rounds of 32 blocks, exclusive scan of counts
      int off = 0;
      for (int base = 0; base < nblk; base += 32) {
        const int b = base + lane;
        uint32_t bits = 0;
        if (b < nblk) {
          const U4 r = rng_at(E, P_BONDS, (uint64_t)b, att, (uint32_t)c);
          const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) if (4 * b + q < nb && w[q] < thr) bits |= 1u << q;
        }
        const int cnt = __popc(bits);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(FULL_MASK, incl, o);
          if (lane >= o) incl += t;
        }
        int k = off + incl - cnt;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (bits & (1u << q)) { if (k < cap - 1) pos[k] = 4 * b + q; ++k; }
        off += __shfl_sync(FULL_MASK, incl, 31);
      }
      break;
    }
  }
  if (Zm1 > cap - 1) Zm1 = cap - 1;  // truncation after 64 rejected draws
  __syncwarp();
  const int Z = Zm1 + 1;
  for (int i = lane; i < Z; i += 32) {
    const int prev = (i == 0) ? -1 : pos[i - 1];
    const int cur = (i == Z - 1) ? nk - 1 : pos[i];
    sN[i] = cur - prev;
  }
  __syncwarp();
  float4* gq = E.QN + (size_t)c * cap;
  float* gt = E.tau + (size_t)c * cap;
  float* gq2 = (float*)pos;  // reuse: Q^2 per strand (positions no longer needed)
  __syncwarp();
  for (int i = lane; i < Z; i += 32) {
    const int N = sN[i];
    float x = 0.f, y = 0.f, z = 0.f;
    if (i >= 1 && i <= Z - 2) {
      const U4 r = rng_at(E, P_QINIT, (uint64_t)i, 0, (uint32_t)c);
      float g0, g1, g2, g3;
      m_gauss2(r.x, r.y, &g0, &g1);
      m_gauss2(r.z, r.w, &g2, &g3);
      const float sg = __fsqrt_rn(__fdiv_rn((float)N, 3.0f));
      x = __fmul_rn(g0, sg); y = __fmul_rn(g1, sg); z = __fmul_rn(g2, sg);
    }
    gq[i] = make_float4(x, y, z, (float)N);
    gq2[i] = m_q2(x, y, z);
    float tr = 0.0f;
    if (i < Z - 1) {
      const U4 r = rng_at(E, P_TAUINIT, (uint64_t)i, 0, (uint32_t)c);
      const PcdDev pp = partner_pcd(E, r.y, false);
      tr = E.cd_flag ? rate_f_t(pp, u01(r.x)) : 0.0f;
    }
    gt[i] = tr;
  }
  __syncwarp();
  // initial fixed-point scale: min(s0, 47 - max exponent of all rate components)
  int emax = -200;
  for (int p = lane; p < Z - 1; p += 32) {
    const int N1 = sN[p], N2 = sN[p + 1];
    const float q1 = gq2[p], q2 = gq2[p + 1];
    const float4 a = __ldg(&E.NT[N1]), b = __ldg(&E.NT[N2]);
    emax = max(emax, fexp(E.cd_flag ? gt[p] : 0.0f));
    emax = max(emax, fexp(shift_plus(E, N1, q1, N2, q2, a, b)));
    emax = max(emax, fexp(shift_minus(E, N1, q1, N2, q2, a, b)));
    emax = max(emax, fexp(E.cd_flag ? __ldg(&E.NE[N1]).w : 0.0f));
  }
  if (lane < NEND) {
    const float wz1 = __double2float_rn(__ddiv_rn(1.0, __dmul_rn(E.beta_d, (double)nk)));
    emax = max(emax, fexp(end_comp(E, lane, Z, sN, wz1)));
  }
  emax = warp_max_i(emax);
  if (lane == 0) {
    ChainState st;
    st.Z = Z; st.stall = 0; st.S = min(E.s0, LIMIT_E - emax); st.dt_prev = 0.f;
    st.T = 0; st.step = 0; st.hash = 0xCBF29CE484222325ull; st.k_next = 0;
    st.nk = nk; st.r1[0] = st.r1[1] = st.r1[2] = 0.f;
    E.cs[c] = st;
  }
}

// ------------------------------------------------------------------ reductions
// G(t) numerator per (level k, lag j): sum over chains of acc/count, FP64,
// fixed tree order (deterministic).  count = values inserted at level k - j.
__global__ void k_gt_reduce(const EnsDev* __restrict__ ensp, double* gsum, long long* gcount) {
  const EnsDev& E = *ensp;
  const int L = E.corr_levels, p = E.corr_p;
  const int kj = blockIdx.x;
  const int k = kj / p, j = kj % p;
  __shared__ double red[256];
  double acc = 0.0;
  for (int c = threadIdx.x; c < E.n_chains; c += blockDim.x) {
    const int4 cn = E.corr_cnt[(size_t)c * L + k];
    const long long nins = ((long long)(unsigned)cn.w) << 32 | (unsigned)cn.z;
    const long long n = nins - j;
    if (n > 0 && !(k > 0 && j < p / E.corr_m)) acc += E.corr_acc[((size_t)c * L + k) * p + j] / (double)n;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    gsum[kj] = red[0];
    const int4 cn = E.corr_cnt[(size_t)0 * L + k];
    const long long nins = ((long long)(unsigned)cn.w) << 32 | (unsigned)cn.z;
    const long long n = nins - j;
    gcount[kj] = (n > 0 && !(k > 0 && j < p / E.corr_m)) ? n : 0;
  }
}

// Ensemble average of the window-end stress over non-stalled, non-NaN chains
// (ensemble_call_block.cu:471-491), FP64, fixed tree order.  out[0..7] sums,
// out[8] chain count.
// per_chain: n_chains x 8 floats (NULL: the flow kernel's E.out_stress)
__global__ void k_stress_reduce(const EnsDev* __restrict__ ensp, const float* __restrict__ per_chain, double* out) {
  const EnsDev& E = *ensp;
  __shared__ double red[9][256];
  double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const float* src = per_chain != nullptr ? per_chain : E.out_stress;
  for (int c = threadIdx.x; c < E.n_chains; c += blockDim.x) {
    const float* s = src + (size_t)c * 8;
    if (E.cs[c].stall != 0 || s[0] != s[0]) continue;
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] += (double)s[q];
    a[8] += 1.0;
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) red[q][threadIdx.x] = a[q];
  __syncthreads();
  for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
#pragma unroll
      for (int q = 0; q < 9; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x < 9) out[threadIdx.x] = red[threadIdx.x][0];
}

// Slots beyond a chain's strands are not maintained by the step kernel; the
// reference layout has them zero.  One thread per (chain, slot).
// Stress of every chain from its state in HBM, for ensembles whose step
// kernel keeps no per-chain stress (equilibrium): the sums of flow_stress
// (ensemble_kernel.cu:504-538) in the same order, strand i into partial
// i mod 16 and a 16-lane tree, one warp per chain; out8 gets n_chains x 8.
__global__ void k_state_stress(const EnsDev* __restrict__ ensp, float* out8) {
  const EnsDev& E = *ensp;
  const int lane = threadIdx.x & 31;
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= E.n_chains) return;
  const int Z = E.cs[c].Z;
  const float4* q = E.QN + (size_t)c * E.cap;
  float s[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int i = lane; lane < 16 && i < Z; i += 16) {
    const float4 v = q[i];
    const float w = __ldg(&E.INV3N[(int)v.w]);
    s[0] = __fmaf_rn(-__fmul_rn(v.x, v.x), w, s[0]);
    s[1] = __fmaf_rn(-__fmul_rn(v.y, v.y), w, s[1]);
    s[2] = __fmaf_rn(-__fmul_rn(v.z, v.z), w, s[2]);
    s[3] = __fmaf_rn(-__fmul_rn(v.x, v.y), w, s[3]);
    s[4] = __fmaf_rn(-__fmul_rn(v.y, v.z), w, s[4]);
    s[5] = __fmaf_rn(-__fmul_rn(v.x, v.z), w, s[5]);
    s[6] = __fadd_rn(s[6], __fsqrt_rn(m_q2(v.x, v.y, v.z)));
  }
#pragma unroll
  for (int k = 0; k < 7; ++k) {
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) s[k] = __fadd_rn(s[k], __shfl_xor_sync(FULL_MASK, s[k], o));
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 7; ++k) out8[c * 8 + k] = s[k];
    out8[c * 8 + 7] = (float)Z;
  }
}

__global__ void k_clear_tail(float4* QN, float* tau, const ChainState* __restrict__ cs, int n_chains, int cap) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)n_chains * cap) return;
  const int c = (int)(i / cap), k = (int)(i - (long long)c * cap);
  const int Z = cs[c].Z;
  if (k >= Z) QN[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (k >= Z - 1) tau[i] = 0.f;
}

// Flow series: windows d_win[0 .. n) with event caps at d_win[stride + w];
// every chain starts at window 0
__global__ void k_series_begin(EnsDev* ens, const long long* d_win, int stride, int n, ChainState* cs,
                               int n_chains) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    ens->win = d_win;
    ens->win_stride = stride;
    ens->n_win = n;
  }
  if (i < n_chains) cs[i].k_next = 0;
}

// Stress sums of window blockIdx.x of a flow series, in the order of
// k_stress_reduce (same per-thread strides, same tree)
__global__ void k_series_reduce(const EnsDev* __restrict__ ensp, double* out) {
  const EnsDev& E = *ensp;
  __shared__ double red[9][256];
  double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const float* base = E.win_stress + (size_t)blockIdx.x * E.n_chains * 8;
  for (int c = threadIdx.x; c < E.n_chains; c += blockDim.x) {
    const float* s = base + (size_t)c * 8;
    if (s[0] != s[0]) continue;
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] += (double)s[q];
    a[8] += 1.0;
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) red[q][threadIdx.x] = a[q];
  __syncthreads();
  for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
#pragma unroll
      for (int q = 0; q < 9; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x < 9) out[(size_t)blockIdx.x * 9 + threadIdx.x] = red[threadIdx.x][0];
}

// Window w of a captured series: end time d_win[w] and event cap d_win[n+w]
__global__ void k_window_begin(EnsDev* ens, const long long* __restrict__ d_win, int n, int w) {
  ens->t_end_ticks = d_win[w];
  ens->watchdog_events = d_win[n + w];
}

// ------------------------------------------------------------------ launchers
template <bool FLOW, int CK, int W, int MB>
static void* step_fn() { return (void*)k_step<FLOW, CK, W, MB, false>; }

// hi: the variant compiled for DSM_MINB_HI blocks per SM
template <int W>
static void* pick_step_w(bool flow, int ck, bool hi) {
  if (flow) return hi ? step_fn<true, 0, W, DSM_MINB_HI>() : step_fn<true, 0, W, DSM_MINB>();
  if (ck == 0) return hi ? step_fn<false, 0, W, DSM_MINB_HI>() : step_fn<false, 0, W, DSM_MINB>();
  if (ck == 2) return hi ? step_fn<false, 2, W, DSM_MINB_HI>() : step_fn<false, 2, W, DSM_MINB>();
  return hi ? step_fn<false, 1, W, DSM_MINB_HI>() : step_fn<false, 1, W, DSM_MINB>();
}
static void* pick_step(bool flow, int ck, int lanes, bool hi) {
  return lanes == 16 ? pick_step_w<16>(flow, ck, hi) : pick_step_w<32>(flow, ck, hi);
}

static int tile_lanes(const LaunchCfg& cfg) { return cfg.lanes == 16 ? 16 : 32; }
static size_t step_smem(const LaunchCfg& cfg) {
  const int tiles = cfg.warps_per_block * 32 / tile_lanes(cfg);
  return step_slot_bytes(cfg.slot_cap, cfg.pmax) * tiles;
}

// Function attributes are process-wide: one thread setting a smaller
// dynamic shared-memory limit between another thread's set and launch would
// make that launch fail.  Each step kernel is therefore prepared once per
// device with the device's opt-in maximum (an upper bound only: occupancy
// follows the size given at launch) and the largest carveout (the slots are
// the working set), and never changed afterwards.
static cudaError_t prep_step(void* fn, size_t sm) {
  static std::mutex mu;
  static std::vector<std::pair<void*, int>> done;  // (kernel, device)
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  std::lock_guard<std::mutex> lk(mu);
  for (const auto& d : done)
    if (d.first == fn && d.second == dev) return cudaSuccess;
  int optin = 0;
  err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (err != cudaSuccess) return err;
  if (sm > (size_t)optin) return cudaErrorInvalidValue;
  err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if (err != cudaSuccess) return err;
  err = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (err != cudaSuccess) return err;
  done.push_back({fn, dev});
  return cudaSuccess;
}

static int blocks_per_sm(void* fn, const LaunchCfg& cfg, size_t sm) {
  if (prep_step(fn, sm) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, cfg.warps_per_block * 32, sm) != cudaSuccess) return 0;
  return nb;
}

// The step kernel of a launch shape and its resident blocks per SM.  Every
// kind has a second build for more resident blocks; it is taken when the
// shape's shared memory lets more of its blocks reside than of the standard
// build's (its smaller register budget costs a little per warp, so a tie
// keeps the standard build).  The choice depends on the shape and the device
// only and is cached, so planning and launching always agree.
struct StepChoice {
  void* fn;
  int bps;
};
static StepChoice choose_step(bool flow, int ck, const LaunchCfg& cfg) {
  struct Key {
    int dev, flow, ck, lanes, warps;
    size_t sm;
    StepChoice v;
  };
  static std::mutex mu;
  static std::vector<Key> cache;
  const size_t sm = step_smem(cfg);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return {pick_step(flow, ck, tile_lanes(cfg), false), 0};
  const int lanes = tile_lanes(cfg), fl = flow ? 1 : 0, kk = flow ? 0 : ck;
  {
    std::lock_guard<std::mutex> lk(mu);
    for (const Key& k : cache)
      if (k.dev == dev && k.flow == fl && k.ck == kk && k.lanes == lanes && k.warps == cfg.warps_per_block && k.sm == sm)
        return k.v;
  }
  void* std_fn = pick_step(flow, ck, lanes, false);
  StepChoice c{std_fn, blocks_per_sm(std_fn, cfg, sm)};
  {
    void* hi_fn = pick_step(flow, ck, lanes, true);
    const int nb = blocks_per_sm(hi_fn, cfg, sm);
    // with a correlator the smaller register budget costs more per warp: the
    // 6-block build pays only with half as many blocks again (measured: +6 %
    // at N_K = 50, p = 16 with 6 blocks; 2-11 % slower with 5 blocks at
    // N_K = 100 and 150, p = 64)
    const bool take = (flow || ck == 0) ? nb > c.bps : 2 * nb >= 3 * c.bps;
    if (take && nb > c.bps) c = StepChoice{hi_fn, nb};
  }
  if (c.bps > 0) {
    std::lock_guard<std::mutex> lk(mu);
    cache.push_back(Key{dev, fl, kk, lanes, cfg.warps_per_block, sm, c});
  }
  return c;
}

int step_max_blocks_per_sm(bool flow, int corr, const LaunchCfg& cfg) { return choose_step(flow, corr, cfg).bps; }

// carved launches: equilibrium kinds, 16-lane tiles, the standard build
template <int CK>
static void* carved_fn() { return (void*)k_step<false, CK, 16, DSM_MINB, true>; }
static void* pick_carved(int ck) { return ck == 0 ? carved_fn<0>() : ck == 2 ? carved_fn<2>() : carved_fn<1>(); }

int step_carved_blocks_per_sm(int corr, size_t smem_bytes) {
  void* fn = pick_carved(corr);
  if (prep_step(fn, smem_bytes) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, smem_bytes) != cudaSuccess) return 0;
  return nb;
}

cudaError_t launch_step_carved(const EnsDev* d_ens, const long long* d_prefix, int corr, int pmax, size_t smem_bytes,
                               const volatile int* abort_flag, int* d_status, int grid, cudaStream_t st,
                               const StepList& lst) {
  void* fn = pick_carved(corr);
  cudaError_t err = prep_step(fn, smem_bytes);
  if (err != cudaSuccess) return err;
  int n_ens = 1, slot_cap = 0;
  long long total = 0;
  unsigned int* work = nullptr;
  StepList l = lst;
  void* args[] = {(void*)&d_ens, (void*)&n_ens, (void*)&d_prefix, (void*)&total, (void*)&work,
                  (void*)&slot_cap, (void*)&pmax, (void*)&abort_flag, (void*)&d_status, (void*)&l};
  return cudaLaunchKernel(fn, dim3(grid), dim3(128), args, smem_bytes, st);
}

size_t step_block_smem(const LaunchCfg& cfg) { return step_smem(cfg); }

cudaError_t launch_step(const EnsDev* d_ens, int n_ens, const long long* d_prefix, long long total,
                        unsigned int* d_work, bool flow, int corr, const LaunchCfg& cfg,
                        const volatile int* abort_flag, int* d_status, int grid, cudaStream_t st,
                        const StepList& lst) {
  const size_t sm = step_smem(cfg);
  void* fn = choose_step(flow, corr, cfg).fn;
  cudaError_t err = prep_step(fn, sm);
  if (err != cudaSuccess) return err;
  StepList l = lst;
  void* args[] = {(void*)&d_ens, (void*)&n_ens, (void*)&d_prefix, (void*)&total, (void*)&d_work,
                  (void*)&cfg.slot_cap, (void*)&cfg.pmax, (void*)&abort_flag, (void*)&d_status, (void*)&l};
  return cudaLaunchKernel(fn, dim3(grid), dim3(cfg.warps_per_block * 32), args, sm, st);
}

cudaError_t launch_init(const EnsDev* d_ens, const EnsDev& h_ens, int slot_cap, cudaStream_t st) {
  const int wpb = 4;
  const size_t sm = (size_t)(slot_cap + 1) * 8 * wpb;
  cudaError_t err = prep_step((void*)k_init, sm);  // one-time attribute setup, as for the step kernels
  if (err != cudaSuccess) return err;
  const int grid = (h_ens.n_chains + wpb - 1) / wpb;
  k_init<<<grid, wpb * 32, sm, st>>>(d_ens, slot_cap);
  return cudaGetLastError();
}

cudaError_t launch_gt_reduce_dev(const EnsDev* d_ens, int levels, int p, double* d_gsum, long long* d_count,
                                 cudaStream_t st) {
  k_gt_reduce<<<levels * p, 256, 0, st>>>(d_ens, d_gsum, d_count);
  return cudaGetLastError();
}
cudaError_t launch_window_begin(EnsDev* d_ens, const long long* d_win, int n, int w, cudaStream_t st) {
  k_window_begin<<<1, 1, 0, st>>>(d_ens, d_win, n, w);
  return cudaGetLastError();
}
cudaError_t launch_clear_tail(float4* d_QN, float* d_tau, const ChainState* d_cs, int n_chains, int cap,
                              cudaStream_t st) {
  const long long n = (long long)n_chains * cap;
  if (n == 0) return cudaSuccess;
  k_clear_tail<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_QN, d_tau, d_cs, n_chains, cap);
  return cudaGetLastError();
}
cudaError_t launch_series_begin(EnsDev* d_ens, const long long* d_win, int stride, int n, int n_chains,
                                ChainState* d_cs, cudaStream_t st) {
  k_series_begin<<<(n_chains + 255) / 256, 256, 0, st>>>(d_ens, d_win, stride, n, d_cs, n_chains);
  return cudaGetLastError();
}
cudaError_t launch_series_reduce(const EnsDev* d_ens, double* out, int n, cudaStream_t st) {
  k_series_reduce<<<n, 256, 0, st>>>(d_ens, out);
  return cudaGetLastError();
}
cudaError_t launch_stress_reduce_dev(const EnsDev* d_ens, double* d_out9, cudaStream_t st) {
  k_stress_reduce<<<1, 256, 0, st>>>(d_ens, nullptr, d_out9);
  return cudaGetLastError();
}
cudaError_t launch_state_stress(const EnsDev* d_ens, int n_chains, float* d_out8, double* d_out9, cudaStream_t st) {
  const long long threads = 32LL * n_chains;
  k_state_stress<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(d_ens, d_out8);
  k_stress_reduce<<<1, 256, 0, st>>>(d_ens, d_out8, d_out9);
  return cudaGetLastError();
}

}  // namespace dsm

#ifdef DSM_PHASE_CLOCKS
// phase counters of the debug build: 32 sums (see the phase clocks above)
extern "C" int dsm_phase_read(unsigned long long* out32) {
  return (int)cudaMemcpyFromSymbol(out32, dsm::g_phase, sizeof(dsm::g_phase));
}
extern "C" int dsm_phase_clear() {
  const unsigned long long z[32] = {};
  return (int)cudaMemcpyToSymbol(dsm::g_phase, z, sizeof(z));
}
#endif
