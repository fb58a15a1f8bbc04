// ORACLE — test infrastructure only.  Only tests/, __graft_entry__.smoke() and
// bench.py (its cpu_baseline leg and the `--impl reference` arm) load this
// library, and only as the checker / the timed CPU restatement.  The product
// (gpu_dsm_gb300/) never links, imports or calls anything under oracle/.
//
// CPU restatement of the reference DSM (Discrete Slip-Link Model) kinetic Monte
// Carlo path of ktaletsk/gpu_dsm, written in "immediate-apply" form: the
// reference defers strand insertions/removals to the next step (delayed
// dynamics, common/ensemble_kernel.cu:64-102); here an event is applied as soon
// as it is picked, which yields the same state sequence.
//
// Three arithmetic modes:
//   mode 0 (FP32 mirror): FP32 strand state, rates from per-N tables and the
//       element-wise functions of orc_math.h, rates quantised to int64 fixed
//       point so that the event pick is an exact integer computation.  This is
//       the arithmetic the sm_103a kernel implements; integer state and Q must
//       agree with it bit for bit.
//   mode 1 (FP64 transcription): the reference formulas evaluated literally in
//       double precision with libm (pow/exp/log/sin/cos), double state, double
//       sums.  Used as the accuracy reference for statistics.
//   mode 2 (reference arithmetic): the reference's chain-parallel kernels
//       restated expression for expression in immediate-apply form: FP32
//       rates with libm expf/powf, the running-subtraction scan with FP32 sums
//       (flow kernel) or FP64 sums (equilibrium kernel), FP32 time relative to
//       sync windows of at most 1e5, the reference's sample and stop rules,
//       and random numbers from ref_tape.h.  The reference's own kernels,
//       compiled for the host by ref_step.cpp with the same random stream,
//       must give the same states bit for bit.
// The measurement path (stress samples, multi-tau correlator, flow stress) is
// accumulated in FP64 in both modes.
//
// Reference functions restated here (file:line in ktaletsk/gpu_dsm):
//   p_cd constants ................ common/pcd_tau.h:32-66
//   lifetime samplers ............. common/gpu_random.cu:78-99,143-148
//   CD creation prefactor ......... common/ensemble.cu:136-150
//   equilibrium initialiser ....... common/chain.cu:106-156,158-170,199-283
//   flow deformation kappa() ...... common/ensemble_kernel.cu:105-110
//   pair (shift + CD) rates ....... common/ensemble_kernel.cu:149-181,
//                                   common/eq_ensemble_kernel.cu:97-127
//   end rates, dt, pick, events ... common/ensemble_kernel.cu:199-501,
//                                   common/eq_ensemble_kernel.cu:260-662
//   stress sample ................. common/eq_ensemble_kernel.cu:281-296
//   multi-tau correlator .......... common/eq_ensemble_kernel.cu:133-227,
//                                   common/correlator.cu:104-187
//   flow stress ................... common/ensemble_kernel.cu:504-538,
//                                   common/ensemble_call_block.cu:452-505
//   reach / sync semantics ........ common/ensemble_kernel.cu:199-207,
//                                   common/eq_ensemble_kernel.cu:260-331
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "orc_math.h"
#include "ref_tape.h"

using namespace orc;

extern "C" {
typedef struct orc_params {
  double beta;           // entanglement activity (input.dat line 1)
  int32_t nk;            // Kuhn steps per chain (input.dat line 2); max for polydisperse
  int32_t n_chains;      // input.dat line 3
  int32_t z_max;         // strand capacity per chain (reference: NK, ensemble.cu:99)
  int32_t cd_flag;       // input.dat line 5
  float kappa[9];        // velocity-gradient transpose, row-major (input.dat line 4)
  int32_t mode;          // 0 FP32 mirror, 1 FP64 transcription, 2 reference arithmetic
  uint32_t stream;       // Philox counter word 3 (ensemble id)
  uint64_t seed;         // Philox key (job_ID)
  int32_t corr_type;     // -1 none, 0 stress G(t), 1 centre-of-mass MSD(t)
  int32_t corr_p, corr_m, corr_levels;
  double corr_dt;        // sample interval
  int64_t corr_nsamples; // samples per chain over the run
  const int32_t* nk_chain;  // per-chain Kuhn steps (NULL: all nk)
  int32_t s0;            // initial fixed-point scale exponent (0 -> 40)
  int32_t gex;           // 1: GEX background partner law from the tables below
  const float* gex_M;    // M/mp at probabilities j*gex_step (common/gamma.cpp:174-263)
  const float* gex_Md;   // the CD-weighted counterpart, step gex_step_d
  int32_t gex_n, gex_nd;
  float gex_step, gex_step_d, gex_scale;  // scale = mp/Mk
  int32_t pad2_;
  double gex_prefact;    // CD creation prefactor of the background law (ensemble.cu:137-146)
  uint32_t chain_offset; // global id of chain 0 (Philox keyed by global chain id)
  int32_t partner_n;     // > 0: per-chain N_K of the whole ensemble that partners are drawn
  const int32_t* partner_nk;  // from, and the CD prefactor averaged over, when these chains
                              // are a slice of a larger polydisperse ensemble
} orc_params;
}

namespace {

constexpr double TICKS = 4294967296.0;  // time unit: 2^-32 tau_K
constexpr int LIMIT_E = 47;             // components kept below 2^48 in fixed point

// Event codes (shared with the kernel's event hash)
enum Ev { CDD = 0, SDP = 1, SDM = 2, CDC_MID = 3, CDC_TAIL = 4, SDC_HEAD = 5,
          SDC_TAIL = 6, SDD_HEAD = 7, SDD_TAIL = 8, NULL_FLAG = 16 };

static inline uint64_t hash_step(uint64_t h, uint32_t code) {
  return (h ^ (uint64_t)code) * 0x100000001B3ull;
}

// ------------------------------------------------------------------ p_cd
struct PCD {
  double alpha, tau_0, tau_max, tau_d, g, c1, cm1, rcm1c1, At, Adt, Bdt, normdt;
  float At_, Dt_, Ct_, Adt_, Bdt_, Cdt_, Ddt_, tau_d_inv, one_minus_g;
};

// common/pcd_tau.h:32-66 (constants), common/gpu_random.cu:78-99 (device form)
PCD make_pcd(double Be, double Nk) {
  PCD p{};
  const double z = (Nk + Be) / (Be + 1.0);
  p.g = 0.667;
  if ((float)Be != 1.0f) {
    p.alpha = (0.053 * std::log(Be) + 0.31) * std::pow(z, -0.012 * std::log(Be) - 0.024);
    p.tau_0 = 0.285 * std::pow(Be + 2.0, 0.515);
    p.tau_max = (Nk < 2) ? p.tau_0 : 0.025 * std::pow(Be + 2.0, 2.6) * std::pow(z, 2.83);
    p.tau_d = (Nk < 2) ? p.tau_0 : 0.036 * std::pow(Be + 2.0, 3.07) * std::pow(z - 1.0, 3.02);
  } else {
    p.alpha = 0.267096 - 0.375571 * std::exp(-0.0838237 * Nk);
    p.tau_0 = 0.460277 + 0.298913 * std::exp(-0.0705314 * Nk);
    p.tau_max = (Nk < 4) ? p.tau_0 : 0.0156137 * std::pow(Nk, 3.18849);
    p.tau_d = (Nk < 4) ? p.tau_0 : 0.0740131 * std::pow(Nk, 3.18363);
  }
  p.c1 = std::pow(p.tau_max, p.alpha) - std::pow(p.tau_0, p.alpha);
  p.cm1 = std::pow(p.tau_max, p.alpha - 1.0) - std::pow(p.tau_0, p.alpha - 1.0);
  p.rcm1c1 = (p.c1 == 0.0) ? (p.alpha - 1.0) / p.alpha / p.tau_0 : p.cm1 / p.c1;
  p.At = 1.0 - p.g;
  p.Adt = p.At * p.alpha / (p.alpha - 1.0);
  p.Bdt = p.Adt * p.rcm1c1;
  p.normdt = p.Bdt + p.g / p.tau_d;
  p.At_ = (float)(p.c1 / p.At);
  p.Dt_ = (float)std::pow(p.tau_0, p.alpha);
  p.Ct_ = (float)(-1.0 / p.alpha);
  p.Adt_ = (float)(p.normdt * p.c1 / p.Adt);
  p.Bdt_ = (float)(p.Bdt / p.normdt);
  p.Cdt_ = (float)(-1.0 / (p.alpha - 1.0));
  p.Ddt_ = (float)std::pow(p.tau_0, p.alpha - 1.0);
  p.tau_d_inv = (float)(1.0 / p.tau_d);
  p.one_minus_g = (float)(1.0 - p.g);
  return p;
}

// Lifetime samplers, returning rates 1/tau (gpu_random.cu:143-148).
// SD-created entanglement: f_t ; CD-created entanglement: f_d*t.
static inline float rate_f_t(const PCD& p, float u) {
  return (u < p.one_minus_g) ? m_pow(std::fmaf(u, p.At_, p.Dt_), p.Ct_) : p.tau_d_inv;
}
static inline float rate_f_dt(const PCD& p, float u) {
  return (u < p.Bdt_) ? m_pow(std::fmaf(u, p.Adt_, p.Ddt_), p.Cdt_) : p.tau_d_inv;
}
// FP64 forms (pcd_tau.h:67-82 literally)
static inline double rate_f_t_d(const PCD& p, double u) {
  if (u < 1.0 - p.g) return 1.0 / std::pow(u * p.c1 / p.At + std::pow(p.tau_0, p.alpha), 1.0 / p.alpha);
  return 1.0 / p.tau_d;
}
static inline double rate_f_dt_d(const PCD& p, double u) {
  const double q = u * p.normdt;
  if (q < p.Bdt) return 1.0 / std::pow(q * p.c1 / p.Adt + std::pow(p.tau_0, p.alpha - 1.0), 1.0 / (p.alpha - 1.0));
  return 1.0 / p.tau_d;
}

// ------------------------------------------------------------------ tables
// Per-N factors of the sliding rates (ensemble_kernel.cu:153-178), evaluated
// once in double and rounded to float.  x^0.75 = sqrt(x)*sqrt(sqrt(x)).
struct Tables {
  int nmax = 0;
  std::vector<float> SIGP, SIGM, PWP, PWM, FRIC, SDC, SDD2, SDDN, CDC;
};
static double pow075(double x) { return std::sqrt(x) * std::sqrt(std::sqrt(x)); }

Tables make_tables(int nmax, double beta_f, float prefact) {
  Tables t;
  t.nmax = nmax;
  const int n = nmax + 2;
  t.SIGP.assign(n, 0.f); t.SIGM.assign(n, 0.f); t.PWP.assign(n, 0.f); t.PWM.assign(n, 0.f);
  t.SDC.assign(n, 0.f); t.SDD2.assign(n, 0.f); t.SDDN.assign(n, 0.f); t.CDC.assign(n, 0.f);
  t.FRIC.assign(8 * (size_t)n + 8, 0.f);
  for (int N = 1; N < n; ++N) {
    const double d = N;
    t.SIGP[N] = (float)(0.75 / (d * (d + 1.0)));
    t.SIGM[N] = N >= 2 ? (float)(0.75 / (d * (d - 1.0))) : 0.f;
    t.PWP[N] = (float)pow075(d / (d + 1.0));
    t.PWM[N] = N >= 2 ? (float)pow075(d / (d - 1.0)) : 0.f;
    t.SDC[N] = (float)(2.0 / (beta_f * (d + 0.5)));
    t.SDD2[N] = (float)(1.0 / (0.75 + (d + 0.25)));
    t.SDDN[N] = (float)(1.0 / (0.75 + 0.5 * d));
    t.CDC[N] = (float)((double)prefact * (d - 1.0));
  }
  for (size_t i = 1; i < t.FRIC.size(); ++i) t.FRIC[i] = (float)(4.0 / (double)i);
  return t;
}

// Sliding + CD components of pair (strand i, strand i+1) in the order the
// reference tests them inside a pair: CD destruction, shift N_i+1, shift
// N_i-1, CD creation inside strand i (ensemble_kernel.cu:304-414).
static inline void pair_rates_f(const Tables& T, int cd, int N1, float q1, int N2, float q2,
                                float taurate, float out[4]) {
  const bool z1 = (q1 == 0.0f), z2 = (q2 == 0.0f);
  float wp = 0.0f, wm = 0.0f;
  if (N2 > 1) {
    const int i = (z1 ? 4 * N1 + 1 : 2 * N1) + (z2 ? 4 * N2 - 1 : 2 * N2);
    const float t2 = q2 * T.SIGM[N2];
    const float arg = std::fmaf(q1, T.SIGP[N1], -t2);
    const float pw = (z1 ? 1.0f : T.PWP[N1]) * (z2 ? 1.0f : T.PWM[N2]);
    wp = (T.FRIC[i] * pw) * m_exp(arg);
  }
  if (N1 > 1) {
    const int i = (z1 ? 4 * N1 - 1 : 2 * N1) + (z2 ? 4 * N2 + 1 : 2 * N2);
    const float t1 = q1 * T.SIGM[N1];
    const float arg = std::fmaf(q2, T.SIGP[N2], -t1);
    const float pw = (z1 ? 1.0f : T.PWM[N1]) * (z2 ? 1.0f : T.PWP[N2]);
    wm = (T.FRIC[i] * pw) * m_exp(arg);
  }
  out[0] = cd ? taurate : 0.0f;
  out[1] = wp;
  out[2] = wm;
  out[3] = cd ? T.CDC[N1] : 0.0f;
}

// FP64 literal transcription of the same rates
static inline void pair_rates_d(double beta_unused, int cd, double prefact, int N1, double q1,
                                int N2, double q2, double taurate, double out[4]) {
  (void)beta_unused;
  double wp = 0.0, wm = 0.0;
  const double n1 = N1, n2 = N2;
  if (N2 > 1) {
    const double sig1 = 0.75 / (n1 * (n1 + 1)), sig2 = 0.75 / (n2 * (n2 - 1));
    const double pf1 = (q1 == 0.0) ? 1.0 : n1 / (n1 + 1), pf2 = (q2 == 0.0) ? 1.0 : n2 / (n2 - 1);
    const double f1 = (q1 == 0.0) ? 2.0 * n1 + 0.5 : n1, f2 = (q2 == 0.0) ? 2.0 * n2 - 0.5 : n2;
    wp = 2.0 / (f1 + f2) * std::pow(pf1 * pf2, 0.75) * std::exp(q1 * sig1 - q2 * sig2);
  }
  if (N1 > 1) {
    const double sig1 = 0.75 / (n1 * (n1 - 1)), sig2 = 0.75 / (n2 * (n2 + 1));
    const double pf1 = (q1 == 0.0) ? 1.0 : n1 / (n1 - 1), pf2 = (q2 == 0.0) ? 1.0 : n2 / (n2 + 1);
    const double f1 = (q1 == 0.0) ? 2.0 * n1 - 0.5 : n1, f2 = (q2 == 0.0) ? 2.0 * n2 + 0.5 : n2;
    wm = 2.0 / (f1 + f2) * std::pow(pf1 * pf2, 0.75) * std::exp(-q1 * sig1 + q2 * sig2);
  }
  out[0] = cd ? taurate : 0.0;
  out[1] = wp;
  out[2] = wm;
  out[3] = cd ? prefact * (n1 - 1.0) : 0.0;
}

// ------------------------------------------------------------------ chains
template <class R>
struct Chain {
  int nk = 0, Z = 0, stall = 0, S = 40;
  int64_t T = 0;          // ticks (mode 0); unused in mode 1
  double Td = 0.0;        // time (mode 1)
  uint64_t step = 0, hash = 0xCBF29CE484222325ull;
  R dt_prev = 0;
  int64_t k_next = 0;     // next sample index
  R r1[3] = {0, 0, 0};    // MSD mode: first entanglement in the lab frame (eq_ensemble_kernel.cu:275-277)
  float tf = 0.0f;        // mode 2: FP32 time since the window start (chain_head.time, chain.h:47-50)
  bool halted = false;    // mode 2: stopped by the event limit in the current run
  std::vector<int32_t> N;
  std::vector<R> Qx, Qy, Qz, q2, tau;
  // multi-tau correlator (FP64), common/eq_ensemble_kernel.cu:133-227
  std::vector<double> cshift, cacc, cavg;
  std::vector<int64_t> cnins;
  std::vector<int32_t> cins, cnavg;
};

struct Ensemble {
  orc_params P{};
  std::vector<int32_t> nk_chain;
  std::vector<int32_t> partner;  // polydisperse partner list (default: nk_chain)
  PCD pcd{};                    // monodisperse / prefactor source
  std::vector<PCD> pcd_by_nk;   // polydisperse partner laws (index = NK)
  float prefact = 0.f;          // CD creation prefactor (ensemble.cu:136-148)
  double prefact_d = 0.0;
  Tables tab;
  float kap[9]{};
  int z_max = 0, s0 = 40;
  int64_t dt_sample_ticks = 0;
  std::vector<Chain<float>> cf;
  std::vector<Chain<double>> cd;
  bool poly = false;
  double block_time = 0.0;  // mode 2: time the block has been advanced to (ensemble_call_block.cu:67,218)
  reftape::Key key{};
  reftape::Law law{};
};

static inline U4 rng(const Ensemble& E, uint32_t purpose, uint64_t ctr, uint32_t hi24, uint32_t chain) {
  return philox((uint32_t)ctr, (purpose << 24) | (hi24 & 0xffffffu), chain + E.P.chain_offset, E.P.stream,
                (uint32_t)E.P.seed, (uint32_t)(E.P.seed >> 32));
}
static inline U4 rng_step(const Ensemble& E, uint32_t purpose, uint64_t step, uint32_t chain) {
  return rng(E, purpose, step, (uint32_t)(step >> 32), chain);
}

// p_cd constants of a partner of N_K = nk, in float (the FP32 mirror of the
// kernel's GEX partner law; common/pcd_tau.h:32-66 evaluated per sample as
// gpu_random.cu:212-228 does)
static PCD pcd_from_nk_f(float be, float nk) {
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
  PCD d{};
  d.At_ = c1 / At; d.Dt_ = p0; d.Ct_ = -1.0f / alpha;
  d.Adt_ = normdt * c1 / Adt; d.Bdt_ = Bdt / normdt; d.Cdt_ = -1.0f / (alpha - 1.0f); d.Ddt_ = p0m1;
  d.tau_d_inv = 1.0f / tau_d; d.one_minus_g = 1.0f - g; d.normdt = normdt;
  return d;
}

// Partner law for a new entanglement: monodisperse -> the ensemble's p_cd;
// per-chain N_K -> p_cd of a partner chain drawn uniformly from the ensemble;
// GEX background -> partner mass from the inverse tables (the CD-weighted one
// for CD-created entanglements), linear interpolation at u/step
// (common/chain.cu:141-149, gpu_random.cu:212-228).
static inline PCD partner_pcd(const Ensemble& E, uint32_t w, bool cd_created) {
  if (E.P.gex) {
    const float* T = cd_created ? E.P.gex_Md : E.P.gex_M;
    const int n = cd_created ? E.P.gex_nd : E.P.gex_n;
    const float st = cd_created ? E.P.gex_step_d : E.P.gex_step;
    if (E.P.mode != 1) {
      const float x = u01(w) / st;
      int i = (int)std::floor(x);
      float di = x - (float)i;
      if (i > n - 2) { i = n - 2; di = 1.0f; }
      const float mw = T[i] * (1.0f - di) + T[i + 1] * di;
      return pcd_from_nk_f((float)E.P.beta, mw * E.P.gex_scale);
    }
    const double x = ((w >> 8) + 1u) * (1.0 / 16777216.0) / (double)st;
    int i = (int)std::floor(x);
    double di = x - (double)i;
    if (i > n - 2) { i = n - 2; di = 1.0; }
    const double mw = (double)T[i] * (1.0 - di) + (double)T[i + 1] * di;
    return make_pcd(E.P.beta, mw * (double)E.P.gex_scale);
  }
  if (!E.poly) return E.pcd;
  const uint32_t idx = (uint32_t)(((uint64_t)w * (uint64_t)E.partner.size()) >> 32);
  return E.pcd_by_nk[E.partner[idx]];
}

template <class R>
void corr_alloc(const Ensemble& E, Chain<R>& c) {
  if (E.P.corr_type < 0) return;
  const int L = E.P.corr_levels, p = E.P.corr_p;
  c.cshift.assign((size_t)L * p * 3, 0.0);
  c.cacc.assign((size_t)L * p, 0.0);
  c.cavg.assign((size_t)L * 3, 0.0);
  c.cnins.assign(L, 0);
  c.cins.assign(L, 0);
  c.cnavg.assign(L, 0);
}

// common/eq_ensemble_kernel.cu:133-227.  Type 0 (stress): level k+1 gets the
// block average of m values of level k, lag products v(t)·v(t-j).  Type 1 (MSD,
// :181-189,203,218): level k+1 gets the first value of each block of m (a
// position must not be averaged), lag terms |v(t) - v(t-j)|^2.
template <class R>
void corr_add(const Ensemble& E, Chain<R>& c, const double v[3], int k) {
  const int L = E.P.corr_levels, p = E.P.corr_p, m = E.P.corr_m, dmin = p / m;
  const bool msd = E.P.corr_type == 1;
  if (k >= L) return;
  const int ins = c.cins[k];
  double* sh = &c.cshift[((size_t)k * p) * 3];
  sh[ins * 3 + 0] = v[0]; sh[ins * 3 + 1] = v[1]; sh[ins * 3 + 2] = v[2];
  double* av = &c.cavg[(size_t)k * 3];
  if (!msd) {
    av[0] += v[0]; av[1] += v[1]; av[2] += v[2];
  } else if (c.cnavg[k] == 0) {
    av[0] = v[0]; av[1] = v[1]; av[2] = v[2];
  }
  c.cnavg[k]++;
  if (c.cnavg[k] == m) {
    const double w[3] = {msd ? av[0] : av[0] / m, msd ? av[1] : av[1] / m, msd ? av[2] : av[2] / m};
    av[0] = av[1] = av[2] = 0.0;
    c.cnavg[k] = 0;
    corr_add(E, c, w, k + 1);
  }
  c.cnins[k]++;
  double* acc = &c.cacc[(size_t)k * p];
  for (int j = (k == 0 ? 0 : dmin); j < p; ++j) {
    if ((int64_t)j >= c.cnins[k]) break;
    int i2 = ins - j;
    if (i2 < 0) i2 += p;
    if (msd) {
      const double dx = v[0] - sh[i2 * 3 + 0], dy = v[1] - sh[i2 * 3 + 1], dz = v[2] - sh[i2 * 3 + 2];
      acc[j] += dx * dx + dy * dy + dz * dz;
    } else {
      acc[j] += v[0] * sh[i2 * 3 + 0] + v[1] * sh[i2 * 3 + 1] + v[2] * sh[i2 * 3 + 2];
    }
  }
  c.cins[k] = (ins + 1 == p) ? 0 : ins + 1;
}

// shear stress sample (xy, yz, xz) of common/eq_ensemble_kernel.cu:282-294
template <class R>
void stress_sample(const Chain<R>& c, double v[3]) {
  double sxy = 0, syz = 0, sxz = 0;
  for (int i = 0; i < c.Z; ++i) {
    const double x = c.Qx[i], y = c.Qy[i], z = c.Qz[i], n = c.N[i];
    sxy -= 3.0 * x * y / n;
    syz -= 3.0 * y * z / n;
    sxz -= 3.0 * x * z / n;
  }
  v[0] = sxy; v[1] = syz; v[2] = sxz;
}

// Centre of mass of the chain (eq_ensemble_kernel.cu:297-321): strand j
// contributes N_j/N_K times the position of its midpoint, R1 + sum_{i<j} Q_i
// + Q_j/2 (the dangling head strand has Q = 0, so R1 is where strand 1 starts).
template <class R>
void com_sample(const Chain<R>& c, double v[3]) {
  double px = 0, py = 0, pz = 0, cx = 0, cy = 0, cz = 0;
  const double nk = (double)c.nk;
  for (int i = 0; i < c.Z; ++i) {
    const double x = c.Qx[i], y = c.Qy[i], z = c.Qz[i], n = c.N[i];
    cx += (px + 0.5 * x) * n / nk;
    cy += (py + 0.5 * y) * n / nk;
    cz += (pz + 0.5 * z) * n / nk;
    px += x; py += y; pz += z;
  }
  v[0] = cx + (double)c.r1[0]; v[1] = cy + (double)c.r1[1]; v[2] = cz + (double)c.r1[2];
}

// ------------------------------------------------------------------ initialiser
// Equilibrium state of common/chain.cu:199-283: Z-1 ~ Binomial(NK-1, 1/(1+beta))
// with N uniform over compositions (chain.cu:106-156) is generated as
// independent entanglement of each of the NK-1 bonds with probability
// 1/(1+beta); Q ~ N(0, N/3) for internal strands, 0 for the dangling ends
// (chain.cu:158-170,247-249); tau_CD rates from f_t (chain.cu:207-226).
template <class R>
void init_chain(const Ensemble& E, Chain<R>& c, uint32_t ci) {
  const int nk = c.nk;
  const double pe = 1.0 / (1.0 + E.P.beta);
  double thr_d = std::floor(pe * 4294967296.0);
  if (thr_d > 4294967295.0) thr_d = 4294967295.0;
  const uint32_t thr = (uint32_t)thr_d;
  std::vector<int> pos;
  for (uint32_t att = 0; att < 64; ++att) {
    pos.clear();
    for (int b = 0; b < nk - 1; b += 4) {
      const U4 r = rng(E, P_BONDS, (uint64_t)(b >> 2), att, ci);
      const uint32_t w[4] = {r.x, r.y, r.z, r.w};
      for (int q = 0; q < 4 && b + q < nk - 1; ++q)
        if (w[q] < thr) pos.push_back(b + q);
    }
    if ((int)pos.size() + 1 <= E.z_max) break;
  }
  if ((int)pos.size() + 1 > E.z_max) pos.resize(E.z_max - 1);
  c.Z = (int)pos.size() + 1;
  const int cap = E.z_max;
  c.N.assign(cap + 1, 0);
  c.Qx.assign(cap + 1, 0); c.Qy.assign(cap + 1, 0); c.Qz.assign(cap + 1, 0);
  c.q2.assign(cap + 1, 0); c.tau.assign(cap + 1, 0);
  int prev = -1;
  for (int i = 0; i < c.Z - 1; ++i) { c.N[i] = pos[i] - prev; prev = pos[i]; }
  c.N[c.Z - 1] = nk - 1 - prev;
  for (int i = 1; i < c.Z - 1; ++i) {
    const U4 r = rng(E, P_QINIT, (uint64_t)i, 0, ci);
    if (E.P.mode != 1) {
      float g0, g1, g2, g3;
      m_gauss2(r.x, r.y, &g0, &g1);
      m_gauss2(r.z, r.w, &g2, &g3);
      const float sg = std::sqrt((float)c.N[i] / 3.0f);
      c.Qx[i] = (R)(g0 * sg); c.Qy[i] = (R)(g1 * sg); c.Qz[i] = (R)(g2 * sg);
    } else {
      const double u1a = ((r.x >> 8) + 1u) * (1.0 / 16777216.0), u2a = (r.y >> 8) * (1.0 / 16777216.0);
      const double u1b = ((r.z >> 8) + 1u) * (1.0 / 16777216.0);
      const double ra = std::sqrt(-2.0 * std::log(u1a)), rb = std::sqrt(-2.0 * std::log(u1b));
      const double tha = 2.0 * M_PI * u2a, thb = 2.0 * M_PI * ((r.w >> 8) * (1.0 / 16777216.0));
      const double sg = std::sqrt(c.N[i] / 3.0);
      c.Qx[i] = (R)(ra * std::cos(tha) * sg); c.Qy[i] = (R)(ra * std::sin(tha) * sg);
      c.Qz[i] = (R)(rb * std::cos(thb) * sg);
    }
  }
  for (int i = 0; i < c.Z; ++i) {
    if (E.P.mode != 1) c.q2[i] = (R)m_q2((float)c.Qx[i], (float)c.Qy[i], (float)c.Qz[i]);
    else c.q2[i] = c.Qx[i] * c.Qx[i] + c.Qy[i] * c.Qy[i] + c.Qz[i] * c.Qz[i];
  }
  for (int k = 0; k < c.Z - 1; ++k) {
    const U4 r = rng(E, P_TAUINIT, (uint64_t)k, 0, ci);
    const PCD pp = partner_pcd(E, r.y, false);
    if (!E.P.cd_flag) { c.tau[k] = 0; continue; }
    if (E.P.mode != 1) c.tau[k] = (R)rate_f_t(pp, u01(r.x));
    else c.tau[k] = (R)rate_f_t_d(pp, ((r.x >> 8) + 1u) * (1.0 / 16777216.0));
  }
  c.T = 0; c.Td = 0; c.step = 0; c.dt_prev = 0; c.stall = 0; c.k_next = 0;
  c.r1[0] = c.r1[1] = c.r1[2] = 0;
  c.hash = 0xCBF29CE484222325ull;
  c.S = E.s0;
  corr_alloc(E, c);
}

// ------------------------------------------------------------------ structural edits
template <class R>
void insert_at(Chain<R>& c, int i) {  // open strand slot i and tau slot i
  for (int s = c.Z; s > i; --s) {
    c.N[s] = c.N[s - 1]; c.Qx[s] = c.Qx[s - 1]; c.Qy[s] = c.Qy[s - 1];
    c.Qz[s] = c.Qz[s - 1]; c.q2[s] = c.q2[s - 1]; c.tau[s] = c.tau[s - 1];
  }
}
template <class R>
void remove_strand(Chain<R>& c, int i) {  // close strand slot i
  for (int s = i; s < c.Z - 1; ++s) {
    c.N[s] = c.N[s + 1]; c.Qx[s] = c.Qx[s + 1]; c.Qy[s] = c.Qy[s + 1];
    c.Qz[s] = c.Qz[s + 1]; c.q2[s] = c.q2[s + 1];
  }
}
template <class R>
void remove_tau(Chain<R>& c, int i) {  // close entanglement slot i
  for (int s = i; s < c.Z - 2; ++s) c.tau[s] = c.tau[s + 1];
}

static inline float q2f(float x, float y, float z) { return m_q2(x, y, z); }
static inline double q2f(double x, double y, double z) { return x * x + y * y + z * z; }

// Apply a picked event (immediate form of ensemble_kernel.cu:312-501).
// g[3]: normals for a new strand; trate: lifetime rate of a new entanglement;
// newn: Kuhn steps of the new strand for a CD creation.
template <class R>
void apply_event(Chain<R>& c, int ev, int j, int newn, const R g[3], R trate, bool track_r1) {
  const int Z = c.Z;
  // MSD mode: the first entanglement moves when the head changes
  // (eq_ensemble_kernel.cu:447-455,531-539,606-614,645-653)
  auto r1_add = [&](R x, R y, R z) { c.r1[0] = c.r1[0] + x; c.r1[1] = c.r1[1] + y; c.r1[2] = c.r1[2] + z; };
  auto r1_sub = [&](R x, R y, R z) { c.r1[0] = c.r1[0] - x; c.r1[1] = c.r1[1] - y; c.r1[2] = c.r1[2] - z; };
  auto setQ = [&](int i, R x, R y, R z) {
    c.Qx[i] = x; c.Qy[i] = y; c.Qz[i] = z; c.q2[i] = q2f(x, y, z);
  };
  switch (ev) {
    case CDD: {  // merge strands j, j+1 (ensemble_kernel.cu:312-323)
      const int n = c.N[j] + c.N[j + 1];
      R x = c.Qx[j] + c.Qx[j + 1], y = c.Qy[j] + c.Qy[j + 1], z = c.Qz[j] + c.Qz[j + 1];
      if (j == Z - 2 || j == 0) { x = 0; y = 0; z = 0; }
      if (track_r1 && j == 0) r1_add(c.Qx[1], c.Qy[1], c.Qz[1]);
      remove_strand(c, j + 1);  // strands > j+1 move down one slot
      remove_tau(c, j);         // entanglement j disappears
      c.N[j] = n; setQ(j, x, y, z);
      c.Z = Z - 1;
      break;
    }
    case SDP: c.N[j] += 1; c.N[j + 1] -= 1; break;
    case SDM: c.N[j] -= 1; c.N[j + 1] += 1; break;
    case CDC_MID: {  // split strand j (ensemble_kernel.cu:378-411)
      const int N1 = c.N[j];
      if (j == 0) {
        const int nn = N1 - newn;
        const R sg = (R)std::sqrt((R)nn / (R)3);
        insert_at(c, 0);
        c.N[0] = newn; setQ(0, 0, 0, 0);
        c.N[1] = nn; setQ(1, g[0] * sg, g[1] * sg, g[2] * sg);
        c.tau[0] = trate;
        if (track_r1) r1_sub(c.Qx[1], c.Qy[1], c.Qz[1]);
      } else {
        const R sg = (R)std::sqrt((R)(newn * (N1 - newn)) / (R)(3 * N1));
        const R ra = (R)newn / (R)N1;
        const R x1 = c.Qx[j], y1 = c.Qy[j], z1 = c.Qz[j];
        R x, y, z;
        if constexpr (sizeof(R) == 4) {
          x = std::fmaf(x1, ra, g[0] * sg); y = std::fmaf(y1, ra, g[1] * sg); z = std::fmaf(z1, ra, g[2] * sg);
        } else {
          x = g[0] * sg + x1 * ra; y = g[1] * sg + y1 * ra; z = g[2] * sg + z1 * ra;
        }
        insert_at(c, j);
        c.N[j] = newn; setQ(j, x, y, z);
        c.N[j + 1] = N1 - newn; setQ(j + 1, x1 - x, y1 - y, z1 - z);
        c.tau[j] = trate;
      }
      c.Z = Z + 1;
      break;
    }
    case CDC_TAIL: {  // split the tail strand (ensemble_kernel.cu:422-443)
      const int Nt = c.N[Z - 1];
      const R sg = (Z == 1) ? (R)0 : (R)std::sqrt((R)newn / (R)3);
      c.N[Z] = Nt - newn; setQ(Z, 0, 0, 0);
      c.N[Z - 1] = newn; setQ(Z - 1, g[0] * sg, g[1] * sg, g[2] * sg);
      c.tau[Z - 1] = trate;
      c.Z = Z + 1;
      break;
    }
    case SDC_HEAD: {  // ensemble_kernel.cu:459-468
      const int n0 = c.N[0] - 1;
      const R sg = (Z == 1) ? (R)0 : (R)std::sqrt((R)n0 / (R)3);
      insert_at(c, 0);
      c.N[0] = 1; setQ(0, 0, 0, 0);
      c.N[1] = n0; setQ(1, g[0] * sg, g[1] * sg, g[2] * sg);
      c.tau[0] = trate;
      if (track_r1) r1_sub(c.Qx[1], c.Qy[1], c.Qz[1]);
      c.Z = Z + 1;
      break;
    }
    case SDC_TAIL: {  // ensemble_kernel.cu:469-479
      const int nt = c.N[Z - 1] - 1;
      const R sg = (Z == 1) ? (R)0 : (R)std::sqrt((R)nt / (R)3);
      c.N[Z] = 1; setQ(Z, 0, 0, 0);
      c.N[Z - 1] = nt; setQ(Z - 1, g[0] * sg, g[1] * sg, g[2] * sg);
      c.tau[Z - 1] = trate;
      c.Z = Z + 1;
      break;
    }
    case SDD_HEAD: {  // ensemble_kernel.cu:492-494
      const int n = c.N[1] + 1;
      if (track_r1) r1_add(c.Qx[1], c.Qy[1], c.Qz[1]);
      remove_strand(c, 0);
      remove_tau(c, 0);
      c.N[0] = n; setQ(0, 0, 0, 0);
      c.Z = Z - 1;
      break;
    }
    case SDD_TAIL: {  // ensemble_kernel.cu:495-498
      c.N[Z - 2] = c.N[Z - 2] + 1; setQ(Z - 2, 0, 0, 0);
      c.Z = Z - 1;
      break;
    }
  }
}

// ------------------------------------------------------------------ FP32 mirror step
struct Ends { float w[5]; };  // CD creation at tail, SD creation head, tail, SD destruction head, tail

static inline Ends end_rates_f(const Ensemble& E, const Chain<float>& c) {
  Ends e{};
  const Tables& T = E.tab;
  const int Z = c.Z;
  const int Nh = c.N[0], Nt = c.N[Z - 1];
  e.w[0] = E.P.cd_flag ? T.CDC[Nt] : 0.0f;
  if (Z == 1) {
    const float w1 = (float)(1.0 / (E.P.beta * (double)c.nk));
    e.w[1] = w1; e.w[2] = w1; e.w[3] = 0; e.w[4] = 0;
  } else {
    if (Nh == 1) { e.w[1] = 0; e.w[3] = (Z == 2) ? T.SDD2[c.N[1]] : T.SDDN[c.N[1]]; }
    else { e.w[1] = T.SDC[Nh]; e.w[3] = 0; }
    if (Nt == 1) { e.w[2] = 0; e.w[4] = (Z == 2) ? T.SDD2[c.N[Z - 2]] : T.SDDN[c.N[Z - 2]]; }
    else { e.w[2] = T.SDC[Nt]; e.w[4] = 0; }
  }
  return e;
}

static inline int fexp(float x) {  // floor(log2 x) for normal positive x, -200 otherwise
  const uint32_t b = as_u(x);
  const int e = (int)((b >> 23) & 0xff);
  if (e == 0) return -200;
  return e - 127;
}

static inline float pow2f(int s) {  // 2^s, s in [-126, 127]
  return f_as((uint32_t)(s + 127) << 23);
}

// One kMC event of a chain in FP32-mirror arithmetic.  Returns false when the
// chain stalls (the event is then not applied).
// Position of a CD creation inside a strand of N1 Kuhn steps
// (common/ensemble_kernel.cu:386: newn = floor(0.5 + pr (N1 - 2) / w) + 1) on the
// quantised values rem < wsel: x = floor((2 rem (N1 - 2) + wsel) / (2 wsel)),
// exactly, in 128-bit integers (the sm_103a kernel gets the same x from an FP32
// estimate and an exact integer correction).
static int split_exact(uint64_t rem, uint64_t wsel, int N1) {
  const uint64_t m = (uint64_t)std::max(N1 - 2, 0);
  if (m == 0 || wsel == 0) return 0;
  const unsigned __int128 num = (unsigned __int128)rem * m * 2u + wsel;
  const unsigned __int128 den = (unsigned __int128)wsel * 2u;
  return (int)(num / den);
}

bool step_mirror(const Ensemble& E, Chain<float>& c, uint32_t ci) {
  const int Z = c.Z;
  const int cd = E.P.cd_flag;
  const int npair = Z - 1;
  // all components (the reference recomputes every pair each step,
  // ensemble_kernel.cu:114-186)
  static thread_local std::vector<float> comp;
  comp.resize((size_t)4 * (npair > 0 ? npair : 1));
  int emax = -200;
  bool bad_nan = false, bad_inf = false;
  for (int j = 0; j < npair; ++j) {
    float* o = &comp[(size_t)4 * j];
    pair_rates_f(E.tab, cd, c.N[j], c.q2[j], c.N[j + 1], c.q2[j + 1], c.tau[j], o);
    for (int q = 0; q < 4; ++q) {
      if (o[q] != o[q]) bad_nan = true;
      else if (o[q] == INFINITY) bad_inf = true;
      else emax = std::max(emax, fexp(o[q]));
    }
  }
  const Ends en = end_rates_f(E, c);
  for (int q = 0; q < 5; ++q) emax = std::max(emax, fexp(en.w[q]));
  if (bad_nan) { c.stall = 2; return false; }
  if (bad_inf) { c.stall = 3; return false; }
  // Fixed-point scale 2^S of the rate components.  Every component must stay
  // below 2^(LIMIT_E+1); equilibrium only ever lowers S, flow also raises it
  // again (up to s0) once 2^16 of headroom is free.
  const bool flow = (E.kap[0] != 0 || E.kap[1] != 0 || E.kap[2] != 0 || E.kap[3] != 0 ||
                     E.kap[4] != 0 || E.kap[5] != 0 || E.kap[6] != 0 || E.kap[7] != 0 ||
                     E.kap[8] != 0);
  if (emax + c.S > LIMIT_E) c.S = LIMIT_E - emax;
  else if (flow && c.S < E.s0 && emax + c.S < LIMIT_E - 16) c.S = std::min(E.s0, LIMIT_E - emax);
  const float sf = pow2f(c.S);
  static thread_local std::vector<uint64_t> qc;
  qc.resize((size_t)4 * (npair > 0 ? npair : 1));
  uint64_t pair_total = 0;
  for (int j = 0; j < npair; ++j)
    for (int q = 0; q < 4; ++q) {
      const uint64_t v = (uint64_t)std::llrint(comp[(size_t)4 * j + q] * sf);
      qc[(size_t)4 * j + q] = v;
      pair_total += v;
    }
  uint64_t qe[5], ends_total = 0;
  for (int q = 0; q < 5; ++q) { qe[q] = (uint64_t)std::llrint(en.w[q] * sf); ends_total += qe[q]; }
  const uint64_t total = pair_total + ends_total;
  // dt = 1/sum W (ensemble_kernel.cu:262-272)
  const float sumw = (float)(int64_t)total * pow2f(-c.S);
  const float dt = 1.0f / sumw;
  if (dt == 0.0f) { c.stall = 1; return false; }
  if (!(dt < 2.0e9f)) { c.stall = 3; return false; }
  const int64_t dtt = (int64_t)std::llrint(dt * 4294967296.0f);
  // pick (ensemble_kernel.cu:274-288): pr uniform in [0,total)
  const U4 r = rng_step(E, P_EVENT, c.step, ci);
  const uint64_t u64 = ((uint64_t)r.y << 32) | r.x;
  uint64_t pr = (uint64_t)(((unsigned __int128)total * u64) >> 64);
  int ev = -1, j = -1;
  uint64_t rem = 0, wsel = 0;
  if (pr < pair_total) {
    j = 0;
    while (pr >= qc[(size_t)4 * j] + qc[(size_t)4 * j + 1] + qc[(size_t)4 * j + 2] + qc[(size_t)4 * j + 3]) {
      pr -= qc[(size_t)4 * j] + qc[(size_t)4 * j + 1] + qc[(size_t)4 * j + 2] + qc[(size_t)4 * j + 3];
      ++j;
    }
    const uint64_t* q4 = &qc[(size_t)4 * j];
    if (pr < q4[0]) ev = CDD;
    else if ((pr -= q4[0]) < q4[1]) ev = SDP;
    else if ((pr -= q4[1]) < q4[2]) ev = SDM;
    else { pr -= q4[2]; ev = CDC_MID; rem = pr; wsel = q4[3]; }
  } else {
    pr -= pair_total;
    if (pr < qe[0]) { ev = CDC_TAIL; rem = pr; wsel = qe[0]; }
    else if ((pr -= qe[0]) < qe[1]) ev = SDC_HEAD;
    else if ((pr -= qe[1]) < qe[2]) ev = SDC_TAIL;
    else if ((pr -= qe[2]) < qe[3]) ev = SDD_HEAD;
    else ev = SDD_TAIL;
  }
  c.T += dtt;
  const bool create = (ev == CDC_MID || ev == CDC_TAIL || ev == SDC_HEAD || ev == SDC_TAIL);
  uint32_t code = (uint32_t)ev << 24 | (uint32_t)(j < 0 ? 0 : j);
  if (create && Z >= E.z_max) {
    code |= (uint32_t)NULL_FLAG << 24;  // refused at capacity (ensemble_kernel.cu:380,423,451)
  } else if (create) {
    int newn = 0;
    if (ev == CDC_MID || ev == CDC_TAIL) {
      const int N1 = (ev == CDC_MID) ? c.N[j] : c.N[Z - 1];
      newn = split_exact(rem, wsel, N1) + 1;
      if (newn < 1) newn = 1;
      if (newn > N1 - 1) newn = N1 - 1;
    }
    const U4 gr = rng_step(E, P_CREATE, c.step, ci);
    float g[3], g3;
    m_gauss2(gr.x, gr.y, &g[0], &g[1]);
    m_gauss2(gr.z, gr.w, &g[2], &g3);
    const PCD pp = partner_pcd(E, r.w, ev == CDC_MID || ev == CDC_TAIL);
    const float u = u01(r.z);
    const float trate = cd ? ((ev == CDC_MID || ev == CDC_TAIL) ? rate_f_dt(pp, u) : rate_f_t(pp, u)) : 0.0f;
    apply_event<float>(c, ev, j, newn, g, trate, E.P.corr_type == 1);
    code |= (uint32_t)newn << 8;
  } else {
    apply_event<float>(c, ev, j, 0, nullptr, 0.0f, E.P.corr_type == 1);
  }
  c.hash = hash_step(c.hash, code);
  c.step++;
  c.dt_prev = dt;
  return true;
}

// ------------------------------------------------------------------ FP64 step
bool step_fp64(const Ensemble& E, Chain<double>& c, uint32_t ci) {
  const int Z = c.Z;
  const int cd = E.P.cd_flag;
  const int npair = Z - 1;
  static thread_local std::vector<double> comp;
  comp.resize((size_t)4 * (npair > 0 ? npair : 1));
  double pair_total = 0;
  for (int j = 0; j < npair; ++j) {
    pair_rates_d(E.P.beta, cd, E.prefact_d, c.N[j], c.q2[j], c.N[j + 1], c.q2[j + 1], c.tau[j],
                 &comp[(size_t)4 * j]);
    pair_total += comp[(size_t)4 * j] + comp[(size_t)4 * j + 1] + comp[(size_t)4 * j + 2] + comp[(size_t)4 * j + 3];
  }
  double w[5] = {0, 0, 0, 0, 0};
  const double be = E.P.beta;
  const int Nh = c.N[0], Nt = c.N[Z - 1];
  w[0] = cd ? E.prefact_d * (Nt - 1.0) : 0.0;
  if (Z == 1) { w[1] = w[2] = 1.0 / (be * c.nk); }
  else {
    if (Nh == 1) w[3] = 1.0 / (0.75 + ((Z == 2) ? c.N[1] + 0.25 : 0.5 * c.N[1]));
    else w[1] = 2.0 / (be * (Nh + 0.5));
    if (Nt == 1) w[4] = 1.0 / (0.75 + ((Z == 2) ? c.N[Z - 2] + 0.25 : 0.5 * c.N[Z - 2]));
    else w[2] = 2.0 / (be * (Nt + 0.5));
  }
  const double sumw = pair_total + w[0] + w[1] + w[2] + w[3] + w[4];
  const double dt = 1.0 / sumw;
  if (!(sumw == sumw)) { c.stall = 2; return false; }
  if (dt == 0.0) { c.stall = 1; return false; }
  if (std::isinf(dt)) { c.stall = 3; return false; }
  const U4 r = rng_step(E, P_EVENT, c.step, ci);
  const uint64_t u64 = ((uint64_t)r.y << 32) | r.x;
  double pr = sumw * ((double)(u64 >> 11) * (1.0 / 9007199254740992.0));
  int ev = -1, j = 0;
  double rem = 0, wsel = 1;
  while (j < npair - 1) {
    const double t = comp[(size_t)4 * j] + comp[(size_t)4 * j + 1] + comp[(size_t)4 * j + 2] + comp[(size_t)4 * j + 3];
    if (pr < t) break;
    pr -= t;
    ++j;
  }
  if (npair > 0) {
    const double* q4 = &comp[(size_t)4 * j];
    const double t = q4[0] + q4[1] + q4[2] + q4[3];
    if (pr < t) {
      if (pr < q4[0]) ev = CDD;
      else if ((pr -= q4[0]) < q4[1]) ev = SDP;
      else if ((pr -= q4[1]) < q4[2]) ev = SDM;
      else { pr -= q4[2]; ev = CDC_MID; rem = pr; wsel = q4[3]; }
    } else pr -= t;
  }
  if (ev < 0) {
    j = -1;
    if (pr < w[0]) { ev = CDC_TAIL; rem = pr; wsel = w[0]; }
    else if ((pr -= w[0]) < w[1]) ev = SDC_HEAD;
    else if ((pr -= w[1]) < w[2]) ev = SDC_TAIL;
    else if ((pr -= w[2]) < w[3]) ev = SDD_HEAD;
    else if ((pr -= w[3]) < w[4]) ev = SDD_TAIL;
    else ev = -2;  // roundoff past the last rate: null event
  }
  c.Td += dt;
  if (ev >= 0) {
    const bool create = (ev == CDC_MID || ev == CDC_TAIL || ev == SDC_HEAD || ev == SDC_TAIL);
    if (create && Z >= E.z_max) {
    } else if (create) {
      int newn = 0;
      if (ev == CDC_MID || ev == CDC_TAIL) {
        const int N1 = (ev == CDC_MID) ? c.N[j] : c.N[Z - 1];
        newn = (int)std::floor(0.5 + rem * (N1 - 2) / wsel) + 1;
        newn = std::max(1, std::min(N1 - 1, newn));
      }
      const U4 gr = rng_step(E, P_CREATE, c.step, ci);
      const double u1a = ((gr.x >> 8) + 1u) * (1.0 / 16777216.0), u2a = (gr.y >> 8) * (1.0 / 16777216.0);
      const double u1b = ((gr.z >> 8) + 1u) * (1.0 / 16777216.0), u2b = (gr.w >> 8) * (1.0 / 16777216.0);
      const double ra = std::sqrt(-2.0 * std::log(u1a)), rb = std::sqrt(-2.0 * std::log(u1b));
      const double g[3] = {ra * std::cos(2 * M_PI * u2a), ra * std::sin(2 * M_PI * u2a), rb * std::cos(2 * M_PI * u2b)};
      const PCD pp = partner_pcd(E, r.w, ev == CDC_MID || ev == CDC_TAIL);
      const double u = ((r.z >> 8) + 1u) * (1.0 / 16777216.0);
      const double trate = cd ? ((ev == CDC_MID || ev == CDC_TAIL) ? rate_f_dt_d(pp, u) : rate_f_t_d(pp, u)) : 0.0;
      apply_event<double>(c, ev, j, newn, g, trate, E.P.corr_type == 1);
    } else {
      apply_event<double>(c, ev, j, 0, nullptr, 0.0, E.P.corr_type == 1);
    }
  }
  c.step++;
  c.dt_prev = dt;
  return true;
}

// flow deformation Q += dt kappa Q (ensemble_kernel.cu:105-110)
void deform_f(const Ensemble& E, Chain<float>& c) {
  const float dt = c.dt_prev;
  float a[9];
  for (int q = 0; q < 9; ++q) a[q] = dt * E.kap[q];
  for (int i = 0; i < c.Z; ++i) {
    const float x = c.Qx[i], y = c.Qy[i], z = c.Qz[i];
    const float nx = std::fmaf(a[2], z, std::fmaf(a[1], y, std::fmaf(a[0], x, x)));
    const float ny = std::fmaf(a[5], z, std::fmaf(a[4], y, std::fmaf(a[3], x, y)));
    const float nz = std::fmaf(a[8], z, std::fmaf(a[7], y, std::fmaf(a[6], x, z)));
    c.Qx[i] = nx; c.Qy[i] = ny; c.Qz[i] = nz; c.q2[i] = m_q2(nx, ny, nz);
  }
}
void deform_d(const Ensemble& E, Chain<double>& c) {
  const double dt = c.dt_prev;
  for (int i = 0; i < c.Z; ++i) {
    const double x = c.Qx[i], y = c.Qy[i], z = c.Qz[i];
    const double* k = nullptr; (void)k;
    c.Qx[i] = x + dt * E.kap[0] * x + dt * E.kap[1] * y + dt * E.kap[2] * z;
    c.Qy[i] = y + dt * E.kap[3] * x + dt * E.kap[4] * y + dt * E.kap[5] * z;
    c.Qz[i] = z + dt * E.kap[6] * x + dt * E.kap[7] * y + dt * E.kap[8] * z;
    c.q2[i] = c.Qx[i] * c.Qx[i] + c.Qy[i] * c.Qy[i] + c.Qz[i] * c.Qz[i];
  }
}

static bool is_flow(const Ensemble& E) {
  for (int q = 0; q < 9; ++q) if (E.kap[q] != 0.0f) return true;
  return false;
}

// ------------------------------------------------------------------ mode 2: reference arithmetic
// The reference's chain-parallel kernels (chain_kernel, ensemble_kernel.cu:188-502;
// EQ_chain_kernel, eq_ensemble_kernel.cu:242-663) with the strand-parallel pass
// (strent_kernel :114-186, EQ_strent_kernel :50-130), evaluated with the same
// float/double expressions, written in immediate-apply form: a creation or
// destruction is applied to the chain at once instead of through the offset
// codec that the next step's strand pass applies.  The intrinsics are taken as
// IEEE a/b, powf, expf, sqrtf, and fdivide(1, sumW) as (float)(1.0 / sumW),
// as the host build of the reference kernels (refshim/cuda_runtime.h) does.

static inline float rq2(float x, float y, float z) { return x * x + y * y + z * z; }

// SD shift rates of pair (strand 1, strand 2): W+ moves a Kuhn step into
// strand 1, W- out of it (ensemble_kernel.cu:149-179, :335-358)
static inline void ref_shift(float n1, float Q, float n2, float Q2, float& wx, float& wy) {
  wx = 0.0f;
  wy = 0.0f;
  if (n2 > 1.0f) {
    const float sig1 = 0.75f / (n1 * (n1 + 1));
    const float sig2 = 0.75f / (n2 * (n2 - 1));
    const float pf1 = (Q == 0.0f) ? 1.0f : n1 / (n1 + 1);
    const float pf2 = (Q2 == 0.0f) ? 1.0f : n2 / (n2 - 1);
    const float f1 = (Q == 0.0f) ? 2.0f * n1 + 0.5f : n1;
    const float f2 = (Q2 == 0.0f) ? 2.0f * n2 - 0.5f : n2;
    const float fr = 2.0f / (f1 + f2);
    wx = fr * powf(pf1 * pf2, 0.75f) * expf(Q * sig1 - Q2 * sig2);
  }
  if (n1 > 1.0f) {
    const float sig1 = 0.75f / (n1 * (n1 - 1.0f));
    const float sig2 = 0.75f / (n2 * (n2 + 1.0f));
    const float pf1 = (Q == 0.0f) ? 1.0f : n1 / (n1 - 1.0f);
    const float pf2 = (Q2 == 0.0f) ? 1.0f : n2 / (n2 + 1.0f);
    const float f1 = (Q == 0.0f) ? 2.0f * n1 - 0.5f : n1;
    const float f2 = (Q2 == 0.0f) ? 2.0f * n2 + 0.5f : n2;
    const float fr = 2.0f / (f1 + f2);
    wy = fr * powf(pf1 * pf2, 0.75f) * expf(-Q * sig1 + Q2 * sig2);
  }
}

// pair rate sum written by the strand pass (ensemble_kernel.cu:181,
// eq_ensemble_kernel.cu:126)
static inline float ref_pair_total(const Ensemble& E, const Chain<float>& c, int j) {
  const float n1 = (float)c.N[j], n2 = (float)c.N[j + 1];
  float wx, wy;
  ref_shift(n1, rq2(c.Qx[j], c.Qy[j], c.Qz[j]), n2, rq2(c.Qx[j + 1], c.Qy[j + 1], c.Qz[j + 1]), wx, wy);
  const float tcd = E.P.cd_flag ? c.tau[j] : 0.0f;
  return wx + wy + (float)E.P.cd_flag * (tcd + E.prefact * (n1 - 1.0f));
}

// flow deformation kappa() (ensemble_kernel.cu:105-110)
static inline void ref_kappa(const float* k, float dt, float& x, float& y, float& z) {
  const float nx = x + dt * k[0] * x + dt * k[1] * y + dt * k[2] * z;
  const float ny = y + dt * k[3] * x + dt * k[4] * y + dt * k[5] * z;
  const float nz = z + dt * k[6] * x + dt * k[7] * y + dt * k[8] * z;
  x = nx;
  y = ny;
  z = nz;
}

static inline void set_strand(Chain<float>& c, int i, float x, float y, float z, float n) {
  c.Qx[i] = x; c.Qy[i] = y; c.Qz[i] = z; c.N[i] = (int32_t)n;
  c.q2[i] = rq2(x, y, z);
}

// scan and event of one step (the part of the chain kernel after dt):
// P = double for the equilibrium kernel (FP64 sums, eq_ensemble_kernel.cu:334-662),
// float for the flow kernel (ensemble_kernel.cu:211-501)
template <class P>
static uint32_t ref_scan(const Ensemble& E, Chain<float>& c, uint32_t ci, bool eq, P pr, const float* tsum, P Wcdz,
                         P Wc1, P Wcz, P Wd1, P Wdz) {
  const int Z = c.Z, cd = E.P.cd_flag;
  const float pf = E.prefact;
  const bool msd = eq && E.P.corr_type == 1;
  const uint64_t ev = c.step - 1;
  float g[4];
  auto draw = [&](bool cd_created) { reftape::creation(E.key, E.law, ev, ci, cd_created, g); };
  int j = 0;
  float tpr = 0.0f;
  if (Z != 1) tpr = tsum[0];
  while ((pr >= tpr) && (j < Z - 2)) {
    pr -= tpr;
    j++;
    tpr = tsum[j];
  }
  if (pr < tpr) {
    const float n1 = (float)c.N[j], n2 = (float)c.N[j + 1];
    const float x1 = c.Qx[j], y1 = c.Qy[j], z1 = c.Qz[j];
    const float x2 = c.Qx[j + 1], y2 = c.Qy[j + 1], z2 = c.Qz[j + 1];
    // 1. CD destruction of entanglement j: strands j, j+1 merge
    const float wcdd = cd ? c.tau[j] : 0.0f;
    if (pr < wcdd) {
      float tx = x1 + x2, ty = y1 + y2, tz = z1 + z2;
      if ((j == Z - 2) || (j == 0)) { tx = 0.0f; ty = 0.0f; tz = 0.0f; }
      if (msd && j == 0) { c.r1[0] = c.r1[0] + x2; c.r1[1] = c.r1[1] + y2; c.r1[2] = c.r1[2] + z2; }
      remove_strand(c, j + 1);
      remove_tau(c, j);
      set_strand(c, j, tx, ty, tz, n1 + n2);
      c.Z = Z - 1;
      return (uint32_t)CDD << 24 | (uint32_t)j;
    }
    pr -= wcdd;
    // 2. SD shift
    float wx, wy;
    ref_shift(n1, rq2(x1, y1, z1), n2, rq2(x2, y2, z2), wx, wy);
    if (pr < wx + wy) {
      if (pr < wx) { c.N[j] += 1; c.N[j + 1] -= 1; return (uint32_t)SDP << 24 | (uint32_t)j; }
      c.N[j] -= 1; c.N[j + 1] += 1;
      return (uint32_t)SDM << 24 | (uint32_t)j;
    }
    pr -= wx + wy;
    // 3. CD creation inside strand j
    const P wcdc = eq ? (P)((float)cd * pf * (n1 - 1.0f)) : (P)(pf * (n1 - 1.0f));
    if (pr < wcdc) {
      if (Z == E.z_max) return (uint32_t)(CDC_MID | NULL_FLAG) << 24 | (uint32_t)j;
      draw(true);
      const float trate = g[3];
      const float newn = floorf(0.5f + (float)(pr * (P)(n1 - 2.0f)) / (float)wcdc) + 1.0f;
      if (j == 0) {
        const float tw = n1 - newn;
        const float sg = sqrtf(tw / 3.0f);
        const float tx = g[0] * sg, ty = g[1] * sg, tz = g[2] * sg;
        insert_at(c, 0);
        set_strand(c, 0, 0.0f, 0.0f, 0.0f, newn);
        set_strand(c, 1, tx, ty, tz, tw);
        c.tau[0] = trate;
        if (msd) { c.r1[0] = c.r1[0] + -tx; c.r1[1] = c.r1[1] + -ty; c.r1[2] = c.r1[2] + -tz; }
      } else {
        const float sg = sqrtf((newn * (n1 - newn)) / (3.0f * n1));
        const float ra = newn / n1;
        float tx = g[0] * sg, ty = g[1] * sg, tz = g[2] * sg;
        tx = tx + x1 * ra;
        ty = ty + y1 * ra;
        tz = tz + z1 * ra;
        insert_at(c, j);
        set_strand(c, j, tx, ty, tz, newn);
        set_strand(c, j + 1, x1 - tx, y1 - ty, z1 - tz, n1 - newn);
        c.tau[j] = trate;
      }
      c.Z = Z + 1;
      return (uint32_t)CDC_MID << 24 | (uint32_t)j | (uint32_t)newn << 8;
    }
    pr -= wcdc;
  } else {
    pr -= tpr;
  }
  const float Nh = (float)c.N[0], Nt = (float)c.N[Z - 1];
  // 4. CD creation in the tail strand
  if (pr < Wcdz) {
    if (Z == E.z_max) return (uint32_t)(CDC_TAIL | NULL_FLAG) << 24;
    draw(true);
    const float newn = 1.0f + floorf(0.5f + (float)(pr * (P)(Nt - 2.0f)) / (float)Wcdz);
    const float sg = (Z == 1) ? 0.0f : sqrtf(newn / 3.0f);
    c.tau[Z] = c.tau[Z - 1];
    set_strand(c, Z, 0.0f, 0.0f, 0.0f, Nt - newn);
    set_strand(c, Z - 1, g[0] * sg, g[1] * sg, g[2] * sg, newn);
    c.tau[Z - 1] = g[3];
    c.Z = Z + 1;
    return (uint32_t)CDC_TAIL << 24 | (uint32_t)newn << 8;
  }
  pr -= Wcdz;
  // 5. SD creation at the head or the tail
  if (pr < Wc1 + Wcz) {
    if (Z == E.z_max) return (uint32_t)(SDC_HEAD | NULL_FLAG) << 24;
    draw(false);
    if (pr < Wc1) {
      const float tw = Nh - 1.0f;
      const float sg = (Z == 1) ? 0.0f : sqrtf(tw / 3.0f);
      const float tx = g[0] * sg, ty = g[1] * sg, tz = g[2] * sg;
      insert_at(c, 0);
      set_strand(c, 0, 0.0f, 0.0f, 0.0f, 1.0f);
      set_strand(c, 1, tx, ty, tz, tw);
      c.tau[0] = g[3];
      if (msd) { c.r1[0] = c.r1[0] + -tx; c.r1[1] = c.r1[1] + -ty; c.r1[2] = c.r1[2] + -tz; }
      c.Z = Z + 1;
      return (uint32_t)SDC_HEAD << 24;
    }
    const float tw = Nt - 1.0f;
    const float sg = (Z == 1) ? 0.0f : sqrtf(tw / 3.0f);
    c.tau[Z] = c.tau[Z - 1];
    set_strand(c, Z, 0.0f, 0.0f, 0.0f, 1.0f);
    set_strand(c, Z - 1, g[0] * sg, g[1] * sg, g[2] * sg, tw);
    c.tau[Z - 1] = g[3];
    c.Z = Z + 1;
    return (uint32_t)SDC_TAIL << 24;
  }
  pr -= Wc1 + Wcz;
  // 6. SD destruction at the head or the tail
  if (pr < Wd1 + Wdz) {
    if (pr < Wd1) {
      const float n1 = (float)c.N[1];
      if (msd) { c.r1[0] = c.r1[0] + c.Qx[1]; c.r1[1] = c.r1[1] + c.Qy[1]; c.r1[2] = c.r1[2] + c.Qz[1]; }
      remove_strand(c, 0);
      remove_tau(c, 0);
      set_strand(c, 0, 0.0f, 0.0f, 0.0f, n1 + 1.0f);
      c.Z = Z - 1;
      return (uint32_t)SDD_HEAD << 24;
    }
    set_strand(c, Z - 2, 0.0f, 0.0f, 0.0f, (float)c.N[Z - 2] + 1.0f);
    c.Z = Z - 1;
    return (uint32_t)SDD_TAIL << 24;
  }
  return (uint32_t)NULL_FLAG << 24 | 0xffffu;  // no process matched (roundoff)
}

// rates, dt, clock, uniform, then ref_scan (chain_kernel :211-290,
// EQ_chain_kernel :333-417)
static void ref_event(const Ensemble& E, Chain<float>& c, uint32_t ci, bool eq) {
  const int Z = c.Z, cd = E.P.cd_flag;
  const float be = (float)E.P.beta, pf = E.prefact;
  static thread_local std::vector<float> tsum;
  tsum.resize(Z > 1 ? (size_t)(Z - 1) : 1);
  for (int j = 0; j < Z - 1; ++j) tsum[j] = ref_pair_total(E, c, j);
  const float Nh = (float)c.N[0], Nt = (float)c.N[Z - 1];
  float wc1 = 0.0f, wd1 = 0.0f, wcz = 0.0f, wdz = 0.0f;
  if (Z == 1) {
    wc1 = 1.0f / (be * (float)c.nk);
    wcz = wc1;
  } else {
    if (Nh == 1.0f) {
      const float nn = (float)c.N[1];
      const float f2 = (Z == 2) ? nn + 0.25f : 0.5f * nn;
      wd1 = 1.0f / (0.75f + f2);
    } else {
      wc1 = 2.0f / (be * (Nh + 0.5f));
    }
    if (Nt == 1.0f) {
      const float np = (float)c.N[Z - 2];
      const float f1 = (Z == 2) ? np + 0.25f : 0.5f * np;
      wdz = eq ? 1.0f / (0.75f + f1) : 1.0f / (f1 + 0.75f);
    } else {
      wcz = 2.0f / (be * (Nt + 0.5f));
    }
  }
  float dt;
  uint32_t code;
  if (eq) {
    double swp = 0.0;
    for (int j = 0; j < Z - 1; ++j) swp += tsum[j];
    const double wcdz = (double)cd * (double)pf * (Nt - 1.0f);
    const double sumw = swp + (double)wc1 + (double)wcz + (double)wd1 + (double)wdz + wcdz;
    dt = (float)(1.0 / sumw);
    if (dt == 0.0f) c.stall = 1;
    if (std::isnan(dt)) c.stall = 2;
    if (std::isinf(dt)) c.stall = 3;
    c.tf += dt;
    const float u = reftape::uniform(E.key, c.step, ci);
    c.step++;
    code = ref_scan<double>(E, c, ci, true, sumw * u, tsum.data(), wcdz, wc1, wcz, wd1, wdz);
  } else {
    float swp = 0.0f;
    for (int j = 0; j < Z - 1; ++j) swp += tsum[j];
    const float wcdz = pf * (Nt - 1.0f);
    const float sumw = swp + wc1 + wcz + wd1 + wdz + wcdz;
    dt = 1.0f / sumw;
    if (dt == 0.0f) c.stall = 1;
    if (std::isnan(dt)) c.stall = 2;
    if (std::isinf(dt)) c.stall = 3;
    c.tf += dt;
    const float u = reftape::uniform(E.key, c.step, ci);
    c.step++;
    code = ref_scan<float>(E, c, ci, false, sumw * u, tsum.data(), wcdz, wc1, wcz, wd1, wdz);
  }
  c.dt_prev = dt;
  c.hash = hash_step(c.hash, code);
}

// One chain through one sync window (universal time ut, window length sync),
// one iteration per step of the reference's loop: the strand pass (flow
// deformation by the previous dt), then the chain kernel's stop test, its
// sample (equilibrium, eq_ensemble_kernel.cu:260-331) and its event.
static int64_t run_ref_window(const Ensemble& E, Chain<float>& c, uint32_t ci, float ut, float sync,
                              int64_t limit, bool flow) {
  const bool eq = !flow;
  const bool corr = eq && E.P.corr_type >= 0;
  const int res = (int)E.P.corr_dt;
  int64_t done = 0;
  if (c.halted) return 0;
  for (;;) {
    if (flow)
      for (int i = 0; i < c.Z; ++i) ref_kappa(E.kap, c.dt_prev, c.Qx[i], c.Qy[i], c.Qz[i]);
    if (limit >= 0 && (int64_t)c.step >= limit) {
      c.halted = true;
      c.dt_prev = 0.0f;
      return done;
    }
    bool reach;
    if (corr) reach = ((c.tf >= sync) && (ut + sync <= (float)((int)c.k_next * res))) || (c.stall != 0);
    else reach = (c.tf >= sync) || (c.stall != 0);
    if (reach) {
      c.tf -= sync;
      c.dt_prev = 0.0f;
      return done;
    }
    if (corr && ut + c.tf > (float)((int)c.k_next * res)) {
      double v[3];
      if (E.P.corr_type == 1) com_sample(c, v); else stress_sample(c, v);
      corr_add(E, c, v, 0);
      c.k_next++;
      if (ut + c.tf > (float)((int)c.k_next * res)) continue;
    }
    ref_event(E, c, ci, eq);
    ++done;
  }
}

// the step loops of time_step_call_block / EQ_time_step_call_block
// (ensemble_call_block.cu:106-379): sync windows of at most 1e5 from the
// block's time to reach_time; limit >= 0 also stops a chain after that many
// steps in this run.
int64_t run_ref(Ensemble& E, double reach_time, int64_t limit, int nthreads) {
  const bool flow = is_flow(E);
  const int n = E.P.n_chains;
  for (auto& c : E.cf) c.halted = false;
  const float interval = (float)(reach_time - E.block_time);
  const int nsync = int(std::floor((interval - 0.5) / 1e5)) + 1;
  int64_t total = 0;
  for (int is = 0; is < nsync; ++is) {
    float sync = 1e5f;
    if (is + 1 == nsync) sync = (float)(interval - is * 1e5);
    const float ut = (float)(E.block_time + is * 1e5);
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < n; ++i) total += run_ref_window(E, E.cf[i], (uint32_t)i, ut, sync, limit, flow);
  }
  E.block_time = reach_time;
  return total;
}

// Run one chain until its time reaches t_end (or step_limit events).  Per
// iteration (common/ensemble_kernel.cu:114-207, eq_ensemble_kernel.cu:260-331):
// deform by the previous dt (flow), take due stress samples (equilibrium),
// stop if time >= t_end or stalled, else do one event.
template <class R>
int64_t run_chain(const Ensemble& E, Chain<R>& c, uint32_t ci, double t_end, int64_t step_limit) {
  const bool flow = is_flow(E);
  const int64_t tend_ticks = (int64_t)std::llrint(t_end * TICKS);
  const bool corr = E.P.corr_type >= 0 && !flow;
  int64_t done = 0;
  for (;;) {
    if (flow && c.dt_prev != (R)0) {
      if constexpr (sizeof(R) == 4) deform_f(E, c); else deform_d(E, c);
    }
    if (corr) {
      for (;;) {
        if (c.k_next >= E.P.corr_nsamples) break;
        bool due;
        if constexpr (sizeof(R) == 4) due = c.T > c.k_next * E.dt_sample_ticks;
        else due = c.Td > (double)c.k_next * E.P.corr_dt;
        if (!due) break;
        double v[3];
        if (E.P.corr_type == 1) com_sample(c, v); else stress_sample(c, v);
        corr_add(E, c, v, 0);
        c.k_next++;
      }
    }
    bool reached;
    if constexpr (sizeof(R) == 4) reached = c.T >= tend_ticks;
    else reached = c.Td >= t_end;
    if (c.stall || reached || (step_limit >= 0 && (int64_t)c.step >= step_limit)) {
      c.dt_prev = 0;
      break;
    }
    bool ok;
    if constexpr (sizeof(R) == 4) ok = step_mirror(E, c, ci); else ok = step_fp64(E, c, ci);
    if (!ok) { c.dt_prev = 0; break; }
    ++done;
  }
  return done;
}

}  // namespace

// ====================================================================== C API
extern "C" {

void* orc_create(const orc_params* p) {
  Ensemble* E = new Ensemble();
  E->P = *p;
  E->poly = p->nk_chain != nullptr;
  E->z_max = p->z_max > 0 ? p->z_max : p->nk;
  E->s0 = p->s0 > 0 ? p->s0 : 40;
  for (int q = 0; q < 9; ++q) E->kap[q] = p->kappa[q];
  E->nk_chain.assign(p->n_chains, p->nk);
  if (E->poly) for (int i = 0; i < p->n_chains; ++i) E->nk_chain[i] = p->nk_chain[i];
  E->P.nk_chain = nullptr;
  if (E->poly && p->partner_nk && p->partner_n > 0) E->partner.assign(p->partner_nk, p->partner_nk + p->partner_n);
  else E->partner = E->nk_chain;
  E->P.partner_nk = nullptr;
  const float be_f = (float)p->beta;
  E->P.beta = (double)be_f;
  int nkmax = 0;
  for (int v : E->nk_chain) nkmax = std::max(nkmax, v);
  if (E->poly) {
    // CD creation prefactor = <normdt>/beta over the partner law
    // (role of ensemble.cu:137-146)
    int pmax = nkmax;
    for (int v : E->partner) pmax = std::max(pmax, v);
    E->pcd_by_nk.assign(pmax + 1, PCD{});
    std::vector<char> seen(pmax + 1, 0);
    for (int v : E->partner) if (!seen[v]) { seen[v] = 1; E->pcd_by_nk[v] = make_pcd(E->P.beta, v); }
    double s = 0;
    for (int v : E->partner) s += E->pcd_by_nk[v].normdt;
    E->prefact = (float)((s / (double)E->partner.size()) / E->P.beta);
    E->pcd = make_pcd(E->P.beta, p->nk);
  } else {
    E->pcd = make_pcd(E->P.beta, p->nk);
    E->prefact = p->gex ? (float)p->gex_prefact : (float)(E->pcd.normdt / E->P.beta);
  }
  E->prefact_d = E->prefact;
  E->tab = make_tables(nkmax, E->P.beta, E->prefact);
  E->dt_sample_ticks = (int64_t)std::llrint(p->corr_dt * TICKS);
  if (p->mode != 1) E->cf.resize(p->n_chains); else E->cd.resize(p->n_chains);
  E->key = reftape::Key{p->seed, p->stream, p->chain_offset};
  E->law = reftape::Law{E->pcd.c1, E->pcd.At, E->pcd.tau_0, E->pcd.alpha, E->pcd.normdt,
                        E->pcd.Adt, E->pcd.Bdt, E->pcd.tau_d, E->pcd.g};
  for (int i = 0; i < p->n_chains; ++i) {
    if (p->mode != 1) E->cf[i].nk = E->nk_chain[i]; else E->cd[i].nk = E->nk_chain[i];
  }
  return E;
}

void orc_destroy(void* h) { delete (Ensemble*)h; }

int orc_init_equilibrium(void* h, int nthreads) {
  Ensemble* E = (Ensemble*)h;
  const int n = E->P.n_chains;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
  for (int i = 0; i < n; ++i) {
    if (E->P.mode != 1) init_chain(*E, E->cf[i], (uint32_t)i);
    else init_chain(*E, E->cd[i], (uint32_t)i);
  }
  if (E->P.mode == 0) {
    // initial fixed-point scale: min(s0, 47 - max exponent of all rates)
    for (int i = 0; i < n; ++i) {
      Chain<float>& c = E->cf[i];
      int emax = -200;
      for (int j = 0; j < c.Z - 1; ++j) {
        float o[4];
        pair_rates_f(E->tab, E->P.cd_flag, c.N[j], c.q2[j], c.N[j + 1], c.q2[j + 1], c.tau[j], o);
        for (int q = 0; q < 4; ++q) emax = std::max(emax, fexp(o[q]));
      }
      const Ends en = end_rates_f(*E, c);
      for (int q = 0; q < 5; ++q) emax = std::max(emax, fexp(en.w[q]));
      c.S = std::min(E->s0, LIMIT_E - emax);
    }
  }
  return 0;
}

// Load chain state in the reference layout: per chain z_max float4 {Qx,Qy,Qz,N}
// and z_max float tau rates (chain.h:37-53).  Optional extended scalars.
int orc_set_state(void* h, const int32_t* Z, const float* QN, const float* tau, const int64_t* T,
                  const uint64_t* step, const float* dt_prev, const int32_t* stall, const int32_t* S) {
  Ensemble* E = (Ensemble*)h;
  if (E->P.mode == 1) return -3;
  const int cap = E->z_max;
  for (int i = 0; i < E->P.n_chains; ++i) {
    Chain<float>& c = E->cf[i];
    c.Z = Z[i];
    c.N.assign(cap + 1, 0);
    c.Qx.assign(cap + 1, 0); c.Qy.assign(cap + 1, 0); c.Qz.assign(cap + 1, 0);
    c.q2.assign(cap + 1, 0); c.tau.assign(cap + 1, 0);
    for (int s = 0; s < c.Z; ++s) {
      const float* q = &QN[((size_t)i * cap + s) * 4];
      c.Qx[s] = q[0]; c.Qy[s] = q[1]; c.Qz[s] = q[2]; c.N[s] = (int32_t)q[3];
      c.q2[s] = m_q2(q[0], q[1], q[2]);
      c.tau[s] = tau[(size_t)i * cap + s];
    }
    c.T = T ? T[i] : 0;
    c.step = step ? step[i] : 0;
    c.dt_prev = dt_prev ? dt_prev[i] : 0.f;
    c.stall = stall ? stall[i] : 0;
    c.S = S ? S[i] : E->s0;
    c.hash = 0xCBF29CE484222325ull;
    c.k_next = 0;
    c.tf = 0.0f;
    c.halted = false;
    c.r1[0] = c.r1[1] = c.r1[2] = 0.0f;
    corr_alloc(*E, c);
  }
  E->block_time = 0.0;
  return 0;
}

int orc_get_state(void* h, int32_t* Z, float* QN, float* tau, int64_t* T, uint64_t* step,
                  float* dt_prev, int32_t* stall, int32_t* S, uint64_t* hash) {
  Ensemble* E = (Ensemble*)h;
  const int cap = E->z_max;
  for (int i = 0; i < E->P.n_chains; ++i) {
    if (E->P.mode != 1) {
      const Chain<float>& c = E->cf[i];
      if (Z) Z[i] = c.Z;
      if (QN) for (int s = 0; s < cap; ++s) {
        float* q = &QN[((size_t)i * cap + s) * 4];
        if (s < c.Z) { q[0] = c.Qx[s]; q[1] = c.Qy[s]; q[2] = c.Qz[s]; q[3] = (float)c.N[s]; }
        else { q[0] = q[1] = q[2] = q[3] = 0.f; }
      }
      if (tau) for (int s = 0; s < cap; ++s) tau[(size_t)i * cap + s] = (s < c.Z - 1) ? c.tau[s] : 0.f;
      if (T) T[i] = c.T;
      if (step) step[i] = c.step;
      if (dt_prev) dt_prev[i] = c.dt_prev;
      if (stall) stall[i] = c.stall;
      if (S) S[i] = c.S;
      if (hash) hash[i] = c.hash;
    } else {
      const Chain<double>& c = E->cd[i];
      if (Z) Z[i] = c.Z;
      if (QN) for (int s = 0; s < cap; ++s) {
        float* q = &QN[((size_t)i * cap + s) * 4];
        if (s < c.Z) { q[0] = (float)c.Qx[s]; q[1] = (float)c.Qy[s]; q[2] = (float)c.Qz[s]; q[3] = (float)c.N[s]; }
        else { q[0] = q[1] = q[2] = q[3] = 0.f; }
      }
      if (tau) for (int s = 0; s < cap; ++s) tau[(size_t)i * cap + s] = (s < c.Z - 1) ? (float)c.tau[s] : 0.f;
      if (T) T[i] = (int64_t)std::llrint(c.Td * TICKS);
      if (step) step[i] = c.step;
      if (dt_prev) dt_prev[i] = (float)c.dt_prev;
      if (stall) stall[i] = c.stall;
      if (S) S[i] = 0;
      if (hash) hash[i] = 0;
    }
  }
  return 0;
}

// Advance every chain to time t_end (or step_limit events; -1 = none).
// Returns the number of kMC events done.
int64_t orc_run(void* h, double t_end, int64_t step_limit, int nthreads) {
  Ensemble* E = (Ensemble*)h;
  if (E->P.mode == 2) return run_ref(*E, t_end, step_limit, nthreads);
  const int n = E->P.n_chains;
  int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total) num_threads(nthreads > 0 ? nthreads : 1)
  for (int i = 0; i < n; ++i) {
    if (E->P.mode == 0) total += run_chain(*E, E->cf[i], (uint32_t)i, t_end, step_limit);
    else total += run_chain(*E, E->cd[i], (uint32_t)i, t_end, step_limit);
  }
  return total;
}

// Ensemble-average stress at the current state (flow output; stress_calc of
// ensemble_kernel.cu:504-538 averaged as in ensemble_call_block.cu:452-505):
// out = {xx, yy, zz, xy, yz, zx, Lpp, Z} over non-stalled, non-NaN chains.
int orc_stress(void* h, double* out, int32_t* count) {
  Ensemble* E = (Ensemble*)h;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int cnt = 0;
  for (int i = 0; i < E->P.n_chains; ++i) {
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int Z, stall;
    auto sum = [&](auto& c) {
      Z = c.Z; stall = c.stall;
      for (int j = 0; j < c.Z; ++j) {
        const double x = c.Qx[j], y = c.Qy[j], z = c.Qz[j], n = c.N[j];
        s[0] -= 3 * x * x / n; s[1] -= 3 * y * y / n; s[2] -= 3 * z * z / n;
        s[3] -= 3 * x * y / n; s[4] -= 3 * y * z / n; s[5] -= 3 * x * z / n;
        s[6] += std::sqrt(x * x + y * y + z * z);
      }
      s[7] = c.Z;
    };
    if (E->P.mode != 1) sum(E->cf[i]); else sum(E->cd[i]);
    if (stall != 0 || s[0] != s[0]) continue;
    for (int q = 0; q < 8; ++q) acc[q] += s[q];
    ++cnt;
  }
  for (int q = 0; q < 8; ++q) out[q] = cnt ? acc[q] / cnt : 0.0;
  if (count) *count = cnt;
  return 0;
}

// Correlator output: gsum[k*p + j] = sum over chains of acc/count, count[k*p+j]
// (count of chain 0).  G(t) = gsum/3/N_cha at lag j*m^k samples
// (correlator.cu:146-187, ensemble.cu:318-321).
int orc_gt(void* h, double* gsum, int64_t* count) {
  Ensemble* E = (Ensemble*)h;
  if (E->P.corr_type < 0) return -3;
  const int L = E->P.corr_levels, p = E->P.corr_p;
  for (int q = 0; q < L * p; ++q) { gsum[q] = 0; if (count) count[q] = 0; }
  for (int i = 0; i < E->P.n_chains; ++i) {
    auto add = [&](auto& c) {
      for (int k = 0; k < L; ++k)
        for (int j = 0; j < p; ++j) {
          const int64_t n = c.cnins[k] - j;
          if (n <= 0) continue;
          if (k > 0 && j < p / E->P.corr_m) continue;
          gsum[k * p + j] += c.cacc[(size_t)k * p + j] / (double)n;
          if (count && i == 0) count[k * p + j] = n;
        }
    };
    if (E->P.mode != 1) add(E->cf[i]); else add(E->cd[i]);
  }
  return 0;
}

// Per-chain correlator output: out[(i*L + k)*p + j] = acc/count of chain i
// (0 where the lag has no entries), for error bars of the ensemble average.
int orc_gt_chains(void* h, double* out) {
  Ensemble* E = (Ensemble*)h;
  if (E->P.corr_type < 0) return -3;
  const int L = E->P.corr_levels, p = E->P.corr_p;
  for (int i = 0; i < E->P.n_chains; ++i) {
    auto put = [&](auto& c) {
      for (int k = 0; k < L; ++k)
        for (int j = 0; j < p; ++j) {
          const int64_t n = c.cnins[k] - j;
          double v = 0.0;
          if (n > 0 && !(k > 0 && j < p / E->P.corr_m)) v = c.cacc[(size_t)k * p + j] / (double)n;
          out[((size_t)i * L + k) * p + j] = v;
        }
    };
    if (E->P.mode != 1) put(E->cf[i]); else put(E->cd[i]);
  }
  return 0;
}

// p_cd constants: out[12] fp64 fit values, outf[9] device-form floats
int orc_pcd(double beta, double nk, double* out, float* outf) {
  const PCD p = make_pcd((double)(float)beta, nk);
  const double v[12] = {p.alpha, p.tau_0, p.tau_max, p.tau_d, p.g, p.c1, p.cm1, p.rcm1c1, p.At, p.Adt, p.Bdt, p.normdt};
  for (int q = 0; q < 12; ++q) out[q] = v[q];
  if (outf) {
    const float f[9] = {p.At_, p.Dt_, p.Ct_, p.Adt_, p.Bdt_, p.Cdt_, p.Ddt_, p.tau_d_inv, p.one_minus_g};
    for (int q = 0; q < 9; ++q) outf[q] = f[q];
  }
  return 0;
}

void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  const U4 r = philox(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

// element-wise math spec, for unit tests: which = 0 exp, 1 log, 2 gauss pair
// from words (x as bits), 3 sin2pi, 4 cos2pi
void orc_math(int which, const float* x, const uint32_t* w, float* y, int n) {
  for (int i = 0; i < n; ++i) {
    switch (which) {
      case 0: y[i] = m_exp(x[i]); break;
      case 1: y[i] = m_log(x[i]); break;
      case 2: { float a, b; m_gauss2(w[2 * i], w[2 * i + 1], &a, &b); y[2 * i] = a; y[2 * i + 1] = b; break; }
      case 3: { float s, c; m_sincos2pi(w[i] & 0xffffffu, &s, &c); y[i] = s; break; }
      case 4: { float s, c; m_sincos2pi(w[i] & 0xffffffu, &s, &c); y[i] = c; break; }
      default: y[i] = 0; break;
    }
  }
}

// lifetime samplers for tests: kind 0 f_t, 1 f_d*t; mode 0 float spec, 1 fp64
void orc_tau_sample(double beta, double nk, int kind, int mode, const float* u, double* out, int n) {
  const PCD p = make_pcd((double)(float)beta, nk);
  for (int i = 0; i < n; ++i) {
    if (mode == 0) out[i] = kind == 0 ? rate_f_t(p, u[i]) : rate_f_dt(p, u[i]);
    else out[i] = kind == 0 ? rate_f_t_d(p, u[i]) : rate_f_dt_d(p, u[i]);
  }
}

// Multi-tau correlator alone on a series of n 3-vectors (unit test of the
// correlator semantics of eq_ensemble_kernel.cu:133-227).
int orc_corr_series(int type, int p, int m, int levels, int64_t n, const double* series, double* acc,
                    int64_t* nins) {
  Ensemble E;
  E.P.corr_type = type; E.P.corr_p = p; E.P.corr_m = m; E.P.corr_levels = levels;
  Chain<double> c;
  corr_alloc(E, c);
  for (int64_t t = 0; t < n; ++t) corr_add(E, c, &series[3 * t], 0);
  for (int q = 0; q < levels * p; ++q) acc[q] = c.cacc[q];
  for (int k = 0; k < levels; ++k) nins[k] = c.cnins[k];
  return 0;
}

// MSD mode: position of every chain's first entanglement (n_chains x 3)
int orc_get_r1(void* h, double* r1) {
  Ensemble* E = (Ensemble*)h;
  for (int i = 0; i < E->P.n_chains; ++i) {
    if (E->P.mode != 1) {
      for (int q = 0; q < 3; ++q) r1[3 * i + q] = E->cf[i].r1[q];
    } else {
      for (int q = 0; q < 3; ++q) r1[3 * i + q] = E->cd[i].r1[q];
    }
  }
  return 0;
}

// Mode 2: FP32 clocks since the window start, sample counters, R1 (n x 3).
int orc_get_ref(void* h, float* tf, int32_t* corr_k, float* r1) {
  Ensemble* E = (Ensemble*)h;
  if (E->P.mode == 1) return -3;
  for (int i = 0; i < E->P.n_chains; ++i) {
    const Chain<float>& c = E->cf[i];
    if (tf) tf[i] = c.tf;
    if (corr_k) corr_k[i] = (int32_t)c.k_next;
    if (r1) for (int q = 0; q < 3; ++q) r1[3 * i + q] = c.r1[q];
  }
  return 0;
}

// Parameters the compiled reference kernels need to run this ensemble: the
// CD creation prefactor and the lifetime-law constants of the random stream
// (c1, At, tau0, alpha, normdt, Adt, Bdt, tau_d, g).
int orc_ref_params(void* h, float* prefact, double* law) {
  Ensemble* E = (Ensemble*)h;
  *prefact = E->prefact;
  const double v[9] = {E->law.c1, E->law.At, E->law.tau0, E->law.alpha, E->law.normdt,
                       E->law.Adt, E->law.Bdt, E->law.tau_d, E->law.g};
  for (int q = 0; q < 9; ++q) law[q] = v[q];
  return 0;
}

// the CD creation split of the FP32 mirror (for the tests)
int orc_split(uint64_t rem, uint64_t wsel, int n1) { return split_exact(rem, wsel, n1); }

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
