// Host runtime of the C ABI (include/dsm.h): owns one ensemble on one GPU,
// builds the per-N rate tables and the lifetime-law constants, launches the
// sm_103a kernels of dsm_kernels.cu and moves conformations in the reference
// layout.  Replaces the process-global ensemble / call-block machinery of the
// reference (common/ensemble.cu, common/ensemble_call_block.cu).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dsm.h"
#include "dsm_host.h"
#include "dsm_internal.h"

using namespace dsm;

// ------------------------------------------------------------------ p_cd
// common/pcd_tau.h:32-66 evaluated in double; device form gpu_random.cu:78-99
HostPcd dsm::make_pcd(double Be, double Nk) {
  HostPcd p{};
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
  PcdDev& d = p.dev;
  d.At_ = (float)(p.c1 / p.At);
  d.Dt_ = (float)std::pow(p.tau_0, p.alpha);
  d.Ct_ = (float)(-1.0 / p.alpha);
  d.Adt_ = (float)(p.normdt * p.c1 / p.Adt);
  d.Bdt_ = (float)(p.Bdt / p.normdt);
  d.Cdt_ = (float)(-1.0 / (p.alpha - 1.0));
  d.Ddt_ = (float)std::pow(p.tau_0, p.alpha - 1.0);
  d.tau_d_inv = (float)(1.0 / p.tau_d);
  d.one_minus_g = (float)(1.0 - p.g);
  d.normdt = (float)p.normdt;
  d.pad_[0] = d.pad_[1] = 0.f;
  return p;
}

extern "C" int dsm_pcd(double beta, int32_t nk, double* out) {
  if (!out || !(beta > 0.0) || nk < 1) return DSM_ERR_INVALID;
  const HostPcd p = make_pcd(beta, (double)nk);
  out[0] = p.alpha; out[1] = p.tau_0; out[2] = p.tau_max; out[3] = p.tau_d; out[4] = p.g; out[5] = p.normdt;
  return DSM_OK;
}

// Per-N factors of the sliding rates (ensemble_kernel.cu:153-178,219-260)
// in double, rounded to float.  x^0.75 = sqrt(x)*sqrt(sqrt(x)).
static double pow075(double x) { return std::sqrt(x) * std::sqrt(std::sqrt(x)); }

size_t dsm::table_floats(int nmax) {
  const size_t n = (size_t)nmax + 2;
  return 8 * n + (8 * n + 8) + n + 4;
}

void dsm::make_tables(int nmax, double beta_f, float prefact, float* buf, TableOffsets& off) {
  const size_t n = (size_t)nmax + 2;
  const size_t nf = 8 * n + 8;
  off.NT = 0; off.NE = 4 * n; off.FRIC = 8 * n; off.INV3N = 8 * n + nf;
  std::memset(buf, 0, table_floats(nmax) * sizeof(float));
  for (size_t N = 1; N < n; ++N) {
    const double d = (double)N;
    float* nt = &buf[off.NT + 4 * N];
    nt[0] = (float)(0.75 / (d * (d + 1.0)));
    nt[1] = N >= 2 ? (float)(0.75 / (d * (d - 1.0))) : 0.f;
    nt[2] = (float)pow075(d / (d + 1.0));
    nt[3] = N >= 2 ? (float)pow075(d / (d - 1.0)) : 0.f;
    float* ne = &buf[off.NE + 4 * N];
    ne[0] = (float)(2.0 / (beta_f * (d + 0.5)));
    ne[1] = (float)(1.0 / (0.75 + (d + 0.25)));
    ne[2] = (float)(1.0 / (0.75 + 0.5 * d));
    ne[3] = (float)((double)prefact * (d - 1.0));
    buf[off.INV3N + N] = (float)(3.0 / d);
  }
  for (size_t i = 1; i < nf; ++i) buf[off.FRIC + i] = (float)(4.0 / (double)i);
}

void dsm::make_tables(int nmax, double beta_f, float prefact, std::vector<float>& buf, TableOffsets& off) {
  buf.assign(table_floats(nmax), 0.f);
  make_tables(nmax, beta_f, prefact, buf.data(), off);
}

// ------------------------------------------------------------------ helpers
static int fail(dsm_sim* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}
#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(s, DSM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

int dsm::corr_levels_for(double t_end, double dt, int p, int m) {
  // main_cuda.cu:70
  const double v = std::ceil(std::log(t_end / dt / p) / std::log((double)m)) + 1.0;
  return v < 1.0 ? 1 : (int)v;
}

static int plan_single(dsm_sim* s);
static int default_schedule(dsm_sim* s);
static void series_free(dsm_sim* s);
static int enqueue_readback(dsm_sim* s);
static int window_collect(dsm_sim* s, uint64_t* events);

static bool is_flow(const float* k) {
  for (int q = 0; q < 9; ++q) if (k[q] != 0.0f) return true;
  return false;
}

// ------------------------------------------------------------------ host words
// Small pinned, mapped host words of every handle (abort flag polled by the
// running kernel; end-of-window counters and stress sums copied back
// asynchronously) come from one slab allocated once per process: pinning
// memory per handle costs milliseconds.
namespace {
constexpr int kSlab = 4096;
std::mutex g_slab_mu;
dsm::HostWords* g_slab = nullptr;
std::vector<int> g_slab_free;
}  // namespace

dsm::HostWords* dsm::host_words_take() {
  std::lock_guard<std::mutex> lk(g_slab_mu);
  if (!g_slab) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, sizeof(HostWords) * kSlab, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess)
      return nullptr;
    g_slab = (HostWords*)p;
    for (int i = kSlab - 1; i >= 0; --i) g_slab_free.push_back(i);
  }
  if (g_slab_free.empty()) return nullptr;
  const int i = g_slab_free.back();
  g_slab_free.pop_back();
  std::memset(&g_slab[i], 0, sizeof(HostWords));
  return &g_slab[i];
}

void dsm::host_words_give(HostWords* w) {
  if (!w) return;
  std::lock_guard<std::mutex> lk(g_slab_mu);
  g_slab_free.push_back((int)(w - g_slab));
}

void dsm::keep_pool_memory(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lk(mu);
  if (std::find(done.begin(), done.end(), device) != done.end()) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done.push_back(device);
}

// ------------------------------------------------------------------ lifecycle
extern "C" int dsm_create(const dsm_params* p, dsm_sim** out) {
  if (!p || !out) return DSM_ERR_INVALID;
  *out = nullptr;
  dsm_sim* s = new dsm_sim();
  s->P = *p;
  const int rc = dsm::sim_setup(s);
  if (rc != DSM_OK) {
    // keep the handle so that dsm_last_error can report; caller destroys it
    *out = s;
    return rc;
  }
  *out = s;
  return DSM_OK;
}

int dsm::sim_setup(dsm_sim* s) {
  dsm_params& P = s->P;
  if (P.nk < 1 || P.n_chains < 1 || !(P.beta > 0.0f)) return fail(s, DSM_ERR_INVALID, "invalid nk / n_chains / beta");
  if (P.pd_flag != 0 && P.nk_chain != nullptr)
    return fail(s, DSM_ERR_INVALID, "GEX background (pd_flag=1) with per-chain N_K is not supported");
  s->flow = is_flow(P.kappa);
  s->cap = P.z_max > 0 ? P.z_max : P.nk;
  if (s->cap < 1) return fail(s, DSM_ERR_INVALID, "z_max");
  if (s->cap > 4096) return fail(s, DSM_ERR_INVALID, "z_max above 4096 strands per chain");
  s->poly = P.nk_chain != nullptr;
  s->nk_chain.assign(P.n_chains, P.nk);
  int nkmax = P.nk;
  if (s->poly) {
    nkmax = 0;
    for (int i = 0; i < P.n_chains; ++i) {
      if (P.nk_chain[i] < 1) return fail(s, DSM_ERR_INVALID, "nk_chain entry < 1");
      s->nk_chain[i] = P.nk_chain[i];
      nkmax = std::max(nkmax, P.nk_chain[i]);
    }
  }
  P.nk_chain = nullptr;
  s->nkmax = nkmax;
  const double be = (double)P.beta;
  s->pcd = make_pcd(be, (double)P.nk);
  if (s->poly) {
    s->pcd_by_nk.assign(nkmax + 1, PcdDev{});
    std::vector<char> seen(nkmax + 1, 0);
    std::vector<double> normdt(nkmax + 1, 0.0);
    for (int v : s->nk_chain)
      if (!seen[v]) { seen[v] = 1; HostPcd h = make_pcd(be, v); s->pcd_by_nk[v] = h.dev; normdt[v] = h.normdt; }
    double acc = 0.0;
    for (int v : s->nk_chain) acc += normdt[v];
    s->prefact = (float)((acc / P.n_chains) / be);
  } else if (P.pd_flag != 0) {
    // GEX background: partner masses from the inverse tables, CD creation
    // prefactor averaged over the background law (ensemble.cu:137-146)
    const int rc = make_gex_table(P.gex_a, P.gex_b, P.gex_mp, P.gex_mk, be, &s->gex);
    if (rc != DSM_OK) return fail(s, DSM_ERR_INVALID, "invalid GEX parameters (polydisp.dat a b mp Mk)");
    s->prefact = (float)s->gex.prefact;
  } else {
    s->prefact = (float)(s->pcd.normdt / be);  // ensemble.cu:148
  }
  // eq_type 1: stress relaxation G(t); 2: centre-of-mass MSD(t) (main_cuda.cu:76-82)
  s->corr = (!s->flow) && (P.eq_type == 1 || P.eq_type == 2) && P.sync_dt > 0 && P.t_end > 0;
  s->msd = s->corr && P.eq_type == 2;
  s->ck = s->corr ? (s->msd ? 2 : 1) : 0;
  s->cp = P.corr_p > 0 ? P.corr_p : 64;
  s->cm = P.corr_m > 0 ? P.corr_m : 8;
  if (s->cp % s->cm != 0 || s->cp > 256) return fail(s, DSM_ERR_INVALID, "correlator p must be a multiple of m and <= 256");
  s->levels = P.corr_levels > 0 ? P.corr_levels : (s->corr ? corr_levels_for(P.t_end, P.sync_dt, s->cp, s->cm) : 1);
  s->nsamples = s->corr ? (int64_t)std::ceil(P.t_end / P.sync_dt) : 0;

  CK(cudaSetDevice(P.device));
  {
    int lo = 0, hi = 0;  // least (numerically largest) and greatest priority
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    s->prio = std::max(hi, std::min(lo, P.stream_priority));
  }
  CK(cudaStreamCreateWithPriority(&s->st, cudaStreamNonBlocking, s->prio));
  CK(cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, P.device));
  // device buffers come from the device's stream-ordered pool, which keeps
  // freed memory for reuse: creating and destroying ensembles (a serving loop)
  // then costs no device-wide synchronisation
  keep_pool_memory(P.device);

  // device memory budget
  const size_t n = (size_t)P.n_chains, cap = (size_t)s->cap;
  size_t need = n * cap * (16 + 4) + n * sizeof(ChainState) + n * 8 * 4;
  if (s->corr) need += n * s->levels * ((size_t)s->cp * (12 + 8) + 12 + 16);
  size_t fre = 0, tot = 0;
  CK(cudaMemGetInfo(&fre, &tot));
  if (need + (64ull << 20) > fre) return fail(s, DSM_ERR_MEMORY, "ensemble needs " + std::to_string(need >> 20) + " MiB of device memory, " + std::to_string(fre >> 20) + " MiB free");
  s->bytes = need;

  // tables
  std::vector<float> tb;
  TableOffsets to;
  make_tables(nkmax, be, s->prefact, tb, to);
  CK(cudaMallocAsync((void**)&s->d_tables, tb.size() * sizeof(float), s->st));
  CK(cudaMemcpyAsync(s->d_tables, tb.data(), tb.size() * sizeof(float), cudaMemcpyHostToDevice, s->st));

  // state
  CK(cudaMallocAsync((void**)&s->d_QN, n * cap * sizeof(float4), s->st));
  CK(cudaMallocAsync((void**)&s->d_tau, n * cap * sizeof(float), s->st));
  CK(cudaMallocAsync((void**)&s->d_cs, n * sizeof(ChainState), s->st));
  CK(cudaMallocAsync((void**)&s->d_stress, n * 8 * sizeof(float), s->st));
  CK(cudaMemsetAsync(s->d_QN, 0, n * cap * sizeof(float4), s->st));
  CK(cudaMemsetAsync(s->d_tau, 0, n * cap * sizeof(float), s->st));
  CK(cudaMemsetAsync(s->d_cs, 0, n * sizeof(ChainState), s->st));
  CK(cudaMemsetAsync(s->d_stress, 0, n * 8 * sizeof(float), s->st));
  if (s->corr) {
    const size_t L = s->levels, pp = s->cp;
    CK(cudaMallocAsync((void**)&s->d_cshift, n * L * pp * 3 * sizeof(float), s->st));
    CK(cudaMallocAsync((void**)&s->d_cacc, n * L * pp * sizeof(double), s->st));
    CK(cudaMallocAsync((void**)&s->d_cavg, n * L * 3 * sizeof(float), s->st));
    CK(cudaMallocAsync((void**)&s->d_ccnt, n * L * sizeof(int4), s->st));
    CK(cudaMallocAsync((void**)&s->d_gsum, L * pp * sizeof(double), s->st));
    CK(cudaMallocAsync((void**)&s->d_gcnt, L * pp * sizeof(long long), s->st));
  }
  if (s->poly) {
    CK(cudaMallocAsync((void**)&s->d_pcd_by_nk, s->pcd_by_nk.size() * sizeof(PcdDev), s->st));
    CK(cudaMemcpyAsync(s->d_pcd_by_nk, s->pcd_by_nk.data(), s->pcd_by_nk.size() * sizeof(PcdDev), cudaMemcpyHostToDevice, s->st));
    CK(cudaMallocAsync((void**)&s->d_nk_chain, n * sizeof(int32_t), s->st));
    CK(cudaMemcpyAsync(s->d_nk_chain, s->nk_chain.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, s->st));
  }
  if (P.pd_flag != 0) {
    const size_t nm = s->gex.M.size(), nd = s->gex.Md.size();
    CK(cudaMallocAsync((void**)&s->d_gex, (nm + nd) * sizeof(float), s->st));
    CK(cudaMemcpyAsync(s->d_gex, s->gex.M.data(), nm * sizeof(float), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->d_gex + nm, s->gex.Md.data(), nd * sizeof(float), cudaMemcpyHostToDevice, s->st));
  }
  CK(cudaMallocAsync((void**)&s->d_ens, sizeof(EnsDev), s->st));
  CK(cudaMallocAsync((void**)&s->d_prefix, 2 * sizeof(long long), s->st));
  CK(cudaMallocAsync((void**)&s->d_work, sizeof(unsigned int), s->st));
  CK(cudaMallocAsync((void**)&s->d_status, sizeof(int), s->st));
  CK(cudaMallocAsync((void**)&s->d_counters, 4 * sizeof(unsigned long long), s->st));
  CK(cudaMallocAsync((void**)&s->d_red, 16 * sizeof(double), s->st));
  CK(cudaEventCreate(&s->ev0));
  CK(cudaEventCreate(&s->ev1));
  CK(cudaEventCreateWithFlags(&s->ev_done, cudaEventDisableTiming));
  s->hw = host_words_take();
  if (!s->hw) return fail(s, DSM_ERR_CUDA, "pinned host memory for the abort flag and counters");
  s->hw->abort = 0;
  s->h_abort = &s->hw->abort;
  CK(cudaHostGetDevicePointer((void**)&s->d_abort, (void*)&s->hw->abort, 0));
  const long long pre[2] = {0, (long long)P.n_chains};
  CK(cudaMemcpyAsync(s->d_prefix, pre, sizeof(pre), cudaMemcpyHostToDevice, s->st));

  // device descriptor
  EnsDev& E = s->h;
  std::memset(&E, 0, sizeof(E));
  E.n_chains = P.n_chains; E.cap = s->cap; E.nk = P.nk; E.cd_flag = P.cd_flag ? 1 : 0;
  E.flow = s->flow ? 1 : 0; E.s0 = P.s0 > 0 ? P.s0 : 40; E.poly = s->poly ? 1 : 0;
  E.corr_type = s->corr ? (s->msd ? 1 : 0) : -1; E.corr_p = s->cp; E.corr_m = s->cm; E.corr_levels = s->levels;
  E.beta = P.beta; E.prefact = s->prefact; E.beta_d = (double)P.beta;
  for (int q = 0; q < 9; ++q) E.kap[q] = P.kappa[q];
  E.seed_lo = (uint32_t)P.seed; E.seed_hi = (uint32_t)(P.seed >> 32); E.stream = P.stream;
  E.chain_offset = P.chain_offset;
  E.dt_sample_ticks = s->corr ? (int64_t)std::llrint(P.sync_dt * TICKS) : 0;
  E.nsamples = s->nsamples;
  E.t_end_ticks = 0; E.step_limit = INT64_MAX; E.watchdog_events = INT64_MAX;
  E.pcd = s->pcd.dev;
  E.pcd_by_nk = s->d_pcd_by_nk; E.nk_chain = s->d_nk_chain;
  if (P.pd_flag != 0) {
    E.gex = 1;
    E.gex_n = (int32_t)s->gex.M.size(); E.gex_nd = (int32_t)s->gex.Md.size();
    E.gex_step = s->gex.step; E.gex_step_d = s->gex.step_d; E.gex_scale = P.gex_mp / P.gex_mk;
    E.gex_M = s->d_gex; E.gex_Md = s->d_gex + s->gex.M.size();
  }
  E.NT = (const float4*)(s->d_tables + to.NT); E.NE = (const float4*)(s->d_tables + to.NE);
  E.FRIC = s->d_tables + to.FRIC; E.INV3N = s->d_tables + to.INV3N;
  E.QN = s->d_QN; E.tau = s->d_tau; E.cs = s->d_cs;
  E.corr_shift = s->d_cshift; E.corr_acc = s->d_cacc; E.corr_avg = s->d_cavg; E.corr_cnt = s->d_ccnt;
  E.out_stress = s->d_stress; E.counters = s->d_counters;
  CK(cudaMemcpyAsync(s->d_ens, &E, sizeof(E), cudaMemcpyHostToDevice, s->st));

  // launch shape
  s->cfg.slot_cap = s->cap;
  s->cfg.pmax = s->corr ? s->cp : 0;
  s->cfg.warps_per_block = P.warps_per_block > 0 ? P.warps_per_block : 4;
  if (s->cfg.warps_per_block > 4) s->cfg.warps_per_block = 4;  // __launch_bounds__(128)
  if (P.lanes_per_chain != 0 && P.lanes_per_chain != 16 && P.lanes_per_chain != 32)
    return fail(s, DSM_ERR_INVALID, "lanes_per_chain must be 16 or 32");
  s->cfg.lanes = P.lanes_per_chain > 0 ? P.lanes_per_chain : 32;
  {
    const int rc = s->poly ? plan_classes(s, 0, 0, 0, 0.f) : default_schedule(s);
    if (rc != DSM_OK) return rc;
  }
  CK(cudaStreamSynchronize(s->st));  // host-side sources of the copies above
  s->ready = true;
  return DSM_OK;
}

// Largest slot (strands) at which the step kernel keeps `bps_want` blocks of
// `cfg.warps_per_block` warps resident per SM (0 if even one strand does not)
static int largest_slot(bool flow, int corr, LaunchCfg cfg, int bps_want, int hi) {
  int lo = 0;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    cfg.slot_cap = mid;
    if (step_max_blocks_per_sm(flow, corr, cfg) >= bps_want) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Fewer warps per block while the block's slots exceed the per-block shared
// memory (long chains: one warp per block holds one slot of z_max strands)
static void fit_block(LaunchCfg& cfg, int optin) {
  while (cfg.warps_per_block > 1 && step_block_smem(cfg) > (size_t)optin) cfg.warps_per_block /= 2;
}

// One launch over all chains with slots of the full capacity
static int plan_single(dsm_sim* s) {
  s->classes.clear();
  ++s->sched_version;
  s->cfg.slot_cap = s->cap;
  int smem_optin = 0;
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->P.device));
  fit_block(s->cfg, smem_optin);
  if (step_block_smem(s->cfg) > (size_t)smem_optin)
    return fail(s, DSM_ERR_INVALID, "chain capacity z_max=" + std::to_string(s->cap) + " does not fit one shared-memory slot");
  const int bps = step_max_blocks_per_sm(s->flow, s->ck, s->cfg);
  if (bps < 1) return fail(s, DSM_ERR_CUDA, "step kernel cannot be resident (occupancy 0)");
  s->blocks_per_sm = bps;
  const int tiles = s->cfg.warps_per_block * 32 / s->cfg.lanes;
  const long long want = ((long long)s->P.n_chains + tiles - 1) / tiles;
  s->grid = (int)std::min<long long>(want, (long long)bps * s->sm_count);
  return DSM_OK;
}

int dsm::plan_classes(dsm_sim* s, int small_cap, int big_grid, int lanes, float margin_sd) {
  s->classes.clear();
  s->carved = false;
  s->margin_sd = margin_sd;
  ++s->sched_version;
  const dsm_params& P = s->P;
  const int n = P.n_chains;
  LaunchCfg sc = s->cfg;
  if (lanes == 16 || lanes == 32) sc.lanes = lanes;
  sc.warps_per_block = 4;
  // full occupancy of the step kernel is 4 blocks x 4 warps per SM (register bound)
  const int full_cap = largest_slot(s->flow, s->ck, sc, 4, s->cap);
  if (small_cap <= 0) small_cap = full_cap;
  // one slot size fits all chains at full occupancy (or no useful split)
  if (small_cap >= s->cap || small_cap < 8) return plan_single(s);
  // with two chains per warp in the small class, chains that outgrow its slot
  // but fit a one-chain-per-warp slot at full occupancy run in a middle class
  int mid_cap = 0;
  if (sc.lanes == 16) {
    LaunchCfg mc = sc;
    mc.lanes = 32;
    mid_cap = largest_slot(s->flow, s->ck, mc, 4, s->cap);
    if (mid_cap <= small_cap) mid_cap = 0;
  }
  // chains whose strand count is expected to stay below the small slot
  // (mean + margin_sd sd of 1 + Binomial(N_K - 1, 1/(1+beta)), plus 2) go there
  const double pe = 1.0 / (1.0 + (double)P.beta);
  const double msd = margin_sd > 0.f ? (double)margin_sd : 5.0;
  std::vector<int> huge, big, mid, small;
  int nk_big = 0, nk_huge = 0;
  double w_big = 0.0, w_all = 0.0;
  // chains beyond the middle (or small) slot: a large class with slots sized
  // for twice that bound, and the few longer ones in a huge class with slots
  // of the longest chain -- one slot size for all of them would spend most of
  // its shared memory on strands the typical large chain never has
  const int large_cap = std::min(s->cap, 2 * std::max(small_cap, mid_cap));
  for (int i = 0; i < n; ++i) {
    const int nk = s->nk_chain[i];
    const double m = 1.0 + (nk - 1) * pe, sd = std::sqrt(std::max(0.0, (nk - 1) * pe * (1.0 - pe)));
    const double zb = std::min((double)nk, m + msd * sd + 2.0);
    // work per tau_K: events ~ N_K, cost per event ~ strands + fixed part
    const double w = (double)nk * (m + 40.0);
    w_all += w;
    if (zb <= small_cap) small.push_back(i);
    else if (zb <= mid_cap) mid.push_back(i);
    else if (zb <= large_cap) { big.push_back(i); nk_big = std::max(nk_big, nk); w_big += w; }
    else { huge.push_back(i); nk_huge = std::max(nk_huge, nk); }
  }
  auto by_nk = [&](int a, int b) { return s->nk_chain[a] != s->nk_chain[b] ? s->nk_chain[a] > s->nk_chain[b] : a < b; };
  std::sort(huge.begin(), huge.end(), by_nk);
  std::sort(big.begin(), big.end(), by_nk);
  std::sort(mid.begin(), mid.end(), by_nk);
  std::sort(small.begin(), small.end(), by_nk);
  std::vector<int> order(huge);
  order.insert(order.end(), big.begin(), big.end());
  order.insert(order.end(), mid.begin(), mid.end());
  order.insert(order.end(), small.begin(), small.end());
  if (!s->d_order) {
    CK(cudaMallocAsync((void**)&s->d_order, (size_t)n * sizeof(int), s->st));
    CK(cudaMallocAsync((void**)&s->d_defer, (size_t)n * sizeof(int), s->st));
    CK(cudaMallocAsync((void**)&s->d_works, 16 * sizeof(unsigned int), s->st));
    CK(cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, s->prio));
    CK(cudaStreamCreateWithPriority(&s->side2, cudaStreamNonBlocking, s->prio));
    CK(cudaStreamCreateWithPriority(&s->side3, cudaStreamNonBlocking, s->prio));
    CK(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&s->ev_join2, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&s->ev_join3, cudaEventDisableTiming));
  }
  CK(cudaMemcpyAsync(s->d_order, order.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s->st));
  const int tiles_per_sm_full = 16;
  SizeClass H, B, M, Sm;
  H.stream = 3;
  B.stream = 1;
  M.stream = 2;
  if (!huge.empty()) {
    // few chains: one warp each, all at once
    H.cfg = LaunchCfg{1, std::min(s->cap, nk_huge), s->cfg.pmax, 32};
    H.bps = step_max_blocks_per_sm(s->flow, s->ck, H.cfg);
    if (H.bps < 1) return fail(s, DSM_ERR_INVALID, "largest chains do not fit one shared-memory slot");
    H.first = 0;
    H.count = (long long)huge.size();
    H.grid = (int)std::min<long long>(H.count, (long long)H.bps * s->sm_count);
  }
  if (!big.empty()) {
    B.cfg = LaunchCfg{1, std::min(s->cap, std::min(nk_big, large_cap)), s->cfg.pmax, 32};
    B.bps = step_max_blocks_per_sm(s->flow, s->ck, B.cfg);
    if (B.bps < 1) return fail(s, DSM_ERR_INVALID, "large chains do not fit one shared-memory slot");
    B.first = H.count;
    B.count = (long long)big.size();
    int g = big_grid > 0 ? big_grid
                         : (int)std::ceil(w_big / std::max(w_all, 1.0) * tiles_per_sm_full * s->sm_count);
    g = (int)std::max<long long>(1, std::min<long long>(g, std::min<long long>(B.count, (long long)B.bps * s->sm_count)));
    B.grid = g;
  }
  if (!mid.empty()) {
    // persistent blocks of 4 chains, a full grid: the middle class competes
    // with the small one for block slots, and a work-share grid left it
    // finishing alone at the end of every window (measured 9.6e8 vs 1.2e9
    // events/s on the 262144-chain log-normal melt)
    M.cfg = LaunchCfg{4, mid_cap, s->cfg.pmax, 32};
    M.bps = step_max_blocks_per_sm(s->flow, s->ck, M.cfg);
    if (M.bps < 1) return fail(s, DSM_ERR_INVALID, "middle slot does not fit shared memory");
    M.first = H.count + B.count;
    M.count = (long long)mid.size();
    M.grid = (int)std::max<long long>(1, std::min<long long>((M.count + 3) / 4, (long long)M.bps * s->sm_count));
  }
  Sm.cfg = LaunchCfg{4, small_cap, s->cfg.pmax, sc.lanes};
  Sm.bps = step_max_blocks_per_sm(s->flow, s->ck, Sm.cfg);
  if (Sm.bps < 1) return fail(s, DSM_ERR_INVALID, "small slot does not fit shared memory");
  Sm.first = H.count + B.count + M.count;
  Sm.count = (long long)small.size();
  {
    const int tiles = 4 * 32 / Sm.cfg.lanes;
    Sm.grid = (int)std::max<long long>(1, std::min<long long>((Sm.count + tiles - 1) / tiles,
                                                                (long long)Sm.bps * s->sm_count));
  }
  s->cleanup = SizeClass{};
  s->cleanup.cfg = LaunchCfg{1, s->cap, s->cfg.pmax, 32};
  s->cleanup.bps = step_max_blocks_per_sm(s->flow, s->ck, s->cleanup.cfg);
  if (s->cleanup.bps < 1) return fail(s, DSM_ERR_INVALID, "chain capacity does not fit one shared-memory slot");
  s->cleanup.grid = s->cleanup.bps * s->sm_count;
  if (H.count > 0) s->classes.push_back(H);
  if (B.count > 0) s->classes.push_back(B);
  if (M.count > 0) s->classes.push_back(M);
  s->classes.push_back(Sm);
  s->blocks_per_sm = Sm.bps;
  s->grid = Sm.grid;
  if (s->carve && !s->flow && sc.lanes == 16) {
    LaunchCfg full = sc;
    full.slot_cap = full_cap;
    plan_carve(s, B, M, Sm, step_block_smem(full));
  }
  return DSM_OK;
}

// The carved form of a class plan: the large, middle and small classes run in
// one launch of 4-warp blocks of 16-lane tiles.  Every block has the shared
// memory of a full-occupancy block (8 slots of the largest size that keeps 4
// blocks per SM, the register limit) and carves it into as many slots of its
// class's size as fit (8 small, about 4 middle, 2 large).  Blocks are ordered large, middle,
// small, so that the block scheduler starts the long chains first; each class
// gets the blocks the concurrent launches would have (large: its tile count in
// blocks, middle and small: up to a full persistent grid), and blocks beyond
// the resident ones start as earlier blocks finish.  Not carved (the plan
// stays as it is) when a class's slot does not fit the block.
int dsm::plan_carve(dsm_sim* s, const SizeClass& B, const SizeClass& M, const SizeClass& Sm, size_t smem) {
  const int bps = step_carved_blocks_per_sm(s->ck, smem);
  if (bps < 1) return DSM_OK;
  StepList l;
  int blk = 0, k = 0;
  auto add = [&](const SizeClass& c, int tiles_want) {
    if (c.count <= 0) return true;
    const int tiles = std::min(8, (int)(smem / step_slot_bytes(c.cfg.slot_cap, c.cfg.pmax)));
    if (tiles < 1) return false;
    const long long need = (c.count + tiles - 1) / tiles;
    const long long want = tiles_want > 0 ? (tiles_want + tiles - 1) / tiles : (long long)bps * s->sm_count;
    const int g = (int)std::max<long long>(1, std::min(need, want));
    l.carve_blk[k] = blk;
    l.carve_slot[k] = c.cfg.slot_cap;
    l.carve_tiles[k] = tiles;
    l.carve_first[k] = (int)c.first;
    l.carve_count[k] = (int)c.count;
    blk += g;
    ++k;
    return true;
  };
  // the large class's grid counts one-warp blocks, one chain each
  if (!add(B, B.grid) || !add(M, 0) || !add(Sm, 0)) return DSM_OK;
  l.carve_n = k;
  l.carve_blk[k] = blk;
  l.order = s->d_order;
  l.defer = s->d_defer;
  l.n_defer = s->d_works + 3;
  l.carve_work = s->d_works + 8;
  s->carve_list = l;
  s->carve_grid = blk;
  s->carve_smem = smem;
  s->carved = true;
  return DSM_OK;
}

extern "C" void dsm_destroy(dsm_sim* s) {
  if (!s) return;
  if (s->st) cudaStreamSynchronize(s->st);
  if (s->st) series_free(s);
  if (s->side) cudaStreamSynchronize(s->side);
  if (s->side2) cudaStreamSynchronize(s->side2);
  if (s->side3) cudaStreamSynchronize(s->side3);
  void* ptrs[] = {s->d_tables, s->d_QN, s->d_tau, s->d_cs, s->d_stress, s->d_cshift, s->d_cacc, s->d_cavg,
                  s->d_ccnt, s->d_gsum, s->d_gcnt, s->d_pcd_by_nk, s->d_nk_chain, s->d_ens, s->d_prefix,
                  s->d_work, s->d_status, s->d_counters, s->d_red, s->d_order, s->d_defer, s->d_works, s->d_gex};
  // stream-ordered frees: no device-wide synchronisation
  for (void* p : ptrs) if (p) cudaFreeAsync(p, s->st);
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->ev_join) cudaEventDestroy(s->ev_join);
  if (s->ev_join2) cudaEventDestroy(s->ev_join2);
  if (s->ev_join3) cudaEventDestroy(s->ev_join3);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->side2) cudaStreamDestroy(s->side2);
  if (s->side3) cudaStreamDestroy(s->side3);
  dsm::host_words_give(s->hw);
  if (s->ev_done) cudaEventDestroy(s->ev_done);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->st) cudaStreamDestroy(s->st);
  delete s;
}

extern "C" const char* dsm_last_error(const dsm_sim* s) { return s ? s->err.c_str() : "null handle"; }

// Default launch schedule of a monodisperse ensemble.  Chains run two per warp
// (16 lanes each) with slots of the size that keeps 4 blocks of 4 warps per
// SM, when the chains' strand count (mean + 5 sd of its equilibrium law) fits
// such a slot: 32 chains per SM instead of 16 (measured +14 % at N_K = 200
// with G(t), +24 % for shear at N_K = 100).  A chain that still outgrows the
// slot finishes in the overflow launch.  Otherwise one warp per chain with
// full-capacity slots.
static int default_schedule(dsm_sim* s) {
  if (s->P.lanes_per_chain != 0) return plan_single(s);
  LaunchCfg c = s->cfg;
  c.lanes = 16;
  c.warps_per_block = 4;
  int cap16 = largest_slot(s->flow, s->ck, c, 4, s->cap);
  const double pe = 1.0 / (1.0 + (double)s->P.beta), nk = (double)s->P.nk;
  const double zb = 1.0 + (nk - 1.0) * pe + 5.0 * std::sqrt(std::max(0.0, (nk - 1.0) * pe * (1.0 - pe))) + 2.0;
  // more resident blocks pay (the second build): the largest slot that keeps
  // 6, else 5, blocks per SM when the chains' bound still fits it; with a
  // correlator only 6 (the second build is taken only at half as many blocks
  // again)
  for (int b : {6, 5}) {
    if (b == 5 && !(s->flow || s->ck == 0)) break;
    const int cb = largest_slot(s->flow, s->ck, c, b, s->cap);
    if (cb >= 8 && zb <= cb) {
      cap16 = cb;
      break;
    }
  }
  if (cap16 >= s->cap) {
    s->cfg.lanes = 16;
    return plan_single(s);
  }
  if (cap16 >= 8 && zb <= cap16) {
    s->cfg.lanes = 16;
    return plan_classes(s, cap16, 0, 16, 0.f);
  }
  return plan_single(s);
}

extern "C" int dsm_set_schedule(dsm_sim* s, int32_t small_slot, int32_t large_grid, int32_t lanes,
                                float z_margin_sd) {
  if (!s || !s->ready) return DSM_ERR_INVALID;
  if (lanes != 0 && lanes != 16 && lanes != 32) return fail(s, DSM_ERR_INVALID, "lanes must be 16 or 32");
  CK(cudaStreamSynchronize(s->st));
  if (lanes) s->cfg.lanes = lanes;
  // monodisperse ensembles keep one launch with full-capacity slots unless a
  // smaller slot is asked for (chains that outgrow it finish in the overflow launch)
  if (!s->poly && small_slot <= 0) return plan_single(s);
  return plan_classes(s, small_slot, large_grid, lanes, z_margin_sd);
}

extern "C" int dsm_set_class_form(dsm_sim* s, int32_t form) {
  if (!s || !s->ready || (form != 0 && form != 1) || s->pending) return DSM_ERR_INVALID;
  CK(cudaStreamSynchronize(s->st));
  s->carve = form == 1;
  if (s->classes.empty()) return DSM_OK;
  // the same classes again, in the form asked for
  int small = 0, grid = 0;
  for (const SizeClass& k : s->classes) {
    if (k.stream == 0) small = k.cfg.slot_cap;
    if (k.stream == 1) grid = k.grid;
  }
  return plan_classes(s, small, grid, s->classes.back().cfg.lanes, s->margin_sd);
}

extern "C" int dsm_get_class_form(const dsm_sim* s, int32_t* form) {
  if (!s || !form) return DSM_ERR_INVALID;
  *form = s->carved ? 1 : 0;
  return DSM_OK;
}

// ------------------------------------------------------------------ autotuner
// Online: every candidate schedule runs one real window of the simulation
// (trajectories do not depend on the schedule, so nothing is restored and no
// trial is wasted) and the one with the most events per kernel millisecond is
// kept.
extern "C" int dsm_autotune(dsm_sim* s, double window, int32_t* best, float* best_ms) {
  const dsm::NvtxRange nvtx_range("dsm_autotune");
  if (!s || !s->ready || !(window > 0.0) || s->pending) return DSM_ERR_INVALID;
  struct Cand { int small, grid, lanes, carve = 0; };
  std::vector<Cand> cands;
  for (int lanes : {32, 16}) {
    if (!s->poly) cands.push_back({0, 0, lanes});  // one launch, full-capacity slots
    // small slot: the largest with 4, 3 or 2 blocks of 4 warps per SM
    LaunchCfg c = s->cfg;
    c.lanes = lanes;
    c.warps_per_block = 4;
    std::vector<int> smalls;
    for (int bps : {4, 3, 2}) {
      const int cap = largest_slot(s->flow, s->ck, c, bps, s->cap);
      if (cap >= 8 && std::find(smalls.begin(), smalls.end(), cap) == smalls.end()) smalls.push_back(cap);
    }
    for (int sm : smalls) {
      if (!s->poly) {
        // a smaller slot pays only if the chains' strand counts stay below it
        const double pe = 1.0 / (1.0 + (double)s->P.beta), nk = (double)s->P.nk;
        const double zb = 1.0 + (nk - 1.0) * pe + 5.0 * std::sqrt((nk - 1.0) * pe * (1.0 - pe)) + 2.0;
        if (sm >= s->cap || zb > sm) continue;
      }
      const int rc = plan_classes(s, sm, 0, lanes, 0.f);
      if (rc != DSM_OK) return rc;
      int g0 = 0;  // grid of the large class, whose size the candidates vary
      for (const SizeClass& k : s->classes)
        if (k.stream == 1) g0 = k.grid;
      if (g0 == 0) { cands.push_back({sm, 0, lanes}); continue; }
      for (int g : {std::max(1, g0 / 2), g0, 2 * g0}) cands.push_back({sm, g, lanes});
      // the carved one-launch form of the same classes
      if (s->poly && lanes == 16 && !s->flow) cands.push_back({sm, g0, lanes, 1});
    }
  }
  const bool carve0 = s->carve;
  int bi = -1;
  double brate = 0.0;
  float bms = 0.f;
  for (size_t i = 0; i < cands.size(); ++i) {
    const Cand& c = cands[i];
    s->cfg.lanes = c.lanes;
    s->carve = c.carve != 0;
    int rc = (s->poly || c.small > 0) ? plan_classes(s, c.small, c.grid, c.lanes, 0.f) : plan_single(s);
    if (rc != DSM_OK) return rc;
    rc = sim_launch_window(s, s->t_done + window, -1);
    if (rc == DSM_OK) rc = sim_finish_window(s, nullptr);
    if (rc != DSM_OK) return rc;
    const double rate = (double)s->last_events / std::max(1e-6, (double)s->last_kernel_ms);
    // A short window tells schedules of different tile widths apart only
    // coarsely: over whole windows two 16-lane tiles per warp ran the
    // polydisperse melt 1.5x faster than one 32-lane tile, while single trial
    // windows of a few tau_K came out within a few percent of each other.  So
    // a change of tile width must win its trial by kLaneMargin: 32 lanes must
    // be that much faster than the best 16-lane schedule, and 16 lanes may be
    // that much slower than the best 32-lane one.
    constexpr double kLaneMargin = 0.03;
    double need = brate;
    if (bi >= 0 && c.lanes != cands[bi].lanes) need = brate * (c.lanes == 16 ? 1.0 - kLaneMargin : 1.0 + kLaneMargin);
    if (bi < 0 || rate > need) { bi = (int)i; brate = rate; bms = s->last_kernel_ms; }
  }
  const Cand& b = cands[bi];
  s->cfg.lanes = b.lanes;
  s->carve = b.carve != 0 || (carve0 && !s->poly);
  const int rc = (s->poly || b.small > 0) ? plan_classes(s, b.small, b.grid, b.lanes, 0.f) : plan_single(s);
  if (best) { best[0] = b.small; best[1] = b.grid; best[2] = b.lanes; best[3] = (int32_t)cands.size(); }
  if (best_ms) *best_ms = bms;
  return rc;
}

extern "C" int dsm_get_r1(dsm_sim* s, float* r1) {
  if (!s || !s->ready || !r1) return DSM_ERR_INVALID;
  const size_t n = s->P.n_chains;
  std::vector<ChainState> cs(n);
  CK(cudaMemcpyAsync(cs.data(), s->d_cs, n * sizeof(ChainState), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  for (size_t i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) r1[3 * i + q] = cs[i].r1[q];
  return DSM_OK;
}

extern "C" int dsm_window_stats(const dsm_sim* s, uint64_t* events, uint64_t* chains_done, uint64_t* deferred) {
  if (!s || !s->hw) return DSM_ERR_INVALID;
  if (events) *events = s->hw->cnt[0];
  if (chains_done) *chains_done = s->hw->cnt[1];
  if (deferred) *deferred = s->hw->cnt[2];
  return DSM_OK;
}

extern "C" int dsm_get_schedule(const dsm_sim* s, int32_t* n_classes, int32_t* info) {
  if (!s || !n_classes) return DSM_ERR_INVALID;
  *n_classes = (int32_t)s->classes.size();
  if (info) {
    for (int i = 0; i < DSM_SCHEDULE_INFO; ++i) info[i] = 0;
    int i = 0;
    auto put = [&](const SizeClass& k, long long count) {
      info[5 * i + 0] = k.cfg.slot_cap; info[5 * i + 1] = k.cfg.warps_per_block; info[5 * i + 2] = k.cfg.lanes;
      info[5 * i + 3] = k.grid; info[5 * i + 4] = (int32_t)count;
      ++i;
    };
    for (const SizeClass& k : s->classes) put(k, k.count);
    if (!s->classes.empty()) put(s->cleanup, 0);
  }
  return DSM_OK;
}

extern "C" int dsm_corr_shape(const dsm_sim* s, int32_t* levels, int32_t* p, int32_t* m) {
  if (!s) return DSM_ERR_INVALID;
  if (levels) *levels = s->corr ? s->levels : 0;
  if (p) *p = s->cp;
  if (m) *m = s->cm;
  return DSM_OK;
}

static int reset_corr(dsm_sim* s) {
  if (!s->corr) return DSM_OK;
  const size_t n = s->P.n_chains, L = s->levels, pp = s->cp;
  CK(cudaMemsetAsync(s->d_cshift, 0, n * L * pp * 3 * sizeof(float), s->st));
  CK(cudaMemsetAsync(s->d_cacc, 0, n * L * pp * sizeof(double), s->st));
  CK(cudaMemsetAsync(s->d_cavg, 0, n * L * 3 * sizeof(float), s->st));
  CK(cudaMemsetAsync(s->d_ccnt, 0, n * L * sizeof(int4), s->st));
  return DSM_OK;
}

extern "C" int dsm_init_equilibrium(dsm_sim* s) {
  const dsm::NvtxRange nvtx_range("dsm_init_equilibrium");
  if (!s || !s->ready) return DSM_ERR_INVALID;
  CK(cudaMemsetAsync(s->d_QN, 0, (size_t)s->P.n_chains * s->cap * sizeof(float4), s->st));
  CK(cudaMemsetAsync(s->d_tau, 0, (size_t)s->P.n_chains * s->cap * sizeof(float), s->st));
  int rc = reset_corr(s);
  if (rc) return rc;
  CK(launch_init(s->d_ens, s->h, s->cap, s->st));
  CK(cudaStreamSynchronize(s->st));
  return DSM_OK;
}

// ------------------------------------------------------------------ state transfer
extern "C" int dsm_set_chains(dsm_sim* s, const dsm_chain_head* heads, const dsm_float4* QN, const float* tau) {
  const dsm::NvtxRange nvtx_range("dsm_set_chains");
  if (!s || !s->ready || !heads || !QN || !tau) return DSM_ERR_INVALID;
  const size_t n = s->P.n_chains, cap = s->cap;
  std::vector<ChainState> cs(n);
  // validate and build the chain states in parallel over chain ranges; the
  // first bad chain in chain order is reported, as a serial pass would
  const size_t nt = std::max<size_t>(1, std::min<size_t>({16, std::thread::hardware_concurrency(), n / 4096 + 1}));
  std::vector<size_t> bad(nt, n);
  std::vector<int> why(nt, 0);
  auto work = [&](size_t r) {
    const size_t i0 = n * r / nt, i1 = n * (r + 1) / nt;
    for (size_t i = i0; i < i1; ++i) {
      const int Z = heads[i].Z;
      int code = 0;
      if (Z < 1 || Z > (int)cap) code = 1;
      long long sumN = 0;
      for (int k = 0; k < Z && code == 0; ++k) {
        const float w = QN[i * cap + k].w;
        if (!(w >= 1.0f) || w != std::floor(w)) code = 2;
        sumN += (long long)w;
      }
      if (code == 0 && sumN != s->nk_chain[i]) code = 3;
      if (code != 0) { bad[r] = i; why[r] = code; return; }
      ChainState& c = cs[i];
      std::memset(&c, 0, sizeof(c));
      c.Z = Z; c.stall = heads[i].stall_flag; c.S = s->h.s0; c.dt_prev = 0.f;
      c.T = (int64_t)std::llrint((double)heads[i].time * TICKS);
      c.step = 0; c.hash = 0xCBF29CE484222325ull; c.k_next = 0; c.nk = s->nk_chain[i];
    }
  };
  std::vector<std::thread> pool;
  for (size_t r = 1; r < nt; ++r) pool.emplace_back(work, r);
  work(0);
  for (auto& th : pool) th.join();
  for (size_t r = 0; r < nt; ++r) {
    if (bad[r] == n) continue;
    static const char* const msg[] = {"", ": Z out of [1, z_max]", ": strand with N < 1 or fractional N",
                                      ": sum of N differs from N_K"};
    return fail(s, DSM_ERR_INVALID, "chain " + std::to_string(bad[r]) + msg[why[r]]);
  }
  CK(cudaMemcpyAsync(s->d_QN, QN, n * cap * sizeof(float4), cudaMemcpyHostToDevice, s->st));
  CK(cudaMemcpyAsync(s->d_tau, tau, n * cap * sizeof(float), cudaMemcpyHostToDevice, s->st));
  CK(cudaMemcpyAsync(s->d_cs, cs.data(), n * sizeof(ChainState), cudaMemcpyHostToDevice, s->st));
  int rc = reset_corr(s);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s->st));
  return DSM_OK;
}

extern "C" int dsm_get_chains(dsm_sim* s, dsm_chain_head* heads, dsm_float4* QN, float* tau) {
  const dsm::NvtxRange nvtx_range("dsm_get_chains");
  if (!s || !s->ready) return DSM_ERR_INVALID;
  const size_t n = s->P.n_chains, cap = s->cap;
  // slots beyond Z are not maintained on the device: zero them there, so the
  // copies come back in the reference layout without a host pass
  if (QN || tau) CK(launch_clear_tail(s->d_QN, s->d_tau, s->d_cs, (int)n, (int)cap, s->st));
  if (QN) CK(cudaMemcpyAsync(QN, s->d_QN, n * cap * sizeof(float4), cudaMemcpyDeviceToHost, s->st));
  if (tau) CK(cudaMemcpyAsync(tau, s->d_tau, n * cap * sizeof(float), cudaMemcpyDeviceToHost, s->st));
  std::vector<ChainState> cs(heads ? n : 0);
  if (heads) CK(cudaMemcpyAsync(cs.data(), s->d_cs, n * sizeof(ChainState), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (heads)
    for (size_t i = 0; i < n; ++i) {
      heads[i].Z = cs[i].Z;
      heads[i].time = (float)((double)cs[i].T / TICKS);
      heads[i].dummy = 0.f;
      heads[i].stall_flag = cs[i].stall;
    }
  return DSM_OK;
}

extern "C" int dsm_get_ext(dsm_sim* s, int64_t* T, uint64_t* steps, float* dt_prev, int32_t* stall,
                           int32_t* scale, uint64_t* hash) {
  if (!s || !s->ready) return DSM_ERR_INVALID;
  const size_t n = s->P.n_chains;
  std::vector<ChainState> cs(n);
  CK(cudaMemcpyAsync(cs.data(), s->d_cs, n * sizeof(ChainState), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  for (size_t i = 0; i < n; ++i) {
    if (T) T[i] = cs[i].T;
    if (steps) steps[i] = cs[i].step;
    if (dt_prev) dt_prev[i] = cs[i].dt_prev;
    if (stall) stall[i] = cs[i].stall;
    if (scale) scale[i] = cs[i].S;
    if (hash) hash[i] = cs[i].hash;
  }
  return DSM_OK;
}

extern "C" int dsm_set_ext(dsm_sim* s, const int64_t* T, const uint64_t* steps, const float* dt_prev,
                           const int32_t* stall, const int32_t* scale) {
  if (!s || !s->ready) return DSM_ERR_INVALID;
  const size_t n = s->P.n_chains;
  std::vector<ChainState> cs(n);
  CK(cudaMemcpyAsync(cs.data(), s->d_cs, n * sizeof(ChainState), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  for (size_t i = 0; i < n; ++i) {
    if (T) cs[i].T = T[i];
    if (steps) cs[i].step = steps[i];
    if (dt_prev) cs[i].dt_prev = dt_prev[i];
    if (stall) cs[i].stall = stall[i];
    if (scale) cs[i].S = scale[i];
  }
  CK(cudaMemcpyAsync(s->d_cs, cs.data(), n * sizeof(ChainState), cudaMemcpyHostToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  return DSM_OK;
}

// ------------------------------------------------------------------ time evolution
// Per-chain event cap of one launch: a chain whose dt collapses (rates blowing
// up) stops with stall code 5 instead of keeping the GPU busy.  The cap is
// 100x the expected events of a window of dt_tau (<sum W> ~ 0.25 N_K per
// tau_K), at least 2^24.
static int64_t window_watchdog(const dsm_sim* s, double dt_tau) {
  if (s->watchdog_events > 0) return s->watchdog_events;
  const double expect = 0.25 * (double)s->nkmax * std::max(0.0, dt_tau) * 100.0;
  return (int64_t)std::max(16777216.0, std::min(expect, 9.0e18));
}

// The step launch(es) of one window on s->st (the descriptor already holds
// the window): one launch over all chains, or the size classes
static int enqueue_classes(dsm_sim* s) {
  // concurrent form: large-slot chains on the side stream first, then the
  // middle class on the second side stream (their blocks are placed first),
  // small-slot chains on the main stream, the huge class on the third
  CK(cudaEventRecord(s->ev_fork, s->st));
  CK(cudaStreamWaitEvent(s->side, s->ev_fork, 0));
  CK(cudaStreamWaitEvent(s->side2, s->ev_fork, 0));
  CK(cudaStreamWaitEvent(s->side3, s->ev_fork, 0));
  for (const SizeClass& k : s->classes) {
    StepList l;
    l.order = s->d_order + k.first;
    l.defer = s->d_defer;
    l.n_defer = s->d_works + 3;
    cudaStream_t st = k.stream == 1 ? s->side : k.stream == 2 ? s->side2 : k.stream == 3 ? s->side3 : s->st;
    unsigned int* work = s->d_works + (k.stream == 1 ? 1 : k.stream == 2 ? 4 : k.stream == 3 ? 5 : 0);
    CK(launch_step(s->d_ens, 1, s->d_prefix, k.count, work, s->flow, s->ck, k.cfg, s->d_abort, s->d_status,
                   k.grid, st, l));
  }
  CK(cudaEventRecord(s->ev_join, s->side));
  CK(cudaEventRecord(s->ev_join2, s->side2));
  CK(cudaEventRecord(s->ev_join3, s->side3));
  CK(cudaStreamWaitEvent(s->st, s->ev_join, 0));
  CK(cudaStreamWaitEvent(s->st, s->ev_join2, 0));
  CK(cudaStreamWaitEvent(s->st, s->ev_join3, 0));
  return DSM_OK;
}

static int enqueue_carved(dsm_sim* s) {
  // carved form: the huge class on its stream, the other classes in one
  // launch on the main stream
  CK(cudaEventRecord(s->ev_fork, s->st));
  CK(cudaStreamWaitEvent(s->side3, s->ev_fork, 0));
  for (const SizeClass& k : s->classes) {
    if (k.stream != 3) continue;
    StepList l;
    l.order = s->d_order + k.first;
    l.defer = s->d_defer;
    l.n_defer = s->d_works + 3;
    CK(launch_step(s->d_ens, 1, s->d_prefix, k.count, s->d_works + 5, s->flow, s->ck, k.cfg, s->d_abort,
                   s->d_status, k.grid, s->side3, l));
  }
  CK(launch_step_carved(s->d_ens, s->d_prefix, s->ck, s->cfg.pmax, s->carve_smem, s->d_abort, s->d_status,
                        s->carve_grid, s->st, s->carve_list));
  CK(cudaEventRecord(s->ev_join3, s->side3));
  CK(cudaStreamWaitEvent(s->st, s->ev_join3, 0));
  return DSM_OK;
}

static int enqueue_step(dsm_sim* s) {
  if (s->classes.empty()) {
    CK(cudaMemsetAsync(s->d_work, 0, sizeof(unsigned int), s->st));
    CK(launch_step(s->d_ens, 1, s->d_prefix, (long long)s->P.n_chains, s->d_work, s->flow, s->ck, s->cfg,
                   s->d_abort, s->d_status, s->grid, s->st));
    return DSM_OK;
  }
  CK(cudaMemsetAsync(s->d_works, 0, 16 * sizeof(unsigned int), s->st));
  const int rc = s->carved ? enqueue_carved(s) : enqueue_classes(s);
  if (rc != DSM_OK) return rc;
  // then the chains that outgrew their slot, in slots of the ensemble's full capacity
  StepList l;
  l.order = s->d_defer;
  l.dyn_total = s->d_works + 3;
  CK(launch_step(s->d_ens, 1, s->d_prefix, 0, s->d_works + 2, s->flow, s->ck, s->cleanup.cfg, s->d_abort,
                 s->d_status, s->cleanup.grid, s->st, l));
  return DSM_OK;
}

int dsm::sim_launch_window(dsm_sim* s, double t_end, int64_t step_limit) {
  EnsDev& E = s->h;
  E.t_end_ticks = (int64_t)std::llrint(t_end * TICKS);
  s->t_window = t_end;
  E.step_limit = step_limit < 0 ? INT64_MAX : step_limit;
  E.watchdog_events = window_watchdog(s, t_end - s->t_done);
  CK(cudaMemcpyAsync(s->d_ens, &E, sizeof(EnsDev), cudaMemcpyHostToDevice, s->st));
  CK(cudaMemsetAsync(s->d_status, 0, sizeof(int), s->st));
  CK(cudaMemsetAsync(s->d_counters, 0, 4 * sizeof(unsigned long long), s->st));
  CK(cudaEventRecord(s->ev0, s->st));
  const int rc = enqueue_step(s);
  if (rc != DSM_OK) return rc;
  CK(cudaEventRecord(s->ev1, s->st));
  return DSM_OK;
}

// ------------------------------------------------------------------ graph series
// n windows as one CUDA graph, replayed with new end times; one graph is
// captured per (n, launch schedule).  Equilibrium: per window a one-thread
// kernel sets the end time and event cap from a device array, then the step
// launch(es).  Flow: groups of up to kSeriesGroup windows run inside one step
// launch (each chain records its stress at every window end it crosses and
// keeps its state resident), followed by the stress sums of each window of
// the group.  At the end the sums and counters go to pinned host memory.
static constexpr int kSeriesGroup = 16;

// bytes of the series buffer: window ends and caps, stress sums, and (flow)
// the per-chain stress of one group of windows
static size_t series_bytes(const dsm_sim* s, int cap) {
  size_t b = (size_t)cap * (2 * sizeof(long long) + 9 * sizeof(double));
  if (s->flow) b = (b + 255) / 256 * 256 + (size_t)std::min(cap, kSeriesGroup) * s->P.n_chains * 8 * sizeof(float);
  return b;
}
static void series_free(dsm_sim* s) {
  for (auto& g : s->ser_graphs) cudaGraphExecDestroy(g.second);
  s->ser_graphs.clear();
  if (s->ser_d) cudaFreeAsync(s->ser_d, s->st);
  if (s->ser_h) cudaFreeHost(s->ser_h);
  s->h.win_stress = nullptr;
  s->ser_d = nullptr;
  s->ser_h = nullptr;
  s->ser_cap = 0;
}

static long long* ser_win_h(dsm_sim* s) { return (long long*)s->ser_h; }
static double* ser_out_h(dsm_sim* s) { return (double*)((char*)s->ser_h + (size_t)s->ser_cap * 2 * sizeof(long long)); }

// The work of n windows on s->st: window ends in, per window (equilibrium) or
// per group of windows (flow) the step launch(es), sums and counters out.
// Captured into a graph, or (capturing = false) issued directly.
static int series_enqueue(dsm_sim* s, int n, bool capturing) {
  const size_t win_bytes = (size_t)s->ser_cap * 2 * sizeof(long long);
  long long* d_win = (long long*)s->ser_d;
  double* d_out = (double*)((char*)s->ser_d + win_bytes);
  int rc = DSM_OK;
  auto cap = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && rc == DSM_OK) rc = fail(s, DSM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  // timing events inside a capture must be real event-record nodes (a plain
  // record there only orders streams)
  auto record = [&](cudaEvent_t ev) {
    cap(capturing ? cudaEventRecordWithFlags(ev, s->st, cudaEventRecordExternal) : cudaEventRecord(ev, s->st), "event");
  };
  cap(cudaMemcpyAsync(d_win, s->ser_h, win_bytes, cudaMemcpyHostToDevice, s->st), "series window copy");
  cap(cudaMemsetAsync(s->d_status, 0, sizeof(int), s->st), "memset");
  cap(cudaMemsetAsync(s->d_counters, 0, 4 * sizeof(unsigned long long), s->st), "memset");
  record(s->ev0);
  if (s->flow) {
    for (int w0 = 0; w0 < n && rc == DSM_OK; w0 += kSeriesGroup) {
      const int k = std::min(kSeriesGroup, n - w0);
      cap(launch_series_begin(s->d_ens, d_win + w0, s->ser_cap, k, s->P.n_chains, s->d_cs, s->st), "series begin");
      if (rc == DSM_OK) rc = enqueue_step(s);
      if (rc == DSM_OK) cap(launch_series_reduce(s->d_ens, d_out + 9 * w0, k, s->st), "stress");
    }
  } else {
    for (int w = 0; w < n && rc == DSM_OK; ++w) {
      cap(launch_window_begin(s->d_ens, d_win, s->ser_cap, w, s->st), "window begin");
      if (rc == DSM_OK) rc = enqueue_step(s);
    }
  }
  record(s->ev1);
  cap(cudaMemcpyAsync(ser_out_h(s), d_out, (size_t)n * 9 * sizeof(double), cudaMemcpyDeviceToHost, s->st), "copy");
  cap(cudaMemcpyAsync(s->hw->cnt, s->d_counters, sizeof(s->hw->cnt), cudaMemcpyDeviceToHost, s->st), "copy");
  cap(cudaMemcpyAsync(&s->hw->status, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, s->st), "copy");
  return rc;
}

static int series_capture(dsm_sim* s, int n, cudaGraphExec_t* exec) {
  CK(cudaStreamSynchronize(s->st));
  CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
  const int rc = series_enqueue(s, n, true);
  cudaGraph_t g = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(s->st, &g);
  if (rc != DSM_OK) { if (g) cudaGraphDestroy(g); return rc; }
  CK(ee);
  const cudaError_t ie = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  CK(ie);
  return DSM_OK;
}

// Graph for n windows with buffers for at least n; recaptured when the launch
// schedule changed
static int series_prepare(dsm_sim* s, int n, cudaGraphExec_t* exec) {
  if (s->ser_version != s->sched_version || n > s->ser_cap) {
    int cap = std::max(n, s->ser_cap);
    if (s->ser_version == s->sched_version || cap < 16) cap = std::max(cap, 16);
    series_free(s);
    const size_t hbytes = (size_t)cap * (2 * sizeof(long long) + 9 * sizeof(double));
    CK(cudaMallocAsync(&s->ser_d, series_bytes(s, cap), s->st));
    CK(cudaHostAlloc(&s->ser_h, hbytes, cudaHostAllocDefault));
    s->ser_cap = cap;
    if (s->flow) s->h.win_stress = (float*)((char*)s->ser_d + (hbytes + 255) / 256 * 256);
    s->ser_version = s->sched_version;
  }
  if (!exec) return DSM_OK;  // buffers only (windows issued directly)
  for (auto& g : s->ser_graphs)
    if (g.first == n) { *exec = g.second; return DSM_OK; }
  cudaGraphExec_t e = nullptr;
  const int rc = series_capture(s, n, &e);
  if (rc != DSM_OK) return rc;
  s->ser_graphs.push_back({n, e});
  *exec = e;
  return DSM_OK;
}

// Enqueue windows ending at ends[0..n) (ascending, after the current time)
static int series_start(dsm_sim* s, const double* ends, int n) {
  double t_prev = s->t_done;
  for (int w = 0; w < n; ++w) {
    if (!(ends[w] >= t_prev) || ends[w] * TICKS >= 9.0e18)
      return fail(s, DSM_ERR_INVALID, "series end times must ascend from the current time");
    t_prev = ends[w];
  }
  // size classes: the windows (flow: the groups of windows) are issued
  // directly.  Replayed from one graph, every window after the first ran
  // 10-20 % slower on the 262144-chain log-normal melt (a graph of one window
  // did not), while a few launches per window cost nothing next to windows of
  // seconds.
  const bool direct = !s->classes.empty();
  cudaGraphExec_t exec = nullptr;
  int rc = series_prepare(s, n, direct ? nullptr : &exec);
  if (rc != DSM_OK) return rc;
  long long* h_win = ser_win_h(s);
  t_prev = s->t_done;
  for (int w = 0; w < n; ++w) {
    h_win[w] = (long long)std::llrint(ends[w] * TICKS);  // as dsm_advance(ends[w])
    h_win[s->ser_cap + w] = (long long)window_watchdog(s, ends[w] - t_prev);
    t_prev = ends[w];
  }
  s->t_window = t_prev;
  s->ser_n = n;
  EnsDev& E = s->h;
  E.step_limit = INT64_MAX;
  CK(cudaMemcpyAsync(s->d_ens, &E, sizeof(EnsDev), cudaMemcpyHostToDevice, s->st));
  if (direct) {
    rc = series_enqueue(s, n, false);
    if (rc != DSM_OK) return rc;
  } else {
    CK(cudaGraphLaunch(exec, s->st));
  }
  CK(cudaEventRecord(s->ev_done, s->st));
  return DSM_OK;
}

static void stress_out(const double* r, dsm_stress_plus* o) {
  const double d = r[8] > 0 ? r[8] : 1.0;
  o->xx = (float)(r[0] / d); o->yy = (float)(r[1] / d); o->zz = (float)(r[2] / d);
  o->xy = (float)(r[3] / d); o->yz = (float)(r[4] / d); o->zx = (float)(r[5] / d);
  o->Lpp = (float)(r[6] / d); o->Z = (float)(r[7] / d);
}

static int series_collect(dsm_sim* s, dsm_stress_plus* out, uint64_t* events) {
  CK(cudaGetLastError());
  const int n = s->ser_n;
  const double* h_out = ser_out_h(s);
  const unsigned long long ev = s->hw->cnt[0];
  if (events) *events = ev;
  s->events_total += ev;
  s->last_events = ev;
  s->t_done = s->t_window;
  CK(cudaEventElapsedTime(&s->last_kernel_ms, s->ev0, s->ev1));
  if (s->flow) {
    for (int q = 0; q < 9; ++q) s->hw->red[q] = h_out[9 * (n - 1) + q];
    if (out) for (int w = 0; w < n; ++w) stress_out(h_out + 9 * w, &out[w]);
  }
  if (s->hw->status & 1) return DSM_ABORTED;
  return DSM_OK;
}

// wait for the pending work of s, forwarding the caller's abort flag
static int wait_pending(dsm_sim* s, const volatile int32_t* abort_flag) {
  if (abort_flag) {
    while (cudaEventQuery(s->ev_done) == cudaErrorNotReady) {
      if (*abort_flag) *s->h_abort = 1;
      std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
  }
  CK(cudaEventSynchronize(s->ev_done));
  return DSM_OK;
}

static std::vector<double> series_ends(const dsm_sim* s, double dt, int n) {
  std::vector<double> e(n);
  for (int w = 0; w < n; ++w) e[w] = s->t_done + dt * (w + 1);  // as dsm_advance(t + dt*(w+1))
  return e;
}

extern "C" int dsm_advance_series(dsm_sim* s, double dt, int32_t n, const volatile int32_t* abort_flag,
                                  dsm_stress_plus* out, uint64_t* events) {
  const dsm::NvtxRange nvtx_range("dsm_advance_series");
  if (!s || !s->ready || n < 1 || !(dt > 0.0) || s->pending) return DSM_ERR_INVALID;
  *s->h_abort = (abort_flag && *abort_flag) ? 1 : 0;
  const std::vector<double> e = series_ends(s, dt, n);
  int rc = series_start(s, e.data(), n);
  if (rc == DSM_OK) rc = wait_pending(s, abort_flag);
  if (rc == DSM_OK) rc = series_collect(s, out, events);
  *s->h_abort = 0;
  return rc;
}

// ------------------------------------------------------------------ asynchronous form
extern "C" int dsm_advance_start(dsm_sim* s, double t_end, int64_t step_limit) {
  const dsm::NvtxRange nvtx_range("dsm_advance_start");
  if (!s || !s->ready || s->pending) return DSM_ERR_INVALID;
  if (!(t_end >= 0.0) || t_end * TICKS >= 9.0e18) return fail(s, DSM_ERR_INVALID, "t_end out of range");
  *s->h_abort = 0;
  int rc = sim_launch_window(s, t_end, step_limit);
  if (rc == DSM_OK) rc = enqueue_readback(s);
  if (rc == DSM_OK) s->pending = 1;
  return rc;
}

extern "C" int dsm_series_start(dsm_sim* s, const double* t_ends, int32_t n) {
  const dsm::NvtxRange nvtx_range("dsm_series_start");
  if (!s || !s->ready || !t_ends || n < 1 || s->pending) return DSM_ERR_INVALID;
  *s->h_abort = 0;
  const int rc = series_start(s, t_ends, n);
  if (rc == DSM_OK) s->pending = 2;
  return rc;
}

extern "C" int dsm_poll(dsm_sim* s, uint64_t* events, dsm_stress_plus* out, int32_t* n_out) {
  if (!s || !s->ready || !s->pending) return DSM_ERR_INVALID;
  const cudaError_t q = cudaEventQuery(s->ev_done);
  if (q == cudaErrorNotReady) return DSM_PENDING;
  CK(q);
  const int kind = s->pending;
  s->pending = 0;
  if (kind == 2) {
    if (n_out) *n_out = s->ser_n;
    return series_collect(s, out, events);
  }
  const int rc = window_collect(s, events);
  if (n_out) *n_out = s->flow ? 1 : 0;
  if (out && s->flow) stress_out(s->hw->red, out);
  return rc;
}

extern "C" int dsm_set_priority(dsm_sim* s, int32_t priority) {
  if (!s || !s->ready || s->pending) return DSM_ERR_INVALID;
  int lo = 0, hi = 0;
  CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  const int pr = std::max(hi, std::min(lo, (int)priority));
  if (pr == s->prio) return DSM_OK;
  // the handle is idle: everything enqueued so far has completed or is ordered
  // before the new streams' work by the synchronisation below
  CK(cudaStreamSynchronize(s->st));
  if (s->side) CK(cudaStreamSynchronize(s->side));
  if (s->side2) CK(cudaStreamSynchronize(s->side2));
  if (s->side3) CK(cudaStreamSynchronize(s->side3));
  cudaStream_t st = nullptr, side = nullptr, side2 = nullptr, side3 = nullptr;
  CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, pr));
  if (s->side) CK(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, pr));
  if (s->side2) CK(cudaStreamCreateWithPriority(&side2, cudaStreamNonBlocking, pr));
  if (s->side3) CK(cudaStreamCreateWithPriority(&side3, cudaStreamNonBlocking, pr));
  cudaStreamDestroy(s->st);
  s->st = st;
  if (s->side) { cudaStreamDestroy(s->side); s->side = side; }
  if (s->side2) { cudaStreamDestroy(s->side2); s->side2 = side2; }
  if (s->side3) { cudaStreamDestroy(s->side3); s->side3 = side3; }
  s->prio = pr;
  return DSM_OK;
}

extern "C" int dsm_abort(dsm_sim* s) {
  if (!s || !s->ready) return DSM_ERR_INVALID;
  *s->h_abort = 1;
  return DSM_OK;
}

// End of a window on s->st: counters, status and (flow) the stress sums into
// pinned memory, then the done event
static int enqueue_readback(dsm_sim* s) {
  CK(cudaMemcpyAsync(s->hw->cnt, s->d_counters, sizeof(s->hw->cnt), cudaMemcpyDeviceToHost, s->st));
  CK(cudaMemcpyAsync(&s->hw->status, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, s->st));
  if (s->flow) {
    CK(launch_stress_reduce_dev(s->d_ens, s->d_red, s->st));
    CK(cudaMemcpyAsync(s->hw->red, s->d_red, 9 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  }
  CK(cudaEventRecord(s->ev_done, s->st));
  return DSM_OK;
}

// Host bookkeeping of a completed window (its readback has landed)
static int window_collect(dsm_sim* s, uint64_t* events) {
  CK(cudaGetLastError());
  const unsigned long long* cnt = s->hw->cnt;
  const int status = s->hw->status;
  if (events) *events = cnt[0];
  s->events_total += cnt[0];
  s->t_done = std::max(s->t_done, s->t_window);
  s->last_events = cnt[0];
  CK(cudaEventElapsedTime(&s->last_kernel_ms, s->ev0, s->ev1));
  if (status & 1) return DSM_ABORTED;
  return DSM_OK;
}

int dsm::sim_finish_window(dsm_sim* s, uint64_t* events) {
  const int rc = enqueue_readback(s);
  if (rc != DSM_OK) return rc;
  CK(cudaStreamSynchronize(s->st));
  return window_collect(s, events);
}

extern "C" int dsm_advance(dsm_sim* s, double t_end, int64_t step_limit, const volatile int32_t* abort_flag,
                           uint64_t* events) {
  const dsm::NvtxRange nvtx_range("dsm_advance");
  if (!s || !s->ready) return DSM_ERR_INVALID;
  if (!(t_end >= 0.0) || t_end * TICKS >= 9.0e18) return fail(s, DSM_ERR_INVALID, "t_end out of range");
  *s->h_abort = (abort_flag && *abort_flag) ? 1 : 0;
  if (s->pending) return fail(s, DSM_ERR_INVALID, "an asynchronous advance is pending (dsm_poll it first)");
  int rc = sim_launch_window(s, t_end, step_limit);
  if (rc == DSM_OK) rc = enqueue_readback(s);
  // forward the caller's flag into the mapped word the kernel polls
  if (rc == DSM_OK) rc = wait_pending(s, abort_flag);
  if (rc == DSM_OK) rc = window_collect(s, events);
  *s->h_abort = 0;
  return rc;
}

extern "C" int dsm_stress(dsm_sim* s, dsm_stress_plus* out, int32_t* count) {
  if (!s || !s->ready || !out) return DSM_ERR_INVALID;
  if (!s->flow) {
    // equilibrium ensembles keep no per-chain stress: evaluate it from the
    // current state, with the sums and the reduction of a flow window end
    // (the per-chain buffer the flow kernel writes is free here)
    if (s->pending) return fail(s, DSM_ERR_INVALID, "asynchronous work pending");
    CK(launch_state_stress(s->d_ens, s->P.n_chains, s->d_stress, s->d_red, s->st));
    CK(cudaMemcpyAsync(s->hw->red, s->d_red, 9 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  }
  // sums of the last window end, copied back with its counters
  CK(cudaStreamSynchronize(s->st));
  const double* r = s->hw->red;
  const double c = r[8];
  const double d = c > 0 ? c : 1.0;
  out->xx = (float)(r[0] / d); out->yy = (float)(r[1] / d); out->zz = (float)(r[2] / d);
  out->xy = (float)(r[3] / d); out->yz = (float)(r[4] / d); out->zx = (float)(r[5] / d);
  out->Lpp = (float)(r[6] / d); out->Z = (float)(r[7] / d);
  if (count) *count = (int32_t)c;
  return DSM_OK;
}

extern "C" int dsm_gt_raw(dsm_sim* s, double* gsum, int64_t* count) {
  const dsm::NvtxRange nvtx_range("dsm_gt_raw");
  if (!s || !s->ready) return DSM_ERR_INVALID;
  if (!s->corr) return fail(s, DSM_ERR_INVALID, "no correlator in this simulation (eq_type != 1 or flow)");
  const size_t m = (size_t)s->levels * s->cp;
  CK(launch_gt_reduce_dev(s->d_ens, s->levels, s->cp, s->d_gsum, s->d_gcnt, s->st));
  std::vector<long long> c(m);
  if (gsum) CK(cudaMemcpyAsync(gsum, s->d_gsum, m * sizeof(double), cudaMemcpyDeviceToHost, s->st));
  CK(cudaMemcpyAsync(c.data(), s->d_gcnt, m * sizeof(long long), cudaMemcpyDeviceToHost, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (count) for (size_t i = 0; i < m; ++i) count[i] = c[i];
  return DSM_OK;
}

// G(t) (or MSD(t)) points in the order and count gpu_Gt_PCS writes them
// (ensemble.cu:298-335, correlator.cu:242-257)
extern "C" int dsm_gt(dsm_sim* s, float* t, float* G, int32_t* n) {
  const dsm::NvtxRange nvtx_range("dsm_gt");
  if (!s || !n) return DSM_ERR_INVALID;
  const int L = s->levels, p = s->cp, m = s->cm, dmin = p / m;
  std::vector<double> gs((size_t)L * p);
  int rc = dsm_gt_raw(s, gs.data(), nullptr);
  if (rc) return rc;
  const double res = s->P.sync_dt;
  const long long np = p + (long long)(L - 1) * (p - dmin);
  long long actual = np - p + (long long)std::floor(s->P.t_end / (res * std::pow((double)m, L - 1)));
  if (actual > np) actual = np;
  if (actual < 0) actual = 0;
  if (*n < actual) { *n = (int32_t)actual; return fail(s, DSM_ERR_INVALID, "output capacity too small"); }
  long long im = 0;
  // G(t): mean of the three shear components per chain (correlator.cu:172);
  // MSD(t): |dr|^2 summed over the components (correlator.cu:173)
  const double inv = 1.0 / ((s->msd ? 1.0 : 3.0) * s->P.n_chains);
  for (int k = 0; k < L && im < actual; ++k)
    for (int j = (k == 0 ? 0 : dmin); j < p && im < actual; ++j) {
      if (t) t[im] = (float)(long long)((double)j * std::pow((double)m, k));
      if (G) G[im] = (float)(gs[(size_t)k * p + j] * inv);
      ++im;
    }
  *n = (int32_t)im;
  return DSM_OK;
}

// ------------------------------------------------------------------ reference files
extern "C" int dsm_save_file(dsm_sim* s, const char* path) {
  if (!s || !path) return DSM_ERR_INVALID;
  const size_t n = s->P.n_chains, cap = s->cap;
  std::vector<dsm_chain_head> h(n);
  std::vector<dsm_float4> q(n * cap);
  std::vector<float> t(n * cap);
  int rc = dsm_get_chains(s, h.data(), q.data(), t.data());
  if (rc) return rc;
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(s, DSM_ERR_INVALID, std::string("cannot open ") + path);
  const int32_t nc = (int32_t)n;
  f.write((const char*)&nc, 4);  // ensemble.cu:346
  for (size_t i = 0; i < n; ++i) {  // chain.cu:304-310
    f.write((const char*)&h[i], sizeof(dsm_chain_head));
    f.write((const char*)&q[i * cap], (std::streamsize)(sizeof(dsm_float4) * h[i].Z));
    f.write((const char*)&t[i * cap], (std::streamsize)(sizeof(float) * h[i].Z));
  }
  return f ? DSM_OK : fail(s, DSM_ERR_INVALID, "write failed");
}

extern "C" int dsm_load_file(dsm_sim* s, const char* path) {
  if (!s || !path) return DSM_ERR_INVALID;
  const size_t n = s->P.n_chains, cap = s->cap;
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(s, DSM_ERR_INVALID, std::string("cannot open ") + path);
  int32_t nc = 0;
  f.read((char*)&nc, 4);
  if (nc != (int32_t)n) return fail(s, DSM_ERR_INVALID, "ensemble size mismatch");  // ensemble.cu:493-496
  std::vector<dsm_chain_head> h(n);
  std::vector<dsm_float4> q(n * cap, dsm_float4{0, 0, 0, 0});
  std::vector<float> t(n * cap, 0.f);
  for (size_t i = 0; i < n; ++i) {  // chain.cu:312-318
    f.read((char*)&h[i], sizeof(dsm_chain_head));
    if (!f || h[i].Z < 1 || h[i].Z > (int)cap) return fail(s, DSM_ERR_INVALID, "corrupt conformation file");
    f.read((char*)&q[i * cap], (std::streamsize)(sizeof(dsm_float4) * h[i].Z));
    f.read((char*)&t[i * cap], (std::streamsize)(sizeof(float) * h[i].Z));
    if (!f) return fail(s, DSM_ERR_INVALID, "truncated conformation file");
  }
  return dsm_set_chains(s, h.data(), q.data(), t.data());
}

extern "C" int dsm_last_window(const dsm_sim* s, float* kernel_ms, uint64_t* events, int32_t* grid,
                               int32_t* blocks_per_sm) {
  if (!s) return DSM_ERR_INVALID;
  if (kernel_ms) *kernel_ms = s->last_kernel_ms;
  if (events) *events = s->last_events;
  if (grid) *grid = s->grid;
  if (blocks_per_sm) *blocks_per_sm = s->blocks_per_sm;
  return DSM_OK;
}

// ------------------------------------------------------------------ batched windows
// Advance several ensembles in one persistent launch per kind (equilibrium /
// equilibrium+G(t) / flow): the work items of all ensembles of a kind form one
// index space (prefix sums of chain counts) that the warps pull from, so short
// and long ensembles share the GPU without a launch per ensemble.  The
// shared-memory slot is sized for the largest z_max of the kind.
extern "C" int dsm_advance_batch(dsm_sim** sims, int32_t n, const double* t_end, const int64_t* step_limit,
                                 uint64_t* events) {
  const dsm::NvtxRange nvtx_range("dsm_advance_batch");
  if (!sims || n < 1 || !t_end) return DSM_ERR_INVALID;
  dsm_sim* s = sims[0];
  if (!s || !s->ready) return DSM_ERR_INVALID;
  for (int i = 0; i < n; ++i) {
    if (!sims[i] || !sims[i]->ready) return DSM_ERR_INVALID;
    if (sims[i]->pending) return fail(s, DSM_ERR_INVALID, "an ensemble of the batch has asynchronous work pending");
    if (sims[i]->P.device != s->P.device) return fail(s, DSM_ERR_INVALID, "batch spans devices");
    if (!(t_end[i] >= 0.0) || t_end[i] * TICKS >= 9.0e18) return fail(s, DSM_ERR_INVALID, "t_end out of range");
    for (int k = 0; k < i; ++k)
      if (sims[k] == sims[i]) return fail(s, DSM_ERR_INVALID, "ensemble listed twice in a batch");
  }
  CK(cudaSetDevice(s->P.device));
  // one launch per kind and shared-memory size class (slot capacity rounded
  // up to a power of two, correlator p, lanes per chain): ensembles of very
  // different chain lengths then do not share the largest one's slot size
  struct Group {
    std::vector<int> idx;
    bool flow;
    int corr;  // correlator kind (0 none, 1 stress, 2 MSD)
    int cap_class, cp, lanes;
  };
  auto cap_class = [](int cap) { int c = 16; while (c < cap) c <<= 1; return c; };
  std::vector<Group> groups;
  for (int i = 0; i < n; ++i) {
    const bool fl = sims[i]->flow;
    const int co = sims[i]->ck;
    const int cc = cap_class(sims[i]->cap), cp = co ? sims[i]->cp : 0, ln = sims[i]->cfg.lanes;
    Group* g = nullptr;
    for (auto& x : groups)
      if (x.flow == fl && x.corr == co && x.cap_class == cc && x.cp == cp && x.lanes == ln) g = &x;
    if (!g) { groups.push_back(Group{{}, fl, co, cc, cp, ln}); g = &groups.back(); }
    g->idx.push_back(i);
  }
  // windows of every ensemble (same bookkeeping as dsm_advance)
  for (int i = 0; i < n; ++i) {
    dsm_sim* q = sims[i];
    EnsDev& E = q->h;
    const double te = t_end[i];
    const int64_t sl = step_limit ? step_limit[i] : -1;
    E.t_end_ticks = (int64_t)std::llrint(te * TICKS);
    q->t_window = te;
    E.step_limit = sl < 0 ? INT64_MAX : sl;
    const double expect = 0.25 * (double)q->nkmax * std::max(0.0, te - q->t_done) * 100.0;
    const double wd = std::max(16777216.0, std::min(expect, 9.0e18));
    E.watchdog_events = q->watchdog_events > 0 ? q->watchdog_events : (int64_t)wd;
    CK(cudaMemcpyAsync(q->d_ens, &E, sizeof(EnsDev), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemsetAsync(q->d_counters, 0, 4 * sizeof(unsigned long long), s->st));
  }
  // groups run concurrently, each on the stream of its first ensemble, after
  // the descriptor copies on s->st; s->st then waits for all of them.  Every
  // exit of enqueue(), an error included, passes through the clean-up below:
  // events destroyed, stream-ordered temporaries released once nothing that
  // reads them can still run.
  std::vector<void*> tmp;
  std::vector<cudaStream_t> used;
  cudaEvent_t ready = nullptr;
  std::vector<cudaEvent_t> joins;
  const bool fan = groups.size() > 1;
  auto enqueue = [&]() -> int {
    if (fan) {
      CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
      CK(cudaEventRecord(ready, s->st));
    }
    for (auto& g : groups) {
      const int k = (int)g.idx.size();
      std::vector<EnsDev> hE(k);
      std::vector<long long> pre(k + 1, 0);
      LaunchCfg cfg{4, 0, 0, g.lanes};
      cudaStream_t gs = fan ? sims[g.idx[0]]->st : s->st;
      for (int q = 0; q < k; ++q) {
        dsm_sim* x = sims[g.idx[q]];
        hE[q] = x->h;
        pre[q + 1] = pre[q] + x->P.n_chains;
        cfg.slot_cap = std::max(cfg.slot_cap, x->cap);
        if (g.corr) cfg.pmax = std::max(cfg.pmax, x->cp);
      }
      EnsDev* dE = nullptr;
      long long* dP = nullptr;
      unsigned int* dW = nullptr;
      CK(cudaMallocAsync((void**)&dE, sizeof(EnsDev) * k, s->st));
      tmp.push_back(dE);
      CK(cudaMallocAsync((void**)&dP, sizeof(long long) * (k + 1) + 16, s->st));
      tmp.push_back(dP);
      dW = (unsigned int*)(dP + k + 1);
      CK(cudaMemcpyAsync(dE, hE.data(), sizeof(EnsDev) * k, cudaMemcpyHostToDevice, s->st));
      CK(cudaMemcpyAsync(dP, pre.data(), sizeof(long long) * (k + 1), cudaMemcpyHostToDevice, s->st));
      CK(cudaMemsetAsync(dW, 0, 16, s->st));
      int optin = 0;
      CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->P.device));
      // when every ensemble of the group planned a small-slot class (its own
      // schedule), the group runs in the smallest of those slots and the chains
      // that outgrow it finish in an overflow launch with slots of the group's
      // largest capacity, as in dsm_advance; otherwise one launch with slots of
      // that capacity
      bool all_small = true;
      int small = cfg.slot_cap;
      for (int q = 0; q < k && all_small; ++q) {
        const dsm_sim* x = sims[g.idx[q]];
        // the small class is the last of an ensemble's classes
        all_small = !x->classes.empty() && x->classes.back().cfg.lanes == g.lanes;
        if (all_small) small = std::min(small, x->classes.back().cfg.slot_cap);
      }
      const bool overflow = all_small && small < cfg.slot_cap;
      LaunchCfg run = cfg;
      if (overflow) run.slot_cap = small;
      fit_block(run, optin);
      const int bps = step_max_blocks_per_sm(g.flow, g.corr, run);
      if (bps < 1) return fail(s, DSM_ERR_INVALID, "batch slot does not fit shared memory");
      const int tiles = run.warps_per_block * 32 / run.lanes;
      const long long want = (pre[k] + tiles - 1) / tiles;
      const int grid = (int)std::min<long long>(want, (long long)bps * s->sm_count);
      StepList lst;
      LaunchCfg oc{1, cfg.slot_cap, cfg.pmax, 32};
      int ogrid = 0;
      if (overflow) {
        const int obps = step_max_blocks_per_sm(g.flow, g.corr, oc);
        if (obps < 1) return fail(s, DSM_ERR_INVALID, "batch capacity does not fit one shared-memory slot");
        ogrid = obps * s->sm_count;
        int* dDef = nullptr;
        CK(cudaMallocAsync((void**)&dDef, sizeof(int) * (size_t)pre[k], s->st));
        tmp.push_back(dDef);
        lst.defer = dDef;
        lst.n_defer = dW + 2;
      }
      if (fan) {
        CK(cudaEventRecord(ready, s->st));
        CK(cudaStreamWaitEvent(gs, ready, 0));
      }
      used.push_back(gs);
      CK(launch_step(dE, k, dP, pre[k], dW, g.flow, g.corr, run, nullptr, (int*)(dW + 1), grid, gs, lst));
      if (overflow) {
        StepList ol;
        ol.order = lst.defer;
        ol.dyn_total = dW + 2;
        CK(launch_step(dE, k, dP, 0, dW + 3, g.flow, g.corr, oc, nullptr, (int*)(dW + 1), ogrid, gs, ol));
      }
      if (fan) {
        cudaEvent_t j = nullptr;
        CK(cudaEventCreateWithFlags(&j, cudaEventDisableTiming));
        joins.push_back(j);
        CK(cudaEventRecord(j, gs));
      }
    }
    for (cudaEvent_t j : joins) CK(cudaStreamWaitEvent(s->st, j, 0));
    for (int i = 0; i < n; ++i) {
      dsm_sim* q = sims[i];
      if (q->flow) {
        CK(launch_stress_reduce_dev(q->d_ens, q->d_red, s->st));
        CK(cudaMemcpyAsync(q->hw->red, q->d_red, 9 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
      }
      CK(cudaMemcpyAsync(q->hw->cnt, q->d_counters, sizeof(q->hw->cnt), cudaMemcpyDeviceToHost, s->st));
    }
    return DSM_OK;
  };
  const int rc = enqueue();
  // on an error the side streams may still run launches that read the
  // temporaries without s->st waiting for them: wait for each first
  if (rc != DSM_OK)
    for (cudaStream_t u : used) cudaStreamSynchronize(u);
  for (cudaEvent_t j : joins) cudaEventDestroy(j);
  if (ready) cudaEventDestroy(ready);
  for (void* p : tmp) cudaFreeAsync(p, s->st);
  const cudaError_t sync_err = cudaStreamSynchronize(s->st);
  if (rc != DSM_OK) return rc;
  if (sync_err != cudaSuccess)
    return fail(s, DSM_ERR_CUDA, std::string("dsm_advance_batch: ") + cudaGetErrorString(sync_err));
  CK(cudaGetLastError());
  for (int i = 0; i < n; ++i) {
    const unsigned long long* cnt = sims[i]->hw->cnt;
    if (events) events[i] = cnt[0];
    sims[i]->events_total += cnt[0];
    sims[i]->last_events = cnt[0];
    sims[i]->t_done = std::max(sims[i]->t_done, sims[i]->t_window);
  }
  return DSM_OK;
}
