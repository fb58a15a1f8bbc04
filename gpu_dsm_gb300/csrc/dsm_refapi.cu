// The reference's C++ entry points (include/dsm_reference.h) on top of the
// handle API: the ensemble.h functions over one process-global device
// ensemble (common/ensemble.cu:106-539), the ensemble_call_block.h functions
// over a block that owns a device ensemble (common/ensemble_call_block.cu:55-565),
// the reference's globals, and main_cuda with C++ linkage (GUI/main.cpp:22).
#include "../../include/dsm_reference.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iostream>
#include <thread>
#include <vector>

#include "dsm_compat.h"

// ---------------------------------------------------------------- globals
// common/ensemble.cu:50-76, common/main_cuda.cu (Be, CD_flag), common/job_ID.h:30
sstrentp chains = {nullptr, nullptr, nullptr};
chain_head* chain_heads = nullptr;
double universal_time = 0.0;
int N_cha = 0;
int NK = 0;
int z_max = 0;
bool dbug = false;
float kxx = 0.0f, kxy = 0.0f, kxz = 0.0f, kyx = 0.0f, kyy = 0.0f, kyz = 0.0f, kzx = 0.0f, kzy = 0.0f, kzz = 0.0f;
bool PD_flag = false;
float Be = 1.0f;
int CD_flag = 1;
int job_ID = 0;
int dsm_correlator_res = 1;

static_assert(sizeof(chain_head) == sizeof(dsm_chain_head), "chain_head layout");
static_assert(sizeof(stress_plus) == sizeof(dsm_stress_plus), "stress_plus layout");

namespace {

constexpr int kChainsPerCall = 5000;  // common/ensemble.cu:47

struct Global {
  dsm_sim* sim = nullptr;
  uint64_t seed = 0;
  int levels = 0;             // s of gpu_init (main_cuda.cu:70)
  bool draw_on_init = false;  // host_chains_init: gpu_init draws the chains
  int corr_type = -1, corr_res = 0;
  double corr_len = 0.0;
};
Global G;

stress_plus to_ref(const dsm_stress_plus& s) {
  stress_plus r;
  std::memcpy(&r, &s, sizeof(r));
  return r;
}

// dsm_params from the reference's globals; polydisp.dat as chains_malloc /
// main_cuda read it (main_cuda.cu:95-103)
dsm_params params_from_globals(int n, uint32_t offset, uint64_t seed, int eq_type, double sync_dt, double t_end,
                               int levels) {
  dsm_params p;
  std::memset(&p, 0, sizeof(p));
  p.beta = Be;
  p.nk = NK;
  p.n_chains = n;
  const float k[9] = {kxx, kxy, kxz, kyx, kyy, kyz, kzx, kzy, kzz};
  for (int q = 0; q < 9; ++q) p.kappa[q] = k[q];
  p.cd_flag = CD_flag;
  p.pd_flag = PD_flag ? 1 : 0;
  p.eq_type = eq_type;
  p.sync_dt = sync_dt;
  p.t_end = t_end;
  p.seed = seed;
  p.z_max = z_max > 0 ? z_max : NK;
  p.corr_levels = levels;
  p.chain_offset = offset;
  if (PD_flag) {
    std::ifstream pf("polydisp.dat");
    pf >> p.gex_a >> p.gex_b >> p.gex_mp >> p.gex_mk;
  }
  return p;
}

int make_sim(const dsm_params& p, dsm_sim** out) {
  dsm_sim* s = nullptr;
  const int rc = dsm_create(&p, &s);
  if (rc != DSM_OK) {
    std::cout << "device ensemble setup failed: " << dsm_last_error(s) << "\n";
    dsm_destroy(s);
    *out = nullptr;
    return rc;
  }
  *out = s;
  return DSM_OK;
}

// conformations between a device ensemble and the reference's host layout
int upload(dsm_sim* s, const chain_head* heads, const sstrentp& c) {
  return dsm_set_chains(s, reinterpret_cast<const dsm_chain_head*>(heads), c.QN, c.tau_CD);
}
int download(dsm_sim* s, int n, chain_head* heads, const sstrentp& c) {
  int rc = dsm_get_chains(s, reinterpret_cast<dsm_chain_head*>(heads), c.QN, c.tau_CD);
  if (rc == DSM_OK && c.R1) {
    std::vector<float> r(3 * (size_t)n);
    if (dsm_get_r1(s, r.data()) == DSM_OK)
      for (int i = 0; i < n; ++i) c.R1[i] = dsm_float4{r[3 * i], r[3 * i + 1], r[3 * i + 2], 0.0f};
  }
  return rc;
}

// advance to t, polling the caller's run_flag as the reference's step loops do
// (ensemble_call_block.cu:214,353): -1 once it is cleared
int advance_polling(dsm_sim* s, double t, bool* run_flag) {
  if (run_flag && !*run_flag) return DSM_ABORTED;
  int rc = dsm_advance_start(s, t, -1);
  while (rc == DSM_OK) {
    rc = dsm_poll(s, nullptr, nullptr, nullptr);
    if (rc != DSM_PENDING) break;
    rc = DSM_OK;
    if (run_flag && !*run_flag) dsm_abort(s);
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
  return rc;
}

// the offset of a block's chains in the global arrays, when they lie there
uint32_t global_offset(const sstrentp& c) {
  const int zc = z_max > 0 ? z_max : NK;
  if (chains.QN && c.QN >= chains.QN && c.QN < chains.QN + (size_t)N_cha * zc)
    return (uint32_t)((c.QN - chains.QN) / zc);
  return 0;
}

void free_host() {
  delete[] chains.QN;
  delete[] chains.tau_CD;
  delete[] chains.R1;
  delete[] chain_heads;
  chains = sstrentp{nullptr, nullptr, nullptr};
  chain_heads = nullptr;
}

// common/ensemble.cu:95-104
void chains_malloc() {
  free_host();
  z_max = NK;
  chain_heads = new chain_head[N_cha];
  chains.QN = new dsm_float4[(size_t)N_cha * z_max];
  chains.tau_CD = new float[(size_t)N_cha * z_max];
  chains.R1 = new dsm_float4[N_cha];
  std::memset(chain_heads, 0, sizeof(chain_head) * N_cha);
  std::memset(chains.QN, 0, sizeof(dsm_float4) * (size_t)N_cha * z_max);
  std::memset(chains.tau_CD, 0, sizeof(float) * (size_t)N_cha * z_max);
  std::memset(chains.R1, 0, sizeof(dsm_float4) * N_cha);
}

// host statistics of the -distr files from the host arrays, as the reference
// computes them (ensemble.cu:356-484)
void host_histograms(std::vector<uint64_t>* hz, std::vector<uint64_t>* hn, std::vector<float>* q) {
  const int zc = z_max > 0 ? z_max : NK;
  if (hz) hz->assign((size_t)zc + 2, 0);
  if (hn) hn->assign((size_t)NK + 2, 0);
  for (int i = 0; i < N_cha; ++i) {
    const int Z = chain_heads[i].Z;
    if (hz && Z >= 0 && Z < (int)hz->size()) (*hz)[Z]++;
    for (int j = 0; j < Z; ++j) {
      const dsm_float4& s = chains.QN[(size_t)i * zc + j];
      const int n = (int)s.w;
      if (hn && n >= 0 && n < (int)hn->size()) (*hn)[n]++;
      if (q && j > 0 && j < Z - 1) q->push_back(std::sqrt(s.x * s.x + s.y * s.y + s.z * s.z));
    }
  }
  if (q) std::sort(q->begin(), q->end());
}

}  // namespace

// ---------------------------------------------------------------- ensemble.h
sstrentp chain_index(const int i) {  // ensemble.cu:79-85
  const size_t zc = (size_t)(z_max > 0 ? z_max : NK);
  return sstrentp{chains.QN + zc * i, chains.tau_CD + zc * i, chains.R1 + i};
}

// ensemble.cu:87-95 (the reference leaves "+ i" out of its tau_CD pointer)
sstrentp chain_index(const int bi, const int i) { return chain_index(bi * kChainsPerCall + i); }

// ensemble.cu:106-115: the host arrays; the equilibrium chains are drawn on
// the device by gpu_init, keyed by its seed
void host_chains_init(Ran*) {
  chains_malloc();
  universal_time = 0.0;
  G.draw_on_init = true;
}

// ensemble.cu:486-504 (an ensemble-size mismatch leaves the arrays empty,
// which gpu_init then rejects, instead of exit(2))
void load_from_file(char* filename) {
  chains_malloc();
  G.draw_on_init = false;
  std::ifstream file(filename, std::ios::in | std::ios::binary);
  if (!file.is_open()) { std::cout << "file error\n"; return; }
  int ti = 0;
  file.read(reinterpret_cast<char*>(&ti), sizeof(int));
  if (ti != N_cha) { std::cout << "ensemble size mismatch\n"; return; }
  for (int i = 0; i < N_cha; ++i) {
    const sstrentp c = chain_index(i);
    file.read(reinterpret_cast<char*>(&chain_heads[i]), sizeof(chain_head));
    const int Z = std::min(std::max(chain_heads[i].Z, 0), z_max);
    file.read(reinterpret_cast<char*>(c.QN), sizeof(dsm_float4) * Z);
    file.read(reinterpret_cast<char*>(c.tau_CD), sizeof(float) * Z);
  }
}

// ensemble.cu:118-208: the device ensemble of all chains, seeded by `seed`
// (main_cuda passes job_ID); s = correlator levels
void gpu_init(int seed, p_cd*, int s) {
  dsm_destroy(G.sim);
  G.sim = nullptr;
  G.seed = (uint64_t)(uint32_t)seed;
  G.levels = s;
  G.corr_type = -1;
  const dsm_params p = params_from_globals(N_cha, 0, G.seed, 0, 1.0, 0.0, 0);
  if (make_sim(p, &G.sim) != DSM_OK) return;
  const int rc = G.draw_on_init ? dsm_init_equilibrium(G.sim) : upload(G.sim, chain_heads, chains);
  if (rc != DSM_OK) { std::cout << dsm_last_error(G.sim) << "\n"; return; }
  if (G.draw_on_init) download(G.sim, N_cha, chain_heads, chains);
  G.draw_on_init = false;
}

// ensemble.cu:231-236
void get_chains_from_device() {
  if (G.sim) download(G.sim, N_cha, chain_heads, chains);
}

// ensemble.cu:342-354, chain.cu:236-242
void save_to_file(char* filename) {
  std::ofstream file(filename, std::ios::out | std::ios::binary);
  if (!file.is_open()) { std::cout << "file error\n"; return; }
  file.write(reinterpret_cast<const char*>(&N_cha), sizeof(int));
  for (int i = 0; i < N_cha; ++i) {
    const sstrentp c = chain_index(i);
    file.write(reinterpret_cast<const char*>(&chain_heads[i]), sizeof(chain_head));
    file.write(reinterpret_cast<const char*>(c.QN), sizeof(dsm_float4) * chain_heads[i].Z);
    file.write(reinterpret_cast<const char*>(c.tau_CD), sizeof(float) * chain_heads[i].Z);
  }
}

// ensemble.cu:356-484, from the host arrays
void save_Z_distribution_to_file(std::string filename, bool cumulative) {
  std::vector<uint64_t> hz;
  host_histograms(&hz, nullptr, nullptr);
  dsmc::write_Z_distr(filename, hz, N_cha, cumulative);
}
void save_N_distribution_to_file(std::string filename, bool cumulative) {
  std::vector<uint64_t> hn;
  host_histograms(nullptr, &hn, nullptr);
  dsmc::write_N_distr(filename, hn, cumulative);
}
void save_Q_distribution_to_file(std::string filename, bool) {
  std::vector<float> q;
  host_histograms(nullptr, nullptr, &q);
  dsmc::write_Q_distr(filename, q);
}

// ensemble.cu:223-229
int gpu_time_step(double reach_time, bool* run_flag) {
  if (!G.sim) return DSM_ERR_INVALID;
  const int rc = advance_polling(G.sim, reach_time, run_flag);
  if (rc == DSM_ABORTED) return -1;
  if (rc != DSM_OK) { std::cout << dsm_last_error(G.sim) << "\n"; return rc; }
  universal_time = reach_time;
  return 0;
}

// ensemble.cu:289-339: the host conformations go to a device ensemble with
// the correlator of this run (type 0 G(t) of the shear stresses, 1 MSD(t)),
// sampled every res tau_K up to `length`; G[_id].dat / MSD[_id].dat receives
// the same points.  t and x are allocated with new[] and left to the caller
// (the reference deletes them before returning).
int gpu_Gt_PCS(int res, double length, float*& t, float*& x, int s, int correlator_type, bool* run_flag,
               int* progress_bar) {
  if (progress_bar) *progress_bar = 1;
  t = nullptr;
  x = nullptr;
  const dsm_params p = params_from_globals(N_cha, 0, G.seed, correlator_type == 1 ? 2 : 1, (double)res, length, s);
  dsm_sim* sim = nullptr;
  int rc = make_sim(p, &sim);
  if (rc != DSM_OK) return rc;
  rc = upload(sim, chain_heads, chains);
  if (rc != DSM_OK) { std::cout << dsm_last_error(sim) << "\n"; dsm_destroy(sim); return rc; }
  dsm_destroy(G.sim);
  G.sim = sim;
  G.corr_type = correlator_type;
  G.corr_res = res;
  G.corr_len = length;
  for (double tw = 0.0; tw < length;) {  // windows of at most 1e5 (ensemble_call_block.cu:24)
    const double te = std::min(length, tw + 1.0e5);
    rc = advance_polling(sim, te, run_flag);
    if (rc == DSM_ABORTED) return -1;
    if (rc != DSM_OK) { std::cout << dsm_last_error(sim) << "\n"; return rc; }
    tw = te;
    if (progress_bar) *progress_bar = (int)(100.0 * tw / length);
  }
  int32_t levels = 0, pp = 0, mm = 0;
  dsm_corr_shape(sim, &levels, &pp, &mm);
  int32_t n = (int32_t)(pp + (levels - 1) * (pp - pp / std::max(mm, 1)));
  t = new float[n];
  x = new float[n];
  std::fill(t, t + n, 0.0f);
  std::fill(x, x + n, 0.0f);
  rc = dsm_gt(sim, t, x, &n);
  if (rc != DSM_OK) { std::cout << dsm_last_error(sim) << "\n"; return rc; }
  std::ofstream f(dsmc::filename_ID(correlator_type == 1 ? "MSD" : "G", job_ID));
  std::cout << "\n";
  for (int j = 0; j < n; ++j) {
    std::cout << t[j] << '\t' << x[j] << '\n';
    f << t[j] << '\t' << x[j] << '\n';
  }
  download(sim, N_cha, chain_heads, chains);
  universal_time = length;
  return 0;
}

// ensemble.cu:506-539
void gpu_clean() {
  dsm_destroy(G.sim);
  G = Global{};
  free_host();
}

// ensemble.cu:210-221
stress_plus calc_stress() {
  dsm_stress_plus s;
  std::memset(&s, 0, sizeof(s));
  int32_t cnt = 0;
  if (G.sim) dsm_stress(G.sim, &s, &cnt);
  return to_ref(s);
}

// ---------------------------------------------------------------- ensemble_call_block.h
namespace {
void init_block(ensemble_call_block* cb, int nc, sstrentp c, chain_head* heads, int s) {
  cb->nc = nc;
  cb->chains = c;
  cb->chain_heads = heads;
  cb->block_time = universal_time;
  cb->sim = nullptr;
  cb->levels = s;
  cb->corr_type = -1;
  cb->corr_res = 0;
  const dsm_params p = params_from_globals(nc, global_offset(c), G.seed, 0, 1.0, 0.0, 0);
  if (make_sim(p, &cb->sim) != DSM_OK) return;
  if (upload(cb->sim, heads, c) != DSM_OK) std::cout << dsm_last_error(cb->sim) << "\n";
}

// give the block's device ensemble the correlator of an EQ run; its chains,
// clocks, random-stream counters and stall codes carry over
int block_with_correlator(ensemble_call_block* cb, int correlator_type, double length) {
  const int n = cb->nc, zc = z_max > 0 ? z_max : NK;
  std::vector<dsm_chain_head> h(n);
  std::vector<dsm_float4> qn((size_t)n * zc);
  std::vector<float> tau((size_t)n * zc), dtp(n);
  std::vector<int64_t> T(n);
  std::vector<uint64_t> st(n);
  std::vector<int32_t> stall(n), S(n);
  int rc = dsm_get_chains(cb->sim, h.data(), qn.data(), tau.data());
  if (rc == DSM_OK) rc = dsm_get_ext(cb->sim, T.data(), st.data(), dtp.data(), stall.data(), S.data(), nullptr);
  if (rc != DSM_OK) return rc;
  const dsm_params p = params_from_globals(n, global_offset(cb->chains), G.seed, correlator_type == 1 ? 2 : 1,
                                           (double)dsm_correlator_res, length, cb->levels);
  dsm_sim* sim = nullptr;
  rc = make_sim(p, &sim);
  if (rc != DSM_OK) return rc;
  rc = dsm_set_chains(sim, h.data(), qn.data(), tau.data());
  if (rc == DSM_OK) rc = dsm_set_ext(sim, T.data(), st.data(), dtp.data(), stall.data(), S.data());
  if (rc != DSM_OK) { std::cout << dsm_last_error(sim) << "\n"; dsm_destroy(sim); return rc; }
  dsm_destroy(cb->sim);
  cb->sim = sim;
  cb->corr_type = correlator_type;
  cb->corr_res = dsm_correlator_res;
  return DSM_OK;
}
}  // namespace

// ensemble_call_block.cu:55-104 (definition, with correlator levels s) and
// ensemble_call_block.h:55 (declaration without)
void init_call_block(ensemble_call_block* cb, int nc, sstrentp c, chain_head* heads) { init_block(cb, nc, c, heads, 0); }
void init_call_block(ensemble_call_block* cb, int nc, sstrentp c, chain_head* heads, int s) {
  init_block(cb, nc, c, heads, s);
}

// ensemble_call_block.cu:106-222
int time_step_call_block(double reach_time, ensemble_call_block* cb, bool* run_flag) {
  if (!cb || !cb->sim) return DSM_ERR_INVALID;
  const int rc = advance_polling(cb->sim, reach_time, run_flag);
  if (rc == DSM_ABORTED) return -1;
  if (rc != DSM_OK) return rc;
  cb->block_time = reach_time;
  return 0;
}

// ensemble_call_block.cu:224-379: samples every dsm_correlator_res tau_K into
// the block's correlator (type 0 G(t), 1 MSD(t)); the G(t) of the block is
// dsm_gt(cb->sim, ...)
int EQ_time_step_call_block(double reach_time, ensemble_call_block* cb, int correlator_type, bool* run_flag,
                            int* progress_bar) {
  if (!cb || !cb->sim) return DSM_ERR_INVALID;
  if (cb->corr_type != correlator_type || cb->corr_res != dsm_correlator_res) {
    const int rc = block_with_correlator(cb, correlator_type, reach_time);
    if (rc != DSM_OK) return rc;
  }
  const int rc = advance_polling(cb->sim, reach_time, run_flag);
  if (rc == DSM_ABORTED) return -1;
  if (rc != DSM_OK) return rc;
  if (progress_bar) *progress_bar = 100;
  cb->block_time = reach_time;
  return 0;
}

// ensemble_call_block.cu:402-413
void get_chain_to_device_call_block(ensemble_call_block* cb) {
  if (cb && cb->sim) upload(cb->sim, cb->chain_heads, cb->chains);
}

// ensemble_call_block.cu:415-450 (no delayed dynamics are ever pending here)
void get_chain_from_device_call_block(ensemble_call_block* cb) {
  if (cb && cb->sim) download(cb->sim, cb->nc, cb->chain_heads, cb->chains);
}

// ensemble_call_block.cu:452-505
stress_plus calc_stress_call_block(ensemble_call_block* cb, int* r_chain_count) {
  dsm_stress_plus s;
  std::memset(&s, 0, sizeof(s));
  int32_t cnt = 0;
  if (cb && cb->sim) dsm_stress(cb->sim, &s, &cnt);
  if (r_chain_count) *r_chain_count = cnt;
  return to_ref(s);
}

// ensemble_call_block.cu:507-531: the device ensemble; the host arrays are the caller's
void free_block(ensemble_call_block* cb) {
  if (!cb) return;
  dsm_destroy(cb->sim);
  cb->sim = nullptr;
}

// ensemble_call_block.cu:533-565: a block keeps its chains in its own device
// ensemble, so there are no working copies to fill or drain
void activate_block(ensemble_call_block*) {}
void deactivate_block(ensemble_call_block*) {}

// ---------------------------------------------------------------- driver
int main_cuda(bool* run_flag, int job, char* savefile, char* loadfile, int device_ID, bool distr, int* progress_bar) {
  return dsmc::main_cuda_impl(run_flag, job, savefile, loadfile, device_ID, distr, progress_bar);
}
