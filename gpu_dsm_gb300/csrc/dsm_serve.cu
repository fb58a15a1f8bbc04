// Serving loop: continuous batching of rheology requests on one GPU.
//
// A server thread admits queued requests while the device-memory budget allows
// (their ensembles are created and initialised on the device and stay
// resident), then repeatedly advances every active ensemble by one tick in
// batched persistent launches (dsm_advance_batch: one launch per kind and
// shared-memory size class, on separate streams).  A request that reaches its
// t_end is completed (G(t) or its stress time series kept on the host), its
// device memory released, and queued requests are admitted in its place, so
// requests that arrive while others run share the GPU with them.  With
// max_active = 1 the same loop is the plain one-ensemble-at-a-time form.
// The reference runs one ensemble per process (common/main_cuda.cu); there is
// no serving counterpart in it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dsm.h"
#include "dsm_host.h"

namespace {

using clk = std::chrono::steady_clock;

enum : int32_t { RQ_QUEUED = 0, RQ_ACTIVE = 1, RQ_DONE = 2, RQ_FAILED = 3 };

struct Req {
  uint64_t id = 0;
  dsm_params P{};
  clk::time_point t_arrive, t_admit, t_done;
  dsm_sim* sim = nullptr;
  double t_cur = 0.0;
  int32_t state = RQ_QUEUED;
  size_t bytes = 0;
  uint64_t events = 0;
  bool flow = false, corr = false;
  double rate = 0.0;  // kMC events per tau_K of the whole ensemble (last tick)
  int64_t k_out = 0;  // flow: stress outputs written
  std::vector<double> out_t;
  std::vector<dsm_stress_plus> out_s;
  std::vector<float> gt_t, gt_g;
  std::string err;
};

bool is_flow(const dsm_params& P) {
  for (int q = 0; q < 9; ++q) if (P.kappa[q] != 0.0f) return true;
  return false;
}

// device bytes of an ensemble (same estimate as dsm_create's budget check)
size_t ensemble_bytes(const dsm_params& P) {
  const size_t n = (size_t)P.n_chains, cap = (size_t)(P.z_max > 0 ? P.z_max : P.nk);
  size_t b = n * cap * 20 + n * 64 + n * 32 + (size_t)(9 * (P.nk + 2) + 8 * (P.nk + 2) + 8) * 4;
  if (!is_flow(P) && P.eq_type == 1 && P.sync_dt > 0 && P.t_end > 0) {
    const int p = P.corr_p > 0 ? P.corr_p : 64, m = P.corr_m > 0 ? P.corr_m : 8;
    const int L = P.corr_levels > 0 ? P.corr_levels : dsm::corr_levels_for(P.t_end, P.sync_dt, p, m);
    b += n * (size_t)L * ((size_t)p * 20 + 28);
  }
  return b + (1u << 20);
}

}  // namespace

struct dsm_server {
  int device = 0;
  uint64_t budget = 0, used = 0;
  int max_active = 0;
  double tick_s = 0.05;      // target tick duration; < 0: whole-request windows
  double rate_est = 1.0e9;   // aggregate kMC events/s of recent ticks
  int sm_count = 152, blocks_per_sm = 4;
  std::mutex mu;
  std::condition_variable cv;
  std::thread th;
  bool stop = false;
  std::deque<Req*> queue;
  std::vector<Req*> active;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  uint64_t next_id = 1;
  uint64_t events = 0, ticks = 0, completed = 0, peak_bytes = 0;
  int peak_active = 0;
  double busy_s = 0.0;
  std::string err;

  void run();
  void plan_tick(std::vector<double>& targets);
  void admit(std::vector<Req*>& fresh);
  void finish(Req* r);
};

// Next time at which a flow request writes its stress: k*sync_dt, the last
// one clipped to t_end (the output loop of common/main_cuda.cu)
static double next_output(const Req* r) {
  return std::min(r->P.t_end, (double)(r->k_out + 1) * r->P.sync_dt);
}

// Windows of one tick.  The tick's event budget B = rate_est * tick_s is
// shared equally by the active requests (processor sharing), each capped by
// its remaining work and by what its chains can do one after another in one
// tick (per resident chain slot, rate_est * tick_s / min(chains, slots)):
// water-filling, so small requests finish in few ticks and a tick stays near
// tick_s.  Flow requests also stop at their next stress output time.
void dsm_server::plan_tick(std::vector<double>& targets) {
  const size_t k = active.size();
  std::vector<double> cap(k), alloc(k);
  double chains = 0.0;
  for (Req* r : active) chains += r->P.n_chains;
  const double B = rate_est * tick_s;
  double slots = 0.0;
  for (Req* r : active) {
    const int lanes = r->P.lanes_per_chain > 0 ? r->P.lanes_per_chain : 32;
    slots = std::max(slots, (double)sm_count * blocks_per_sm * (128.0 / lanes));
  }
  const double per_chain = B / std::max(1.0, std::min(chains, slots));
  for (size_t i = 0; i < k; ++i) {
    Req* r = active[i];
    const double remaining = (r->P.t_end - r->t_cur) * r->rate;
    cap[i] = std::min(remaining, per_chain * r->P.n_chains);
  }
  if (tick_s < 0) {
    for (size_t i = 0; i < k; ++i) alloc[i] = std::numeric_limits<double>::infinity();
  } else {
    std::vector<size_t> ord(k);
    for (size_t i = 0; i < k; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return cap[a] < cap[b]; });
    double left = B;
    size_t n_left = k;
    for (size_t j = 0; j < k; ++j) {
      const size_t i = ord[j];
      const double share = left / (double)n_left;
      alloc[i] = std::min(cap[i], share);
      left -= alloc[i];
      --n_left;
    }
  }
  for (size_t i = 0; i < k; ++i) {
    Req* r = active[i];
    // at least ~4 events per chain so that a tick always makes progress
    const double win = std::max(alloc[i], 4.0 * r->P.n_chains) / std::max(r->rate, 1.0);
    double t = std::isfinite(win) ? r->t_cur + win : r->P.t_end;
    t = std::min(t, r->P.t_end);
    if (r->flow) t = std::min(t, next_output(r));
    targets[i] = t;
  }
}

void dsm_server::admit(std::vector<Req*>& fresh) {
  std::lock_guard<std::mutex> lk(mu);
  while (!queue.empty() && (max_active <= 0 || (int)active.size() + (int)fresh.size() < max_active)) {
    Req* r = queue.front();
    const bool fits = used + r->bytes <= budget;
    if (!fits && !(active.empty() && fresh.empty())) break;
    queue.pop_front();
    used += r->bytes;
    fresh.push_back(r);
    peak_bytes = std::max<uint64_t>(peak_bytes, used);
    peak_active = std::max<int>(peak_active, (int)(active.size() + fresh.size()));
  }
}

void dsm_server::finish(Req* r) {
  if (r->corr) {
    int32_t n = 8192;
    r->gt_t.assign(n, 0.f);
    r->gt_g.assign(n, 0.f);
    if (dsm_gt(r->sim, r->gt_t.data(), r->gt_g.data(), &n) == DSM_OK) {
      r->gt_t.resize(n);
      r->gt_g.resize(n);
    } else {
      r->gt_t.clear();
      r->gt_g.clear();
    }
  }
  dsm_destroy(r->sim);
  r->sim = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  used -= r->bytes;
  r->t_done = clk::now();
  r->state = RQ_DONE;
  ++completed;
  cv.notify_all();
}

void dsm_server::run() {
  cudaSetDevice(device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu);
      if (stop) break;
      if (queue.empty() && active.empty()) {
        cv.wait_for(lk, std::chrono::milliseconds(1));
        continue;
      }
    }
    std::vector<Req*> fresh;
    admit(fresh);
    for (Req* r : fresh) {
      dsm_sim* s = nullptr;
      int rc = dsm_create(&r->P, &s);
      if (rc == DSM_OK) rc = dsm_init_equilibrium(s);
      std::lock_guard<std::mutex> lk(mu);
      if (rc != DSM_OK) {
        r->err = s ? dsm_last_error(s) : "dsm_create failed";
        if (s) dsm_destroy(s);
        used -= r->bytes;
        r->state = RQ_FAILED;
        r->t_done = clk::now();
        cv.notify_all();
        continue;
      }
      r->sim = s;
      r->state = RQ_ACTIVE;
      r->t_admit = clk::now();
      active.push_back(r);
    }
    if (active.empty()) continue;
    const size_t k = active.size();
    std::vector<dsm_sim*> sims(k);
    std::vector<double> targets(k);
    plan_tick(targets);
    for (size_t i = 0; i < k; ++i) sims[i] = active[i]->sim;
    std::vector<uint64_t> ev(k, 0);
    const auto t0 = clk::now();
    const int rc = dsm_advance_batch(sims.data(), (int32_t)k, targets.data(), nullptr, ev.data());
    const double dt_tick = std::chrono::duration<double>(clk::now() - t0).count();
    busy_s += dt_tick;
    ++ticks;
    if (rc == DSM_OK) {
      uint64_t tot = 0;
      for (uint64_t e : ev) tot += e;
      if (dt_tick > 0 && tot > 0) rate_est = 0.7 * rate_est + 0.3 * ((double)tot / dt_tick);
      int32_t grid = 0, bps = 0;
      if (dsm_last_window(sims[0], nullptr, nullptr, &grid, &bps) == DSM_OK && bps > 0) blocks_per_sm = bps;
    }
    if (rc != DSM_OK) {
      std::lock_guard<std::mutex> lk(mu);
      err = dsm_last_error(sims[0]);
      for (Req* r : active) {
        dsm_destroy(r->sim);
        r->sim = nullptr;
        used -= r->bytes;
        r->state = RQ_FAILED;
        r->err = err;
        r->t_done = clk::now();
      }
      active.clear();
      cv.notify_all();
      continue;
    }
    std::vector<Req*> still;
    for (size_t i = 0; i < k; ++i) {
      Req* r = active[i];
      const double dtau = targets[i] - r->t_cur;
      if (dtau > 0 && ev[i] > 0) r->rate = (double)ev[i] / dtau;
      r->t_cur = targets[i];
      r->events += ev[i];
      events += ev[i];
      if (r->flow && r->t_cur == next_output(r)) {
        dsm_stress_plus sp;
        if (dsm_stress(r->sim, &sp, nullptr) == DSM_OK) {
          r->out_t.push_back(r->t_cur);
          r->out_s.push_back(sp);
        }
        ++r->k_out;
      }
      if (r->t_cur >= r->P.t_end) finish(r);
      else still.push_back(r);
    }
    active.swap(still);
  }
  // shutdown: release what is still resident
  for (Req* r : active) if (r->sim) dsm_destroy(r->sim);
  active.clear();
}

extern "C" int dsm_serve_open(int32_t device, uint64_t hbm_budget_bytes, int32_t max_active, double tick_s,
                              dsm_server** out) {
  if (!out) return DSM_ERR_INVALID;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return DSM_ERR_CUDA;
  size_t fre = 0, tot = 0;
  if (cudaMemGetInfo(&fre, &tot) != cudaSuccess) return DSM_ERR_CUDA;
  dsm_server* s = new dsm_server();
  s->device = device;
  s->budget = hbm_budget_bytes > 0 ? std::min<uint64_t>(hbm_budget_bytes, fre - (fre >> 4)) : (uint64_t)(fre - (fre >> 4));
  s->max_active = max_active;
  s->tick_s = tick_s != 0.0 ? tick_s : 0.05;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0)
    s->sm_count = sms;
  s->th = std::thread([s] { s->run(); });
  *out = s;
  return DSM_OK;
}

extern "C" int dsm_serve_submit(dsm_server* s, const dsm_params* p, uint64_t* id) {
  if (!s || !p || !id) return DSM_ERR_INVALID;
  if (p->nk_chain != nullptr) return DSM_ERR_INVALID;
  auto r = std::make_unique<Req>();
  r->P = *p;
  r->P.device = s->device;
  r->flow = is_flow(*p);
  r->corr = !r->flow && p->eq_type == 1 && p->sync_dt > 0 && p->t_end > 0;
  r->bytes = ensemble_bytes(*p);
  // prior for the events per tau_K of the ensemble (about 0.2 N_K + 2 per
  // chain at beta = 1); replaced by the measured value after the first tick
  r->rate = (0.2 * (double)p->nk + 2.0) * (double)p->n_chains;
  r->t_arrive = clk::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (r->bytes > s->budget) return DSM_ERR_MEMORY;
  r->id = s->next_id++;
  *id = r->id;
  s->queue.push_back(r.get());
  s->reqs.emplace(r->id, std::move(r));
  s->cv.notify_all();
  return DSM_OK;
}

extern "C" int dsm_serve_status(dsm_server* s, uint64_t id, int32_t* state, double* latency_s, double* queue_s,
                                uint64_t* events) {
  if (!s) return DSM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return DSM_ERR_INVALID;
  Req* r = it->second.get();
  if (state) *state = r->state;
  const bool fin = r->state == RQ_DONE || r->state == RQ_FAILED;
  if (latency_s) *latency_s = fin ? std::chrono::duration<double>(r->t_done - r->t_arrive).count() : -1.0;
  if (queue_s)
    *queue_s = (r->state == RQ_QUEUED) ? -1.0 : std::chrono::duration<double>(r->t_admit - r->t_arrive).count();
  if (events) *events = r->events;
  return DSM_OK;
}

extern "C" int dsm_serve_wait_all(dsm_server* s, double timeout_s) {
  if (!s) return DSM_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const auto dl = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
  for (;;) {
    bool all = s->queue.empty() && s->active.empty();
    if (all) {
      for (auto& kv : s->reqs)
        if (kv.second->state == RQ_QUEUED || kv.second->state == RQ_ACTIVE) { all = false; break; }
    }
    if (all) return DSM_OK;
    if (s->cv.wait_until(lk, dl) == std::cv_status::timeout) return DSM_ERR_WATCHDOG;
  }
}

extern "C" int dsm_serve_result_gt(dsm_server* s, uint64_t id, float* t, float* G, int32_t* n) {
  if (!s || !n) return DSM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second->state != RQ_DONE) return DSM_ERR_INVALID;
  Req* r = it->second.get();
  const int32_t m = (int32_t)r->gt_g.size();
  if (*n < m) { *n = m; return DSM_ERR_INVALID; }
  for (int32_t i = 0; i < m; ++i) { if (t) t[i] = r->gt_t[i]; if (G) G[i] = r->gt_g[i]; }
  *n = m;
  return DSM_OK;
}

extern "C" int dsm_serve_result_stress(dsm_server* s, uint64_t id, double* t, dsm_stress_plus* out, int32_t* n) {
  if (!s || !n) return DSM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second->state != RQ_DONE) return DSM_ERR_INVALID;
  Req* r = it->second.get();
  const int32_t m = (int32_t)r->out_s.size();
  if (*n < m) { *n = m; return DSM_ERR_INVALID; }
  for (int32_t i = 0; i < m; ++i) { if (t) t[i] = r->out_t[i]; if (out) out[i] = r->out_s[i]; }
  *n = m;
  return DSM_OK;
}

extern "C" int dsm_serve_stats(dsm_server* s, dsm_serve_totals* out) {
  if (!s || !out) return DSM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->events = s->events;
  out->busy_s = s->busy_s;
  out->ticks = s->ticks;
  out->completed = s->completed;
  out->peak_bytes = s->peak_bytes;
  out->peak_active = s->peak_active;
  return DSM_OK;
}

extern "C" void dsm_serve_close(dsm_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  delete s;
}
