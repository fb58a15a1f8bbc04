// Serving loop: continuous batching of rheology requests on one GPU.
//
// A server thread admits queued requests while the device-memory budget allows
// (their ensembles are created and initialised on the device and stay
// resident) and keeps every admitted ensemble busy on its own CUDA stream:
// whenever one finishes a chunk of work it gets the next one at once
// (dsm_advance_start for equilibrium requests, dsm_series_start for flow
// requests, whose stress outputs of a chunk run as one CUDA graph replay), so
// the kernels of all admitted requests overlap on the device and share its SMs
// through the hardware block scheduler.  Chunks are sized so that each takes
// about chunk_s seconds with every resident chain advancing at the same pace.
// A request that reaches its t_end is completed (G(t) or its stress series
// kept on the host), its device memory released, and queued requests are
// admitted in its place.  With max_active = 1 and chunk_s < 0 the same loop is
// the plain form: one request at a time, each equilibrium request in one
// launch, each flow output one launch followed by a host round trip (the
// reference's flow loop).  The reference runs one ensemble per process
// (common/main_cuda.cu); there is no serving counterpart in it.
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

constexpr int kMaxSeries = 256;  // flow outputs per graph replay

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
  double rate = 0.0;      // kMC events per tau_K of the whole ensemble (last chunk)
  int64_t k_out = 0;      // flow: stress outputs written
  int64_t n_outputs = 0;  // flow: outputs at min(t_end, k * sync_dt), k = 1..n_outputs
  bool inflight = false;
  double target = 0.0;    // end time of the chunk in flight
  double eps = 0.0;       // kMC events per second of its last chunk (wall clock)
  double occupancy = 1.0; // share of the GPU's chain slots its step launch fills
  clk::time_point t_chunk;
  std::vector<double> ends;
  std::vector<dsm_stress_plus> sbuf;
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

// time of flow output k (1-based): the same product wherever it is computed
double output_time(const Req* r, int64_t k) { return std::min(r->P.t_end, (double)k * r->P.sync_dt); }

}  // namespace

struct dsm_server {
  int device = 0;
  uint64_t budget = 0, used = 0;
  int max_active = 0;
  double chunk_s = 0.05;     // target duration of one chunk; < 0: whole-request windows
  double rate_est = 1.0e9;   // aggregate kMC events/s while work is in flight
  int policy = 0;            // 0 first come first served with backfill, 1 equal pace per chain
  double overlap = 1.0;      // running requests may fill up to this many GPUs' worth of chain slots
  double bypass = 0.2;       // requests shorter than bypass * chunk_s of the whole GPU run at once
  int prio_least = 0, prio_greatest = 0;  // CUDA stream priority range
  int sm_slots = 4864;       // chains resident on the GPU at full occupancy (152 SMs x 32)
  std::mutex mu;
  std::condition_variable cv;       // request state changes (waiters)
  std::condition_variable cv_work;  // work for the loader / finisher threads
  std::thread th, loader, finisher;
  bool stop = false;
  std::deque<Req*> queue;      // submitted, not admitted
  std::deque<Req*> to_load;    // admitted: ensemble to create and initialise
  std::vector<Req*> loaded;    // ready to run
  std::deque<Req*> to_finish;  // done: results to read, ensemble to release
  std::vector<Req*> active;    // running (server thread only)
  int resident = 0;            // admitted and not yet released
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
  uint64_t next_id = 1;
  uint64_t events = 0, ticks = 0, completed = 0, peak_bytes = 0;
  int peak_active = 0;
  double busy_s = 0.0, setup_s = 0.0, finish_s = 0.0;
  std::string err;

  void run();
  void load_loop();
  void finish_loop();
  void admit();
  int start_chunk(Req* r, double chains_total, int rank);
  void fail_req(Req* r, const std::string& why);
};

// Admission (under the lock): in arrival order while the budget and the cap on
// resident ensembles allow; a request larger than the whole budget still runs
// alone.  Creation and initialisation happen on the loader thread.
void dsm_server::admit() {
  std::lock_guard<std::mutex> lk(mu);
  bool any = false;
  while (!queue.empty() && (max_active <= 0 || resident < max_active)) {
    Req* r = queue.front();
    if (used + r->bytes > budget && resident > 0) break;
    queue.pop_front();
    used += r->bytes;
    ++resident;
    peak_bytes = std::max<uint64_t>(peak_bytes, used);
    peak_active = std::max(peak_active, resident);
    to_load.push_back(r);
    any = true;
  }
  if (any) cv_work.notify_all();
}

// Loader thread: create and initialise admitted ensembles, so that the server
// thread never waits for SMs held by other requests' kernels
void dsm_server::load_loop() {
  cudaSetDevice(device);
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return stop || !to_load.empty(); });
      if (stop) return;
      r = to_load.front();
      to_load.pop_front();
    }
    const auto t0 = clk::now();
    dsm_sim* sim = nullptr;
    // create and initialise on a highest-priority stream: the initialiser then
    // gets SMs as soon as running blocks retire, not after whole chunks
    dsm_params P = r->P;
    P.stream_priority = prio_greatest;
    int rc = dsm_create(&P, &sim);
    if (rc == DSM_OK) rc = dsm_init_equilibrium(sim);
    if (rc == DSM_OK) {
      int32_t grid = 0, bps = 0;
      dsm_last_window(sim, nullptr, nullptr, &grid, &bps);
      if (grid > 0 && bps > 0) r->occupancy = std::min(1.0, (double)grid / ((double)bps * (double)(sm_slots / 32)));
    }
    std::string why;
    if (rc != DSM_OK) {
      why = sim ? dsm_last_error(sim) : "dsm_create failed";
      if (sim) dsm_destroy(sim);
      sim = nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    setup_s += std::chrono::duration<double>(clk::now() - t0).count();
    if (rc != DSM_OK) {
      used -= r->bytes;
      --resident;
      r->state = RQ_FAILED;
      r->err = why;
      r->t_done = clk::now();
      ++completed;
      cv.notify_all();
      continue;
    }
    r->sim = sim;
    r->state = RQ_ACTIVE;
    r->t_admit = clk::now();
    loaded.push_back(r);
  }
}

// Finisher thread: read results (G(t)) and release the ensemble; the request
// completes when its results are on the host
void dsm_server::finish_loop() {
  cudaSetDevice(device);
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return stop || !to_finish.empty(); });
      if (stop && to_finish.empty()) return;
      r = to_finish.front();
      to_finish.pop_front();
    }
    const auto t0 = clk::now();
    dsm_set_priority(r->sim, prio_greatest);  // the G(t) reduction should not wait for whole chunks
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
    finish_s += std::chrono::duration<double>(clk::now() - t0).count();
    used -= r->bytes;
    --resident;
    r->t_done = clk::now();
    r->state = RQ_DONE;
    ++completed;
    cv.notify_all();
  }
}

// Next chunk of r on its own stream, about chunk_s seconds of work.
//  * policy 0 (first come, first served with backfill): the request's stream
//    priority follows its age rank (the oldest gets the highest), so when SMs
//    free up the block scheduler serves older requests first and younger ones
//    fill what is left; a chunk is chunk_s times the request's own measured
//    events per second (first chunk: its share of the GPU's chain slots).
//  * policy 1 (equal pace): every resident chain advances by the same number of
//    events per chunk (the request's share of rate_est * chunk_s is its share
//    of the resident chains), at the default priority.
// Both give at least 64 events per chain per chunk.
int dsm_server::start_chunk(Req* r, double chains_total, int rank) {
  const double n = (double)r->P.n_chains;
  double dtau = std::numeric_limits<double>::infinity();
  if (chunk_s > 0.0) {
    double ev;
    if (policy != 1) {
      const double slots = (double)sm_slots;
      const double eps = r->eps > 0.0 ? r->eps : rate_est * std::min(1.0, n / slots);
      ev = std::max(eps * chunk_s, 64.0 * n);
    } else {
      ev = std::max(rate_est * chunk_s * n / std::max(chains_total, 1.0), 64.0 * n);
    }
    dtau = ev / std::max(r->rate, 1.0);
  }
  if (policy != 1) dsm_set_priority(r->sim, prio_greatest + std::min(rank, prio_least - prio_greatest));
  r->t_chunk = clk::now();
  if (r->flow) {
    const int64_t left = r->n_outputs - r->k_out;
    int64_t k = 1;
    if (chunk_s > 0.0) {
      k = (int64_t)std::floor(dtau / r->P.sync_dt);
      k = std::max<int64_t>(1, std::min<int64_t>({k, left, kMaxSeries}));
      int64_t p2 = 1;  // a power of two: few distinct graphs per request
      while (p2 * 2 <= k) p2 *= 2;
      k = p2;
    }
    r->ends.resize(k);
    for (int64_t w = 0; w < k; ++w) r->ends[w] = output_time(r, r->k_out + w + 1);
    r->sbuf.resize(k);
    r->target = r->ends[k - 1];
    if (chunk_s > 0.0) return dsm_series_start(r->sim, r->ends.data(), (int32_t)k);
    return dsm_advance_start(r->sim, r->target, -1);
  }
  r->target = std::min(r->P.t_end, r->t_cur + dtau);
  return dsm_advance_start(r->sim, r->target, -1);
}

void dsm_server::fail_req(Req* r, const std::string& why) {
  if (r->sim) dsm_destroy(r->sim);
  r->sim = nullptr;
  std::lock_guard<std::mutex> lk(mu);
  used -= r->bytes;
  --resident;
  r->state = RQ_FAILED;
  r->err = why;
  r->t_done = clk::now();
  ++completed;
  cv.notify_all();
}

void dsm_server::run() {
  cudaSetDevice(device);
  clk::time_point t_mark = clk::now();
  uint64_t ev_mark = 0;
  for (;;) {
    bool idle = false;
    {
      std::unique_lock<std::mutex> lk(mu);
      if (stop) break;
      idle = queue.empty() && loaded.empty() && active.empty();
      if (idle && resident == 0) {
        cv.wait_for(lk, std::chrono::milliseconds(1));
        t_mark = clk::now();
        ev_mark = events;
        continue;
      }
    }
    admit();
    bool changed = false;
    {
      std::lock_guard<std::mutex> lk(mu);
      if (!loaded.empty()) {
        // keep arrival order (request ids ascend with arrival)
        for (Req* r : loaded) active.push_back(r);
        loaded.clear();
        std::sort(active.begin(), active.end(), [](const Req* x, const Req* y) { return x->id < y->id; });
        changed = true;
      }
    }
    (void)changed;
    double chains_total = 0.0;
    for (Req* r : active) chains_total += r->P.n_chains;
    std::vector<Req*> still;
    bool progressed = false;
    int rank = 0;  // age rank among the running requests (active is in arrival order)
    // First come, first served with backfill: in arrival order, a request
    // gets chunks while the older running ones leave part of the GPU's chain
    // slots free (the oldest always runs); a request whose remaining work
    // is below one chunk of the whole GPU runs at once.  Equal pace runs all.
    double occ = 0.0;
    const double short_work = rate_est * std::max(chunk_s, 0.0) * bypass;
    for (Req* r : active) {
      const int my_rank = rank++;
      bool may_run = true;
      if ((policy == 0 || policy == 2) && chunk_s > 0.0) {
        const double rem = (r->P.t_end - r->t_cur) * r->rate;
        may_run = r->inflight || occ < overlap || (policy == 0 && rem < short_work);
        occ += r->occupancy;
      }
      if (!may_run) { still.push_back(r); continue; }
      if (!r->inflight) {
        const int rc = start_chunk(r, chains_total, my_rank);
        if (rc != DSM_OK) { fail_req(r, dsm_last_error(r->sim)); progressed = true; continue; }
        r->inflight = true;
        ++ticks;
      }
      uint64_t ev = 0;
      int32_t nout = 0;
      const int rc = dsm_poll(r->sim, &ev, r->flow ? r->sbuf.data() : nullptr, &nout);
      if (rc == DSM_PENDING) { still.push_back(r); continue; }
      progressed = true;
      r->inflight = false;
      if (rc != DSM_OK) { fail_req(r, dsm_last_error(r->sim)); continue; }
      const double dtau = r->target - r->t_cur;
      if (dtau > 0 && ev > 0) r->rate = (double)ev / dtau;
      const double wall = std::chrono::duration<double>(clk::now() - r->t_chunk).count();
      if (wall > 0 && ev > 0) r->eps = (double)ev / wall;
      r->t_cur = r->target;
      r->events += ev;
      events += ev;
      if (r->flow) {
        for (int32_t w = 0; w < nout && w < (int32_t)r->ends.size(); ++w) {
          r->out_t.push_back(r->ends[w]);
          r->out_s.push_back(r->sbuf[w]);
        }
        r->k_out += (int64_t)r->ends.size();
      }
      if (r->t_cur >= r->P.t_end) {
        std::lock_guard<std::mutex> lk(mu);
        to_finish.push_back(r);
        cv_work.notify_all();
      } else {
        still.push_back(r);
      }
    }
    active.swap(still);
    // aggregate rate over the last >= 20 ms with work in flight
    const auto now = clk::now();
    const double el = std::chrono::duration<double>(now - t_mark).count();
    if (el >= 0.02) {
      if (events > ev_mark) rate_est = 0.5 * rate_est + 0.5 * ((double)(events - ev_mark) / el);
      if (!active.empty()) busy_s += el;
      t_mark = now;
      ev_mark = events;
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  // shutdown: release what is still resident
  for (Req* r : active) {
    if (r->sim) {
      if (r->inflight) dsm_abort(r->sim);
      dsm_destroy(r->sim);
      r->sim = nullptr;
    }
  }
  active.clear();
}

extern "C" int dsm_serve_open(int32_t device, uint64_t hbm_budget_bytes, int32_t max_active, double chunk_s,
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
  s->chunk_s = chunk_s != 0.0 ? chunk_s : 0.05;
  cudaDeviceGetStreamPriorityRange(&s->prio_least, &s->prio_greatest);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && sms > 0)
    s->sm_slots = sms * 32;
  s->th = std::thread([s] { s->run(); });
  s->loader = std::thread([s] { s->load_loop(); });
  s->finisher = std::thread([s] { s->finish_loop(); });
  *out = s;
  return DSM_OK;
}

extern "C" int dsm_serve_set_policy(dsm_server* s, int32_t policy) {
  if (!s || policy < 0 || policy > 2) return DSM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->policy = policy;
  return DSM_OK;
}

extern "C" int dsm_serve_tune(dsm_server* s, double overlap, double bypass) {
  if (!s || !(overlap >= 1.0) || !(bypass >= 0.0)) return DSM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->overlap = overlap;
  s->bypass = bypass;
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
  if (r->flow) {
    if (!(p->sync_dt > 0) || !(p->t_end > 0)) return DSM_ERR_INVALID;
    r->n_outputs = (int64_t)std::ceil(p->t_end / p->sync_dt - 1e-9);
    if (r->n_outputs < 1) r->n_outputs = 1;
  }
  r->bytes = ensemble_bytes(*p);
  // prior for the events per tau_K of the ensemble (about 0.2 N_K + 2 per
  // chain at beta = 1); replaced by the measured value after the first chunk
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
    bool all = true;
    for (auto& kv : s->reqs)
      if (kv.second->state == RQ_QUEUED || kv.second->state == RQ_ACTIVE) { all = false; break; }
    if (all) return DSM_OK;
    if (s->cv.wait_until(lk, dl) == std::cv_status::timeout) return DSM_ERR_WATCHDOG;
  }
}

extern "C" const char* dsm_serve_error(dsm_server* s, uint64_t id) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return "unknown request";
  return it->second->err.c_str();
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
  out->setup_s = s->setup_s;
  out->finish_s = s->finish_s;
  return DSM_OK;
}

extern "C" void dsm_serve_close(dsm_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv.notify_all();
    s->cv_work.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  if (s->loader.joinable()) s->loader.join();
  if (s->finisher.joinable()) s->finisher.join();
  // requests loaded or finishing when the server stopped
  for (Req* r : s->loaded) if (r->sim) dsm_destroy(r->sim);
  for (Req* r : s->to_finish) if (r->sim) dsm_destroy(r->sim);
  delete s;
}
