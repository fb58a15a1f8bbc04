// Host-side state of one simulation handle (dsm_sim of include/dsm.h).
#pragma once
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/dsm.h"
#include "dsm_internal.h"

namespace dsm {

struct HostPcd {  // p_cd fit (common/pcd_tau.h:26-66) in double + device form
  double alpha, tau_0, tau_max, tau_d, g, c1, cm1, rcm1c1, At, Adt, Bdt, normdt;
  PcdDev dev;
};

struct TableOffsets { size_t NT, NE, FRIC, INV3N; };  // float offsets into one buffer

HostPcd make_pcd(double beta, double nk);

// GEX background molecular-weight tables (dsm_gex.cpp)
struct GexTable {
  std::vector<float> M, Md;  // M/mp at probabilities j*step (plain and CD-weighted law)
  float step = 0.f, step_d = 0.f, mp = 0.f, mk = 0.f;
  double prefact = 0.0;      // CD creation prefactor step * sum normdt / beta
};
int make_gex_table(float a, float b, float mp, float mk, double beta, GexTable* out);
// Per-N rate tables (sliding factors, end rates, CD creation, 3/N, 4/i
// frictions) in one buffer of table_floats(nmax) floats; the vector form
// sizes the buffer itself.
size_t table_floats(int nmax);
void make_tables(int nmax, double beta_f, float prefact, float* buf, TableOffsets& off);
void make_tables(int nmax, double beta_f, float prefact, std::vector<float>& buf, TableOffsets& off);
int corr_levels_for(double t_end, double dt, int p, int m);

}  // namespace dsm

namespace dsm {
// Pinned, mapped host words of one handle
struct HostWords {
  int abort;
  int status;
  unsigned long long cnt[4];
  double red[16];
  double pad_[3];
};
HostWords* host_words_take();
void host_words_give(HostWords* w);
void keep_pool_memory(int device);

// One persistent launch of a polydisperse ensemble's size-class plan: chains
// order[first .. first+count) with slots of cfg.slot_cap strands
// NVTX range over one phase of the host API (a no-op unless a tool such as
// ncu --nvtx is attached)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

struct SizeClass {
  LaunchCfg cfg{4, 0, 0, 32};
  long long first = 0, count = 0;
  int grid = 0, bps = 0;
  int stream = 0;  // 0 the handle's stream, 1 side, 2 side2, 3 side3
};
}  // namespace dsm

struct dsm_sim {
  dsm_params P{};
  std::string err;
  bool ready = false, flow = false, corr = false, poly = false, msd = false;
  int ck = 0;  // correlator kind of the step kernel: 0 none, 1 stress, 2 MSD
  int cap = 0, nkmax = 0, cp = 64, cm = 8, levels = 1;
  int64_t nsamples = 0;
  float prefact = 0.f;
  dsm::HostPcd pcd{};
  std::vector<dsm::PcdDev> pcd_by_nk;
  std::vector<int32_t> nk_chain;
  size_t bytes = 0;
  int sm_count = 0, blocks_per_sm = 0, grid = 0;
  int64_t watchdog_events = 0;
  double t_done = 0.0, t_window = 0.0;  // lowest time all chains reached / target of the window
  unsigned long long events_total = 0, last_events = 0;
  float last_kernel_ms = 0.f;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  dsm::LaunchCfg cfg{4, 0, 0, 32};
  dsm::EnsDev h{};
  cudaStream_t st = nullptr;
  // device buffers
  float* d_tables = nullptr;
  float4* d_QN = nullptr;
  float* d_tau = nullptr;
  dsm::ChainState* d_cs = nullptr;
  float* d_stress = nullptr;
  float* d_cshift = nullptr;
  double* d_cacc = nullptr;
  float* d_cavg = nullptr;
  int4* d_ccnt = nullptr;
  double* d_gsum = nullptr;
  long long* d_gcnt = nullptr;
  dsm::PcdDev* d_pcd_by_nk = nullptr;
  int32_t* d_nk_chain = nullptr;
  dsm::EnsDev* d_ens = nullptr;
  dsm::GexTable gex;        // GEX background tables (pd_flag = 1)
  float* d_gex = nullptr;   // device copy: M then Md
  long long* d_prefix = nullptr;
  unsigned int* d_work = nullptr;
  int* d_status = nullptr;
  unsigned long long* d_counters = nullptr;
  double* d_red = nullptr;
  volatile int* h_abort = nullptr;
  int* d_abort = nullptr;
  dsm::HostWords* hw = nullptr;
  // size classes (polydisperse ensembles whose largest chains do not fit a
  // full-occupancy slot): huge and large slots (one warp per block), middle
  // slots (one warp per chain, when the small class runs two chains per warp)
  // and small slots, run concurrently on four streams; chains that outgrow a
  // slot finish in the cleanup launch
  std::vector<dsm::SizeClass> classes;
  dsm::SizeClass cleanup;
  int* d_order = nullptr;
  int* d_defer = nullptr;
  unsigned int* d_works = nullptr;  // [0] small, [1] large, [2] cleanup, [3] deferred count, [4] middle, [5] huge,
                                    // [8 ..) the classes of a carved launch
  // carved form (dsm_set_class_form): the large, middle and small classes in
  // one launch of 16-lane tiles whose blocks carve the same shared memory into
  // per-class slot counts; the huge class (if any) beside it on its stream
  bool carve = false;       // asked for
  bool carved = false;      // the current plan is carved
  float margin_sd = 0.f;    // strand-count margin of the current class plan (0: 5 sd)
  dsm::StepList carve_list;
  int carve_grid = 0;
  size_t carve_smem = 0;
  cudaStream_t side = nullptr, side2 = nullptr, side3 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr, ev_join3 = nullptr;
  int prio = 0;  // CUDA stream priority of st and side
  int sched_version = 0;  // bumped whenever the launch schedule changes
  cudaEvent_t ev_done = nullptr;  // end of the last enqueued window / series, readback included
  int pending = 0;                // asynchronous work in flight: 1 window, 2 series
  // captured window series (dsm_advance_series / dsm_series_start): one graph
  // per window count, buffers for ser_cap windows
  std::vector<std::pair<int, cudaGraphExec_t>> ser_graphs;
  int ser_cap = 0, ser_n = 0, ser_version = -1;
  void* ser_d = nullptr;  // device: [cap end ticks][cap event caps][cap x 9 stress sums]
  void* ser_h = nullptr;  // pinned host mirror
};

namespace dsm {
int sim_setup(dsm_sim* s);
// Size-class plan of a polydisperse ensemble; small_cap / big_grid / lanes
// <= 0 pick the defaults (full-occupancy small slot, large-class grid by work share)
int plan_classes(dsm_sim* s, int small_cap, int big_grid, int lanes, float margin_sd);
// carved form of a class plan (dsm_set_class_form) in blocks of block_smem
// bytes; leaves the plan as it is if a class's slot does not fit the block
int plan_carve(dsm_sim* s, const SizeClass& big, const SizeClass& mid, const SizeClass& small, size_t block_smem);
int sim_launch_window(dsm_sim* s, double t_end, int64_t step_limit);
int sim_finish_window(dsm_sim* s, uint64_t* events);
}  // namespace dsm
