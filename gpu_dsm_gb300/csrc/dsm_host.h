// Host-side state of one simulation handle (dsm_sim of include/dsm.h).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dsm.h"
#include "dsm_internal.h"

namespace dsm {

struct HostPcd {  // p_cd fit (common/pcd_tau.h:26-66) in double + device form
  double alpha, tau_0, tau_max, tau_d, g, c1, cm1, rcm1c1, At, Adt, Bdt, normdt;
  PcdDev dev;
};

struct TableOffsets { size_t NT, NE, FRIC, INV3N; };  // float offsets into one buffer

HostPcd make_pcd(double beta, double nk);
void make_tables(int nmax, double beta_f, float prefact, std::vector<float>& buf, TableOffsets& off);
int corr_levels_for(double t_end, double dt, int p, int m);

}  // namespace dsm

struct dsm_sim {
  dsm_params P{};
  std::string err;
  bool ready = false, flow = false, corr = false, poly = false;
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
  long long* d_prefix = nullptr;
  unsigned int* d_work = nullptr;
  int* d_status = nullptr;
  unsigned long long* d_counters = nullptr;
  double* d_red = nullptr;
  volatile int* h_abort = nullptr;
  int* d_abort = nullptr;
};

namespace dsm {
int sim_setup(dsm_sim* s);
int sim_launch_window(dsm_sim* s, double t_end, int64_t step_limit);
int sim_finish_window(dsm_sim* s, uint64_t* events);
}  // namespace dsm
