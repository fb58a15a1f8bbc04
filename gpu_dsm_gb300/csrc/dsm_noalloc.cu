// dsm_advance_noalloc: advance caller-owned chains without allocating memory.
//
// Who needs this: callers that cannot call cudaMalloc / cudaFree around a time
// step — a serving loop or host framework that owns every byte of device
// memory through its own allocator or HBM budget (a hidden allocation would
// break its accounting or fail once it has reserved the device), and loops
// that cannot afford the implicit device-wide synchronisation that
// cudaMalloc/cudaFree impose.  dsm_create allocates per-ensemble tables,
// descriptors and counters; this entry point keeps all of that in one
// file-scope device array instead, so the only memory it touches is the
// caller's state buffers and that array.
//
// The array below is a module-scope __device__ variable: every GPU that loads
// libgpudsm.so holds DSM_NOALLOC_SCRATCH_BYTES of it until the process exits.
// All calls share it and it keeps the last call's contents, so calls that
// overlap on the GPU (two streams, two host threads) race: serialise them.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/dsm.h"
#include "dsm_host.h"
#include "dsm_internal.h"

namespace {

constexpr size_t kScratchBytes = DSM_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxNk = DSM_NOALLOC_MAX_NK;
constexpr int kMaxDevices = 64;

// descriptor, launch bookkeeping and rate tables of one call
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;                                  // serialises host staging
void* g_dev_ptr[kMaxDevices] = {nullptr};         // device address of the array, per device
alignas(256) unsigned char g_host_stage[kScratchBytes];  // host image copied into the array
thread_local std::string g_err;

// layout of the array (bytes, 256-aligned blocks)
constexpr size_t kOffEns = 0;                          // EnsDev
constexpr size_t kOffPrefix = 1024;                    // long long[2]
constexpr size_t kOffWork = 1040;                      // unsigned int
constexpr size_t kOffStatus = 1044;                    // int
constexpr size_t kOffCounters = 1056;                  // unsigned long long[4]
constexpr size_t kOffTables = 2048;                    // float tables
static_assert(sizeof(dsm::EnsDev) <= kOffPrefix, "descriptor block");

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

}  // namespace

extern "C" const char* dsm_noalloc_last_error(void) { return g_err.c_str(); }

extern "C" int dsm_advance_noalloc(const dsm_params* p, dsm_float4* d_QN, float* d_tau, dsm_chain_state* d_state,
                                   float* d_stress_out, double t_end, int64_t step_limit, void* stream,
                                   uint64_t* events) {
  if (!p || !d_QN || !d_tau || !d_state) return fail(DSM_ERR_INVALID, "null argument");
  const int cap = p->z_max > 0 ? p->z_max : p->nk;
  bool flow = false;
  for (int q = 0; q < 9; ++q) flow = flow || (p->kappa[q] != 0.0f);
  if (p->nk < 1 || p->n_chains < 1 || !(p->beta > 0.0f)) return fail(DSM_ERR_INVALID, "invalid nk / n_chains / beta");
  if (p->nk > kMaxNk)
    return fail(DSM_ERR_INVALID, "nk=" + std::to_string(p->nk) + " exceeds the no-allocation limit of " +
                                     std::to_string(kMaxNk) + " Kuhn steps (the rate tables must fit the " +
                                     std::to_string(kScratchBytes >> 10) + " KiB static scratch)");
  if (cap < 1 || cap > 4096) return fail(DSM_ERR_INVALID, "z_max must be in [1, 4096]");
  if (p->nk_chain != nullptr) return fail(DSM_ERR_INVALID, "polydisperse ensembles need per-chain tables: use dsm_create");
  if (p->pd_flag != 0) return fail(DSM_ERR_INVALID, "pd_flag=1 is not supported");
  // dsm_create's rule: a G(t) or MSD correlator runs for equilibrium
  // ensembles with eq_type 1 or 2 and positive sync_dt and t_end
  if (!flow && (p->eq_type == 1 || p->eq_type == 2) && p->sync_dt > 0 && p->t_end > 0)
    return fail(DSM_ERR_INVALID, "the G(t) / MSD correlator needs per-chain buffers: use dsm_create");
  if (flow && d_stress_out == nullptr) return fail(DSM_ERR_INVALID, "flow ensembles need d_stress_out (n_chains x 8 floats)");
  if (!(t_end >= 0.0) || t_end * dsm::TICKS >= 9.0e18) return fail(DSM_ERR_INVALID, "t_end out of range");
  if (dsm::table_floats(p->nk) * sizeof(float) + kOffTables > kScratchBytes)
    return fail(DSM_ERR_INVALID, "tables exceed scratch");

  std::lock_guard<std::mutex> lock(g_mu);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(DSM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(DSM_ERR_INVALID, "device index above 63");
  if (g_dev_ptr[dev] == nullptr) {
    // one-time set-up on this device (the current one): device address of the
    // array.  This first call should come before any stream capture.
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(DSM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_dev_ptr[dev] = ptr;
  }
  unsigned char* dbase = (unsigned char*)g_dev_ptr[dev];
  cudaStream_t st = (cudaStream_t)stream;

  // ---- host image: descriptor, prefix, zeroed counters, tables
  const double be = (double)p->beta;
  const dsm::HostPcd pcd = dsm::make_pcd(be, (double)p->nk);
  const float prefact = (float)(pcd.normdt / be);
  std::memset(g_host_stage, 0, kOffTables);
  dsm::TableOffsets to;
  float* htab = (float*)(g_host_stage + kOffTables);
  dsm::make_tables(p->nk, be, prefact, htab, to);
  const float* dtab = (const float*)(dbase + kOffTables);
  dsm::EnsDev E;
  std::memset(&E, 0, sizeof(E));
  E.n_chains = p->n_chains; E.cap = cap; E.nk = p->nk; E.cd_flag = p->cd_flag ? 1 : 0;
  E.flow = flow ? 1 : 0; E.s0 = p->s0 > 0 ? p->s0 : 40; E.poly = 0; E.corr_type = -1;
  E.corr_p = 64; E.corr_m = 8; E.corr_levels = 1;
  E.beta = p->beta; E.prefact = prefact; E.beta_d = be;
  for (int q = 0; q < 9; ++q) E.kap[q] = p->kappa[q];
  E.seed_lo = (uint32_t)p->seed; E.seed_hi = (uint32_t)(p->seed >> 32); E.stream = p->stream;
  E.chain_offset = p->chain_offset;
  E.t_end_ticks = (int64_t)std::llrint(t_end * dsm::TICKS);
  E.step_limit = step_limit < 0 ? INT64_MAX : step_limit;
  // a chain that does 100x the expected events (at least 2^24) stops with
  // stall code 5; the expectation is taken over [0, t_end], since no window
  // start is known here, so for windows that start later the cap is looser
  // than dsm_advance's, which counts from the window start
  const double expect = 0.25 * (double)p->nk * t_end * 100.0;
  E.watchdog_events = (int64_t)(expect > 16777216.0 ? (expect < 9.0e18 ? expect : 9.0e18) : 16777216.0);
  E.pcd = pcd.dev;
  E.NT = (const float4*)(dtab + to.NT); E.NE = (const float4*)(dtab + to.NE);
  E.FRIC = dtab + to.FRIC; E.INV3N = dtab + to.INV3N;
  E.QN = (float4*)d_QN; E.tau = d_tau; E.cs = (dsm::ChainState*)d_state;
  E.out_stress = d_stress_out;
  E.counters = (unsigned long long*)(dbase + kOffCounters);
  std::memcpy(g_host_stage + kOffEns, &E, sizeof(E));
  const long long pre[2] = {0, (long long)p->n_chains};
  std::memcpy(g_host_stage + kOffPrefix, pre, sizeof(pre));
  const size_t bytes = kOffTables + dsm::table_floats(p->nk) * sizeof(float);
  e = cudaMemcpyAsync(dbase, g_host_stage, bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return fail(DSM_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));

  // ---- launch the step kernel on the staged descriptor
  dsm::LaunchCfg cfg;
  cfg.warps_per_block = 4;
  cfg.slot_cap = cap;
  cfg.pmax = 0;
  int sms = 0, optin = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // long chains: fewer warps (chain slots) per block until the block fits
  while (cfg.warps_per_block > 1 && dsm::step_slot_bytes(cap, 0) * cfg.warps_per_block > (size_t)optin)
    cfg.warps_per_block /= 2;
  if (dsm::step_slot_bytes(cap, 0) * cfg.warps_per_block > (size_t)optin)
    return fail(DSM_ERR_INVALID, "z_max does not fit one shared-memory slot");
  const int bps = dsm::step_max_blocks_per_sm(flow, false, cfg);
  if (bps < 1) return fail(DSM_ERR_CUDA, "step kernel cannot be resident");
  const long long want = ((long long)p->n_chains + cfg.warps_per_block - 1) / cfg.warps_per_block;
  const int grid = (int)(want < (long long)bps * sms ? want : (long long)bps * sms);
  e = dsm::launch_step((const dsm::EnsDev*)(dbase + kOffEns), 1, (const long long*)(dbase + kOffPrefix),
                       (long long)p->n_chains, (unsigned int*)(dbase + kOffWork), flow, false, cfg, nullptr,
                       (int*)(dbase + kOffStatus), grid, st);
  if (e != cudaSuccess) return fail(DSM_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
  if (events) {
    unsigned long long cnt = 0;
    e = cudaMemcpyAsync(&cnt, dbase + kOffCounters, sizeof(cnt), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(DSM_ERR_CUDA, std::string("event count: ") + cudaGetErrorString(e));
    *events = cnt;
  }
  return DSM_OK;
}
