// Internal layouts shared by the host runtime (dsm_host.cu) and the sm_103a
// kernels (dsm_kernels.cu).  Not part of the public C ABI (include/dsm.h).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dsm {

constexpr int LIMIT_E = 47;            // fixed-point rate components stay below 2^48
constexpr int S_HYST = 16;             // flow: raise the scale again when 2^16 headroom is free
constexpr double TICKS = 4294967296.0; // chain time unit: 2^-32 tau_K

// Event codes (also folded into the per-chain event hash)
enum Ev : int { CDD = 0, SDP = 1, SDM = 2, CDC_MID = 3, CDC_TAIL = 4, SDC_HEAD = 5,
                SDC_TAIL = 6, SDD_HEAD = 7, SDD_TAIL = 8, NULL_FLAG = 16 };

// Stall / status codes kept per chain (reference: ensemble_kernel.cu:265-270)
enum Stall : int { ST_OK = 0, ST_DT_ZERO = 1, ST_NAN = 2, ST_INF = 3, ST_WATCHDOG = 5 };

// Device form of the lifetime law of a partner chain (gpu_random.cu:78-99)
struct PcdDev {
  float At_, Dt_, Ct_, Adt_, Bdt_, Cdt_, Ddt_, tau_d_inv, one_minus_g;
  float normdt;
  float pad_[2];
};

// Per-chain scalar state, 64 bytes, array of structs in HBM.
struct ChainState {
  int32_t Z;          // strands
  int32_t stall;      // stall code
  int32_t S;          // fixed-point scale exponent of the rate components
  float dt_prev;      // previous dt (flow deformation is applied at the next step)
  int64_t T;          // chain time in ticks (2^-32 tau_K)
  uint64_t step;      // kMC events done by this chain (Philox counter)
  uint64_t hash;      // running FNV-style hash of the event sequence
  int64_t k_next;     // next stress-sample index
  int32_t nk;         // Kuhn steps of this chain
  float r1[3];        // MSD mode: first entanglement in the lab frame (eq_ensemble_kernel.cu:275-277)
};
static_assert(sizeof(ChainState) == 64, "ChainState layout");

// Everything one kernel needs to know about one ensemble (device copy).
struct EnsDev {
  int32_t n_chains, cap, nk, cd_flag;
  int32_t flow, s0, poly, corr_type;
  int32_t corr_p, corr_m, corr_levels, pad0_;
  float beta, prefact;
  double beta_d;
  float kap[9];
  uint32_t seed_lo, seed_hi, stream;
  uint32_t chain_offset;     // global id of local chain 0 (chains sharded over GPUs)
  uint32_t pad_off_;
  int64_t dt_sample_ticks, nsamples;
  // window of the current launch
  int64_t t_end_ticks;       // chains stop when T >= t_end_ticks
  int64_t step_limit;        // ... or when step >= step_limit
  int64_t watchdog_events;   // max events per chain per launch (stall 5 beyond)
  PcdDev pcd;                // monodisperse partner law
  // GEX background (pd_flag = 1): partner N_K = mp/Mk * M/mp from the inverse
  // tables M (SD-created and initial entanglements) and Md (CD-created)
  int32_t gex, gex_n, gex_nd, gex_pad_;
  float gex_step, gex_step_d, gex_scale, gex_pad2_;
  const float* gex_M;
  const float* gex_Md;
  const PcdDev* pcd_by_nk;   // polydisperse: partner law by N_K
  const int32_t* nk_chain;   // polydisperse: N_K of every chain
  // per-N tables: NT[N] = {0.75/(N(N+1)), 0.75/(N(N-1)), (N/(N+1))^0.75, (N/(N-1))^0.75}
  // (sliding-rate factors, ensemble_kernel.cu:153-178); NE[N] = {2/(beta(N+1/2)),
  // 1/(1+N), 1/(3/4+N/2), prefact*(N-1)} (chain-end and CD creation rates,
  // ensemble_kernel.cu:219-260,378); FRIC[i] = 4/i (friction 2/(f1+f2) with
  // i = 2(f1+f2)); INV3N[N] = 3/N
  const float4* NT;
  const float4* NE;
  const float* FRIC;
  const float* INV3N;
  // state (reference layout: float4 {Qx,Qy,Qz,N} x cap per chain; tau rate x cap)
  float4* QN;
  float* tau;
  ChainState* cs;
  // multi-tau correlator per chain: [chain][level][p][3] shift, [chain][level][p]
  // FP64 correlation sums, [chain][level][3] block averages, [chain][level]
  // counters {insert index, block count, values lo, values hi}
  float* corr_shift;
  double* corr_acc;
  float* corr_avg;
  int4* corr_cnt;
  float* out_stress;               // [chain][8] stress at the end of the launch (flow)
  unsigned long long* counters;    // [0] events this launch, [1] chains done
  // flow output series inside one launch (n_win > 0): window w ends at
  // win[w] ticks with event cap win[win_stride + w]; a chain records its stress
  // at each window end in win_stress[w][chain][8] and keeps running; its next
  // window is ChainState::k_next (reset to 0 before the launch)
  const long long* win;
  float* win_stress;
  int32_t n_win, win_stride;
};

constexpr int kCarveMax = 4;  // size classes of one carved launch

struct LaunchCfg {
  int warps_per_block;
  int slot_cap;        // strands per SMEM slot (max cap of the ensembles launched)
  int pmax;            // correlator points per level (max over ensembles)
  int lanes = 32;      // lanes per chain: 32 (one chain per warp) or 16 (two per warp)
};

__host__ __device__ size_t step_slot_bytes(int slot_cap, int pmax);

// Work list of one step launch.  Items are order[0 .. n) (global chain ids
// across the launched ensembles; order == NULL: the identity over [0, total)),
// n = *dyn_total when dyn_total is given.  With defer set, a chain whose
// strand count reaches the slot capacity while its ensemble allows more
// strands stops at that step boundary (state written back exactly as at a
// window end) and its id is appended to defer, for a launch with larger slots.
struct StepList {
  const int* order = nullptr;
  const unsigned int* dyn_total = nullptr;
  int* defer = nullptr;
  unsigned int* n_defer = nullptr;
  // Carved launch (k_step with CARVED, carve_n > 0): several size classes in one
  // launch.  Blocks
  // [carve_blk[k], carve_blk[k+1]) run class k: the block's shared memory
  // holds carve_tiles[k] slots of carve_slot[k] strands (its other tiles stay
  // idle), and its tiles take the items order[carve_first[k] ..
  // carve_first[k] + carve_count[k]) from the work counter carve_work + k.
  int carve_n = 0;
  int carve_blk[kCarveMax + 1] = {};
  int carve_slot[kCarveMax] = {};
  int carve_tiles[kCarveMax] = {};
  int carve_first[kCarveMax] = {};
  int carve_count[kCarveMax] = {};
  unsigned int* carve_work = nullptr;
};

// kernels (dsm_kernels.cu)
// carved launch of equilibrium size classes in 16-lane tiles (lst.carve_*),
// block shared memory smem_bytes; resident blocks per SM of that kernel
cudaError_t launch_step_carved(const EnsDev* d_ens, const long long* d_prefix, int corr, int pmax, size_t smem_bytes,
                               const volatile int* abort_flag, int* d_status, int grid, cudaStream_t st,
                               const StepList& lst);
int step_carved_blocks_per_sm(int corr, size_t smem_bytes);
cudaError_t launch_init(const EnsDev* d_ens, const EnsDev& h_ens, int slot_cap, cudaStream_t st);
// zero the slots a chain does not use (strands >= Z, entanglements >= Z-1)
cudaError_t launch_clear_tail(float4* d_QN, float* d_tau, const ChainState* d_cs, int n_chains, int cap,
                              cudaStream_t st);
// flow output series: point the descriptor at windows d_win[0 .. n) (event
// caps at d_win[stride + w]) and reset every chain's window index
cudaError_t launch_series_begin(EnsDev* d_ens, const long long* d_win, int stride, int n, int n_chains,
                                ChainState* d_cs, cudaStream_t st);
// stress sums of windows 0 .. n of a flow series into out[9 w .. 9 w + 9)
cudaError_t launch_series_reduce(const EnsDev* d_ens, double* out, int n, cudaStream_t st);
cudaError_t launch_step(const EnsDev* d_ens, int n_ens, const long long* d_prefix, long long total,
                        unsigned int* d_work, bool flow, int corr, const LaunchCfg& cfg,
                        const volatile int* abort_flag, int* d_status, int grid, cudaStream_t st,
                        const StepList& lst = StepList{});
// corr: correlator kind, 0 none, 1 stress G(t), 2 centre-of-mass MSD
int step_max_blocks_per_sm(bool flow, int corr, const LaunchCfg& cfg);
size_t step_block_smem(const LaunchCfg& cfg);
cudaError_t launch_gt_reduce_dev(const EnsDev* d_ens, int levels, int p, double* d_gsum, long long* d_count,
                                 cudaStream_t st);
cudaError_t launch_window_begin(EnsDev* d_ens, const long long* d_win, int n, int w, cudaStream_t st);
cudaError_t launch_stress_reduce_dev(const EnsDev* d_ens, double* d_out9, cudaStream_t st);
// stress of every chain from its state in HBM (d_out8: n_chains x 8 floats), then the reduction
cudaError_t launch_state_stress(const EnsDev* d_ens, int n_chains, float* d_out8, double* d_out9, cudaStream_t st);

}  // namespace dsm
