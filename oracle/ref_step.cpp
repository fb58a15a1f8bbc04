// ORACLE — test infrastructure only.  Built by `make ref` from the reference
// tree into oracle/_ref/libdsmrefstep.so; tests/ load it to pin the oracle's
// reference-arithmetic mode (dsm_oracle.cpp, mode 2) against the reference's
// own kernel code.  Nothing in the product links, loads or calls it.
//
// The reference's kMC kernels — strent_kernel, chain_kernel, stress_calc
// (common/ensemble_kernel.cu:114-538) and EQ_strent_kernel, EQ_chain_kernel,
// corr_add, update_correlator (common/eq_ensemble_kernel.cu:50-663) — are
// compiled here unchanged from the reference tree, with oracle/refshim/
// standing in for the CUDA runtime (texture and surface references, thread
// indices, intrinsics).  This file is the host side the reference's
// common/ensemble_call_block.cu would be (that file launches kernels with
// <<<>>> and binds cudaArrays, so it cannot be compiled for the host):
//   * one call block holding every chain, with the reference's arrays: the
//     block's conformations, the two working copies a/b that the kernels
//     ping-pong between, the pair-rate sums, the delayed-dynamics words
//     (d_offset, d_new_strent, d_new_tau_CD), reach flags, dt, the 250-slot
//     stress rings and the per-chain multi-tau correlator
//     (ensemble_call_block.cu:55-104, correlator.cu:29-90);
//   * the step loops of time_step_call_block (:106-222) and
//     EQ_time_step_call_block (:224-379): sync windows of at most 1e5,
//     universal time, parity of steps_count, counter resets every 250 steps,
//     ring drains through update_correlator every 250 steps and at the end;
//   * activate_block / deactivate_block (:533-565);
//   * the ensemble average of corr_function_calc_kernel (correlator.cu:104-144)
//     and the host stress average of calc_stress_call_block (:452-505),
//     restated (both sit behind <<<>>> launches).
// Kernel launches become loops over the launch's thread indices; within one
// kernel the reference's threads never read what another thread writes, so
// the sequential loop gives the GPU's result.
//
// The random textures are bound to hooks that hand out ref_tape.h's stream,
// keyed by the chain's event index (the number of uniforms it has drawn).
//
// One addition for fixed event counts: ref_run's event_limit stops a chain
// after that many kMC steps by setting its reach flag from the host after the
// step that drew its last uniform; its dt is zeroed after the following pass,
// which applies the pending delayed dynamics and the last flow deformation
// (the state a chain has when the kernel itself stops it at a window end).
#include "cuda_runtime.h"  // oracle/refshim: host stand-ins

#include <algorithm>
#include <vector>

#include "correlator.h"       // reference: corr_device, textures_surfaces.h
#include "ensemble_kernel.cu"  // reference kernels (includes eq_ensemble_kernel.cu)
#include "ref_tape.h"

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;
int refshim_error = 0;
// globals the reference's host headers declare (chain.h:30-31,56)
float Be = 1.0f;
int CD_flag = 1;
double universal_time = 0.0;

#define API extern "C" __attribute__((visibility("default")))

namespace {

constexpr int RING = stressarray_count;       // 250 (textures_surfaces.h:23)
constexpr int RANDN = uniformrandom_count;    // 250 (textures_surfaces.h:22)
constexpr double MAX_SYNC = 1e5;               // ensemble_call_block.cu:24

struct Sim {
  int nc = 0, z_max = 0, nk = 0, eq = 1, corr_type = 0, p = 64, m = 8, levels = 1, res = 1;
  reftape::Key key{};
  reftape::Law law{};
  // block arrays and the working copies (ensemble_call_block.cu:26-45)
  std::vector<float4> qn_blk, qn_a, qn_b;
  std::vector<float> tcd_blk, tcd_a, tcd_b, sum_w;
  std::vector<chain_head> heads;
  std::vector<float> dt, reach;
  std::vector<int> offset;
  std::vector<float4> new_strent, r1;
  std::vector<float> new_tau;
  std::vector<int> rand_used, used_cd, used_sd, corr_time;
  std::vector<float4> ring_a, ring_b;  // [RING][nc]
  std::vector<float4> stress_buf;      // [nc][2]
  // correlator (correlator.cu:29-90): [nc][levels][p] and [nc][levels]
  std::vector<float4> c_shift, c_corr, c_acc, c_accval;
  std::vector<float> c_ncorr;
  std::vector<int> c_nacc, c_ins, c_kmax;
  int ci_nc = 0, ci_levels = 0, ci_dmin = 0, ci_p = 0, ci_m = 0;
  corr_device gc{};
  // harness bookkeeping
  std::vector<int64_t> events;  // uniforms drawn per chain
  int steps_count = 0;
  double block_time = 0.0;
};

Sim* cur = nullptr;  // the reference's state is process-global; one block is active

float hook_uniform(int, int chain) {
  return reftape::uniform(cur->key, (uint64_t)cur->events[chain]++, (uint32_t)chain);
}
float4 hook_create(int chain, bool cd) {
  float v[4];
  reftape::creation(cur->key, cur->law, (uint64_t)(cur->events[chain] - 1), (uint32_t)chain, cd, v);
  return make_float4(v[0], v[1], v[2], v[3]);
}
float4 hook_cd(int, int chain) { return hook_create(chain, true); }
float4 hook_sd(int, int chain) { return hook_create(chain, false); }

template <class T>
void bind_tex(texture<T, 2, cudaReadModeElementType>& t, const std::vector<T>& a, int w, int h) {
  t.data = a.data();
  t.width = w;
  t.height = h;
  t.hook = nullptr;
}
template <class T>
void bind_surf(surface<void, 2>& s, std::vector<T>& a, int w, int h) {
  s.data = reinterpret_cast<unsigned char*>(a.data());
  s.width_bytes = w * (int)sizeof(T);
  s.height = h;
}

// the reference's __constant__ parameters and the random textures
void set_globals(Sim& S) {
  cur = &S;
  dn_cha_per_call = S.nc;
  d_z_max = S.z_max;
  dnk = S.nk;
  d_correlator_res = S.res;
  t_uniformrand.hook = hook_uniform;
  t_taucd_gauss_rand_CD.hook = hook_cd;
  t_taucd_gauss_rand_SD.hook = hook_sd;
  bind_surf(s_sum_W, S.sum_w, S.z_max, S.nc);
  s_stress.data = reinterpret_cast<unsigned char*>(S.stress_buf.data());
  s_stress.width_bytes = S.nc * 32;
  s_stress.height = 1;
}

void launch_strent(Sim& S) {
  blockDim = dim3(1, 1, 1);
  threadIdx = uint3{0, 0, 0};
  for (int j = 0; j < S.nc; ++j)
    for (int i = 0; i < S.z_max; ++i) {
      blockIdx = uint3{(unsigned)i, (unsigned)j, 0};
      if (S.eq) EQ_strent_kernel(S.heads.data(), S.offset.data(), S.new_strent.data(), S.new_tau.data());
      else strent_kernel(S.heads.data(), S.dt.data(), S.offset.data(), S.new_strent.data(), S.new_tau.data());
    }
}

void launch_chain(Sim& S, float sync_interval) {
  blockDim = dim3(1, 1, 1);
  threadIdx = uint3{0, 0, 0};
  for (int i = 0; i < S.nc; ++i) {
    blockIdx = uint3{(unsigned)i, 0, 0};
    if (S.eq)
      EQ_chain_kernel(S.heads.data(), S.dt.data(), S.reach.data(), sync_interval, S.offset.data(),
                      S.new_strent.data(), S.new_tau.data(), S.corr_time.data(), S.corr_type, S.rand_used.data(),
                      S.used_cd.data(), S.used_sd.data(), S.steps_count % RING, S.r1.data());
    else
      chain_kernel(S.heads.data(), S.dt.data(), S.reach.data(), sync_interval, S.offset.data(), S.new_strent.data(),
                   S.new_tau.data(), S.rand_used.data(), S.used_cd.data(), S.used_sd.data());
  }
}

void launch_update_correlator(Sim& S, int n) {
  blockDim = dim3(1, 1, 1);
  threadIdx = uint3{0, 0, 0};
  for (int i = 0; i < S.nc; ++i) {
    blockIdx = uint3{(unsigned)i, 0, 0};
    update_correlator(S.gc, n, S.corr_type);
  }
}

// one step of the loop body: bind by parity, strand pass, chain pass
void one_pass(Sim& S, float sync_interval, bool texture_flag) {
  const bool even = !(S.steps_count & 1);
  std::vector<float4>& qa = even ? S.qn_a : S.qn_b;
  std::vector<float4>& qb = even ? S.qn_b : S.qn_a;
  std::vector<float>& ta = even ? S.tcd_a : S.tcd_b;
  std::vector<float>& tb = even ? S.tcd_b : S.tcd_a;
  bind_tex(t_a_QN, qa, S.z_max, S.nc);
  bind_surf(s_b_QN, qb, S.z_max, S.nc);
  bind_tex(t_a_tCD, ta, S.z_max, S.nc);
  bind_surf(s_b_tCD, tb, S.z_max, S.nc);
  if (S.eq) bind_surf(s_corr, texture_flag ? S.ring_b : S.ring_a, S.nc, RING);
  launch_strent(S);
  launch_chain(S, sync_interval);
}

void activate(Sim& S) {  // ensemble_call_block.cu:533-553
  d_universal_time = (float)S.block_time;
  if (!(S.steps_count & 1)) { S.qn_a = S.qn_blk; S.tcd_a = S.tcd_blk; }
  else { S.qn_b = S.qn_blk; S.tcd_b = S.tcd_blk; }
}
void deactivate(Sim& S) {  // ensemble_call_block.cu:555-565
  if (!(S.steps_count & 1)) { S.qn_blk = S.qn_a; S.tcd_blk = S.tcd_a; }
  else { S.qn_blk = S.qn_b; S.tcd_blk = S.tcd_b; }
}

void refill(Sim& S) {  // random_textures_refill (ensemble.cu:265-287): counters restart
  std::fill(S.rand_used.begin(), S.rand_used.end(), 0);
  std::fill(S.used_cd.begin(), S.used_cd.end(), 0);
  std::fill(S.used_sd.begin(), S.used_sd.end(), 0);
}

void drain(Sim& S, bool& texture_flag, int n) {  // ensemble_call_block.cu:329-341,358-370
  bind_tex(t_corr, texture_flag ? S.ring_b : S.ring_a, S.nc, RING);
  texture_flag = !texture_flag;
  launch_update_correlator(S, n);
}

}  // namespace

extern "C" {
typedef struct ref_params {
  int32_t n_chains, nk, z_max, cd_flag;
  float beta, prefact;      // dBe, d_CD_create_prefact (ensemble.cu:123,136-150)
  float kappa[9];           // d_kappa_xx .. d_kappa_zz, row-major
  int32_t eq;               // 1: EQ_* kernels with the correlator, 0: flow kernels
  int32_t corr_type;        // 0 stress G(t), 1 centre-of-mass MSD
  int32_t corr_p, corr_m, corr_levels, corr_res;  // correlator size, averaging, levels, sample interval
  uint64_t seed;
  uint32_t stream, chain_offset;
  double law[9];            // c1, At, tau0, alpha, normdt, Adt, Bdt, tau_d, g
} ref_params;
}

API void* ref_create(const ref_params* p) {
  Sim* S = new Sim();
  S->nc = p->n_chains;
  S->nk = p->nk;
  S->z_max = p->z_max > 0 ? p->z_max : p->nk;
  S->eq = p->eq;
  S->corr_type = p->corr_type;
  S->p = p->corr_p;
  S->m = p->corr_m;
  S->levels = p->corr_levels > 0 ? p->corr_levels : 1;
  S->res = p->corr_res > 0 ? p->corr_res : 1;
  S->key = reftape::Key{p->seed, p->stream, p->chain_offset};
  S->law = reftape::Law{p->law[0], p->law[1], p->law[2], p->law[3], p->law[4],
                        p->law[5], p->law[6], p->law[7], p->law[8]};
  Be = p->beta;
  CD_flag = p->cd_flag;
  dBe = p->beta;
  d_CD_flag = p->cd_flag;
  d_CD_create_prefact = p->prefact;
  d_kappa_xx = p->kappa[0]; d_kappa_xy = p->kappa[1]; d_kappa_xz = p->kappa[2];
  d_kappa_yx = p->kappa[3]; d_kappa_yy = p->kappa[4]; d_kappa_yz = p->kappa[5];
  d_kappa_zx = p->kappa[6]; d_kappa_zy = p->kappa[7]; d_kappa_zz = p->kappa[8];
  const size_t n = S->nc, zc = (size_t)S->nc * S->z_max;
  S->qn_blk.assign(zc, float4{0, 0, 0, 0});
  S->qn_a = S->qn_blk;
  S->qn_b = S->qn_blk;
  S->tcd_blk.assign(zc, 0.0f);
  S->tcd_a = S->tcd_blk;
  S->tcd_b = S->tcd_blk;
  S->sum_w.assign(zc, 0.0f);
  S->heads.assign(n, chain_head{0, 0.0f, 0.0f, 0});
  S->dt.assign(n, 0.0f);
  S->reach.assign(n, 0.0f);
  S->offset.assign(n, -1);
  S->new_strent.assign(n, float4{0, 0, 0, 0});
  S->r1.assign(n, float4{0, 0, 0, 0});
  S->new_tau.assign(n, 0.0f);
  S->rand_used.assign(n, 0);
  S->used_cd.assign(n, 0);
  S->used_sd.assign(n, 0);
  S->corr_time.assign(n, 0);
  S->ring_a.assign((size_t)RING * n, float4{0, 0, 0, 0});
  S->ring_b = S->ring_a;
  S->stress_buf.assign(2 * n, float4{0, 0, 0, 0});
  const size_t cl = n * S->levels;
  S->c_shift.assign(cl * S->p, float4{0, 0, 0, 0});
  S->c_corr = S->c_shift;
  S->c_ncorr.assign(cl * S->p, 0.0f);
  S->c_acc.assign(cl, float4{0, 0, 0, 0});
  S->c_nacc.assign(cl, 0);
  S->c_ins.assign(cl, 0);
  S->c_kmax.assign(n, 0);
  S->c_accval.assign(n, float4{0, 0, 0, 0});
  S->ci_nc = S->nc;
  S->ci_levels = S->levels;
  S->ci_dmin = S->p / S->m;
  S->ci_p = S->p;
  S->ci_m = S->m;
  corr_device& g = S->gc;
  g.d_correlator = nullptr;
  g.d_nc = &S->ci_nc;
  g.d_numcorrelators = &S->ci_levels;
  g.d_dmin = &S->ci_dmin;
  g.d_correlator_size = &S->ci_p;
  g.d_correlator_aver_size = &S->ci_m;
  g.d_shift = cudaPitchedPtr{S->c_shift.data(), (size_t)S->p * sizeof(float4), (size_t)S->p * sizeof(float4),
                             (size_t)S->levels};
  g.d_correlation = cudaPitchedPtr{S->c_corr.data(), (size_t)S->p * sizeof(float4),
                                   (size_t)S->p * sizeof(float4), (size_t)S->levels};
  g.d_ncorrelation = cudaPitchedPtr{S->c_ncorr.data(), (size_t)S->p * sizeof(float),
                                    (size_t)S->p * sizeof(float), (size_t)S->levels};
  g.d_accumulator = S->c_acc.data();
  g.d_accumulator_pitch = (size_t)S->levels * sizeof(float4);
  g.d_naccumulator = S->c_nacc.data();
  g.d_naccumulator_pitch = (size_t)S->levels * sizeof(int);
  g.d_insertindex = S->c_ins.data();
  g.d_insertindex_pitch = (size_t)S->levels * sizeof(int);
  g.d_kmax = S->c_kmax.data();
  g.d_accval = S->c_accval.data();
  S->events.assign(n, 0);
  return S;
}

API void ref_destroy(void* h) {
  if (cur == h) cur = nullptr;
  delete (Sim*)h;
}

// Chains in the reference layout (chain.h:37-53): n*z_max float4 {Qx,Qy,Qz,N},
// n*z_max lifetime rates, optional n float4 R1.  Restarts clocks, counters,
// delayed dynamics and correlators (init_call_block, get_chain_to_device_call_block,
// gpu_Gt_PCS's reset of d_correlator_time).
API int ref_set_chains(void* h, const int32_t* Z, const float* QN, const float* tau, const float* R1) {
  Sim& S = *(Sim*)h;
  const size_t zc = (size_t)S.nc * S.z_max;
  std::memcpy(S.qn_blk.data(), QN, zc * sizeof(float4));
  std::memcpy(S.tcd_blk.data(), tau, zc * sizeof(float));
  for (int i = 0; i < S.nc; ++i) {
    S.heads[i] = chain_head{Z[i], 0.0f, 0.0f, 0};
    S.r1[i] = R1 ? make_float4(R1[4 * i], R1[4 * i + 1], R1[4 * i + 2], R1[4 * i + 3]) : make_float4(0, 0, 0, 0);
  }
  std::fill(S.dt.begin(), S.dt.end(), 0.0f);
  std::fill(S.offset.begin(), S.offset.end(), -1);
  std::fill(S.events.begin(), S.events.end(), 0);
  std::fill(S.corr_time.begin(), S.corr_time.end(), 0);
  refill(S);
  S.steps_count = 0;
  S.block_time = 0.0;
  return 0;
}

// Advance every chain to reach_time as the reference's step loops do; with
// event_limit >= 0 a chain also stops after that many kMC steps (uniforms).
// Returns 0, or the first out-of-range surface access code.
API int ref_run(void* h, double reach_time, int64_t event_limit) {
  Sim& S = *(Sim*)h;
  set_globals(S);
  refshim_error = 0;
  std::vector<int> lim(S.nc, 0);  // 0 running, 1 stopped (flush pass due), 2 stopped and flushed
  if (event_limit >= 0)
    for (int i = 0; i < S.nc; ++i)
      if (S.events[i] >= event_limit) lim[i] = 2;
  bool texture_flag = true;
  if (S.eq) S.steps_count = 0;  // EQ_time_step_call_block:241
  activate(S);
  const float interval = (float)(reach_time - S.block_time);
  const int nsync = int(std::floor((interval - 0.5) / MAX_SYNC)) + 1;
  for (int is = 0; is < nsync; ++is) {
    float sync_interval = (float)MAX_SYNC;
    if (is + 1 == nsync) sync_interval = interval - is * MAX_SYNC;
    std::fill(S.reach.begin(), S.reach.end(), 0.0f);
    d_universal_time = (float)(S.block_time + is * MAX_SYNC);
    for (int i = 0; i < S.nc; ++i)
      if (lim[i]) S.reach[i] = 1.0f;
    for (;;) {
      one_pass(S, sync_interval, texture_flag);
      S.steps_count++;
      if (S.steps_count % RANDN == 0) {
        refill(S);
        S.steps_count = 0;
      }
      if (S.eq && S.steps_count % RING == 0) drain(S, texture_flag, RING);
      bool pending = false;
      if (event_limit >= 0) {
        for (int i = 0; i < S.nc; ++i)
          if (lim[i] == 1) { S.dt[i] = 0.0f; lim[i] = 2; }
        for (int i = 0; i < S.nc; ++i)
          if (lim[i] == 0 && S.events[i] >= event_limit) { S.reach[i] = 1.0f; lim[i] = 1; pending = true; }
      }
      float sumrt = 0.0f;
      for (int i = 0; i < S.nc; ++i) sumrt += S.reach[i];
      if (sumrt == (float)S.nc && !pending) break;
    }
  }
  if (S.eq && S.steps_count % RING != 0) drain(S, texture_flag, S.steps_count);
  S.block_time = reach_time;
  deactivate(S);
  return refshim_error;
}

// State after a run (no delayed dynamics are pending once every chain has
// stopped): Z, conformations, rates, clocks, stall flags, uniforms drawn,
// R1 and sample counters; any pointer may be null.
API int ref_get_chains(void* h, int32_t* Z, float* QN, float* tau, float* time, int32_t* stall, int64_t* events,
                       float* R1, int32_t* corr_time) {
  Sim& S = *(Sim*)h;
  const size_t zc = (size_t)S.nc * S.z_max;
  if (QN) std::memcpy(QN, S.qn_blk.data(), zc * sizeof(float4));
  if (tau) std::memcpy(tau, S.tcd_blk.data(), zc * sizeof(float));
  for (int i = 0; i < S.nc; ++i) {
    if (Z) Z[i] = S.heads[i].Z;
    if (time) time[i] = S.heads[i].time;
    if (stall) stall[i] = S.heads[i].stall_flag;
    if (events) events[i] = S.events[i];
    if (R1) { R1[4 * i] = S.r1[i].x; R1[4 * i + 1] = S.r1[i].y; R1[4 * i + 2] = S.r1[i].z; R1[4 * i + 3] = S.r1[i].w; }
    if (corr_time) corr_time[i] = S.corr_time[i];
  }
  return 0;
}

// stress_calc over the block (ensemble_kernel.cu:504-538) and the host average
// of calc_stress_call_block (ensemble_call_block.cu:471-502): float sums over
// chains that are not stalled and not NaN.  out = xx yy zz xy yz zx Lpp Z.
API int ref_stress(void* h, double* out, int32_t* count) {
  Sim& S = *(Sim*)h;
  set_globals(S);
  refshim_error = 0;
  bind_tex(t_a_QN, S.qn_blk, S.z_max, S.nc);
  blockDim = dim3(1, 1, 1);
  threadIdx = uint3{0, 0, 0};
  for (int i = 0; i < S.nc; ++i) {
    blockIdx = uint3{(unsigned)i, 0, 0};
    stress_calc(S.heads.data(), S.dt.data(), S.offset.data(), S.new_strent.data());
  }
  float4 s1 = make_float4(0, 0, 0, 0), s2 = make_float4(0, 0, 0, 0);
  int cnt = S.nc;
  for (int j = 0; j < S.nc; ++j) {
    if (S.heads[j].stall_flag == 0 && !std::isnan(S.stress_buf[2 * j].x)) {
      s1.x += S.stress_buf[2 * j].x; s1.y += S.stress_buf[2 * j].y;
      s1.z += S.stress_buf[2 * j].z; s1.w += S.stress_buf[2 * j].w;
      s2.x += S.stress_buf[2 * j + 1].x; s2.y += S.stress_buf[2 * j + 1].y;
      s2.z += S.stress_buf[2 * j + 1].z; s2.w += S.stress_buf[2 * j + 1].w;
    } else {
      cnt--;
    }
  }
  const float v[8] = {s1.x / cnt, s1.y / cnt, s1.z / cnt, s1.w / cnt, s2.x / cnt, s2.y / cnt, s2.z / cnt, s2.w / cnt};
  for (int q = 0; q < 8; ++q) out[q] = v[q];
  if (count) *count = cnt;
  return refshim_error;
}

// Ensemble correlation of corr_function_calc_kernel (correlator.cu:104-144):
// corr[k*p + j] = sum over chains of (C.x + C.y + C.z) / count in float, lag
// j * m^k; entries k > 0, j < p/m stay 0.  ncorr0 = chain 0's counts.
API int ref_gt(void* h, float* corr, float* lag, float* ncorr0) {
  Sim& S = *(Sim*)h;
  const int L = S.levels, p = S.p;
  for (int k = 0; k < L; ++k)
    for (int j = 0; j < p; ++j) {
      corr[k * p + j] = 0.0f;
      if (lag) lag[k * p + j] = 0.0f;
      if (ncorr0) ncorr0[k * p + j] = S.c_ncorr[(size_t)k * p + j];
      if (k > 0 && j < S.ci_dmin) continue;
      if (lag) lag[k * p + j] = (float)j * powf((float)S.m, (float)k);
      float st = 0.0f;
      for (int n = 0; n < S.nc; ++n) {
        const size_t o = ((size_t)n * L + k) * p + j;
        const float4 e = S.c_corr[o];
        const float w = S.c_ncorr[o];
        if (w > 0) st += __fdividef(e.x + e.y + e.z, w);
      }
      corr[k * p + j] = st;
    }
  return 0;
}
