/*
 * gpu_dsm_gb300 — C ABI of the GB300-native Discrete Slip-Link Model (DSM)
 * kinetic Monte Carlo simulator.
 *
 * Every entry point is extern "C" with plain pointers and sizes.  Host arrays
 * use the reference's own layouts (ktaletsk/gpu_dsm):
 *   - chain_head  {int Z; float time; float dummy; int stall_flag}  common/chain.h:45-53
 *   - QN          n_chains * z_max float4 {Qx, Qy, Qz, N}            common/chain.h:37-42,
 *                                                                    common/ensemble.cu:79-104
 *   - tau_CD      n_chains * z_max float (rates 1/tau_CD)            common/chain.cu:243-246
 *   - stress_plus {xx, yy, zz, xy, yz, zx, Lpp, Z}                   common/stress.h:23-29
 * Status codes replace the reference's exit(-1) on CUDA errors
 * (common/cuda_call.h:42-49); -1 keeps its meaning "aborted by run_flag".
 */
#ifndef GPU_DSM_GB300_DSM_H
#define GPU_DSM_GB300_DSM_H

#include <stdint.h>

#ifdef __cplusplus
#define DSM_BOOL bool
extern "C" {
#else
#define DSM_BOOL _Bool
#endif

#define DSM_OK 0
#define DSM_ABORTED (-1)        /* run_flag cleared (ensemble_call_block.cu:214,353) */
#define DSM_ERR_CUDA (-2)       /* CUDA runtime error (reference: exit(-1)) */
#define DSM_ERR_INVALID (-3)    /* invalid argument / input */
#define DSM_ERR_MEMORY (-4)     /* device memory budget exceeded */
#define DSM_ERR_WATCHDOG (-5)   /* a chain exceeded the per-launch event cap */
#define DSM_ERR_NOT_BUILT (-6)  /* library built without the CUDA kernels */
#define DSM_PENDING 1           /* dsm_poll: the asynchronous advance is still running */

typedef struct dsm_float4 { float x, y, z, w; } dsm_float4;

/* chain_head of the reference, same field order and size (16 bytes) */
typedef struct dsm_chain_head {
  int32_t Z;
  float time;
  float dummy;
  int32_t stall_flag;
} dsm_chain_head;

/* stress_plus of the reference (32 bytes) */
typedef struct dsm_stress_plus {
  float xx, yy, zz, xy, yz, zx, Lpp, Z;
} dsm_stress_plus;

/*
 * Simulation parameters.  The first block is the reference's input.dat
 * (common/main_cuda.cu:55-68, CLI/input.dat:1-22); the rest are the
 * reference's compile-time constants made runtime knobs.
 */
typedef struct dsm_params {
  float beta;              /* input.dat 1: entanglement activity */
  int32_t nk;              /* input.dat 2: Kuhn steps per chain (max for polydisperse) */
  int32_t n_chains;        /* input.dat 3 */
  float kappa[9];          /* input.dat 4: transpose of the velocity gradient, row-major */
  int32_t cd_flag;         /* input.dat 5: 0 SD only, 1 SD+CD */
  int32_t pd_flag;         /* input.dat 6: 1 = GEX background polydispersity (gex_* below) */
  int32_t eq_type;         /* input.dat 7: 1 G(t), 2 MSD(t); other values: no correlator */
  double sync_dt;          /* input.dat 8: sync / sample interval (tau_K) */
  double t_end;            /* input.dat 9: total simulation time (tau_K) */
  uint64_t seed;           /* job_ID: Philox key */
  int32_t device;          /* CUDA device (-d) */
  int32_t z_max;           /* strand capacity per chain; 0 = nk (ensemble.cu:99) */
  int32_t corr_p;          /* correlator points per level; 0 = 64 (correlator.h:21) */
  int32_t corr_m;          /* correlator averaging; 0 = 8 (correlator.h:22) */
  int32_t corr_levels;     /* 0 = ceil(log(t_end/sync_dt/p)/log m)+1 (main_cuda.cu:70) */
  uint32_t stream;         /* Philox counter word 3 (ensemble id) */
  const int32_t* nk_chain; /* per-chain N_K (polydisperse melt) or NULL */
  int32_t warps_per_block; /* step-kernel block size in warps; 0 = autotuned */
  int32_t s0;              /* initial fixed-point scale exponent; 0 = 40 */
  int32_t lanes_per_chain; /* 32: one chain per warp, 16: two chains per warp; 0 = auto */
  int32_t stream_priority; /* CUDA priority of the handle's streams (0 = default; lower
                              values are scheduled first, clamped to the device's range) */
  float gex_a, gex_b;      /* pd_flag = 1: polydisp.dat a, b of the GEX background law */
  float gex_mp, gex_mk;    /* polydisp.dat mp (mass scale) and Mk (Kuhn-step mass) */
  uint32_t chain_offset;   /* global id of chain 0 when an ensemble is sharded over GPUs:
                              random streams are keyed by global chain id */
  int32_t pad2_;
} dsm_params;

typedef struct dsm_sim dsm_sim;

/* Lifecycle.  Replaces gpu_init/gpu_clean (common/ensemble.cu:118-208,506-539)
 * with an owning handle instead of process globals. */
int dsm_create(const dsm_params* params, dsm_sim** out);
void dsm_destroy(dsm_sim* sim);
const char* dsm_last_error(const dsm_sim* sim);

/* Equilibrium initial state on the device, keyed by (seed, chain).
 * Replaces host_chains_init/chain_init (common/ensemble.cu:106-115,
 * common/chain.cu:199-283). */
int dsm_init_equilibrium(dsm_sim* sim);

/* Host <-> device conformations in the reference layout.  Replace
 * get_chain_to_device_call_block / get_chain_from_device_call_block
 * (common/ensemble_call_block.cu:402-450) and get_chains_from_device
 * (common/ensemble.cu:231-236).  On set, heads[i].time is the chain time,
 * stall_flag the stall code; pending flow dt, event counters and correlator
 * state are reset. */
int dsm_set_chains(dsm_sim* sim, const dsm_chain_head* heads, const dsm_float4* QN, const float* tau);
int dsm_get_chains(dsm_sim* sim, dsm_chain_head* heads, dsm_float4* QN, float* tau);

/* Extended per-chain scalars (time in 2^-32 tau_K ticks, event counter,
 * pending flow dt, stall code, fixed-point scale, event-sequence hash).
 * Any pointer may be NULL. */
int dsm_get_ext(dsm_sim* sim, int64_t* time_ticks, uint64_t* steps, float* dt_prev, int32_t* stall,
                int32_t* scale, uint64_t* hash);
int dsm_set_ext(dsm_sim* sim, const int64_t* time_ticks, const uint64_t* steps, const float* dt_prev,
                const int32_t* stall, const int32_t* scale);

/* Advance every chain until its time reaches t_end (tau_K), or it has done
 * step_limit events in total (step_limit < 0: no limit).  Replaces
 * time_step_call_block / EQ_time_step_call_block
 * (common/ensemble_call_block.cu:106-379) and gpu_time_step
 * (common/ensemble.cu:223-229).  abort_flag: host int polled by the running
 * kernel (mapped memory), non-zero aborts with DSM_ABORTED; may be NULL.
 * events (may be NULL) receives the number of kMC events done. */
int dsm_advance(dsm_sim* sim, double t_end, int64_t step_limit, const volatile int32_t* abort_flag,
                uint64_t* events);

/* Advance through n windows of dt tau_K from the current time (window w ends
 * at t + dt*(w+1), the times dsm_advance calls would use) as one CUDA graph
 * launch, captured on the first call for this n and launch schedule and
 * replayed afterwards (with size classes the same launches are issued
 * directly, with no host synchronisation between windows).  Flow ensembles: out[w] (n entries, may be NULL)
 * receives the stress at the end of window w, as dsm_stress would after each
 * window.  Replaces the host loop of time_step_call_block +
 * calc_stress_call_block per output time (common/main_cuda.cu flow loop,
 * common/ensemble_call_block.cu:106-379,452-505). */
int dsm_advance_series(dsm_sim* sim, double dt, int32_t n, const volatile int32_t* abort_flag,
                       dsm_stress_plus* out, uint64_t* events);

/* Asynchronous forms: enqueue a window (dsm_advance_start) or windows ending
 * at t_ends[0..n) (ascending; dsm_series_start, one graph replay as in
 * dsm_advance_series) on the handle's own stream and return at once; dsm_poll
 * returns DSM_PENDING while it runs and, once done, the events, the stress
 * (flow: 1 entry for a window, n for a series; may be NULL) with *n_out its
 * count, and the status dsm_advance / dsm_advance_series would have returned.
 * One asynchronous advance per handle at a time; handles on the same GPU run
 * concurrently.  dsm_abort sets the handle's abort word (the running kernels
 * stop within 4096 events per chain; dsm_poll then returns DSM_ABORTED). */
int dsm_advance_start(dsm_sim* sim, double t_end, int64_t step_limit);
int dsm_series_start(dsm_sim* sim, const double* t_ends, int32_t n);
int dsm_poll(dsm_sim* sim, uint64_t* events, dsm_stress_plus* out, int32_t* n_out);
int dsm_abort(dsm_sim* sim);
/* Move an idle handle to streams of another CUDA priority (lower values are
 * scheduled first; clamped to the device's range).  Used by the serving loop
 * to favour older requests. */
int dsm_set_priority(dsm_sim* sim, int32_t priority);

/* Advance n ensembles (same device) to their own t_end[i] / step_limit[i]
 * (step_limit may be NULL) in one persistent launch per kind (equilibrium,
 * equilibrium with G(t), flow).  No counterpart in the reference, which runs
 * one ensemble per process; used for multi-condition runs (several flow
 * rates) and by the serving loop.  When every ensemble of a launch planned a
 * small-slot class, the launch uses the smallest of those slots and the chains
 * that outgrow it finish in an overflow launch with full-capacity slots.
 * events[i] (may be NULL) receives the kMC events of ensemble i.  Results
 * equal per-ensemble dsm_advance calls. */
int dsm_advance_batch(dsm_sim** sims, int32_t n, const double* t_end, const int64_t* step_limit,
                      uint64_t* events);

/* Ensemble-average stress of the current state over non-stalled chains
 * (the flow output; for equilibrium ensembles evaluated from the current
 * state on call).  Replaces calc_stress / calc_stress_call_block
 * (common/ensemble.cu:210-221, common/ensemble_call_block.cu:452-505). */
int dsm_stress(dsm_sim* sim, dsm_stress_plus* out, int32_t* chain_count);

/* Stress relaxation G(t) as written to G.dat by gpu_Gt_PCS
 * (common/ensemble.cu:289-339, common/correlator.cu:146-187): t in sample
 * units, G averaged over xy/yz/xz and chains.  n: in = capacity, out = points. */
int dsm_gt(dsm_sim* sim, float* t, float* G, int32_t* n);
/* Raw correlator sums: gsum[k*p+j] = sum over chains of C/count, count of chain 0 */
/* eq_type = 2 (MSD mode, main_cuda.cu:79-82): dsm_gt returns MSD(t), the
 * centre-of-mass mean-square displacement, written to MSD[_id].dat by
 * main_cuda.  dsm_get_r1: position of every chain's first entanglement in the
 * lab frame (n_chains x 3 floats), the MSD reference point
 * (eq_ensemble_kernel.cu:275-277,447-653). */
int dsm_get_r1(dsm_sim* sim, float* r1);
int dsm_gt_raw(dsm_sim* sim, double* gsum, int64_t* count);

/* Device time (CUDA events on the launching stream) and kMC events of the
 * step kernel of the last dsm_advance, plus its launch shape. */
int dsm_last_window(const dsm_sim* sim, float* kernel_ms, uint64_t* events, int32_t* grid,
                    int32_t* blocks_per_sm);

/* Constraint-dynamics lifetime law p_cd(beta, N_K) of common/pcd_tau.h:26-66:
 * out[0..5] = alpha, tau_0, tau_max, tau_d, g, normdt (tau_K units).  tau_d is
 * the disentanglement time the GUI uses to turn a Weissenberg number into a
 * shear rate, kappa_xy = Wi / tau_d (GUI/mainwindow.cpp:836). */
int dsm_pcd(double beta, int32_t nk, double* out);

/* Launch schedule of a polydisperse ensemble whose longest chains do not fit
 * a full-occupancy shared-memory slot.  Chains are sorted by N_K and split in
 * two size classes run as concurrent persistent launches: small slots
 * (small_slot strands, 4 warps per block) and one warp per block with slots
 * for the longest chains (large_grid blocks); a chain that outgrows its slot
 * stops at a step boundary and finishes in a third launch with slots of the
 * full capacity.  A chain goes to the small class when the mean of its
 * equilibrium strand count plus z_margin_sd standard deviations fits the
 * small slot.  Results do not depend on the schedule (state, flow stress and
 * G(t) to the bit; the MSD centre-of-mass sums to rounding).  Arguments <= 0 choose
 * the defaults (largest slot with 4 blocks per SM; large-class blocks in
 * proportion to its share of the work; lanes of the handle; 5 sd).  No
 * counterpart in the reference (one thread per chain, ensemble_kernel.cu). */
int dsm_set_schedule(dsm_sim* sim, int32_t small_slot, int32_t large_grid, int32_t lanes, float z_margin_sd);
/* Current schedule: n_classes (0 = one launch over all chains), then per
 * class {slot strands, warps per block, lanes, grid, chains} in info[5*i..]
 * (info holds DSM_SCHEDULE_INFO = 25 ints: up to four classes -- huge, large,
 * middle, small -- and the overflow launch, which has no fixed chain count). */
#define DSM_SCHEDULE_INFO 25
int dsm_get_schedule(const dsm_sim* sim, int32_t* n_classes, int32_t* info);

/* How size classes launch (equilibrium ensembles whose small class runs 16
 * lanes per chain).  form 0 (default): each class its own persistent launch,
 * the four launched concurrently on four streams.  form 1: the large, middle
 * and small classes in one launch whose blocks carve the same shared memory
 * into per-class slot counts (8 small, about 4 middle, 2 large slots per
 * block, all in 16-lane tiles), the huge class beside it on its stream.
 * Trajectories do not depend on the form.  The plan is made again; a form
 * that does not apply leaves the concurrent launches.  dsm_get_class_form
 * reports the form of the current plan. */
int dsm_set_class_form(dsm_sim* sim, int32_t form);
int dsm_get_class_form(const dsm_sim* sim, int32_t* form);

/* Autotuner (online): runs one real window of `window` tau_K with each
 * candidate schedule (lanes per chain 32/16; the small slot at 4/3/2 blocks per
 * SM when the strand-count bound fits it; for polydisperse ensembles the
 * large-class grid at 1/2, 1 and 2 times its default, and with 16 lanes each
 * small slot also in the carved one-launch form of dsm_set_class_form) and
 * keeps the one with
 * the most kMC events per kernel millisecond; a change of lanes per chain must
 * win by 3 % (32 lanes over the best 16-lane schedule; 16 lanes within 3 % of
 * the best 32-lane one), since trial windows resolve tile widths only
 * coarsely.  The ensemble advances by
 * candidates x window; its trajectory is the one it would have had without
 * the autotuner.  best (may be NULL) receives {small_slot, large_grid, lanes,
 * candidates}; best_ms the winner's kernel time.  No counterpart in the
 * reference (fixed launch shapes). */
int dsm_autotune(dsm_sim* sim, double window, int32_t* best, float* best_ms);

/* Counters of the last window: kMC events, chains that completed the window
 * in their first slot, chains moved to a larger slot on the way. */
int dsm_window_stats(const dsm_sim* sim, uint64_t* events, uint64_t* chains_done, uint64_t* deferred);

/* GEX background molecular-weight tables of a polydisperse melt
 * (polydisp.dat "a b mp Mk", common/gamma.cpp:174-263): m[0..n) = M/mp at
 * cumulative probabilities j*step, md[0..n_d) the same for the law weighted by
 * the partner's mean CD destruction rate; info = {step, step_d, CD creation
 * prefactor}.  n, n_d: in = capacities, out = sizes.  Host only. */
int dsm_gex_table(float a, float b, float mp, float mk, double beta, float* m, int32_t* n, float* md,
                  int32_t* n_d, double* info);

/* Correlator geometry of a simulation: levels, p, m */
int dsm_corr_shape(const dsm_sim* sim, int32_t* levels, int32_t* p, int32_t* m);

/* Conformation statistics of the -distr files, computed on the device
 * (ensemble.cu:356-484 does them on the host): z_counts[Z] chains with Z
 * strands (z_bins >= z_max + 1), n_counts[N] strands with N Kuhn steps
 * (n_bins >= max N_K + 1); dsm_q_sorted: |Q| of every internal strand in
 * ascending order (q NULL: *n receives the count; else *n in = capacity). */
int dsm_zn_hist(dsm_sim* sim, uint64_t* z_counts, int32_t z_bins, uint64_t* n_counts, int32_t n_bins);
int dsm_q_sorted(dsm_sim* sim, float* q, int64_t* n);

/* Reference-format checkpoint (common/ensemble.cu:342-354,486-504):
 * int N_cha, then per chain chain_head, Z float4 QN, Z float tau. */
int dsm_save_file(dsm_sim* sim, const char* path);
int dsm_load_file(dsm_sim* sim, const char* path);
/* Full-state checkpoint for an exact resume (no counterpart in the reference,
 * whose conformation file above restarts clocks, random streams and G(t)):
 * per-chain time, Philox event counter, event hash, scale and stall code, the
 * conformations, every correlator level, and the ensemble's time, behind a
 * versioned header and a payload checksum.  dsm_checkpoint_load checks that
 * the file was written by an ensemble of the same shape (chains, z_max, N_K,
 * per-chain N_K, flow / correlator kind, levels, p, m) and the same random
 * streams (seed, stream, chain offset), and verifies the checksum, before it
 * changes anything; on any mismatch it returns DSM_ERR_INVALID with the reason
 * in dsm_last_error and leaves the ensemble as it was.  Advancing a restored
 * ensemble gives the same bits as advancing the one that wrote the file. */
int dsm_checkpoint_save(dsm_sim* sim, const char* path);
int dsm_checkpoint_load(dsm_sim* sim, const char* path);

/* ---------------------------------------------------------------------
 * Allocation-free time step.  No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc/cudaFree around a step (a serving loop
 * or host framework that owns every byte of device memory through its own
 * allocator or budget, or a loop that cannot take the device-wide
 * synchronisation those calls imply).  The caller passes device buffers for
 * the chains; tables, descriptor and counters live in one static device array
 * of DSM_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits.  Limits: nk <= DSM_NOALLOC_MAX_NK (larger is rejected with
 * DSM_ERR_INVALID), z_max <= 4096, monodisperse, and no correlator: params
 * for which dsm_create would run one (no flow, eq_type 1 or 2, sync_dt > 0 and
 * t_end > 0) are rejected with DSM_ERR_INVALID.  The first
 * call on a device looks up the array's device address (make it before any
 * stream capture).  All calls share the array and it keeps the last call's
 * contents: calls that overlap on the GPU race and must be serialised.
 * --------------------------------------------------------------------- */
#define DSM_NOALLOC_SCRATCH_BYTES (160 * 1024)
#define DSM_NOALLOC_MAX_NK 2048

/* Per-chain scalars in the device layout (64 bytes): strands, stall code,
 * fixed-point scale of the rates, pending flow dt, time in 2^-32 tau_K ticks,
 * events done (Philox counter), event-sequence hash, next stress-sample
 * index, Kuhn steps.  dsm_get_ext / dsm_get_chains report the same values. */
typedef struct dsm_chain_state {
  int32_t Z;
  int32_t stall_flag;
  int32_t scale;
  float dt_prev;
  int64_t time_ticks;
  uint64_t steps;
  uint64_t hash;
  int64_t next_sample;
  int32_t nk;
  int32_t pad_[3];
} dsm_chain_state;

/* Advance n_chains chains held in caller-owned device memory (d_QN: n*z_max
 * float4 {Qx,Qy,Qz,N}; d_tau: n*z_max rates; d_state: n dsm_chain_state) to
 * time t_end or step_limit events, on `stream` (a cudaStream_t, NULL = legacy
 * default stream).  Flow ensembles (kappa != 0) also need d_stress_out
 * (n*8 floats: xx yy zz xy yz zx Lpp Z of every chain at the end).  d_QN,
 * d_tau and d_state must hold chains as dsm_get_chains / dsm_get_ext report
 * them (or as a previous call left them): in particular every state's nk must
 * equal params->nk and Z must lie in [1, z_max]; the kernel does not check
 * them, and a zeroed state gives infinite or NaN rates.  Results are identical
 * to dsm_advance on the same inputs, with one exception: the runaway-chain cap
 * (a chain doing 100x the expected events, at least 2^24, stops with stall
 * code 5) is sized from [0, t_end] here and from the window [t_start, t_end]
 * in dsm_advance, so a chain whose time step collapses in a window that
 * starts after t = 0 is stopped later here.  If events is non-NULL the call
 * waits for the kernel and stores the number of kMC events done. */
int dsm_advance_noalloc(const dsm_params* params, dsm_float4* d_QN, float* d_tau, dsm_chain_state* d_state,
                        float* d_stress_out, double t_end, int64_t step_limit, void* stream, uint64_t* events);
/* Message of the last failed dsm_advance_noalloc of the calling thread */
const char* dsm_noalloc_last_error(void);

/* ---------------------------------------------------------------------
 * Serving loop (no counterpart in the reference, which runs one ensemble per
 * process through main_cuda).  A server owns a thread that admits submitted
 * requests (each a dsm_params, monodisperse) while their device memory fits
 * in hbm_budget_bytes (0: 15/16 of the free memory), keeps their ensembles
 * resident and keeps each one busy on its own stream with chunks of about
 * chunk_s seconds (0: 0.05), every resident chain advancing at the same pace,
 * so that the kernels of all admitted requests overlap on the GPU.
 * Equilibrium requests with eq_type=1 produce G(t); flow requests (kappa != 0)
 * produce the stress at t = min(t_end, k*sync_dt), k = 1, 2, ... (the tau.dat
 * series), a chunk of outputs per CUDA graph replay.  max_active > 0 caps the
 * ensembles resident at once; max_active = 1 with chunk_s < 0 is the plain
 * form (one request at a time, one launch per request or flow output).
 * --------------------------------------------------------------------- */
typedef struct dsm_server dsm_server;
enum { DSM_REQ_QUEUED = 0, DSM_REQ_ACTIVE = 1, DSM_REQ_DONE = 2, DSM_REQ_FAILED = 3 };

int dsm_serve_open(int32_t device, uint64_t hbm_budget_bytes, int32_t max_active, double chunk_s,
                   dsm_server** out);
/* Scheduling policy (default 0): 0 first come, first served with backfill
 * (in arrival order while the older running requests leave GPU chain slots
 * free; stream priority by age; chunks of chunk_s of each request's own
 * measured speed) and requests shorter than one chunk of the whole GPU run at
 * once; 2 the same without that bypass; 1 equal pace for every resident chain
 * at the default priority. */
#define DSM_SERVE_FCFS 0
#define DSM_SERVE_EQUAL_PACE 1
#define DSM_SERVE_FCFS_STRICT 2
int dsm_serve_set_policy(dsm_server* srv, int32_t policy);
/* First-come policies: requests run in arrival order while the running ones
 * fill fewer than `overlap` GPUs' worth of chain slots (1: backfill of idle
 * slots only; above 1, younger requests also run at lower stream priority and
 * take the SMs the older ones leave free at the ends of their launches);
 * policy 0 also starts at once any request whose remaining work is below
 * bypass x chunk_s of the whole GPU.  Defaults 1 and 0.2 (on the 200-request
 * stream: p50 about 20x and p99 1.1x better than one-at-a-time serving). */
int dsm_serve_tune(dsm_server* srv, double overlap, double bypass);
/* Queue a request; *id identifies it.  DSM_ERR_MEMORY if it can never fit. */
int dsm_serve_submit(dsm_server* srv, const dsm_params* params, uint64_t* id);
/* State, latency (arrival to completion, s; -1 while unfinished), queueing
 * delay (arrival to admission, s; -1 while queued), kMC events so far. */
int dsm_serve_status(dsm_server* srv, uint64_t id, int32_t* state, double* latency_s, double* queue_s,
                     uint64_t* events);
/* Message of a failed request ("" otherwise); valid until the server closes */
const char* dsm_serve_error(dsm_server* srv, uint64_t id);
/* Wait until every submitted request finished; DSM_ERR_WATCHDOG on timeout. */
int dsm_serve_wait_all(dsm_server* srv, double timeout_s);
/* Results of a finished request (n: in = capacity, out = points) */
int dsm_serve_result_gt(dsm_server* srv, uint64_t id, float* t, float* G, int32_t* n);
int dsm_serve_result_stress(dsm_server* srv, uint64_t id, double* t, dsm_stress_plus* out, int32_t* n);
/* Totals since dsm_serve_open */
typedef struct dsm_serve_totals {
  uint64_t events;       /* kMC events of all requests */
  double busy_s;         /* seconds with work in flight */
  uint64_t ticks;        /* chunks launched */
  uint64_t completed;    /* requests finished (done or failed) */
  uint64_t peak_bytes;   /* most device memory admitted at once */
  int32_t peak_active;   /* most ensembles resident at once */
  int32_t pad_;
  double setup_s;        /* host seconds creating and initialising admitted ensembles */
  double finish_s;       /* host seconds reading results and releasing ensembles */
} dsm_serve_totals;
int dsm_serve_stats(dsm_server* srv, dsm_serve_totals* out);
/* Stop the server thread and release every resident ensemble */
void dsm_serve_close(dsm_server* srv);

/* ---------------------------------------------------------------------
 * Reference driver entry point (common/main_cuda.cu:34), same signature and
 * return convention (0 ok, -1 aborted): reads input.dat from the working
 * directory, writes tau[_id].dat / G[_id].dat, honours -s/-l/-distr.
 * C linkage here; dsm_reference.h declares the same function with the C++
 * linkage of the reference's GUI (GUI/main.cpp:22) and defines
 * DSM_NO_C_MAIN_CUDA so that one translation unit sees one of the two.
 * --------------------------------------------------------------------- */
#ifndef DSM_NO_C_MAIN_CUDA
int main_cuda(DSM_BOOL* run_flag, int job_ID, char* savefile, char* loadfile, int device_ID,
              DSM_BOOL distr, int* progress_bar);
#endif

#ifdef __cplusplus
}
#endif

#endif /* GPU_DSM_GB300_DSM_H */
