/*
 * gpu_dsm_gb300 — the reference's own C++ entry points, for callers written
 * against ktaletsk/gpu_dsm's headers (common/ensemble.h, common/ensemble_call_block.h,
 * common/chain.h, common/stress.h) or its GUI (GUI/main.cpp:22,
 * GUI/mainwindow.cpp:47).  C++ linkage, the reference's names, argument
 * meanings and return conventions; implemented in libgpudsm.so on top of the
 * handle API of dsm.h (gpu_dsm_gb300/csrc/dsm_refapi.cu).
 *
 * Include this header before, or instead of, dsm.h: it declares main_cuda with
 * C++ linkage, as the reference's GUI does, and so hides dsm.h's extern "C"
 * declaration of the same function (both symbols are exported).
 *
 * Differences from the reference, all in where state lives:
 *  - The ensemble.h functions drive one process-global device ensemble (one
 *    persistent launch over every chain) instead of blocks of chains_per_call
 *    chains; the host arrays `chains` / `chain_heads` and the globals
 *    (N_cha, NK, z_max, Be, CD_flag, PD_flag, kxx..kzz, universal_time)
 *    keep the reference's meaning.
 *  - host_chains_init only allocates the host arrays; gpu_init draws the
 *    equilibrium chains on the device (Philox keyed by the gpu_init seed and
 *    the chain) and copies them into the host arrays, unless load_from_file
 *    filled them.  The Ran and p_cd arguments are accepted and not used: the
 *    reference's host MT19937 stream and p_cd object are replaced by the
 *    device initialiser and the library's own p_cd.
 *  - ensemble_call_block owns one device ensemble for its chains
 *    (random streams keyed by the chain's global index, so blocks of one
 *    ensemble are shards of it); activate_block / deactivate_block have
 *    nothing to copy and return at once; free_block releases the device
 *    ensemble but not the caller's host arrays.
 */
#ifndef GPU_DSM_GB300_DSM_REFERENCE_H
#define GPU_DSM_GB300_DSM_REFERENCE_H

#ifndef __cplusplus
#error "dsm_reference.h declares the reference's C++ entry points; C callers use dsm.h"
#endif

#define DSM_NO_C_MAIN_CUDA
#include "dsm.h"

#include <string>

struct Ran;   /* common/random.h:77, accepted and unused */
struct p_cd;  /* common/pcd_tau.h:26, accepted and unused */

/* common/chain.h:37-42 */
typedef struct sstrentp {
  dsm_float4* QN;   /* {Qx, Qy, Qz, N} x z_max per chain */
  float* tau_CD;    /* lifetime rates 1/tau_CD x z_max per chain */
  dsm_float4* R1;   /* first entanglement in the lab frame, one per chain */
} sstrentp;

/* common/chain.h:45-53 */
typedef struct chain_head {
  int Z;
  float time;
  float dummy;
  int stall_flag;
} chain_head;

/* common/stress.h:23-29 */
typedef struct stress_plus {
  float xx, yy, zz;
  float xy, yz, zx;
  float Lpp;
  float Z;
} stress_plus;

/* common/ensemble_call_block.h:24-56: the host members the reference's
 * callers use; the device part is one ensemble of the library. */
typedef struct ensemble_call_block {
  int nc;                  /* number of chains */
  sstrentp chains;         /* host conformations of the block's chains */
  chain_head* chain_heads; /* host chain heads of the block's chains */
  double block_time;       /* time the block has been advanced to */
  dsm_sim* sim;            /* device ensemble of the block */
  int levels;              /* correlator levels given to init_call_block (0: from the run length) */
  int corr_type;           /* correlator of the device ensemble: -1 none, 0 G(t), 1 MSD(t) */
  int corr_res;            /* its sample interval */
} ensemble_call_block;

/* ---------------------------------------------------------------- globals
 * common/ensemble.h:33-55, common/chain.h:30-31,56, common/job_ID.h:30 */
extern sstrentp chains;
extern chain_head* chain_heads;
extern double universal_time;
extern int N_cha;
extern int NK;
extern int z_max;
extern bool dbug;
extern float kxx, kxy, kxz, kyx, kyy, kyz, kzx, kzy, kzz;
extern bool PD_flag;
extern float Be;
extern int CD_flag;
extern int job_ID;
/* Sample interval of the call-block correlator: the value gpu_Gt_PCS copies
 * into the reference's __constant__ d_correlator_res (ensemble.cu:296)
 * before EQ_time_step_call_block runs. */
extern int dsm_correlator_res;

/* ---------------------------------------------------------------- ensemble.h
 * common/ensemble.h:37-77 */
sstrentp chain_index(const int i);
sstrentp chain_index(const int bi, const int i);
void host_chains_init(Ran* eran);
void gpu_init(int seed, p_cd* pcd, int s);
void get_chains_from_device();
void save_to_file(char* filename);
void save_Z_distribution_to_file(std::string filename, bool cumulative);
void save_N_distribution_to_file(std::string filename, bool cumulative);
void save_Q_distribution_to_file(std::string filename, bool cumulative);
void load_from_file(char* filename);
int gpu_time_step(double reach_time, bool* run_flag);
int gpu_Gt_PCS(int res, double length, float*& t, float*& x, int s, int correlator_type, bool* run_flag,
               int* progress_bar);
void gpu_clean();
stress_plus calc_stress();

/* ---------------------------------------------------------------- ensemble_call_block.h
 * common/ensemble_call_block.h:55-75; init_call_block in both the header's
 * 4-argument and the definition's 5-argument form (ensemble_call_block.cu:55) */
void init_call_block(ensemble_call_block* cb, int nc, sstrentp chains, chain_head* chain_heads);
void init_call_block(ensemble_call_block* cb, int nc, sstrentp chains, chain_head* chain_heads, int s);
int time_step_call_block(double reach_time, ensemble_call_block* cb, bool* run_flag);
int EQ_time_step_call_block(double reach_time, ensemble_call_block* cb, int correlator_type, bool* run_flag,
                            int* progress_bar);
void get_chain_to_device_call_block(ensemble_call_block* cb);
void get_chain_from_device_call_block(ensemble_call_block* cb);
stress_plus calc_stress_call_block(ensemble_call_block* cb, int* r_chain_count);
void free_block(ensemble_call_block* cb);
void activate_block(ensemble_call_block* cb);
void deactivate_block(ensemble_call_block* cb);

/* ---------------------------------------------------------------- driver
 * common/main_cuda.cu:34 with C++ linkage, as GUI/main.cpp:22 and
 * GUI/mainwindow.cpp:47 declare it; same behaviour as dsm.h's main_cuda. */
int main_cuda(bool* run_flag, int job_ID, char* savefile, char* loadfile, int device_ID, bool distr,
              int* progress_bar);

#endif /* GPU_DSM_GB300_DSM_REFERENCE_H */
