// ORACLE — test infrastructure only.  C shim over the reference's own host code
// (common/chain.cu, common/pcd_tau.h, common/random.h of ktaletsk/gpu_dsm),
// compiled from the reference tree by `make ref` into _ref/libdsmref.so.  It is
// used to pin the oracle (p_cd constants, equilibrium-initialiser statistics)
// and to generate the golden fixtures under tests/golden/.  Never shipped.
#include <cstring>
#include "chain.h"
#include "gamma.h"

// globals the reference host code expects (defined in its ensemble.cu /
// gpu_random.cu / main_cuda.cu, which are not compiled here)
float Be = 1.0f;
float step = 0.0f;
float mp = 0.0f, Mk = 0.0f;
float* GEX_table = 0;
double universal_time = 0.0;
// GEX background tables of common/gamma.cpp
float a = 0.0f, b = 0.0f;
float step_d = 0.0f;
int table_size = 0, table_size_d = 0;
float gamma_table_cutoff = 0.0f;
float* GEXd_table = 0;

extern "C" {

// p_cd fit constants as the reference computes them in float (pcd_tau.h:32-66)
int ref_pcd(float beta, float nk, double* out) {
  Be = beta;
  p_cd p(beta, nk, 0);
  const double v[12] = {p.alpha, p.tau_0, p.tau_max, p.tau_d, p.g, p.c1, p.cm1, p.rcm1c1,
                        p.At, p.Adt, p.Bdt, p.normdt};
  for (int i = 0; i < 12; ++i) out[i] = v[i];
  return 0;
}

// Equilibrium chains from the reference initialiser chain_init (chain.cu:199),
// seeded as main_cuda.cu:106 does (seed = job_ID * N_cha).  QN: n*z_max float4,
// tau: n*z_max rates.
int ref_chain_init(int seed, int n_chains, int nk, float beta, int cd_flag, int z_max,
                   int* Z, float* QN, float* tau) {
  Be = beta;
  CD_flag = cd_flag;
  Ran eran(1);
  eran.seed(seed);
  chain_head h;
  float4 r1;
  for (int i = 0; i < n_chains; ++i) {
    sstrentp d;
    d.QN = (float4*)(QN + (size_t)i * z_max * 4);
    d.tau_CD = tau + (size_t)i * z_max;
    d.R1 = &r1;
    chain_init(&h, d, nk, z_max, false, &eran);
    Z[i] = h.Z;
  }
  return 0;
}

// Lifetime samples from the reference host sampler p_cd::tau_CD_f_t /
// tau_CD_f_d_t (pcd_tau.h:67-82), returned as times tau.
int ref_tau_samples(float beta, float nk, int kind, int seed, int n, float* out) {
  Ran eran(seed);
  p_cd p(beta, nk, &eran);
  for (int i = 0; i < n; ++i) out[i] = kind == 0 ? p.tau_CD_f_t() : p.tau_CD_f_d_t();
  return 0;
}

// GEX background molecular-weight tables built by the reference's own
// make_gamma_table (gamma.cpp:174-263): the M/mp table and its CD-weighted
// counterpart, their probability steps and the table cutoff.  The caller's
// arrays hold up to cap entries; sizes are returned.
int ref_gex_table(float ga, float gb, float gmp, float gmk, float beta, int cap, float* tab_m, int* n_m,
                  float* tab_md, int* n_md, float* steps_out) {
  Be = beta; a = ga; b = gb; mp = gmp; Mk = gmk;
  step = 0.0f; step_d = 0.0f;
  make_gamma_table(ga, gb);
  *n_m = table_size;
  *n_md = table_size_d;
  for (int i = 0; i < table_size && i < cap; ++i) tab_m[i] = GEX_table[i];
  for (int i = 0; i < table_size_d && i < cap; ++i) tab_md[i] = GEXd_table[i];
  steps_out[0] = step;
  steps_out[1] = step_d;
  steps_out[2] = gamma_table_cutoff;
  delete[] GEX_table;
  delete[] GEXd_table;
  GEX_table = 0;
  GEXd_table = 0;
  return 0;
}

}  // extern "C"
