/* A C11 caller of the handle API (include/dsm.h), linked against libgpudsm.so:
 * equilibrium ensemble with G(t), advanced to t_end; writes the chains and
 * the raw correlator sums to out_path for comparison with other callers.
 * Usage: c_caller <nk> <n_chains> <seed> <t_end> <out_path> */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dsm.h"

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  dsm_params p;
  memset(&p, 0, sizeof(p));
  p.beta = 1.0f;
  p.nk = atoi(argv[1]);
  p.n_chains = atoi(argv[2]);
  p.seed = (uint64_t)atoi(argv[3]);
  p.cd_flag = 1;
  p.eq_type = 1;
  p.sync_dt = 1.0;
  p.t_end = atof(argv[4]);
  p.corr_p = 16;
  p.corr_m = 2;
  dsm_sim* sim = NULL;
  int rc = dsm_create(&p, &sim);
  if (rc != DSM_OK) { fprintf(stderr, "dsm_create: %d %s\n", rc, dsm_last_error(sim)); return 1; }
  rc = dsm_init_equilibrium(sim);
  uint64_t events = 0;
  if (rc == DSM_OK) rc = dsm_advance(sim, p.t_end, -1, NULL, &events);
  const size_t n = (size_t)p.n_chains, cap = (size_t)p.nk;
  dsm_chain_head* heads = (dsm_chain_head*)calloc(n, sizeof(dsm_chain_head));
  dsm_float4* qn = (dsm_float4*)calloc(n * cap, sizeof(dsm_float4));
  float* tau = (float*)calloc(n * cap, sizeof(float));
  int32_t L = 0, cp = 0, cm = 0;
  if (rc == DSM_OK) rc = dsm_get_chains(sim, heads, qn, tau);
  if (rc == DSM_OK) rc = dsm_corr_shape(sim, &L, &cp, &cm);
  double* g = (double*)calloc((size_t)L * cp + 1, sizeof(double));
  int64_t* c = (int64_t*)calloc((size_t)L * cp + 1, sizeof(int64_t));
  if (rc == DSM_OK) rc = dsm_gt_raw(sim, g, c);
  if (rc != DSM_OK) { fprintf(stderr, "failed: %d %s\n", rc, dsm_last_error(sim)); dsm_destroy(sim); return 1; }
  FILE* f = fopen(argv[5], "wb");
  if (!f) return 1;
  fwrite(&events, sizeof(events), 1, f);
  fwrite(heads, sizeof(dsm_chain_head), n, f);
  fwrite(qn, sizeof(dsm_float4), n * cap, f);
  fwrite(tau, sizeof(float), n * cap, f);
  fwrite(&L, sizeof(L), 1, f);
  fwrite(&cp, sizeof(cp), 1, f);
  fwrite(g, sizeof(double), (size_t)L * cp, f);
  fclose(f);
  printf("events=%llu levels=%d p=%d\n", (unsigned long long)events, L, cp);
  free(heads); free(qn); free(tau); free(g); free(c);
  dsm_destroy(sim);
  return 0;
}
