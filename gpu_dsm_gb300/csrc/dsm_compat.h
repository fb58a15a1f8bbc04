// Reference-compatible file formats and driver helpers (dsm_compat.cu).
#pragma once
#include <string>

#include "../../include/dsm.h"

namespace dsmc {

// input.dat (common/main_cuda.cu:55-68)
struct InputDat {
  float beta = 1.0f;
  int nk = 0, n_chains = 0;
  float kappa[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int cd_flag = 1, pd_flag = 0, eq_type = 0;
  double sync_dt = 1.0, t_end = 0.0;
};

std::string filename_ID(const std::string& name, int job_ID);
int read_input(const char* path, InputDat* in);
int write_distributions(dsm_sim* sim, int n_chains, int cap, bool cd_flag);

}  // namespace dsmc
