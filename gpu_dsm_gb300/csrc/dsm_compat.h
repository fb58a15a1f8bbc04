// Reference-compatible file formats and driver helpers (dsm_compat.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

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
// -distr file writers from histograms (common/ensemble.cu:356-484)
void write_Z_distr(const std::string& fn, const std::vector<uint64_t>& hist, int n_chains, bool cumulative);
void write_N_distr(const std::string& fn, const std::vector<uint64_t>& hist, bool cumulative);
void write_Q_distr(const std::string& fn, const std::vector<float>& Q);
// the reference driver main_cuda (common/main_cuda.cu:34-185)
int main_cuda_impl(bool* run_flag, int job_ID, char* savefile, char* loadfile, int device_ID, bool distr,
                   int* progress_bar);

}  // namespace dsmc
