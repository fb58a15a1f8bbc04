// Reference-compatible driver on top of the C ABI: main_cuda() with the
// reference's signature (common/main_cuda.cu:34), the input.dat format
// (common/main_cuda.cu:53-68, CLI/input.dat:1-22), tau/G output files
// (common/main_cuda.cu:122-159, common/ensemble.cu:326-335), the job_ID file
// suffix (common/job_ID.h:33-68) and the -distr histograms
// (common/ensemble.cu:356-484).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/dsm.h"
#include "dsm_compat.h"

namespace dsmc {

// common/job_ID.h:33-68: "<name>_<id>.dat", or "<name>.dat" for id 0
std::string filename_ID(const std::string& name, int job_ID) {
  if (job_ID != 0) return name + "_" + std::to_string(job_ID) + ".dat";
  return name + ".dat";
}

// common/main_cuda.cu:53-68
int read_input(const char* path, InputDat* in) {
  std::ifstream f(path);
  if (!f) return DSM_ERR_INVALID;
  f >> in->beta >> in->nk >> in->n_chains;
  for (int q = 0; q < 9; ++q) f >> in->kappa[q];
  f >> in->cd_flag >> in->pd_flag >> in->eq_type >> in->sync_dt >> in->t_end;
  if (!f) return DSM_ERR_INVALID;
  return DSM_OK;
}

// common/ensemble.cu:394-431, from the device histogram of N over all strands
void write_N_distr(const std::string& fn, const std::vector<uint64_t>& hist, bool cumulative) {
  std::ofstream f(fn);
  if (!f) { std::cout << "file error\n"; return; }
  int nmin = -1, nmax = -1;
  unsigned long long nstr = 0;
  for (size_t n = 0; n < hist.size(); ++n)
    if (hist[n]) { if (nmin < 0) nmin = (int)n; nmax = (int)n; nstr += hist[n]; }
  if (hist.size() > 0 && hist[0]) std::cout << "Zero length strands: " << hist[0] << "\n";
  unsigned long long run = 0;
  for (int n = nmin; n >= 0 && n <= nmax; ++n) {
    run += hist[n];
    const unsigned long long cnt = cumulative ? run : hist[n];
    f << n << "\t" << (float)cnt / (float)nstr << "\n";
  }
}

// common/ensemble.cu:356-392, from the device histogram of Z over chains
void write_Z_distr(const std::string& fn, const std::vector<uint64_t>& hist, int n_chains, bool cumulative) {
  std::ofstream f(fn);
  if (!f) { std::cout << "file error\n"; return; }
  int zmin = -1, zmax = -1;
  for (size_t z = 0; z < hist.size(); ++z)
    if (hist[z]) { if (zmin < 0) zmin = (int)z; zmax = (int)z; }
  unsigned long long run = 0;
  for (int j = zmin; j >= 0 && j <= zmax; ++j) {
    run += hist[j];
    const unsigned long long cnt = cumulative ? run : hist[j];
    f << j << "\t" << (float)cnt / (float)n_chains << "\n";
  }
}

// common/ensemble.cu:439-484: cumulative distribution of |Q| of the internal
// strands, every 10th of the sorted lengths (sorted on the device)
void write_Q_distr(const std::string& fn, const std::vector<float>& Q) {
  std::ofstream f(fn);
  if (!f) { std::cout << "file error\n"; return; }
  const size_t n = Q.size();
  std::vector<float> P(n);
  for (size_t i = 0; i < n; ++i) {
    if (i != 0 && Q[i] == Q[i - 1]) P[i - 1] = (float)i / (float)n;
    P[i] = (float)i / (float)n;
  }
  const size_t quant = 10;
  for (size_t i = 0; i < n / quant; ++i) f << Q[i * quant] << "\t" << P[i * quant] << "\n";
}

int write_distributions(dsm_sim* sim, int n_chains, int cap, bool cd_flag) {
  std::vector<uint64_t> hz((size_t)cap + 2), hn((size_t)cap + 2);
  int rc = dsm_zn_hist(sim, hz.data(), (int32_t)hz.size(), hn.data(), (int32_t)hn.size());
  if (rc) return rc;
  int64_t nq = 0;
  rc = dsm_q_sorted(sim, nullptr, &nq);
  if (rc) return rc;
  std::vector<float> Q((size_t)nq);
  rc = dsm_q_sorted(sim, Q.data(), &nq);
  if (rc) return rc;
  // common/main_cuda.cu:169-180
  const std::string sfx = cd_flag ? "" : "_";
  write_Z_distr("distr_Z" + sfx + ".dat", hz, n_chains, false);
  write_N_distr("distr_N" + sfx + ".dat", hn, false);
  write_Q_distr("distr_Q" + sfx + ".dat", Q);
  return DSM_OK;
}

}  // namespace dsmc

using namespace dsmc;

extern "C" int main_cuda(bool* run_flag, int job_ID, char* savefile, char* loadfile, int device_ID, bool distr,
                         int* progress_bar) {
  return main_cuda_impl(run_flag, job_ID, savefile, loadfile, device_ID, distr, progress_bar);
}

// common/main_cuda.cu:34-185; exported as main_cuda with C linkage (above) and
// with the reference GUI's C++ linkage (dsm_refapi.cu)
int dsmc::main_cuda_impl(bool* run_flag, int job_ID, char* savefile, char* loadfile, int device_ID, bool distr,
                         int* progress_bar) {
  if (job_ID != 0) {
    std::cout << "job_ID: " << job_ID << '\n';
    std::cout << "using " << job_ID << " as a seed for random number generator\n";
    std::cout << "\"_" << job_ID << "\" will be appended to filename for all files generated\n\n";
  }
  InputDat in;
  if (read_input("input.dat", &in) != DSM_OK) {
    std::cout << "cannot read input.dat\n";
    return DSM_ERR_INVALID;
  }
  dsm_params p;
  std::memset(&p, 0, sizeof(p));
  p.beta = in.beta; p.nk = in.nk; p.n_chains = in.n_chains;
  for (int q = 0; q < 9; ++q) p.kappa[q] = in.kappa[q];
  p.cd_flag = in.cd_flag; p.pd_flag = in.pd_flag; p.eq_type = in.eq_type;
  p.sync_dt = in.sync_dt; p.t_end = in.t_end;
  p.seed = (uint64_t)(uint32_t)job_ID;
  p.device = device_ID;
  if (in.pd_flag) {
    // GEX background: polydisp.dat holds a, b, mp, Mk (main_cuda.cu:95-103)
    std::ifstream pf("polydisp.dat");
    if (!(pf >> p.gex_a >> p.gex_b >> p.gex_mp >> p.gex_mk)) {
      std::cout << "cannot read polydisp.dat\n";
      return DSM_ERR_INVALID;
    }
  }
  const bool flow = std::any_of(in.kappa, in.kappa + 9, [](float k) { return k != 0.0f; });
  const int s_levels = (int)std::ceil(std::log(in.t_end / in.sync_dt / 64.0) / std::log(8.0)) + 1;

  std::cout << "\nsimulation parameters:\n";
  std::cout << "NK\tBeta\tN_cha" << "\n";
  std::cout << in.nk << '\t' << in.beta << '\t' << in.n_chains << "\n";
  std::cout << "deformation tensor:" << "\n";
  std::cout << in.kappa[0] << '\t' << in.kappa[1] << '\t' << in.kappa[2] << '\n' << in.kappa[3] << '\t'
            << in.kappa[4] << '\t' << in.kappa[5] << '\n' << in.kappa[6] << '\t' << in.kappa[7] << '\t'
            << in.kappa[8] << '\n';
  if (in.eq_type == 1) std::cout << "G(t) calculation is on\n";
  else if (in.eq_type == 2) std::cout << "MSD(t) calculation is on\n";
  std::cout << "simulation time, sync time" << "\n";
  std::cout << in.t_end << '\t' << in.sync_dt << '\n';
  std::cout << "number of correlator levels" << '\t' << s_levels << '\n' << '\n';

  dsm_sim* sim = nullptr;
  int rc = dsm_create(&p, &sim);
  if (rc != DSM_OK) {
    std::cout << "setup failed: " << dsm_last_error(sim) << "\n";
    dsm_destroy(sim);
    return rc;
  }
  if (loadfile != nullptr) {
    std::cout << "loading chain conformations from " << loadfile << "..";
    rc = dsm_load_file(sim, loadfile);
    std::cout << (rc == DSM_OK ? "done.\n" : "failed.\n");
  } else {
    std::cout << "generating equilibrium chain conformations on device..";
    rc = dsm_init_equilibrium(sim);
    std::cout << "done\n";
  }
  if (rc != DSM_OK) {
    std::cout << dsm_last_error(sim) << "\n";
    dsm_destroy(sim);
    return rc;
  }
  volatile int32_t abort_word = 0;
  auto poll = [&]() { if (run_flag && !*run_flag) abort_word = 1; };
  const auto t0 = std::chrono::steady_clock::now();
  if (flow) {
    std::ofstream tau_file(filename_ID("tau", job_ID));
    std::cout << "output file: " << filename_ID("tau", job_ID) << '\n';
    std::cout << "performing time evolution for the ensemble..\n";
    std::cout << "time\tstress tensor(xx yy zz xy yz xz)\t<Lpp>\t<Z>\n";
    // output times of the reference loop (main_cuda.cu:117-133): t_step += sync_dt
    std::vector<double> ends;
    for (double t_step = 0; t_step < in.t_end; t_step += in.sync_dt) ends.push_back(t_step + in.sync_dt);
    // up to 64 outputs per graph replay; the chains run through 16 of them per
    // step launch, recording the stress at each output time
    constexpr size_t kOutGroup = 64;
    std::vector<dsm_stress_plus> sp(kOutGroup);
    for (size_t g0 = 0; g0 < ends.size(); g0 += kOutGroup) {
      const int32_t k = (int32_t)std::min(kOutGroup, ends.size() - g0);
      poll();
      if (abort_word) { dsm_destroy(sim); return -1; }
      rc = dsm_series_start(sim, ends.data() + g0, k);
      int32_t n_out = 0;
      while (rc == DSM_OK) {
        rc = dsm_poll(sim, nullptr, sp.data(), &n_out);
        if (rc != DSM_PENDING) break;
        rc = DSM_OK;
        poll();
        if (abort_word) dsm_abort(sim);
        std::this_thread::sleep_for(std::chrono::microseconds(200));
      }
      if (rc == DSM_ABORTED) { dsm_destroy(sim); return -1; }
      if (rc != DSM_OK) { std::cout << dsm_last_error(sim) << "\n"; dsm_destroy(sim); return rc; }
      for (int32_t w = 0; w < k; ++w) {
        const dsm_stress_plus& q = sp[w];
        std::cout << ends[g0 + w] << '\t' << q.xx << ' ' << q.yy << ' ' << q.zz << ' ' << q.xy << ' ' << q.yz << ' '
                  << q.zx << ' ' << q.Lpp << ' ' << q.Z << '\n';
        tau_file << ends[g0 + w] << '\t' << q.xx << ' ' << q.yy << ' ' << q.zz << ' ' << q.xy << ' ' << q.yz << ' '
                 << q.zx << ' ' << q.Lpp << ' ' << q.Z << '\n';
      }
      tau_file.flush();
      if (progress_bar) *progress_bar = (int)(100.0 * ends[g0 + k - 1] / in.t_end);
    }
    std::cout << "time evolution done.\n";
  } else if (in.eq_type == 1 || in.eq_type == 2) {
    // G(t) (correlator of the shear stresses) or MSD(t) (centre of mass), same
    // correlator and window loop (ensemble.cu:289-339, main_cuda.cu:136-156)
    const bool msd = in.eq_type == 2;
    std::cout << (msd ? "MSD(t) calc...\n" : "G(t) calc...\n");
    if (progress_bar) *progress_bar = 1;
    // windows of at most 1e5 tau_K (max_sync_interval, ensemble_call_block.cu:24)
    const double win = std::max(in.sync_dt, 1.0e5);
    for (double t = 0; t < in.t_end;) {
      const double te = std::min(in.t_end, t + win);
      poll();
      rc = dsm_advance(sim, te, -1, &abort_word, nullptr);
      if (rc == DSM_ABORTED) { dsm_destroy(sim); return -1; }
      if (rc != DSM_OK) { std::cout << dsm_last_error(sim) << "\n"; dsm_destroy(sim); return rc; }
      t = te;
      if (progress_bar) *progress_bar = (int)(100.0 * t / in.t_end);
      std::cout << "\r" << (int)(100.0 * t / in.t_end) << "%\t ";
    }
    int32_t n = 4096;
    std::vector<float> tt(n), gg(n);
    rc = dsm_gt(sim, tt.data(), gg.data(), &n);
    if (rc != DSM_OK) { std::cout << dsm_last_error(sim) << "\n"; dsm_destroy(sim); return rc; }
    std::ofstream gf(filename_ID(msd ? "MSD" : "G", job_ID));
    std::cout << "\n";
    for (int j = 0; j < n; ++j) {
      std::cout << tt[j] << '\t' << gg[j] << '\n';
      gf << tt[j] << '\t' << gg[j] << '\n';
    }
  } else {
    std::cout << "There are no flow and no equilibrium quantity to calculate. Exiting... \n";
  }
  if (savefile != nullptr) {
    std::cout << "saving chain conformations to " << savefile << "..";
    rc = dsm_save_file(sim, savefile);
    std::cout << (rc == DSM_OK ? "done.\n" : "failed.\n");
  }
  if (distr) {
    std::cout << "Saving distribution to file...";
    int32_t zmax = 0;
    (void)zmax;
    write_distributions(sim, in.n_chains, in.nk, in.cd_flag != 0);
  }
  dsm_destroy(sim);
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  std::cout << "Calculation time: " << ms << " milliseconds\n";
  return 0;
}
