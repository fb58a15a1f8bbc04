// A caller of the reference's own entry points (include/dsm_reference.h, the
// functions and globals of common/ensemble.h and common/ensemble_call_block.h),
// driving them as common/main_cuda.cu does; linked against libgpudsm.so.
// Usage:
//   ref_api_caller gt   <nk> <n> <seed> <t_end> <levels>   G(t) through gpu_Gt_PCS,
//       then the ensemble split in two call blocks advanced 100 tau_K further by
//       EQ_time_step_call_block; writes G_<seed>.dat, ens.bin, blocks.bin,
//       blocks_in.bin (the host state the blocks started from) and stress lines
//   ref_api_caller flow <nk> <n> <seed> <kxy> <dt> <n_out>  shear through
//       gpu_time_step + calc_stress at n_out outputs; writes ens.bin
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "dsm_reference.h"

static void print_stress(const char* what, const stress_plus& s, int count) {
  std::printf("%s %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %d\n", what, s.xx, s.yy, s.zz, s.xy, s.yz, s.zx, s.Lpp,
              s.Z, count);
}

int main(int argc, char** argv) {
  if (argc < 8) return 2;
  const std::string mode = argv[1];
  NK = std::atoi(argv[2]);
  N_cha = std::atoi(argv[3]);
  job_ID = std::atoi(argv[4]);
  Be = 1.0f;
  CD_flag = 1;
  bool run = true;
  int progress = 0;
  char ens[] = "ens.bin", blocks[] = "blocks.bin", blocks_in[] = "blocks_in.bin";
  if (mode == "gt") {
    const double t_end = std::atof(argv[5]);
    const int s = std::atoi(argv[6]);
    host_chains_init(nullptr);
    gpu_init(job_ID, nullptr, s);
    float* t = nullptr;
    float* x = nullptr;
    const int rc = gpu_Gt_PCS(1, t_end, t, x, s, 0, &run, &progress);
    if (rc != 0) { std::printf("gpu_Gt_PCS=%d\n", rc); return 1; }
    delete[] t;
    delete[] x;
    save_to_file(ens);
    print_stress("ensemble", calc_stress(), N_cha);
    // two call blocks over the host arrays, each with its own correlator
    save_to_file(blocks_in);
    const int half = N_cha / 2;
    ensemble_call_block cb[2];
    init_call_block(&cb[0], half, chain_index(0), chain_heads, s);
    init_call_block(&cb[1], N_cha - half, chain_index(half), chain_heads + half, s);
    dsm_correlator_res = 1;
    for (int b = 0; b < 2; ++b) {
      activate_block(&cb[b]);
      const int r = EQ_time_step_call_block(t_end + 100.0, &cb[b], 0, &run, &progress);
      deactivate_block(&cb[b]);
      if (r != 0) { std::printf("EQ_time_step_call_block=%d\n", r); return 1; }
      get_chain_from_device_call_block(&cb[b]);
      int count = 0;
      const stress_plus sp = calc_stress_call_block(&cb[b], &count);
      print_stress(b == 0 ? "block0" : "block1", sp, count);
    }
    save_to_file(blocks);
    free_block(&cb[0]);
    free_block(&cb[1]);
  } else if (mode == "flow") {
    kxy = (float)std::atof(argv[5]);
    const double dt = std::atof(argv[6]);
    const int n_out = std::atoi(argv[7]);
    host_chains_init(nullptr);
    gpu_init(job_ID, nullptr, 1);
    for (int k = 1; k <= n_out; ++k) {
      const int rc = gpu_time_step(k * dt, &run);
      if (rc != 0) { std::printf("gpu_time_step=%d\n", rc); return 1; }
      char what[32];
      std::snprintf(what, sizeof(what), "out%d", k);
      print_stress(what, calc_stress(), N_cha);
    }
    get_chains_from_device();
    save_to_file(ens);
  } else {
    return 2;
  }
  gpu_clean();
  std::printf("done universal_time=%g\n", universal_time);
  return 0;
}
