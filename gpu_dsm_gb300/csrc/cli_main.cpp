// gpu_DSM command-line driver: same arguments as the reference CLI
// (CLI/main.cu:20-56): gpu_DSM <job_ID> [-s file] [-l file] [-d device] [-distr]
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "dsm.h"

int main(int narg, char** arg) {
  bool run_flag = true;
  char* savefile = nullptr;
  char* loadfile = nullptr;
  bool distr = false;
  int device_ID = 0;
  int progress_bar = 0;
  int job_ID = 0;
  for (int k = 1; k < narg; ++k) {
    if (k == 1) job_ID = std::atoi(arg[k]);
    if (std::strcmp(arg[k], "-s") == 0 && k + 1 < narg) {
      savefile = arg[++k];
      std::cout << "final chain conformations will be saved to " << savefile << '\n';
    } else if (std::strcmp(arg[k], "-l") == 0 && k + 1 < narg) {
      loadfile = arg[++k];
    } else if (std::strcmp(arg[k], "-d") == 0 && k + 1 < narg) {
      device_ID = std::atoi(arg[++k]);
    } else if (std::strcmp(arg[k], "-distr") == 0) {
      distr = true;
    }
  }
  const int rc = main_cuda(&run_flag, job_ID, savefile, loadfile, device_ID, distr, &progress_bar);
  return rc == 0 ? 0 : 1;
}
