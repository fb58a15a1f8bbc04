// A caller written like the reference's GUI front end: it includes no header
// of this library and declares main_cuda itself, with C++ linkage, exactly as
// GUI/main.cpp:22 and GUI/mainwindow.cpp:47 do; linked against libgpudsm.so.
// Usage: gui_caller <job_ID>  (reads input.dat in the working directory)
#include <cstdio>
#include <cstdlib>

extern int main_cuda(bool* run_flag, int job_ID, char *savefile, char *loadfile, int device_ID, bool distr, int* progress_bar);

int main(int argc, char** argv) {
  bool run_flag = true;
  int progress_bar = 0;
  const int job = argc > 1 ? std::atoi(argv[1]) : 0;
  const int rc = main_cuda(&run_flag, job, nullptr, nullptr, 0, false, &progress_bar);
  std::printf("main_cuda=%d progress=%d\n", rc, progress_bar);
  return rc == 0 ? 0 : 1;
}
