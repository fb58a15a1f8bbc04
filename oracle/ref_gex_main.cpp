// ORACLE — test infrastructure only.  Runs the reference's own GEX table
// builder (common/gamma.cpp:174-263 of ktaletsk/gpu_dsm, compiled from the
// reference tree by `make ref` into _ref/ref_gex) for one parameter set and
// prints the table sizes, steps, cutoff and every k-th entry as JSON.  It runs
// as a separate process: the reference's inversion of the CD-weighted table
// can read past the filled part of its work array (uninitialised memory), so a
// parameter set may crash it without harming the caller.
#include <cstdio>
#include <cstdlib>

#include "gamma.h"

float Be = 1.0f, step = 0.0f, mp = 0.0f, Mk = 0.0f, a = 0.0f, b = 0.0f, step_d = 0.0f, gamma_table_cutoff = 0.0f;
float* GEX_table = 0;
float* GEXd_table = 0;
int table_size = 0, table_size_d = 0;

int main(int argc, char** argv) {
  if (argc < 7) { std::fprintf(stderr, "usage: ref_gex a b mp Mk beta every\n"); return 2; }
  a = (float)std::atof(argv[1]); b = (float)std::atof(argv[2]);
  mp = (float)std::atof(argv[3]); Mk = (float)std::atof(argv[4]); Be = (float)std::atof(argv[5]);
  const int every = std::atoi(argv[6]);
  make_gamma_table(a, b);
  std::printf("{\"n\": %d, \"n_d\": %d, \"step\": %.9g, \"step_d\": %.9g, \"cutoff\": %.9g, \"every\": %d, \"M\": [",
              table_size, table_size_d, step, step_d, gamma_table_cutoff, every);
  for (int i = 0; i < table_size; i += every) std::printf("%s%.9g", i ? ", " : "", GEX_table[i]);
  std::printf("], \"Md\": [");
  for (int i = 0; i < table_size_d; i += every) std::printf("%s%.9g", i ? ", " : "", GEXd_table[i]);
  std::printf("]}\n");
  return 0;
}
