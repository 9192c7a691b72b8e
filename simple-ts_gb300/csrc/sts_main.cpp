// simple_ts_gb300: drop-in replacement for the reference executable.  Run it in (or
// point it at) a directory holding EnteredData.txt and the body files; it writes the
// same dumps and logs as the serial reference solver.
//
//   simple_ts_gb300 [case_dir] [--residual] [--no-graph] [--device N]
//
// --residual selects the residual-terminated p-T loop (the reference built without
// FIXED_NUMBER_OF_ITERATIONS_LOOP_3); the default runs N_I_p_c sweeps like the shipped build.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/sts_gb300.h"

int main(int argc, char** argv) {
  const char* dir = ".";
  sts_options o;
  sts_default_options(&o);
  for (int k = 1; k < argc; k++) {
    if (std::strcmp(argv[k], "--residual") == 0) o.fixed_sweeps = 0;
    else if (std::strcmp(argv[k], "--no-graph") == 0) o.use_graph = 0;
    else if (std::strcmp(argv[k], "--device") == 0 && k + 1 < argc) o.device = std::atoi(argv[++k]);
    else dir = argv[k];
  }
  const int r = sts_run_case(dir, &o);
  if (r != STS_OK) {
    std::fprintf(stderr, "simple_ts_gb300: %s\n", sts_last_error());
    return 1;
  }
  return 0;
}
