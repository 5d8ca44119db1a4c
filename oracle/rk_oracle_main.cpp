// rk_oracle_main.cpp -- command-line driver of the CPU oracle (test infrastructure).
//
// usage: rk_oracle <conf> <outdir> [max_steps] [qrot qdot qddot qnorm vnorm vdiv]
// Runs the reference's console loop (initial NL update, then the integrate
// loop writing conf<N> files into outdir), like `rockable <conf>` does
// (src/Apps/run.cpp:135-212).
#include <cstdio>
#include <cstdlib>

#include "rk_oracle.h"

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <conf> <outdir> [max_steps] [variant x6]\n", argv[0]);
    return 2;
  }
  long max_steps = argc > 3 ? std::atol(argv[3]) : 0;
  if (argc >= 10) {
    orc_variant v;
    v.qrot = std::atoi(argv[4]);
    v.qdot = std::atoi(argv[5]);
    v.qddot = std::atoi(argv[6]);
    v.qnorm = std::atoi(argv[7]);
    v.vnorm = std::atoi(argv[8]);
    v.vdiv = std::atoi(argv[9]);
    orc_set_variant(&v);
  }
  orc_sim* s = orc_load(argv[1]);
  if (!s) {
    std::fprintf(stderr, "error: %s\n", orc_last_error());
    return 1;
  }
  long n = orc_integrate(s, argv[2], max_steps);
  std::printf("steps %ld\n", n);
  orc_free(s);
  return n < 0 ? 1 : 0;
}
