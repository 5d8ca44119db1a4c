// rk_run.cpp -- command-line runner, the GB300 counterpart of Rockable's
// `rockable` application (src/Apps/run.cpp:135-212).
//
//   rockable-gb300 <conf> [-o outdir] [-m max_steps] [-n newconf -r golden]
//
// Runs the conf (initial NL update, integrate loop writing conf<N> files).
// A drivingSystem.txt in the working directory is read like the reference
// does.  With -n/-r, compares the written conf with a golden from the
// `Particles` line on (run.cpp:38-92) and exits 1 on a difference.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "rk_host.hpp"

static std::vector<std::string> tail_lines(const std::string& path) {
  std::ifstream f(path);
  std::vector<std::string> out;
  std::string l;
  bool on = false;
  while (std::getline(f, l)) {
    if (!on && l.rfind("Particles", 0) == 0) on = true;
    if (on) out.push_back(l);
  }
  return out;
}

int main(int argc, char** argv) {
  std::string conf, outdir = ".", newconf, golden;
  long max_steps = 0;
  for (int k = 1; k < argc; k++) {
    std::string a = argv[k];
    if (a == "-o" && k + 1 < argc) outdir = argv[++k];
    else if (a == "-m" && k + 1 < argc) max_steps = std::atol(argv[++k]);
    else if (a == "-n" && k + 1 < argc) newconf = argv[++k];
    else if (a == "-r" && k + 1 < argc) golden = argv[++k];
    else if ((a == "-j" || a == "-v") && k + 1 < argc) ++k;  // threads / verbosity: not used by the GPU engine
    else conf = a;
  }
  if (conf.empty()) {
    std::fprintf(stderr, "usage: %s <conf> [-o outdir] [-m max_steps] [-n newconf -r golden]\n", argv[0]);
    return 2;
  }
  rkhost::Rockable box;
  if (!box.loadConf(conf)) {
    std::fprintf(stderr, "error: %s\n", box.error().c_str());
    return 1;
  }
  {
    std::ifstream ds("drivingSystem.txt");
    if (ds.good() && !box.readDrivingSystem("drivingSystem.txt")) {
      std::fprintf(stderr, "error: %s\n", box.error().c_str());
      return 1;
    }
  }
  long n = box.consoleRun(outdir, max_steps);
  if (n < 0) {
    std::fprintf(stderr, "error: %s\n", box.error().c_str());
    return 1;
  }
  std::printf("steps %ld\n", n);
  if (!newconf.empty() && !golden.empty()) {
    auto a = tail_lines(newconf), b = tail_lines(golden);
    if (a != b) {
      size_t k = 0;
      while (k < a.size() && k < b.size() && a[k] == b[k]) k++;
      std::fprintf(stderr, "regression: %s differs from %s at line %zu of the compared part\n", newconf.c_str(),
                   golden.c_str(), k);
      return 1;
    }
    std::printf("regression: identical\n");
  }
  return 0;
}
