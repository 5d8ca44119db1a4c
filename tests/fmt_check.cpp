// Host build of rockable_gb300/csrc/rk_fmt.cuh for tests/test_fmt_cpu.py.
#include "../rockable_gb300/csrc/rk_fmt.cuh"

extern "C" int rk_fmt_e_host(double x, int prec, int toward_zero, char* out) {
  const int n = rk::fmt_e(x, prec, toward_zero != 0, out);
  out[n] = 0;
  return n;
}
