// rk_conf.cuh -- the Particles and Interactions sections of a conf file,
// formatted on the device (Rockable::saveConf, Rockable.cpp:547-580), for
// rk_format_conf in rk_api.cu.  Each body and each active entry writes its
// line into a fixed-size slot (rk_fmt.cuh's exact printf("%.*e")), the line
// lengths are prefix-summed, and the lines are packed into one text.
#pragma once
#include "rk_engine.cuh"
#include "rk_fmt.cuh"

namespace rk {

constexpr int kConfBodySlot = 1024;  // name (<= 255) + 2 integers + 20 numbers of <= 26 characters
constexpr int kConfEntrySlot = 512;  // 5 integers + 17 numbers
constexpr int kConfMaxName = 255;

// "name group cluster homothety pos vel acc Q vrot arot\n"
__global__ void k_conf_bodies(Scene s, const char* names, const int* name_ofs, int prec, char* slots,
                              int64_t* lens) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= s.n) return;
  char* o = slots + b * (int64_t)kConfBodySlot;
  int L = 0;
  const int sh = s.shape[b];
  const int n0 = name_ofs[sh];
  int nl = name_ofs[sh + 1] - n0;
  if (nl > kConfMaxName) nl = kConfMaxName;
  for (int k = 0; k < nl; k++) o[L++] = names[n0 + k];
  o[L++] = ' ';
  L += fmt_i(s.group[b], o + L);
  o[L++] = ' ';
  L += fmt_i(s.cluster[b], o + L);
  o[L++] = ' ';
  L += fmt_e(s.hom[b], prec, false, o + L);
  const double* f[6] = {s.pos + 3 * b, s.vel + 3 * b, s.acc + 3 * b, s.Q + 4 * b, s.vrot + 3 * b, s.arot + 3 * b};
  const int cnt[6] = {3, 3, 3, 4, 3, 3};
  for (int q = 0; q < 6; q++)
    for (int d = 0; d < cnt[q]; d++) {
      o[L++] = ' ';
      L += fmt_e(f[q][d], prec, false, o + L);
    }
  o[L++] = '\n';
  lens[b] = L;
}

// 1 for the entries saveConf writes: dn < 0 or bonded (Rockable.cpp:3005-3029)
__global__ void k_conf_active(Scene s, int64_t* flag) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= s.ne) return;
  flag[e] = (s.dn[e] < 0.0 || s.bond[e] >= 0) ? 1 : 0;
}

// "i j type isub jsub n dn pos vel fn ft mom damp\n", the normal rounded
// toward zero (Rockable.cpp:569-575); line k of the active entries
__global__ void k_conf_entries(Scene s, const int64_t* pos, int prec, char* slots, int64_t* lens) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= s.ne) return;
  if (!(s.dn[e] < 0.0 || s.bond[e] >= 0)) return;
  const int64_t k = pos[e];
  char* o = slots + k * (int64_t)kConfEntrySlot;
  int L = 0;
  const uint32_t ts = s.etsub[e];
  const long long iv[5] = {s.ei[e], s.ej[e], tsub_type(ts), tsub_isub(ts), tsub_jsub(ts)};
  for (int q = 0; q < 5; q++) {
    if (q) o[L++] = ' ';
    L += fmt_i(iv[q], o + L);
  }
  for (int d = 0; d < 3; d++) {
    o[L++] = ' ';
    L += fmt_e(s.gn[3 * e + d], prec, true, o + L);
  }
  o[L++] = ' ';
  L += fmt_e(s.dn[e], prec, false, o + L);
  const double* f[2] = {s.gpos + 3 * e, s.gvel + 3 * e};
  for (int q = 0; q < 2; q++)
    for (int d = 0; d < 3; d++) {
      o[L++] = ' ';
      L += fmt_e(f[q][d], prec, false, o + L);
    }
  o[L++] = ' ';
  L += fmt_e(s.fn[e], prec, false, o + L);
  const double* g[2] = {s.ft + 3 * e, s.mom + 3 * e};
  for (int q = 0; q < 2; q++)
    for (int d = 0; d < 3; d++) {
      o[L++] = ' ';
      L += fmt_e(g[q][d], prec, false, o + L);
    }
  o[L++] = ' ';
  L += fmt_e(s.damp[e], prec, false, o + L);
  o[L++] = '\n';
  lens[k] = L;
}

// line k of `slots` to out + ofs[k]: one warp per line
__global__ void k_conf_pack(const char* slots, int slot, const int64_t* ofs, const int64_t* lens, int64_t n,
                            char* out) {
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= n) return;
  const char* src = slots + k * (int64_t)slot;
  char* dst = out + ofs[k];
  const int64_t L = lens[k];
  for (int64_t q = lane; q < L; q += 32) dst[q] = src[q];
}

}  // namespace rk
