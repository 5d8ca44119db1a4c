// rk_fmt.cuh -- exact decimal formatting of doubles, on the device and the host.
//
// fmt_e(x, p, toward_zero, out) writes what the C library's printf("%.*e", p,
// x) writes: the decimal value of the binary number x rounded to p + 1
// significant digits -- to nearest with ties to even (the default rounding
// mode) or toward zero (the mode Rockable::saveConf sets around the contact
// normals, Rockable.cpp:569-575) -- as d.ddd...e+XX (at least two exponent
// digits), "inf" / "nan" with their sign.  The rounding is exact: x = m 2^q is
// scaled by the power of ten that leaves p + 2 integer digits, with big
// integers of 32-bit limbs (the scaled value of the smallest subnormal needs
// about 1200 bits), and the extra digit plus a sticky bit decide.  Formatting
// a conf file's numbers this way on the device gives the same text as the
// host's stream would.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define RK_FMT_FN __host__ __device__ __forceinline__
#else
#define RK_FMT_FN inline
#endif

namespace rk {

constexpr int kFmtLimbs = 40;  // 1280 bits

struct BigU {
  uint32_t w[kFmtLimbs];
  int n;  // limbs in use (w[n-1] != 0 unless n == 0)
};

RK_FMT_FN void big_set(BigU& a, uint64_t v) {
  a.n = 0;
  while (v) {
    a.w[a.n++] = (uint32_t)v;
    v >>= 32;
  }
}

RK_FMT_FN void big_mul_small(BigU& a, uint32_t f) {
  uint64_t carry = 0;
  for (int i = 0; i < a.n; i++) {
    const uint64_t t = (uint64_t)a.w[i] * f + carry;
    a.w[i] = (uint32_t)t;
    carry = t >> 32;
  }
  if (carry && a.n < kFmtLimbs) a.w[a.n++] = (uint32_t)carry;
}

// a = a / d, returns the remainder
RK_FMT_FN uint32_t big_div_small(BigU& a, uint32_t d) {
  uint64_t r = 0;
  for (int i = a.n - 1; i >= 0; i--) {
    const uint64_t cur = (r << 32) | a.w[i];
    a.w[i] = (uint32_t)(cur / d);
    r = cur % d;
  }
  while (a.n > 0 && a.w[a.n - 1] == 0) a.n--;
  return (uint32_t)r;
}

RK_FMT_FN void big_shl(BigU& a, int s) {
  if (a.n == 0) return;
  const int limbs = s >> 5, bits = s & 31;
  int n = a.n + limbs + 1;
  if (n > kFmtLimbs) n = kFmtLimbs;
  for (int i = n - 1; i >= 0; i--) {
    const int src = i - limbs;
    uint32_t hi = (src >= 0 && src < a.n) ? a.w[src] : 0u;
    uint32_t lo = (src - 1 >= 0 && src - 1 < a.n) ? a.w[src - 1] : 0u;
    a.w[i] = bits ? ((hi << bits) | (lo >> (32 - bits))) : hi;
  }
  a.n = n;
  while (a.n > 0 && a.w[a.n - 1] == 0) a.n--;
}

// a = a >> s; the highest shifted-out bit goes to *half, and the return
// value is 1 when any other shifted-out bit was set (sticky)
RK_FMT_FN int big_shr(BigU& a, int s, int* half) {
  *half = 0;
  if (s <= 0) return 0;
  int sticky = 0;
  const int hb = s - 1, hl = hb >> 5;
  if (hl < a.n) {
    *half = (int)((a.w[hl] >> (hb & 31)) & 1u);
    if (a.w[hl] & ((1u << (hb & 31)) - 1u)) sticky = 1;
  }
  for (int i = 0; i < hl && i < a.n; i++)
    if (a.w[i]) sticky = 1;
  const int limbs = s >> 5, bits = s & 31;
  const int n = a.n - limbs;
  if (n <= 0) {
    a.n = 0;
    return sticky;
  }
  for (int i = 0; i < n; i++) {
    const uint32_t lo = a.w[i + limbs];
    const uint32_t hi = (i + limbs + 1 < a.n) ? a.w[i + limbs + 1] : 0u;
    a.w[i] = bits ? ((lo >> bits) | (hi << (32 - bits))) : lo;
  }
  a.n = n;
  while (a.n > 0 && a.w[a.n - 1] == 0) a.n--;
  return sticky;
}

RK_FMT_FN void big_mul_pow10(BigU& a, int e) {
  while (e >= 9) {
    big_mul_small(a, 1000000000u);
    e -= 9;
  }
  uint32_t f = 1;
  while (e-- > 0) f *= 10u;
  if (f > 1) big_mul_small(a, f);
}

// a = a / 10^e; the remainder's first decimal digit (of the digits removed)
// goes to *first, whether any other removed digit was non-zero to *sticky
RK_FMT_FN void big_div_pow10(BigU& a, int e, int* first, int* sticky) {
  *first = 0;
  *sticky = 0;
  // all digits but the last removed one first, then that one
  int rest = e - 1;
  while (rest >= 9) {
    if (big_div_small(a, 1000000000u)) *sticky = 1;
    rest -= 9;
  }
  if (rest > 0) {
    uint32_t f = 1;
    for (int i = 0; i < rest; i++) f *= 10u;
    if (big_div_small(a, f)) *sticky = 1;
  }
  if (e > 0) *first = (int)big_div_small(a, 10u);
}

// the decimal digits of a (at most 40 of them) into d[], most significant
// first; returns their count
RK_FMT_FN int big_digits(BigU a, char* d) {
  char tmp[48];
  int k = 0;
  if (a.n == 0) tmp[k++] = '0';
  while (a.n > 0 && k < 48) tmp[k++] = (char)('0' + big_div_small(a, 10u));
  for (int i = 0; i < k; i++) d[i] = tmp[k - 1 - i];
  return k;
}

RK_FMT_FN int fmt_copy(char* out, const char* s) {
  int k = 0;
  while (s[k]) {
    out[k] = s[k];
    k++;
  }
  return k;
}

// printf("%.*e", prec, x) with prec in [0, 17]; returns the length written
// (at most prec + 9 characters; no terminating zero)
RK_FMT_FN int fmt_e(double x, int prec, bool toward_zero, char* out) {
  uint64_t u;
#if defined(__CUDA_ARCH__)
  u = (uint64_t)__double_as_longlong(x);
#else
  __builtin_memcpy(&u, &x, 8);
#endif
  const bool neg = (u >> 63) != 0;
  const int ex = (int)((u >> 52) & 0x7ff);
  const uint64_t frac = u & ((1ull << 52) - 1);
  int len = 0;
  if (neg) out[len++] = '-';
  if (ex == 0x7ff) {
    len += fmt_copy(out + len, frac ? "nan" : "inf");
    return len;
  }
  char dig[48];
  int k;  // decimal exponent of the first digit
  if (ex == 0 && frac == 0) {
    for (int i = 0; i <= prec; i++) dig[i] = '0';
    k = 0;
  } else {
    const uint64_t m = ex ? (frac | (1ull << 52)) : frac;
    const int q = ex ? ex - 1075 : -1074;
    // first estimate of floor(log10 x) from the binary exponent of the top bit
    int top = 63;
    while (!((m >> top) & 1ull)) top--;
    const int b2 = q + top;  // x in [2^b2, 2^(b2+1))
    k = (int)((b2 * 1233) >> 12);  // floor(b2 log10 2) or one less
    if (b2 < 0) k = -(int)(((-b2) * 1233 + 4095) >> 12);
    for (int attempt = 0; attempt < 4; attempt++) {
      // D = x 10^(prec + 1 - k): p + 2 digits, the last one for the rounding
      const int s = prec + 1 - k;
      BigU a;
      big_set(a, m);
      int first = 0, sticky = 0;
      if (s >= 0) {
        big_mul_pow10(a, s);
        if (q >= 0) {
          big_shl(a, q);
        } else {
          int half = 0;
          sticky = big_shr(a, -q, &half);
          sticky |= half;  // below the extra digit: only "non-zero" matters
        }
      } else {
        if (q >= 0) big_shl(a, q);
        else {
          int half = 0;
          sticky = big_shr(a, -q, &half) | half;
        }
        int st2 = 0;
        big_div_pow10(a, -s, &first, &st2);
        sticky |= first != 0 || st2;
      }
      char d[48];
      const int nd = big_digits(a, d);
      if (nd < prec + 2) {  // estimate one too high
        k--;
        continue;
      }
      if (nd > prec + 2) {  // one too low
        k++;
        continue;
      }
      // d = the p + 1 kept digits and one extra digit; sticky = below it
      const int extra = d[prec + 1] - '0';
      bool up = false;
      if (!toward_zero) {
        if (extra > 5) up = true;
        else if (extra == 5) up = sticky || ((d[prec] - '0') & 1);
      }
      if (up) {
        int i = prec;
        while (i >= 0 && d[i] == '9') d[i--] = '0';
        if (i >= 0) d[i]++;
        else {  // 9.99..9 rounded up: 1.00..0 of the next decade
          d[0] = '1';
          for (int j = 1; j <= prec; j++) d[j] = '0';
          k++;
        }
      }
      for (int i = 0; i <= prec; i++) dig[i] = d[i];
      break;
    }
  }
  out[len++] = dig[0];
  if (prec > 0) {
    out[len++] = '.';
    for (int i = 1; i <= prec; i++) out[len++] = dig[i];
  }
  out[len++] = 'e';
  out[len++] = k < 0 ? '-' : '+';
  int ak = k < 0 ? -k : k;
  if (ak >= 100) {
    out[len++] = (char)('0' + ak / 100);
    ak %= 100;
    out[len++] = (char)('0' + ak / 10);
    out[len++] = (char)('0' + ak % 10);
  } else {
    out[len++] = (char)('0' + ak / 10);
    out[len++] = (char)('0' + ak % 10);
  }
  return len;
}

// a signed integer in decimal
RK_FMT_FN int fmt_i(long long v, char* out) {
  char tmp[24];
  int k = 0, len = 0;
  unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  if (v < 0) out[len++] = '-';
  do {
    tmp[k++] = (char)('0' + a % 10ull);
    a /= 10ull;
  } while (a);
  while (k) out[len++] = tmp[--k];
  return len;
}

}  // namespace rk
