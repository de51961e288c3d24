// Host-side check of the double-float helpers (codyfortran_gb300/csrc/dfloat.cuh),
// compiled by nvcc as host code and run by tests/test_double_float.py.
// Prints one line of counts and error maxima as JSON.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "../codyfortran_gb300/csrc/dfloat.cuh"

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;
uint64_t next_u64() {  // splitmix64
  uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform() { return (double)(next_u64() >> 11) * 0x1.0p-53; }

// a double with random sign, 52 random mantissa bits and a binary exponent in [lo, hi]
double random_double(int elo, int ehi) {
  const int e = elo + (int)(next_u64() % (uint64_t)(ehi - elo + 1));
  const uint64_t bits = ((next_u64() & 1) << 63) | ((uint64_t)(e + 1023) << 52) | (next_u64() & ((1ull << 52) - 1));
  double x;
  std::memcpy(&x, &bits, 8);
  return x;
}
// a float with random sign and mantissa, 2^e <= |f| < 2^(e+1), e in [lo, hi]
// (an FP32 subnormal below 2^-126)
float random_float(int elo, int ehi) {
  const int e = elo + (int)(next_u64() % (uint64_t)(ehi - elo + 1));
  const float m = 1.0f + (float)(next_u64() & 0x7FFFFF) * 0x1.0p-23f;
  return std::ldexp((next_u64() & 1) ? -m : m, e);
}
double ulp(double x) {
  const double a = std::fabs(x);
  return std::nextafter(a, INFINITY) - a;
}

}  // namespace

int main() {
  // 1. df_split then df_to_d gives x with the low part rounded to 24 bits
  long split_cases = 0, split_bad = 0;
  double split_rel = 0.0;
  for (int i = 0; i < 2000000; i++) {
    const double x = (i % 7 == 0) ? std::ldexp(std::floor(uniform() * 1e6), -(int)(next_u64() % 40)) : random_double(-90, 120);
    const float2 s = df_split(x);
    uint64_t u;
    std::memcpy(&u, &x, 8);
    const uint32_t r = (uint32_t)(u & 0x1FFFFFFF);
    uint64_t want = u;
    if (r) {
      const int msb = 31 - __builtin_clz(r);
      if (msb > 23) {  // round half to even; a carry out of the 29 bits adds to hi's pattern
        const int sh = msb - 23;
        const uint64_t rr = (uint64_t)(((r + (1u << (sh - 1)) - 1u + ((r >> sh) & 1u)) >> sh) << sh);
        want = (u & ~0x1FFFFFFFull) + rr;
      }
    }
    double w;
    std::memcpy(&w, &want, 8);
    const double back = df_to_d(s);
    split_cases++;
    if (back != w) split_bad++;
    if (x != 0.0) split_rel = std::fmax(split_rel, std::fabs(back - x) / std::fabs(x));
  }
  // bias of the split and back: mean signed relative error over random values
  double bias = 0.0;
  for (int i = 0; i < 2000000; i++) {
    const double x = std::ldexp(1.0 + uniform(), (int)(next_u64() % 40) - 20);
    bias += (df_to_d(df_split(x)) - x) / x;
  }
  bias /= 2000000.0;
  // 2. df_to_d(hi, lo) against the correctly rounded FP64 sum, for any pair
  long conv_cases = 0, conv_flushed = 0, conv_bad = 0, conv_exact_cases = 0, conv_exact_bad = 0;
  double conv_ulps = 0.0;
  for (int i = 0; i < 4000000; i++) {
    float hi = random_float(-120, 120);
    const int kind = i % 8;
    if (kind == 0) hi = df_float(df_bits(hi) & 0xFF800000u);  // a power of two
    const int eh = (int)((df_bits(hi) >> 23) & 0xFF) - 127;
    float lo;
    if (kind == 1)
      lo = 0.0f;
    else if (kind == 2)
      lo = random_float(eh - 60, eh - 30);  // far below the FP64 last place
    else if (kind == 3)
      lo = random_float(eh - 2, eh + 1);  // not normalised: two-sum first
    else
      lo = random_float(eh - 30, eh - 22);
    if (kind == 0 && (i & 16)) lo = -std::fabs(lo) * (hi > 0 ? 1.0f : -1.0f);
    const double want = (double)hi + (double)lo;
    const double got = df_to_d(make_float2(hi, lo));
    if (std::fabs(want) < 0x1.0p-126) {  // below the FP32 normal range: 0 by design
      conv_flushed += got == 0.0;
      continue;
    }
    conv_cases++;
    const double du = std::fabs(got - want) / ulp(want);
    conv_ulps = std::fmax(conv_ulps, du);
    if (du > 1.0) conv_bad++;
    // exactly representable sums (lo at most 29 places below hi's last bit) come out exact
    const int el = (int)((df_bits(lo) >> 23) & 0xFF) - 127;
    if (lo != 0.0f && el - 23 >= eh - 52 && kind != 3) {
      conv_exact_cases++;
      if (got != want) conv_exact_bad++;
    }
  }
  // 3. complex dot products in double-float against long double sums
  double dot_rel = 0.0;
  for (int t = 0; t < 2000; t++) {
    const int n = 1 + (int)(next_u64() % 600);
    zdf_acc a = {0.0f, 0.0f, 0.0f, 0.0f};
    long double wr = 0.0L, wi = 0.0L, mag = 0.0L;
    for (int k = 0; k < n; k++) {
      const double2 h = make_double2(random_double(-8, 2), random_double(-8, 2));
      const double2 x = make_double2(random_double(-8, 2), random_double(-8, 2));
      const bool neg = (next_u64() & 3) == 0;
      zdf_fma(a, zdf_from(h), zdf_from(x), neg);
      const long double sg = neg ? -1.0L : 1.0L;
      wr += sg * ((long double)h.x * x.x - (long double)h.y * x.y);
      wi += sg * ((long double)h.x * x.y + (long double)h.y * x.x);
      mag += std::fabs((long double)h.x * x.x) + std::fabs((long double)h.y * x.y) +
             std::fabs((long double)h.x * x.y) + std::fabs((long double)h.y * x.x);
    }
    const double2 z = zdf_to_z(a);
    const double e = (double)((std::fabs(z.x - wr) + std::fabs(z.y - wi)) / mag);
    dot_rel = std::fmax(dot_rel, e);
  }
  // 4. special values
  const bool specials = df_to_d(make_float2(0.0f, 0.0f)) == 0.0 && std::isinf(df_to_d(make_float2(INFINITY, 0.0f))) &&
                        df_to_d(make_float2(1e-40f, 0.0f)) == 0.0 && df_to_d(make_float2(1.0f, 1e-45f)) == 1.0;
  std::printf("{\"split_cases\": %ld, \"split_bad\": %ld, \"split_rel_max\": %.3e, \"conv_cases\": %ld, "
              "\"conv_flushed\": %ld, \"conv_bad\": %ld, \"conv_ulps_max\": %.3f, \"conv_exact_cases\": %ld, \"conv_exact_bad\": %ld, "
              "\"dot_rel_max\": %.3e, \"split_bias\": %.3e, \"specials\": %s}\n",
              split_cases, split_bad, split_rel, conv_cases, conv_flushed, conv_bad, conv_ulps, conv_exact_cases, conv_exact_bad,
              dot_rel, bias, specials ? "true" : "false");
  return 0;
}
