// dfloat.cuh -- double-float arithmetic: a value as the unevaluated sum hi + lo
// of two FP32 numbers (about 47 significant bits).  The fixed-point forms run
// their vector kernels (CI apply, RDM gathers, one-body apply, Gram partials,
// the Lanczos first pass and update) in it, because GB300 issues FP64 at two
// FMA per cycle per SM and FP32 at 128.  A complex value is float4
// {re.hi, re.lo, im.hi, im.lo} (16 bytes, as an FP64 complex).
//
// Every conversion between FP64 and double-float is done by integer
// operations on the bit patterns, so that no instruction of these kernels
// needs the FP64 pipe.  The helpers compile for the host as well, where the
// CPU tests check them against exact arithmetic.
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <math.h>

#define DF_HD __host__ __device__ __forceinline__

DF_HD unsigned df_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  unsigned u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
DF_HD float df_float(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
DF_HD unsigned long long df_bits64(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
DF_HD double df_double(unsigned long long u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
// index of the most significant set bit of r > 0
DF_HD int df_msb(unsigned r) {
#ifdef __CUDA_ARCH__
  return 31 - __clz((int)r);
#else
  return 31 - __builtin_clz(r);
#endif
}

// x as hi + lo: hi = the leading 24 bits (truncated), lo = the next 29 bits
// rounded to the nearest 24 (an FP32 subnormal, with fewer bits, below
// 2^-126); |x| < 2^-100 becomes 0 and |x| >= 2^128 infinity.  Rounding, not
// truncation: a value split and converted back many times (a state advanced
// over thousands of steps) must not drift by a one-sided bias.
DF_HD float2 df_split(double x) {
  const unsigned long long u = df_bits64(x);
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7FF) - 1023;
  if (e < -100) return make_float2(0.0f, 0.0f);
  if (e > 127) return make_float2(df_float(sign | 0x7F800000u), 0.0f);
  const float hi = df_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((u >> 29) & 0x7FFFFF));
  unsigned r = (unsigned)(u & 0x1FFFFFFF);  // value r 2^(e-52)
  if (r == 0) return make_float2(hi, 0.0f);
  int msb = df_msb(r);
  if (msb > 23) {  // round r to its leading 24 bits (half to even); may carry to 2^(msb+1)
    const int sh = msb - 23;
    r = ((r + (1u << (sh - 1)) - 1u + ((r >> sh) & 1u)) >> sh) << sh;
    msb = df_msb(r);
  }
  const int elo = e - 52 + msb;
  if (elo < -126) {  // lo = r 2^(e-52) in units of 2^-149 (below 2^23 here)
    const int sh = e + 97;
    return make_float2(hi, df_float(sign | (sh >= 0 ? r << sh : r >> -sh)));
  }
  const unsigned mlo = (msb >= 23) ? ((r >> (msb - 23)) & 0x7FFFFF) : ((r << (23 - msb)) & 0x7FFFFF);
  return make_float2(hi, df_float(sign | ((unsigned)(elo + 127) << 23) | mlo));
}

DF_HD float4 zdf_from(double2 z) {
  const float2 r = df_split(z.x), i = df_split(z.y);
  return make_float4(r.x, r.y, i.x, i.y);
}

// (s, c) += p + q with an exact FP32 two-sum of s + p; the rounding errors and
// q accumulate in c.
DF_HD void df_acc(float& s, float& c, float p, float q) {
  const float t = s + p;
  const float bp = t - s;
  const float err = (s - (t - bp)) + (p - bp);
  s = t;
  c += err + q;
}

// (s, c) += a * b for double-floats a, b (error-free FP32 product plus cross terms).
DF_HD void df_mul_acc(float& s, float& c, float a1, float a2, float b1, float b2) {
  const float p = a1 * b1;
  float e = fmaf(a1, b1, -p);
  e = fmaf(a1, b2, e);
  e = fmaf(a2, b1, e);
  df_acc(s, c, p, e);
}
// (s, c) from df_acc as a normalised double-float (hi, lo) by a fast two-sum
// (|c| well below |s|, as the accumulators keep it)
DF_HD float2 df_norm(float s, float c) {
  const float hi = s + c;
  return make_float2(hi, c - (hi - s));
}
// a + b as a normalised double-float for any a, b (exact two-sum)
DF_HD float2 df_two_sum(float a, float b) {
  const float t = a + b;
  const float bp = t - a;
  return make_float2(t, (a - (t - bp)) + (b - bp));
}
// a b + c d for double-floats, normalised
DF_HD float2 df_dot2(float2 a, float2 b, float2 c, float2 d) {
  float s = 0.0f, e = 0.0f;
  df_mul_acc(s, e, a.x, a.y, b.x, b.y);
  df_mul_acc(s, e, c.x, c.y, d.x, d.y);
  return df_norm(s, e);
}
// a b + c d + e f for double-floats, normalised
DF_HD float2 df_dot3(float2 a, float2 b, float2 c, float2 d, float2 e, float2 f) {
  float s = 0.0f, r = 0.0f;
  df_mul_acc(s, r, a.x, a.y, b.x, b.y);
  df_mul_acc(s, r, c.x, c.y, d.x, d.y);
  df_mul_acc(s, r, e.x, e.y, f.x, f.y);
  return df_norm(s, r);
}

// An FP32 value as FP64 (exact; zero and FP32 subnormals, below 2^-126, give 0).
DF_HD double f2d_exact(float f) {
  const unsigned u = df_bits(f);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e == 0) return 0.0;
  const unsigned long long be = (e == 0xFFu) ? 0x7FFull : (unsigned long long)(e - 127 + 1023);
  return df_double(((unsigned long long)(u >> 31) << 63) | (be << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29));
}

// hi + lo as FP64, for any pair: one exact two-sum makes |lo| <= ulp(hi)/2,
// then the FP64 pattern of hi has 29 zero bits below its 24-bit mantissa and
// lo, in units of that pattern's last place (2^(e_hi-52)), is below 2^29.  The
// scaled lo is or-ed into those bits when the signs agree and subtracted from
// the 64-bit pattern when they differ -- in units one place finer when hi is
// a power of two, whose lower neighbours are twice as dense.  Bits of lo below
// the FP64 last place are rounded to the nearest place (half to even);
// a subnormal lo counts with its exponent 2^-126 and no leading bit; hi below
// 2^-126 gives 0, an infinite or NaN hi passes through.
DF_HD double df_to_d(float2 a) {
  const float2 n = df_two_sum(a.x, a.y);
  const unsigned H = df_bits(n.x), L = df_bits(n.y);
  const int eH = (int)((H >> 23) & 0xFFu), eL = (int)((L >> 23) & 0xFFu);
  if (eH == 0) return 0.0;
  const unsigned mH = H & 0x7FFFFFu;
  const unsigned hiw = (H & 0x80000000u) | ((unsigned)(eH == 0xFF ? 0x7FF : eH + 896) << 20) | (mH >> 3);
  const unsigned low = mH << 29;
  if ((L & 0x7FFFFFFFu) == 0 || eH == 0xFF) return df_double(((unsigned long long)hiw << 32) | low);
  const bool opp = ((H ^ L) & 0x80000000u) != 0;
  const int s = (eL ? eL : 1) - eH + 29 + ((opp && mH == 0) ? 1 : 0);
  const unsigned mL = (L & 0x7FFFFFu) | (eL ? 0x800000u : 0u);
  const unsigned k =
      (s >= 0) ? (mL << s) : (s > -25 ? ((mL + (1u << (-s - 1)) - 1u + ((mL >> -s) & 1u)) >> -s) : 0u);
  const unsigned long long u = ((unsigned long long)hiw << 32) | low;
  return df_double(opp ? u - k : (u | k));
}

// a complex accumulator of double-float parts (not normalised)
struct zdf_acc {
  float rs, rc, is, ic;
};

DF_HD double2 zdf_to_z(const zdf_acc& a) {
  return make_double2(df_to_d(make_float2(a.rs, a.rc)), df_to_d(make_float2(a.is, a.ic)));
}

// acc += h * x for complex double-float h, x; x negated when neg (sign bits).
DF_HD void zdf_fma(zdf_acc& a, float4 h, float4 x, bool neg) {
  if (neg) {
    x.x = -x.x;
    x.y = -x.y;
    x.z = -x.z;
    x.w = -x.w;
  }
  // products a b of double-floats: p = a1 b1 exactly as p + e, plus the cross terms
  float p, e;
  p = h.x * x.x;
  e = fmaf(h.x, x.x, -p);
  e = fmaf(h.x, x.y, e);
  e = fmaf(h.y, x.x, e);
  df_acc(a.rs, a.rc, p, e);  // + hr xr
  p = h.z * x.z;
  e = fmaf(h.z, x.z, -p);
  e = fmaf(h.z, x.w, e);
  e = fmaf(h.w, x.z, e);
  df_acc(a.rs, a.rc, -p, -e);  // - hi xi
  p = h.x * x.z;
  e = fmaf(h.x, x.z, -p);
  e = fmaf(h.x, x.w, e);
  e = fmaf(h.y, x.z, e);
  df_acc(a.is, a.ic, p, e);  // + hr xi
  p = h.z * x.x;
  e = fmaf(h.z, x.x, -p);
  e = fmaf(h.z, x.y, e);
  e = fmaf(h.w, x.x, e);
  df_acc(a.is, a.ic, p, e);  // + hi xr
}

// acc += conj(h) * x for complex double-floats; x negated when neg.
DF_HD void zdf_cfma(zdf_acc& a, float4 h, float4 x, bool neg) {
  h.z = -h.z;
  h.w = -h.w;
  zdf_fma(a, h, x, neg);
}
