// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32 numbers
// (|lo| <= ulp(hi)), carrying about 47 significant bits.  GB300 runs FP32 fused multiply-adds
// at roughly 70 times its FP64 rate, so the FP64-bound kernels of precision mode 3 compute in
// this format while the fields stay FP64 in memory.
//
// The building blocks are the error-free transformations of Knuth (two-sum) and Dekker
// (quick-two-sum), with the exact product error taken from a fused multiply-add; the add,
// multiply, divide and square root below follow the published double-word algorithms
// (e.g. Hida, Li and Bailey's double-double arithmetic; Joldes, Muller and Popescu, "Tight and
// rigorous error bounds for basic building blocks of double-word arithmetic", ACM TOMS 2017),
// written here for FP32 words.
//
// Conversions from FP64 split the bit pattern with integer and FP32 instructions (the FP64 pipe,
// where GB300 also does FP64<->FP32 conversions, is the scarce unit): hi takes the leading 24
// significant bits, lo the next 29 rounded to 24.  The range is 2^-70 .. 2^120 (smaller
// magnitudes become zero).  The conversion back to FP64 adds the two widened words with one FP64
// addition.
#pragma once
#include <cuda_runtime.h>

namespace sts {
namespace {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df quick_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df operator+(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df operator-(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ df operator/(df a, df b) {
  const float r = __frcp_rn(b.hi);
  const float q1 = __fmul_rn(a.hi, r);
  df rem = a - b * df{q1, 0.f};
  const float q2 = __fmul_rn(rem.hi, r);
  rem = rem - b * df{q2, 0.f};
  const float q3 = __fmul_rn(rem.hi, r);
  df q = quick_two_sum(q1, q2);
  return q + df{q3, 0.f};
}
__device__ __forceinline__ df dsqrt(df a) {
  if (!(a.hi > 0.f)) return {__fsqrt_rn(a.hi), 0.f};  // 0 (or a negative/NaN argument, as FP32)
  const float s = __fsqrt_rn(a.hi);
  const float p = __fmul_rn(s, s);
  const float pe = __fmaf_rn(s, s, -p);
  const df rem = a - df{p, pe};
  return quick_two_sum(s, __fdiv_rn(rem.hi, __fmul_rn(2.f, s)));
}
__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df to_df(double x);
// mixed operands: an FP64 scalar (a constant or a per-launch parameter) is split first
__device__ __forceinline__ df operator*(double a, df b) { return to_df(a) * b; }
__device__ __forceinline__ df operator*(df a, double b) { return a * to_df(b); }
__device__ __forceinline__ df operator+(double a, df b) { return to_df(a) + b; }
__device__ __forceinline__ df operator+(df a, double b) { return a + to_df(b); }
__device__ __forceinline__ df operator-(double a, df b) { return to_df(a) - b; }
__device__ __forceinline__ df operator-(df a, double b) { return a - to_df(b); }
__device__ __forceinline__ df operator/(double a, df b) { return to_df(a) / b; }
__device__ __forceinline__ df fmax0(df a) { return a.hi > 0.f ? a : df{0.f, 0.f}; }
__device__ __forceinline__ df dabs(df a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ double dabs(double a) { return ::fabs(a); }
__device__ __forceinline__ double dsqrt(double a) { return ::sqrt(a); }
__device__ __forceinline__ double fmax0(double a) { return fmax(0.0, a); }

// FP64 -> double-float by integer splitting of the bit pattern.  No FP64 instruction appears
// even on the rare paths (a predicated FP64 instruction still costs an issue slot on GB300's
// narrow FP64 pipe): magnitudes below 2^-70 become zero, above 2^120 infinity (NaN stays NaN).
__device__ __forceinline__ df to_df(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32);
  const unsigned sign = hi32 & 0x80000000u;
  const int E = (int)((hi32 >> 20) & 0x7ffu) - 1023;
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (E < -70) return {__uint_as_float(sign), 0.f};
  if (E > 120) return {__uint_as_float(sign | (E == 1024 && m ? 0x7fc00000u : 0x7f800000u)), 0.f};
  const float h = __uint_as_float(sign | ((unsigned)(E + 127) << 23) | (unsigned)(m >> 29));
  // the remaining 29 bits ml, times 2^(E-52), rounded once: ml = 64 a + c with a < 2^23, c < 64,
  // each converted exactly by the 2^23 bias trick, then a fused a*64 + c
  const unsigned ml = (unsigned)(m & 0x1FFFFFFFull);
  const float a = __fsub_rn(__uint_as_float(0x4b000000u | (ml >> 6)), 8388608.0f);
  const float c = __fsub_rn(__uint_as_float(0x4b000000u | (ml & 63u)), 8388608.0f);
  const float l = __fmul_rn(__fmaf_rn(a, 64.0f, c), __uint_as_float((unsigned)(E - 52 + 127) << 23));
  return {h, __uint_as_float(__float_as_uint(l) | sign)};
}
// FP32 -> FP64 widening by integer re-biasing (subnormal FP32 values become zero).
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  unsigned long long d;
  if (e == 0u) d = sign;
  else if (e == 0xffu) d = sign | 0x7ff0000000000000ull | ((unsigned long long)(u & 0x7fffffu) << 29);
  else d = sign | ((unsigned long long)(e - 127u + 1023u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}
__device__ __forceinline__ double to_double(df a) { return __dadd_rn(widen(a.hi), widen(a.lo)); }
__device__ __forceinline__ double to_double(double a) { return a; }
__device__ __forceinline__ float to_float(df a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ float to_float(double a) { return (float)a; }

// Number-type plumbing for kernels written once for FP64 (R = double) and double-float.
template <class R>
__device__ __forceinline__ R num(double x);
template <>
__device__ __forceinline__ double num<double>(double x) { return x; }
template <>
__device__ __forceinline__ df num<df>(double x) { return to_df(x); }

template <class R>
struct Arr {
  const double* __restrict__ p;
  __device__ __forceinline__ R operator[](int i) const { return num<R>(p[i]); }
};

}  // namespace
}  // namespace sts
