// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats (|lo| <= ulp(hi)), a 48-bit significand with float's exponent
// range.  On GB300 the FP32 pipes issue about 70 times as many operations per
// cycle as the FP64 pipe, and a double-float add or multiply costs 7-11
// float operations, so the FP64-accuracy transforms run faster this way than
// in IEEE double.
//
// Algorithms (published, restated here): Knuth's TwoSum and Dekker's
// FastTwoSum for exact sums, the FMA form of TwoProduct for exact products,
// and the "sloppy" double-float addition of Dekker (1971) / Shewchuk, whose
// error is bounded relative to |a| + |b| -- the bound FFT error analysis
// uses.  Every step uses the _rn intrinsics so that the compiler neither
// contracts a multiply and an add into an FMA nor reassociates.
//
// Memory keeps IEEE double: conversions split and join the bit patterns with
// integer operations, because f64 <-> f32 conversion instructions run on the
// FP64 pipe.  Twiddle tables of double-float plans are stored as (hi, lo)
// pairs and load without conversion.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace afg {

struct df {
  float hi, lo;
  __host__ __device__ constexpr df() : hi(0.0f), lo(0.0f) {}
  // compile-time constants only: a run-time use would convert on the FP64 pipe
  __host__ __device__ explicit constexpr df(double d) : hi(float(d)), lo(float(d - double(float(d)))) {}
  __host__ __device__ constexpr df(float h, float l, int) : hi(h), lo(l) {}
};
struct dfc {
  df x, y;
};

__device__ __forceinline__ df df_make(float h, float l) { return df(h, l, 0); }

// FastTwoSum (|a| >= |b| or a == 0): s + e == a + b exactly
__device__ __forceinline__ df df_quick(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return df_make(s, e);
}

__device__ __forceinline__ df operator+(df a, df b) {
  // TwoSum of the high parts, then the low parts, then renormalise
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return df_quick(s, e);
}
__device__ __forceinline__ df operator-(df a) { return df_make(-a.hi, -a.lo); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);          // exact error of p
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_quick(p, e);
}
__device__ __forceinline__ df& operator+=(df& a, df b) { return a = a + b; }
__device__ __forceinline__ df& operator-=(df& a, df b) { return a = a - b; }
__device__ __forceinline__ df& operator*=(df& a, df b) { return a = a * b; }
__device__ __forceinline__ bool operator==(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }

// ------------------------------------------------------- IEEE double <-> df
// Both directions scale by an exact power of two: d * 2^k in, v * 2^-k out.
// A transform picks k so that its input's largest magnitude lands in
// [1, 2) (df_shift), which keeps every value of the transform inside float's
// exponent range whatever the data's scale.
//
// hi = the double's sign, exponent and top 23 significand bits (truncated),
// lo = the remaining 29 bits (rounded to 24); after scaling, values below
// 2^-126 flush to zero and lo is dropped below 2^-74 (|value| relative to the
// input's largest is then below 2^-75: far under the transform's rounding).
__device__ __forceinline__ df df_from_double(double d, int k) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const unsigned hw = unsigned(u >> 32), lw = unsigned(u);
  const unsigned sign = hw & 0x80000000u;
  const int e = int((hw >> 20) & 0x7FFu);
  const int ef = e - 896 + k;                    // float biased exponent of hi
  if (e == 0 || ef <= 0) return df_make(__uint_as_float(sign), __uint_as_float(sign));
  if (e == 0x7FF || ef >= 255) {                 // inf or nan, or beyond float range
    const bool nan = e == 0x7FF && ((hw & 0xFFFFFu) | lw) != 0;
    return df_make(__uint_as_float(sign | 0x7F800000u | (nan ? 0x400000u : 0u)), 0.0f);
  }
  const float hi = __uint_as_float(sign | (unsigned(ef) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
  const int el = e - 948 + k;                    // float biased exponent of 2^(e - 1075 + k)
  float lo = 0.0f;
  if (el > 0) lo = __fmul_rn(__uint2float_rn(lw & 0x1FFFFFFFu), __uint_as_float(unsigned(el) << 23));
  return df_make(hi, sign ? -lo : lo);
}

// the double nearest (hi + lo) * 2^-k (ties and the bits below 2^-53 |hi|
// truncated; results below the double normal range flush to zero)
__device__ __forceinline__ double df_to_double(df v, int k) {
  // renormalise so that |lo| <= ulp(hi) / 2 with hi = fl(hi + lo)
  v = df_quick(v.hi, v.lo);
  const unsigned hb = __float_as_uint(v.hi);
  const unsigned eh = (hb >> 23) & 0xFFu;
  if (eh == 0) return __longlong_as_double((long long)((unsigned long long)(hb & 0x80000000u) << 32));
  if (eh == 0xFFu) {                             // inf or nan
    const unsigned long long s = (unsigned long long)(hb & 0x80000000u) << 32;
    return __longlong_as_double((long long)(s | 0x7FF0000000000000ull | ((hb & 0x7FFFFFu) ? 1ull << 51 : 0ull)));
  }
  // significands as integers in units of 2^(eh - 127 - 52): hi = H << 29
  long long m = (long long)((unsigned long long)((hb & 0x7FFFFFu) | 0x800000u) << 29);
  const unsigned lb = __float_as_uint(v.lo);
  const unsigned el = (lb >> 23) & 0xFFu;
  if (el != 0) {
    const long long L = (long long)((lb & 0x7FFFFFu) | 0x800000u);
    const int sh = int(el) - int(eh) + 29;       // lo = L * 2^sh in those units; sh <= 5
    long long lv = sh >= 0 ? (L << sh) : (sh > -40 ? (L >> -sh) : 0);
    if ((lb ^ hb) & 0x80000000u) lv = -lv;       // lo's sign against hi's
    m += lv;
  }
  // |lo| <= ulp(hi)/2 keeps m within [2^52 - 2^28, 2^53 + 2^28]: renormalise one bit
  int ex = int(eh) - 127 + 1023 - k;
  if (m >= (1ll << 53)) {
    m >>= 1;
    ++ex;
  } else if (m < (1ll << 52)) {
    m <<= 1;
    --ex;
  }
  const unsigned long long s = (unsigned long long)(hb & 0x80000000u) << 32;
  if (ex <= 0) return __longlong_as_double((long long)s);
  if (ex >= 0x7FF) return __longlong_as_double((long long)(s | 0x7FF0000000000000ull));
  const unsigned long long bits = s | ((unsigned long long)ex << 52) | ((unsigned long long)m & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

// the scale exponent k of a transform whose input's largest biased double
// exponent is m (0: all zero or subnormal; 0x7FF: an inf or nan)
__device__ __forceinline__ int df_shift_of(int m) { return (m <= 0 || m >= 0x7FF) ? 0 : 1023 - m; }

}  // namespace afg
