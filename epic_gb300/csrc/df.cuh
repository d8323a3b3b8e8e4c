// Double-float arithmetic: a value carried as an unevaluated sum hi + lo of two binary32
// numbers (|lo| <= ulp(hi)/2), about 48 significant bits, computed on the FP32 pipe.
//
// GB300 runs FP32 at ~64 times its FP64 rate, so where the mixed form needs more than FP32
// precision in arithmetic-only code (the finite-volume pressure gradient, whose face integrals
// cancel to a few parts in a thousand), double-float is the fast way to get it.  The algorithms
// are the classical error-free transformations (Knuth's two-sum, Dekker's two-product by FMA)
// and the "sloppy" double-double add, multiply and divide of Hida, Li and Bailey's QD library,
// restated for binary32: relative error of a product or quotient ~ 2^-44, absolute error of a
// sum ~ 2^-44 of the larger operand.  The file is compiled with -fmad=false, so no expression
// here is contracted into an FMA behind the algorithms' back; the FMAs are explicit.
#pragma once
#include <cuda_runtime.h>

namespace epic {

struct dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // from a compile-time constant (the literals of the kernel templates): folded by the compiler
  __host__ __device__ constexpr dfl(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
};

__device__ __forceinline__ dfl df_quick_two_sum(float a, float b) {   // |a| >= |b|
  const float s = a + b;
  return dfl(s, b - (s - a));
}
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return dfl(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ dfl df_two_prod(float a, float b) {
  const float p = a * b;
  return dfl(p, fmaf(a, b, -p));
}

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  dfl s = df_two_sum(a.hi, b.hi);
  return df_quick_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  dfl p = df_two_prod(a.hi, b.hi);
  return df_quick_two_sum(p.hi, p.lo + (a.hi * b.lo + a.lo * b.hi));
}
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float q1 = a.hi / b.hi;                 // first quotient digit
  const dfl r = a - b * dfl(q1, 0.f);           // remainder
  const float q2 = r.hi / b.hi;                 // correction
  return df_quick_two_sum(q1, q2);
}
__device__ __forceinline__ dfl &operator+=(dfl &a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl &operator-=(dfl &a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl &operator*=(dfl &a, dfl b) { return a = a * b; }
__device__ __forceinline__ dfl &operator/=(dfl &a, dfl b) { return a = a / b; }
__device__ __forceinline__ bool operator>(dfl a, dfl b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool operator<(dfl a, dfl b) { return b > a; }
__device__ __forceinline__ bool operator>=(dfl a, dfl b) { return !(a < b); }
__device__ __forceinline__ bool operator<=(dfl a, dfl b) { return !(a > b); }
using ::fabs;   // the binary32/binary64 overloads stay visible beside this one
__device__ __forceinline__ dfl fabs(dfl a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f) ? -a : a; }

// a 2^e for -126 <= e <= 127: the scale is a normal binary32 power of two, so each part is one
// exactly rounded multiplication (the value ldexpf gives, without its range handling)
__device__ __forceinline__ dfl df_ldexp(dfl a, int e) {
  const float s = __int_as_float((e + 127) << 23);
  return dfl(a.hi * s, a.lo * s);
}

// ---- exp and log (relative error ~1e-13 over the arguments the model uses) ----
//
// exp: x = N ln2/32 + r with N = rint(32 x / ln2), |r| <= ln2/64; exp(x) = 2^(N>>5) T[N&31] exp(r),
// T[j] = 2^(j/32) as double-floats (tab, filled on the host), exp(r) by its Taylor polynomial to
// r^5/120 (the first omitted term is below 2.2e-15 relative).  Arguments must keep the result a
// normal binary32 number (|x| < 87).
__device__ __forceinline__ dfl exp_df(dfl x, const float2 *tab) {
  constexpr dfl LN2_32(0.021660849392498290);   // ln(2)/32
  const float nf = rintf(x.hi * 46.166241308446828f);   // 32/ln(2)
  const int n = (int)nf;
  const dfl r = x - dfl(nf, 0.f) * LN2_32;
  // exp(r) = 1 + r (1 + r (1/2 + tail)), tail = r/6 + r^2/24 + r^3/120 < 2e-3: its float
  // rounding moves the result by less than 2e-14 relative
  const float rh = r.hi;
  const float tail = rh * (1.f / 6.f + rh * (1.f / 24.f + rh * (1.f / 120.f)));
  dfl p = dfl(0.5f, 0.f) + dfl(tail, 0.f);
  p = dfl(1.f, 0.f) + p * r;
  p = dfl(1.f, 0.f) + p * r;
  const float2 t = __ldg(tab + (n & 31));
  return df_ldexp(dfl(t.x, t.y) * p, n >> 5);
}
// log: one Newton step y0 + x exp(-y0) - 1 from the hardware's approximate logarithm y0
// (__logf: lg2.approx times ln 2, absolute error ~1e-7 for arguments near 1 and relative error
// a few 2^-23 elsewhere); the step is quadratic, so that error leaves ~1e-14.  x > 0 with
// 2^-120 < x < 2^120 (exp_df's range for -y0).
__device__ __forceinline__ dfl log_df(dfl x, const float2 *tab) {
  const float y0 = __logf(x.hi);
  const dfl t = x * exp_df(dfl(-y0, 0.f), tab);
  return dfl(y0, 0.f) + (t - dfl(1.f, 0.f));
}

}  // namespace epic
