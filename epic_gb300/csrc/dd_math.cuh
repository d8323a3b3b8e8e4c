// Correctly rounded log, exp and pow for binary64, evaluated in double-double arithmetic.
//
// The reference calls glibc's log/exp/pow, whose results are correctly rounded in all but a
// tiny fraction of cases.  Several of the reference's formulas cancel hard (the finite-volume
// pressure gradient differences products of geopotentials), so one-ulp differences in GZ3 or P2
// grow to ~4e-11 in U after a step from rest.  Evaluating these functions to ~2^-84 relative and
// rounding once gives the correctly rounded value in all but ~2^-30 of cases, and so the
// reference's value whenever glibc's is correctly rounded.
//
// Methods (textbook, no vendor code): the error-free transformations TwoSum (Knuth) and TwoProd
// with a fused multiply-add; log by x = 2^e m, m = c (1 + r) with c = k/1024 from a table of
// log(c) and 1/c, log(1+r) by its Taylor series (leading terms in double-double, the tail in
// double); exp by x = (1024 q + j) ln2/1024 + r with a table of 2^(j/1024), exp(r) by its Taylor
// series; pow = exp(y log x) with the double-double logarithm.  The tables are built on the
// host from slow, long double-double series (2 atanh((c-1)/(c+1)) and exp(y/2^10)^(2^10)).
//
// Each function first takes a fast path (Ziv's strategy): the same reductions with a shorter
// evaluation whose error is bounded well below 2^-69 of the result, then a rounding test that
// returns the result only if both ends of the error interval round to the same double.  About
// one call in 2^16 fails the test and goes on to the double-double evaluation above.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace epic {

struct dd { double hi, lo; };

__host__ __device__ __forceinline__ dd two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  const double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__host__ __device__ __forceinline__ dd fast_two_sum(double a, double b) {   // |a| >= |b|
  const double s = a + b;
  return {s, b - (s - a)};
}
__host__ __device__ __forceinline__ dd two_prod(double a, double b) {
  const double p = a * b;
  return {p, fma(a, b, -p)};
}
__host__ __device__ __forceinline__ dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  const dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
__host__ __device__ __forceinline__ dd dd_add_d(dd a, double b) {
  dd s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}
__host__ __device__ __forceinline__ dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
__host__ __device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
__host__ __device__ __forceinline__ dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo = fma(a.hi, b.lo, p.lo);
  p.lo = fma(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__host__ __device__ __forceinline__ dd dd_mul_d(dd a, double b) {
  dd p = two_prod(a.hi, b);
  p.lo = fma(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__host__ __device__ __forceinline__ dd dd_div(dd a, dd b) {
  const double q1 = a.hi / b.hi;
  dd r = dd_sub(a, dd_mul_d(b, q1));
  const double q2 = r.hi / b.hi;
  r = dd_sub(r, dd_mul_d(b, q2));
  const double q3 = r.hi / b.hi;
  return dd_add(fast_two_sum(q1, q2), {q3, 0.});
}

// ---- slow, long series used only to build the tables (host) ----

// 2 atanh(s) summed to 2^-106 for |s| <= 0.18.
inline dd slow_two_atanh(dd s) {
  const dd s2 = dd_mul(s, s);
  dd term = s, sum = s;
  for (int t = 1; t < 45; t++) {
    term = dd_mul(term, s2);
    sum = dd_add(sum, dd_div(term, {(double)(2 * t + 1), 0.}));
  }
  return {2. * sum.hi, 2. * sum.lo};
}
inline dd slow_log(double c) {   // c in [0.7, 1.45]
  return slow_two_atanh(dd_div(dd_sub({c, 0.}, {1., 0.}), dd_add({c, 0.}, {1., 0.})));
}
inline dd slow_exp(dd x) {       // |x| < 1: Taylor of exp(x/2^10), then ten squarings
  dd r = {ldexp(x.hi, -10), ldexp(x.lo, -10)};
  dd term = r, sum = dd_add({1., 0.}, r);
  for (int n = 2; n <= 14; n++) {
    term = dd_div(dd_mul(term, r), {(double)n, 0.});
    sum = dd_add(sum, term);
  }
  for (int q = 0; q < 10; q++) sum = dd_mul(sum, sum);
  return sum;
}

constexpr int LOG_K0 = 724;       // c = k/1024, k = 724 .. 1448 covers m in [sqrt(1/2), sqrt(2)]
constexpr int LOG_N = 725;
constexpr int EXP_N = 1024;

constexpr int ATAN_N = 33;       // atan(k/32), k = 0 .. 32

// atan(x) for 0 <= x <= 1 to 2^-106 by Euler's series
// atan(x) = sum_n (2^2n (n!)^2 / (2n+1)!) x^(2n+1) / (1+x^2)^(n+1), whose ratio x^2/(1+x^2) <= 1/2.
inline dd slow_atan(dd x) {
  const dd x2 = dd_mul(x, x);
  const dd den = dd_add_d(x2, 1.);
  const dd y = dd_div(x2, den);
  dd term = dd_div(x, den), sum = term;
  for (int n = 1; n < 130; n++) {
    term = dd_div(dd_mul(dd_mul(term, y), {(double)(2 * n), 0.}), {(double)(2 * n + 1), 0.});
    sum = dd_add(sum, term);
  }
  return sum;
}

struct MathTable {
  dd ln2;                  // ln 2
  dd ln2_1024;             // ln 2 / 1024
  dd logc[LOG_N];          // log(k/1024)
  double invc[LOG_N];      // 1024/k rounded
  dd exp2j[EXP_N];         // 2^(j/1024)
  dd atanc[ATAN_N];        // atan(k/32)
};

inline void fill_math_table(MathTable &t) {
  const dd third = dd_div({1., 0.}, {3., 0.});
  t.ln2 = slow_two_atanh(third);
  t.ln2_1024 = {ldexp(t.ln2.hi, -10), ldexp(t.ln2.lo, -10)};
  for (int i = 0; i < LOG_N; i++) {
    const double c = (double)(LOG_K0 + i) / 1024.;
    t.logc[i] = slow_log(c);
    t.invc[i] = 1. / c;
  }
  for (int j = 0; j < EXP_N; j++) t.exp2j[j] = slow_exp(dd_mul_d(t.ln2_1024, (double)j));
  for (int k = 0; k < ATAN_N; k++) t.atanc[k] = slow_atan({(double)k / 32., 0.});
}

// log(x) in double-double, x > 0 finite and normal.  Relative error ~2^-84.
__host__ __device__ __forceinline__ dd dd_log(double x, const MathTable &T) {
  int e;
  double m = frexp(x, &e);   // m in [0.5, 1)
  m *= 2.;
  e -= 1;                    // m in [1, 2)
  if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
  const int k = (int)rint(m * 1024.);
  const double c = (double)k * (1. / 1024.);
  const double num = m - c;                          // exact (Sterbenz)
  const double invc = T.invc[k - LOG_K0];
  const double rh = num * invc;
  const double rl = fma(-rh, c, num) * invc;
  const dd r = fast_two_sum(rh, rl);                 // |r| < 7e-4
  const dd r2 = dd_mul(r, r);
  const dd r3 = dd_mul(r2, r);
  // log(1+r) = r - r^2/2 + r^3/3 - r^4 (1/4 - r/5 + r^2/6 - r^3/7 + r^4/8)
  const double x1 = r.hi;
  const double tail = -(r2.hi * r2.hi) * (0.25 - x1 * (0.2 - x1 * (1. / 6. - x1 * (1. / 7. - x1 * 0.125))));
  dd s = dd_add(r, {-0.5 * r2.hi, -0.5 * r2.lo});
  s = dd_add(s, dd_mul(r3, {0.33333333333333331, 1.8503717077085941e-17}));
  s = dd_add_d(s, tail);
  const dd le = dd_mul_d(T.ln2, (double)e);
  return dd_add(dd_add(le, T.logc[k - LOG_K0]), s);
}

// exp(x) for a double-double argument, |x| < 700, rounded to double.
__host__ __device__ __forceinline__ double dd_exp_round(dd x, const MathTable &T) {
  const double nf = rint(x.hi * (1024. / 0.69314718055994529));
  const dd r = dd_sub(x, dd_mul_d(T.ln2_1024, nf));  // |r| <= ln2/2048 (+ rounding)
  const long long n = (long long)nf;
  const int j = (int)(n & 1023);
  const int q = (int)((n - j) / 1024);
  const dd r2 = dd_mul(r, r);
  const double x1 = r.hi;
  // exp(r) - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120 + r^3/720 + r^4/5040)
  const double tail = (r2.hi * x1) * (1. / 6. + x1 * (1. / 24. + x1 * (1. / 120. + x1 * (1. / 720. + x1 * (1. / 5040.)))));
  dd em1 = dd_add(r, {0.5 * r2.hi, 0.5 * r2.lo});
  em1 = dd_add_d(em1, tail);
  const dd e = dd_add_d(em1, 1.);
  const dd v = dd_mul(T.exp2j[j], e);
  return ldexp(v.hi, q);
}

// ---- fast paths ----

__host__ __device__ __forceinline__ uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}
__host__ __device__ __forceinline__ double dfrom(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}
// 2^q for -1022 <= q <= 1023
__host__ __device__ __forceinline__ double pow2i(int q) { return dfrom((uint64_t)(q + 1023) << 52); }

// log(x) as an unevaluated sum hi + lo, x > 0 finite and normal, x != 1.  |error| < 2^-72 |log x|:
// x = 2^e m, m = c (1 + r) as in dd_log; log(1+r) = r - r^2/2 + r^3 (1/3 - r/4 + ... - r^5/8), with
// r^2 split exactly by TwoProd and |r| < 6.9e-4 (the r^9 truncation is < 2^-90 |r|).
__host__ __device__ __forceinline__ dd fast_log(double x, const MathTable &T) {
  const uint64_t u = dbits(x);
  int e = (int)(u >> 52) - 1023;
  double m = dfrom((u & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);   // [1, 2)
  if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
  const int k = (int)rint(m * 1024.);
  const double c = (double)k * (1. / 1024.);
  const double num = m - c;                          // exact (Sterbenz)
  const double invc = T.invc[k - LOG_K0];
  const double rh = num * invc;
  const double rl = fma(-rh, c, num) * invc;
  const dd r2 = two_prod(rh, rh);
  const double tail = (rh * r2.hi) *
                      (1. / 3. - rh * (0.25 - rh * (0.2 - rh * (1. / 6. - rh * (1. / 7. - rh * 0.125)))));
  const dd lc = T.logc[k - LOG_K0];
  const double ed = (double)e;
  const dd a = two_prod(ed, T.ln2.hi);
  const dd s1 = two_sum(a.hi, lc.hi);
  const dd s2 = two_sum(s1.hi, rh);
  const dd s3 = two_sum(s2.hi, -0.5 * r2.hi);
  const double lo = (((a.lo + s1.lo) + (s2.lo + s3.lo)) + (ed * T.ln2.lo + lc.lo)) + ((rl - rh * rl) - 0.5 * r2.lo + tail);
  return fast_two_sum(s3.hi, lo);
}

// exp(x) for x = xh + xl (|xh| < 700, |xl| <= ulp(xh)) as 2^q (hi + lo).  |error| < 2^-72 of the
// result: x = (1024 q + j) ln2/1024 + r, |r| <= ln2/2048 (+ rounding), exp(r) - 1 =
// r + r^2/2 + r^3 (1/6 + r/24 + r^2/120) with r^2 split exactly (the r^6 truncation is < 2^-78).
__host__ __device__ __forceinline__ dd fast_exp(double xh, double xl, const MathTable &T, int &q) {
  const double nf = rint(xh * (1024. / 0.69314718055994529));
  const dd p = two_prod(nf, T.ln2_1024.hi);
  const double rh = xh - p.hi;                       // exact: xh and p.hi are within a factor 2
  const double rl = (xl - p.lo) - nf * T.ln2_1024.lo;
  const long long n = (long long)nf;
  const int j = (int)(n & 1023);
  q = (int)((n - j) / 1024);
  const dd r2 = two_prod(rh, rh);
  const double tail = (rh * r2.hi) * (1. / 6. + rh * (1. / 24. + rh * (1. / 120.)));
  const double qlo = rl + rh * rl + 0.5 * r2.lo + tail;   // exp(r) - 1 = rh + r2.hi/2 + qlo
  const dd t = T.exp2j[j];
  const dd a = two_prod(t.hi, rh);
  const dd b = two_prod(t.hi, 0.5 * r2.hi);
  const dd s1 = fast_two_sum(t.hi, a.hi);
  const dd s2 = fast_two_sum(s1.hi, b.hi);
  const double lo = ((s1.lo + s2.lo) + (a.lo + b.lo)) + (t.hi * qlo + (t.lo + t.lo * (rh + 0.5 * r2.hi)));
  return fast_two_sum(s2.hi, lo);
}

// Round hi + lo if every value within err of it rounds the same way; else report failure.
__host__ __device__ __forceinline__ bool round_test(dd v, double err, double &out) {
  const double a = v.hi + (v.lo - err), b = v.hi + (v.lo + err);
  out = a;
  return a == b;
}

__host__ __device__ __forceinline__ double cr_log(double x, const MathTable &T) {
  if (!(x > 0.) || !(x < INFINITY) || x < 2.2250738585072014e-308) return log(x);
  if (x == 1.) return 0.;
  const dd v = fast_log(x, T);
  double r;
  if (round_test(v, fabs(v.hi) * 0x1p-69, r)) return r;
  return dd_log(x, T).hi;
}
__host__ __device__ __forceinline__ double cr_exp(double x, const MathTable &T) {
  if (!(fabs(x) < 700.)) return exp(x);
  if (x == 0.) return 1.;
  int q;
  const dd v = fast_exp(x, 0., T, q);
  double r;
  if (round_test(v, fabs(v.hi) * 0x1p-69, r)) return r * pow2i(q);
  return dd_exp_round({x, 0.}, T);
}
// pow(x, y) and log(x) of one argument, sharing the fast logarithm; each result equals the
// separate cr_pow / cr_log call.
__host__ __device__ __forceinline__ double cr_pow(double x, double y, const MathTable &T);
__host__ __device__ __forceinline__ double cr_log_pow(double x, double y, const MathTable &T, double &lg) {
  if (!(x > 0.) || !(x < INFINITY) || x < 2.2250738585072014e-308 || x == 1. || y == 0. || y == 2. || !(fabs(y) < 1e6)) {
    lg = cr_log(x, T);
    return cr_pow(x, y, T);
  }
  const dd l = fast_log(x, T);
  double r;
  lg = round_test(l, fabs(l.hi) * 0x1p-69, r) ? r : dd_log(x, T).hi;
  dd yl = two_prod(y, l.hi);
  yl.lo += y * l.lo;
  if (!(fabs(yl.hi) < 700.)) return pow(x, y);
  yl = fast_two_sum(yl.hi, yl.lo);
  int q;
  const dd v = fast_exp(yl.hi, yl.lo, T, q);
  if (round_test(v, fabs(v.hi) * (0x1p-69 + fabs(yl.hi) * 0x1p-68), r)) return r * pow2i(q);
  const dd ls = dd_mul_d(dd_log(x, T), y);
  return dd_exp_round(ls, T);
}

__host__ __device__ __forceinline__ double cr_pow(double x, double y, const MathTable &T) {
  if (y == 0. || x == 1.) return 1.;
  if (y == 2.) return x * x;   // the square rounded once: the correctly rounded x^2 for every x
  if (!(x > 0.) || !(x < INFINITY) || x < 2.2250738585072014e-308 || !(fabs(y) < 1e6)) return pow(x, y);
  const dd l = fast_log(x, T);
  dd yl = two_prod(y, l.hi);
  yl.lo += y * l.lo;
  if (!(fabs(yl.hi) < 700.)) return pow(x, y);
  yl = fast_two_sum(yl.hi, yl.lo);
  int q;
  const dd v = fast_exp(yl.hi, yl.lo, T, q);
  double r;
  // the logarithm's relative error 2^-72 becomes an absolute error in y log x
  if (round_test(v, fabs(v.hi) * (0x1p-69 + fabs(yl.hi) * 0x1p-68), r)) return r * pow2i(q);
  const dd ls = dd_mul_d(dd_log(x, T), y);
  return dd_exp_round(ls, T);
}

// ---- atan and cos (the turbulence closure's wall function and fv1 inversion) ----
//
// One double-double evaluation to ~2^-100, rounded once: the correctly rounded value except
// within ~2^-100 of a rounding boundary, and the same bits on the host and the device.

// atan(t) for a double-double 0 <= t <= 1: t = c + d with c = k/32 from the table,
// atan(t) = atan(c) + atan(r), r = (t - c) / (1 + t c), |r| < 1/63, and
// atan(r) = r (1 - r^2 (1/3 - r^2 (1/5 - r^2 (1/7 - r^2 (1/9 - r^2/11 + r^4/13 - r^6/15))))), the
// innermost bracket in double (the r^17 term is below 2^-100 |r|).
__host__ __device__ __forceinline__ dd dd_atan_unit(dd t, const MathTable &T) {
  const int k = (int)rint(t.hi * 32.);
  const double c = (double)k * (1. / 32.);
  const dd r = dd_div(dd_add_d(t, -c), dd_add_d(dd_mul_d(t, c), 1.));
  const dd r2 = dd_mul(r, r);
  const double x2 = r2.hi;
  const double tail = x2 * (1. / 9. - x2 * (1. / 11. - x2 * (1. / 13. - x2 * (1. / 15.))));
  // Horner in double-double: 1 - r2 (1/3 - r2 (1/5 - r2 (1/7 - tail)))
  dd h = dd_add_d(dd_div({1., 0.}, {7., 0.}), -tail);
  h = dd_sub(dd_div({1., 0.}, {5., 0.}), dd_mul(r2, h));
  h = dd_sub(dd_div({1., 0.}, {3., 0.}), dd_mul(r2, h));
  h = dd_sub({1., 0.}, dd_mul(r2, h));
  return dd_add(T.atanc[k], dd_mul(r, h));
}

__host__ __device__ __forceinline__ double cr_atan(double x, const MathTable &T) {
  if (!(fabs(x) < INFINITY) || x == 0.) return atan(x);
  const double a = fabs(x);
  dd v;
  if (a <= 1.) {
    v = dd_atan_unit({a, 0.}, T);
  } else {   // atan(a) = pi/2 - atan(1/a), pi/2 = 2 atan(1)
    const dd half_pi = {2. * T.atanc[ATAN_N - 1].hi, 2. * T.atanc[ATAN_N - 1].lo};
    v = dd_sub(half_pi, dd_atan_unit(dd_div({1., 0.}, {a, 0.}), T));
  }
  const double r = v.hi + v.lo;
  return x < 0. ? -r : r;
}

// cos(x) for |x| < 1 by its Taylor series to x^30/30! in double-double (Horner:
// 1 - x^2/(1*2) (1 - x^2/(3*4) (1 - ...))); other arguments go to the library's cos.
__host__ __device__ __forceinline__ double cr_cos(double x, const MathTable &T) {
  (void)T;
  if (!(fabs(x) < 1.)) return cos(x);
  const dd x2 = two_prod(x, x);
  dd s = {1., 0.};
  for (int n = 15; n >= 1; n--) {
    const double q = (double)((2 * n - 1) * (2 * n));
    s = dd_sub({1., 0.}, dd_div(dd_mul(x2, s), {q, 0.}));
  }
  return s.hi + s.lo;
}

}  // namespace epic
