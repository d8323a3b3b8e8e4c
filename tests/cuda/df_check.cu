// Accuracy of the double-float arithmetic and exp/log of df.cuh against binary64: prints the
// largest relative error of each operation over seeded arguments in the ranges the mixed form
// uses (products and quotients of O(1)..O(1e5) values, exp of [-12, 3], log of [1e-5, 1e5] and of
// ratios within 20% of 1; log errors are absolute, scaled by max(1, |log x|)).  Exit status 0 when
// every error is below its bound.
#include <cstdio>
#include <cmath>
#include "device_common.cuh"

using namespace epic;

__device__ double rel(double got, double want) { return fabs(got - want) / fabs(want); }

// one hashed uniform in [0, 1) per (t, salt)
__device__ double uni(unsigned long long t, unsigned salt) {
  unsigned long long h = (t + 0x9E3779B97F4A7C15ull * (salt + 1)) * 0xBF58476D1CE4E5B9ull;
  h ^= h >> 31; h *= 0x94D049BB133111EBull; h ^= h >> 29;
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

__device__ unsigned long long as_ull(double x) { return (unsigned long long)__double_as_longlong(x); }

__global__ void k_check(int n, const float2 *tab, unsigned long long *worst) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double a = 1e5 * uni(t, 0) + 1e-3, b = 10. * uni(t, 1) + 1e-2;
  const dfl A = cv<dfl>(a), B = cv<dfl>(b);
  const double e[6] = {
      rel(to_d(A * B), a * b),
      rel(to_d(A / B), a / b),
      fabs(to_d(A - B) - (a - b)) / fmax(a, b),
      rel(to_d(exp_df(cv<dfl>(-12. + 15. * uni(t, 2)), tab)), exp(-12. + 15. * uni(t, 2))),
      fabs(to_d(log_df(cv<dfl>(exp(-11.5 + 23. * uni(t, 3))), tab)) - (-11.5 + 23. * uni(t, 3))) / fmax(1., fabs(-11.5 + 23. * uni(t, 3))),
      fabs(to_d(log_df(cv<dfl>(0.8 + 0.4 * uni(t, 4)), tab)) - log(0.8 + 0.4 * uni(t, 4)))};
  for (int q = 0; q < 6; q++) atomicMax(worst + q, as_ull(e[q]));   // non-negative doubles order as integers
}

// d2df and df2d (device_common.cuh) against the FP64-unit formulas they replace, bit for bit:
// binary64 values of every exponent from 2^-74 to 2^127 with random significands (and every
// eighth one a binary32 value plus a tie or near-tie residual), and double-floats from products
// and sums, plus powers of two with a lo of the opposite sign (the binade-below case).
// Counts the mismatches of each; any at all fails.
__global__ void k_conv(int n, unsigned long long *bad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const unsigned long long h = (unsigned long long)(uni(t, 7) * 18446744073709551616.0);
  const unsigned e = 949u + (unsigned)(uni(t, 8) * 202.);
  unsigned long long bits = ((unsigned long long)(uni(t, 9) < .5) << 63) | ((unsigned long long)e << 52) |
                            (h & 0x000fffffffffffffull);
  if ((t & 7) == 0) bits = (bits & ~0x1fffffffull) | (0x10000000ull ^ (h >> 60));   // residual at or near half
  const double x = __longlong_as_double((long long)bits);
  const dfl d = d2df(x);
  const float rh = d2f(x), rl = d2f(x - f2d(rh));
  if (__float_as_uint(d.hi) != __float_as_uint(rh) || __float_as_uint(d.lo) != __float_as_uint(rl)) atomicAdd(bad, 1ull);
  const double y = 1e3 * uni(t, 10) + 1e-3;
  dfl q[4] = {d, cv<dfl>(y) * d, d + cv<dfl>(y), dfl(0.f, 0.f)};
  // a power of two with lo taking it towards zero
  const float p2 = ldexpf(1.f, (int)(uni(t, 11) * 200.) - 90), sg = uni(t, 12) < .5 ? 1.f : -1.f;
  q[3] = dfl(sg * p2, -sg * p2 * (float)(uni(t, 13) * 5.9604644775390625e-08));   // |lo| < ulp(hi)/2
  for (int m = 0; m < 4; m++) {
    const double want = f2d(q[m].hi) + f2d(q[m].lo);
    if (fabs(q[m].hi) < 2.2e-22f || fabs(q[m].hi) > 1.7e38f) continue;   // outside the documented range
    if (__double_as_longlong(df2d(q[m])) != __double_as_longlong(want)) atomicAdd(bad + 1 + (m == 3), 1ull);
  }
}

int main() {
  float2 host_tab[32];
  for (int j = 0; j < 32; j++) {
    const double v = exp2(j / 32.);
    host_tab[j].x = (float)v;
    host_tab[j].y = (float)(v - (double)host_tab[j].x);
  }
  float2 *tab = nullptr;
  unsigned long long *worst = nullptr, hw[6] = {0, 0, 0, 0, 0, 0};
  if (cudaMalloc(&tab, sizeof(host_tab)) != cudaSuccess || cudaMalloc(&worst, sizeof(hw)) != cudaSuccess) return 2;
  cudaMemcpy(tab, host_tab, sizeof(host_tab), cudaMemcpyHostToDevice);
  cudaMemset(worst, 0, sizeof(hw));
  const int n = 1 << 22;
  k_check<<<(n + 255) / 256, 256>>>(n, tab, worst);
  if (cudaMemcpy(hw, worst, sizeof(hw), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  unsigned long long *cbad = nullptr, hc[3] = {0, 0, 0};
  if (cudaMalloc(&cbad, sizeof(hc)) != cudaSuccess) return 2;
  cudaMemset(cbad, 0, sizeof(hc));
  k_conv<<<(n + 255) / 256, 256>>>(n, cbad);
  if (cudaMemcpy(hc, cbad, sizeof(hc), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  printf("d2df mismatches %llu, df2d mismatches %llu (binade below a power of two: %llu) of %d\n", hc[0], hc[1], hc[2], n);
  const char *name[6] = {"mul", "div", "sub (abs / max(a,b))", "exp", "log (abs / max(1,|y|))", "log near 1 (abs)"};
  const double bound[6] = {2e-13, 2e-13, 2e-13, 2e-13, 2e-13, 2e-13};
  int bad = 0;
  for (int q = 0; q < 6; q++) {
    double v;
    memcpy(&v, &hw[q], sizeof v);
    printf("%-18s max error %.3e (bound %.0e)\n", name[q], v, bound[q]);
    bad |= !(v < bound[q]);
  }
  return bad | (hc[0] + hc[1] + hc[2] != 0);
}
