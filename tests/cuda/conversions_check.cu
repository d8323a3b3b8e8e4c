// Compares the integer-pipe binary64 <-> binary32 conversions of device_common.cuh (d2f, f2d)
// with the hardware conversions, bit for bit: every binary32 pattern for f2d; for d2f, 2^32
// hashed binary64 patterns plus, for every exponent of the normal, subnormal and overflow ranges
// of binary32, mantissas that sit on, just below and just above each rounding boundary.  Inputs
// of magnitude below FLT_MIN are expected as the signed zero that d2f/f2d flush them to.
// Also every finite normal binary32 pattern through cvt.rna.tf32.f32 against the rule the host
// uses to split the tensor-core filter's operator into TF32 parts.
// Prints "mismatches d2f=<n> f2d=<n> tf32=<n>"; exit status 0 when all are zero.
#include <cstdio>
#include "device_common.cuh"

using epic::d2f;
using epic::f2d;

__device__ __forceinline__ float flush(float b) { return fabsf(b) < FLT_MIN ? copysignf(0.f, b) : b; }
// d2f(d) against the hardware conversion, with |d| < FLT_MIN expected as a signed zero
__device__ __forceinline__ bool same_d2f(double d) {
  const float a = d2f(d), b = fabs(d) < (double)FLT_MIN ? copysignf(0.f, (float)d) : __double2float_rn(d);
  return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}
__device__ __forceinline__ bool same(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}

// the host's TF32 rounding of the tensor-core filter's operator tiles (k_filter_gemm.cu, tf32_rna):
// round to nearest, ties away from zero, the 13 low bits cleared
__device__ __forceinline__ unsigned tf32_host_rule(unsigned u) { return (u + 0x1000u) & 0xffffe000u; }
__device__ __forceinline__ unsigned tf32_hw(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__global__ void k_check(unsigned long long n, unsigned long long *bad) {
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < n; t += stride) {
    // every binary32 pattern through f2d
    const float f = __uint_as_float((unsigned)t);
    if (!same(f2d(f), (double)flush(f))) atomicAdd(bad + 1, 1ull);
    // every finite normal binary32 pattern through cvt.rna.tf32 and the host's rule
    const unsigned ex = ((unsigned)t >> 23) & 0xffu;
    if (ex != 0u && ex != 0xffu && tf32_hw(f) != tf32_host_rule((unsigned)t)) atomicAdd(bad + 2, 1ull);
    // a hashed binary64 pattern through d2f
    unsigned long long h = t * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29; h *= 0xBF58476D1CE4E5B9ull; h ^= h >> 32;
    const double d = __longlong_as_double((long long)h);
    if (!same_d2f(d)) atomicAdd(bad, 1ull);
    // rounding boundaries: exponent 850..1160, the 29 dropped bits near 0, 2^28 and 2^29
    const unsigned e = 850u + (unsigned)(t % 311ull);
    const unsigned sel = (unsigned)((t / 311ull) % 9ull);
    const unsigned mhi = (unsigned)(h >> 44) & 0xfffffu;
    const unsigned low3 = (unsigned)(h >> 12) & 7u;
    const unsigned drop[9] = {0u, 1u, 0x0fffffffu, 0x10000000u, 0x10000001u, 0x1fffffffu, 0x1ffffffeu, 0x0ffffffeu, 2u};
    const unsigned lo = (low3 << 29) | drop[sel];
    const unsigned sgn = (unsigned)(h & 1ull) << 31;
    const double b = __hiloint2double((int)(sgn | (e << 20) | mhi), (int)lo);
    if (!same_d2f(b)) atomicAdd(bad, 1ull);
  }
}

int main() {
  unsigned long long *bad = nullptr, host[3] = {0, 0, 0};
  if (cudaMalloc(&bad, sizeof(host)) != cudaSuccess) return 2;
  cudaMemset(bad, 0, sizeof(host));
  k_check<<<2048, 256>>>(1ull << 32, bad);
  const cudaError_t e = cudaMemcpy(host, bad, sizeof(host), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { printf("cuda error: %s\n", cudaGetErrorString(e)); return 2; }
  printf("mismatches d2f=%llu f2d=%llu tf32=%llu\n", host[0], host[1], host[2]);
  return host[0] || host[1] || host[2] ? 1 : 0;
}
