// Column tiles and the sigma-coordinate helpers shared by the column kernels (k_column.cu,
// k_column_acc.cu).
#pragma once
#include "device_common.cuh"

namespace epic {

// ---- column tiles ----
//
// The transcendental work of calc_w, set_p2etc and store_pgrad_vars is pointwise once a
// column's pressures are known; only their running sums are sequential.  A block takes 32
// neighbouring columns (one per lane; neighbouring columns are neighbouring addresses, so every
// level is one coalesced 256-byte access) and stages their levels in shared memory as
// [k][lane].  Pointwise phases spread the levels over CT_WARPS warps; warp 0 alone runs each
// running sum, in the reference's order, so the results are those of one thread per column.
constexpr int CT_WARPS = 8;
constexpr int CT_THREADS = 32 * CT_WARPS;
// levels per warp whose loads a column kernel issues together before using them
constexpr int TILE_SLOTS = 4;

struct ColTile {
  int lane, warp, j, i;
  bool valid;
  long long base;   // M.at(0, j, i)
};
__device__ __forceinline__ ColTile col_tile(const DevModel &M) {
  ColTile c;
  c.lane = (int)(threadIdx.x & 31);
  c.warp = (int)(threadIdx.x >> 5);
  const int t = (int)blockIdx.x * 32 + c.lane;
  c.valid = t < (M.nj + 1) * M.iadim;
  c.j = c.valid ? t / M.iadim : 0;
  c.i = c.valid ? t - c.j * M.iadim : 0;
  c.base = M.at(0, c.j, c.i);
  return c;
}
// level k of a [k][lane] shared array
#define CT(a, k) (a)[(k) * 32 + c.lane]

// Running sum over the levels of every column of a tile, by all CT_WARPS warps: on entry
// A[k] (k = 1..n) holds the increments and A[0] the starting value, on exit
// A[k] = A[0] + A[1] + ... + A[k].  Each warp sums a contiguous chunk of levels, then adds the
// totals of the chunks above it -- binary64 throughout, in an order other than the sequential
// one (the mixed forms; the FP64 form keeps warp 0's sum in the reference's order).  Every
// thread of the block must call it (it holds two barriers).
__device__ __forceinline__ void ct_running_sum(double *A, int n, int lane, int warp) {
  __shared__ double s_part[CT_WARPS * 32];
  const int chunk = (n + CT_WARPS - 1) / CT_WARPS;
  const int k0 = 1 + warp * chunk, k1 = min(n, k0 + chunk - 1);
  double run = 0.;
  for (int k = k0; k <= k1; k++) {
    run += A[k * 32 + lane];
    A[k * 32 + lane] = run;
  }
  s_part[warp * 32 + lane] = run;
  __syncthreads();
  double off = A[lane];
  for (int w = 0; w < warp; w++) off += s_part[w * 32 + lane];
  for (int k = k0; k <= k1; k++) A[k * 32 + lane] += off;
  __syncthreads();
}

// The same from the bottom up: on entry A[n] holds the starting value and A[k] (k = 0..n-1) the
// increments, on exit A[k] = A[n] + A[n-1] + ... + A[k].
__device__ __forceinline__ void ct_running_sum_up(double *A, int n, int lane, int warp) {
  __shared__ double s_part[CT_WARPS * 32];
  const int chunk = (n + CT_WARPS - 1) / CT_WARPS;
  const int k1 = n - 1 - warp * chunk, k0 = max(0, k1 - chunk + 1);
  double run = 0.;
  for (int k = k1; k >= k0; k--) {
    run += A[k * 32 + lane];
    A[k * 32 + lane] = run;
  }
  s_part[warp * 32 + lane] = run;
  __syncthreads();
  double off = A[n * 32 + lane];
  for (int w = 0; w < warp; w++) off += s_part[w * 32 + lane];
  for (int k = k1; k >= k0; k--) A[k * 32 + lane] += off;
  __syncthreads();
}

// f_sigma/g_sigma (epic_funcs_diag.c:1271-1314) in the compute type, one exponential for both
template <class R>
__device__ __forceinline__ R f_and_g_sigma_r(const DevModel &M, R s, R &g) {
  const R ss = mconst<R>(M, DFC_SIGMA_SIGMA, M.sigma_sigma), z0 = mconst<R>(M, DFC_ZETA0, M.zeta0),
          z1 = mconst<R>(M, DFC_ZETA1, M.zeta1);
  if (s <= ss) g = R(0.);
  else if (s >= R(1.)) g = R(1.);
  else g = mconst<R>(M, DFC_G_COEFF, M.g_coeff) * (R(1.) - RMath<R>::exp(M, -mconst<R>(M, DFC_ALPHA, M.alpha) * (s - ss)));
  if (s < R(0.)) return z0;
  if (s <= ss) return z0 + s * (z1 - z0);
  if (s < R(1.)) return (R(1.) - g) * (z0 + s * (z1 - z0));
  return R(0.);
}

// d(return_sigmatheta)/dp at fixed theta and pbot, from f_sigma/g_sigma's derivatives:
// sigma = log(p/pbot)/lp, dsigma/dp = 1/(p lp); sigma_side takes the pure-sigma branch (f linear,
// g = 0) whatever sigma's rounding says.
template <class R>
__device__ __forceinline__ R dsigmatheta_dp(const DevModel &M, R theta, R p, R pbot, R lp, bool sigma_side) {
  const R ss = mconst<R>(M, DFC_SIGMA_SIGMA, M.sigma_sigma), z0 = mconst<R>(M, DFC_ZETA0, M.zeta0),
          z1 = mconst<R>(M, DFC_ZETA1, M.zeta1);
  const R s = RMath<R>::log(M, p / pbot) / lp;
  R dfs, dgs;
  if (sigma_side || (s <= ss && s >= R(0.))) {
    dfs = z1 - z0;
    dgs = R(0.);
  } else if (s > ss && s < R(1.)) {
    const R a = mconst<R>(M, DFC_ALPHA, M.alpha), gc = mconst<R>(M, DFC_G_COEFF, M.g_coeff);
    const R e = RMath<R>::exp(M, -a * (s - ss));
    const R g = gc * (R(1.) - e);
    dgs = gc * a * e;
    dfs = -dgs * (z0 + s * (z1 - z0)) + (R(1.) - g) * (z1 - z0);
  } else {
    dfs = R(0.);
    dgs = R(0.);
  }
  return (dfs + dgs * theta) / (p * lp);
}

// log(b/a) for b/a near 1, from the FP64 difference
__device__ __forceinline__ float log_ratio_f(double a, double b) { return log1pf(d2f(b - a) / d2f(a)); }

// return_sigmatheta (epic_funcs_diag.c:1238-1250) with log(ptop/pbot) supplied
template <class R>
__device__ __forceinline__ R sigmatheta_lp(const DevModel &M, R theta, R p, R pbot, R ptop, R lp) {
  if (p <= ptop) return theta;
  const R s = RMath<R>::log(M, p / pbot) / lp;
  R g;
  const R f = f_and_g_sigma_r<R>(M, s, g);
  return f + g * theta;
}

}  // namespace epic
