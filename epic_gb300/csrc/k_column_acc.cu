// The vertical pressure and geopotential integration of the mixed form (EPIC_PREC_MIXED):
// set_p2etc and the column part of store_pgrad_vars, with the quantities that feed the pressure
// gradient -- the layer pressure P2, the diagnosed THETA, T3, RHO3 and the
// geopotential increments -- evaluated in double-float (df.cuh: ~1e-13 relative, on the FP32
// pipe) instead of binary32, and the running sums in binary64.  Rounding these to binary32 every
// step is what makes the meridional wind of the all-FP32 form (EPIC_PREC_MIXED_FAST) drift from
// FP64 by 6e-4 in a day; with them in double-float the mixed form stays within 1e-4.  Quantities
// that only diagnostics read (THETA2, T2 and RHO2 feed the Richardson number alone; H3, EXNER3,
// MONT3, DZDT3) stay FP32, as in the fast form.
//
// Structure, phases and the restated reference lines are those of k_set_p2etc_mixed and
// k_pgrad_vars_column_mixed (k_column.cu): set_p2etc, epic_funcs_diag.c:3352-3569;
// store_pgrad_vars, epic_funcs_diag.c:3595-3895.
#include "device_common.cuh"
#include "column_tile.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

namespace {

__device__ __forceinline__ dfl one_df() { return dfl(1.f, 0.f); }

// onto_kk(P2_INDEX) at a layer: bot * q^(1/kappa), q = (1 - r^(kappa+1)) / ((kappa+1)(1 - r)),
// r = top/bot, with lr = log r given as the difference of the interfaces' logarithms (absolute
// error ~1e-12, so P2 keeps ~1e-10 relative accuracy down to layers 1% thick -- 500 times
// better than binary32).  Layers thinner than 1e-7 relative take the reference's
// equal-pressure branch (the mean differs from the formula by O(eps^2) there).
__device__ __forceinline__ double layer_p_acc(const DevModel &M, double top, double bot, dfl lr) {
  const dfl B = cv<dfl>(bot);
  const dfl eps = cv<dfl>(bot - top) / B;
  if (!(eps.hi >= 1e-7f)) return .5 * (bot + top);
  const dfl a = mconst<dfl>(M, DFC_KAPPA1, 0.);
  const dfl q = (one_df() - exp_df(a * lr, M.exp2tab)) / (a * eps);
  return to_d(B * exp_df(log_df(q, M.exp2tab) * mconst<dfl>(M, DFC_KAPPA_INV, 0.), M.exp2tab));
}

// theta on the hybrid surface sigmatheta = sg at sigma = log(p/pbot) / log(ptop/pbot) (the
// inversion of return_sigmatheta)
__device__ __forceinline__ double theta_acc(const DevModel &M, double sg, dfl sigma) {
  dfl gs;
  const dfl fs = f_and_g_sigma_r<dfl>(M, sigma, gs);
  return to_d((cv<dfl>(sg) - fs) / gs);
}

}  // namespace

// layers = 0: only P3, HDRY and the interfaces' logarithms (lp3) -- the call inside advection,
// whose P2, H3 and THETA2 stage 11 recomputes before anything reads them.
__global__ void __launch_bounds__(CT_THREADS, 4) k_set_p2etc_acc(DevModel M, int update_theta, int layers) {
  if (epic_member(M)) return;
  extern __shared__ double sm[];
  __shared__ int s_kay[EPIC_MAX_NK + 1];
  __shared__ float s_w[EPIC_MAX_NK + 1];
  if (update_theta && layers) theta2_intervals(M, s_kay, s_w);
  const ColTile c = col_tile(M);
  const int nk = M.nk, ks = M.k_sigma, L = nk + 1;
  const long long n2 = M.n2;
  double *P = sm, *HL = P + 32 * L, *TH = HL + 32 * L;
  float2 *LPS = reinterpret_cast<float2 *>(TH + 32 * L);   // log P3 per interface, double-float
  const double g = M.grav[2 * c.j + 1];
  if (c.valid) {
    double v[TILE_SLOTS][2];
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++) {
      const long long x = c.base + min(c.warp + r * CT_WARPS, nk) * n2;
      v[r][0] = __ldg(M.theta + x); v[r][1] = __ldg(M.hdry + x);
    }
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++) {
      const int k = c.warp + r * CT_WARPS;
      if (k <= nk) { CT(TH, k) = v[r][0]; CT(HL, k) = v[r][1]; }
    }
    for (int k = c.warp + TILE_SLOTS * CT_WARPS; k <= nk; k += CT_WARPS) {
      CT(TH, k) = M.theta[c.base + k * n2];
      CT(HL, k) = M.hdry[c.base + k * n2];
    }
  }
  __syncthreads();
  // P3 from the top down, in FP64: the layer pressure thicknesses dsgth g HDRY in parallel, then
  // their running sum by every warp
  if (c.valid) {
    if (c.warp == 0) CT(P, 0) = M.p3[c.base];
    for (int k = 1 + c.warp; k <= nk; k += CT_WARPS) CT(P, k) = M.dsgth[2 * k] * g * CT(HL, k);
  }
  __syncthreads();
  ct_running_sum(P, nk, c.lane, c.warp);
  const double ptop = CT(P, 0), pbot = CT(P, nk);
  // log(ptop/pbot) and the pure-sigma interfaces pbot (ptop/pbot)^sigma in double-float, by every
  // warp (binary64 log/exp by warp 0 alone kept the other warps waiting at the barrier)
  const dfl LPB = c.valid ? log_df(cv<dfl>(pbot), M.exp2tab) : dfl(0.f, 0.f);
  const dfl LP = c.valid ? log_df(cv<dfl>(ptop), M.exp2tab) - LPB : dfl(1.f, 0.f);   // log(ptop/pbot)
  if (c.valid && ks - 1 < nk) {
    const dfl Z0 = mconst<dfl>(M, DFC_ZETA0, 0.), DZ = mconst<dfl>(M, DFC_ZETA1, 0.) - Z0, PB = cv<dfl>(pbot);
    for (int k = ks - 1 + c.warp; k < nk; k += CT_WARPS)
      CT(P, k) = to_d(PB * exp_df((cv<dfl>(M.sgth[2 * k + 1]) - Z0) / DZ * LP, M.exp2tab));
  }
  __syncthreads();
  if (!c.valid) return;
  const double ginv = to_d(dfl(1.f, 0.f) / cv<dfl>(g));
  const float lpf = LP.hi;
  // the logarithms of the interface pressures, once per interface: the layer-mean pressure, the
  // diagnosed theta here and T3 and the geopotential increments of store_pgrad_vars (lp3) take
  // theirs from these
  for (int k = c.warp; k <= nk; k += CT_WARPS) {
    const double pk = CT(P, k);
    const dfl lpk = k == nk ? LPB : log_df(cv<dfl>(pk), M.exp2tab);
    CT(LPS, k) = make_float2(lpk.hi, lpk.lo);
    M.lp3[c.base + k * n2] = make_float2(lpk.hi, lpk.lo);
    if (k >= 1) {
      const long long x = c.base + k * n2;
      M.p3[x] = pk;
      double hl = CT(HL, k);   // recomputed only next to a rescaled interface (k_set_p2etc_mixed)
      if (k >= ks - 1) {
        hl = (pk - CT(P, k - 1)) * (ginv * M.dsgth_inv[2 * k]);
        CT(HL, k) = hl;
      }
      M.hdry[x] = dmaxr(M.h_min[k], hl);
    }
    if (update_theta && k < ks - 1) {
      const double th = theta_acc(M, M.sgth[2 * k + 1], (lpk - LPB) / LP);
      CT(TH, k) = th;
      M.theta[c.base + k * n2] = th;
    }
  }
  __syncthreads();
  if (!layers) return;
  for (int k = 1 + c.warp; k <= nk; k += CT_WARPS) {
    const long long x = c.base + k * n2;
    const double top = CT(P, k - 1), bot = CT(P, k);
    const float2 lt = CT(LPS, k - 1), lb = CT(LPS, k);
    const double p2 = layer_p_acc(M, top, bot, dfl(lt.x, lt.y) - dfl(lb.x, lb.y));
    M.p2[x] = p2;
    put_split(M.work2, x, p2);
    if (k == 1) {
      M.p2[c.base] = top * top / p2;
      put_split(M.work2, c.base, top * top / p2);
    }
    double h;
    if (k == nk) h = CT(HL, nk);
    else {
      const float topwt = d2f(M.dsgth[2 * k]), botwt = d2f(M.dsgth[2 * k + 2]);
      h = f2d((topwt * d2f(CT(HL, k)) + botwt * d2f(CT(HL, k + 1))) / (topwt + botwt));
    }
    M.h3[x] = h;
    if (k == 1) M.h3[c.base] = h;
    if (!update_theta) continue;
    double t2;
    if (k < ks - 1) {
      const float sigma = log_ratio_f(pbot, p2) / lpf;
      float gs;
      const float fs = f_and_g_sigma_r<float>(M, sigma, gs);
      t2 = f2d((d2f(M.sgth[2 * k]) - fs) / gs);
    } else if (k == ks - 1) {
      t2 = .5 * (CT(TH, ks - 1) + CT(TH, ks - 2));
    } else {   // linint in binary32 with the block's interval and weight of this level (THETA2
               // feeds the Richardson number alone)
      const float y0 = d2f(CT(TH, nk - s_kay[k])), y1 = d2f(CT(TH, nk - s_kay[k] - 1));
      t2 = f2d(y0 + (y1 - y0) * s_w[k]);
    }
    M.theta2[x] = t2;
  }
}

// FULL = false: GZ3 alone (with its monotonicity check) -- the call before the filtered-GZ
// copy, whose other outputs the call after stage 11 rewrites before anything reads them.
// H2: the hydrogen thermodynamics (x_h2 > 0): T3, T2 and the enthalpy of MONT3 from thermo_setup's
// tables in binary64 (hydrogen_temp of the ideal-gas temperature this kernel evaluates anyway,
// return_enthalpy), EXNER3 = cp T3 / THETA as the reference
// stores it (epic_funcs_diag.c:3698, :3717); the ideal-gas power (p/p0)^kappa is then not T3/THETA.
template <bool FULL, bool H2>
__device__ __forceinline__ void pgrad_vars_column_acc(DevModel &M) {
  extern __shared__ double sm[];
  __shared__ double s_rho2_1[32];
  const ColTile c = col_tile(M);
  const int nk = M.nk, L = nk + 1;
  const long long n2 = M.n2;
  double *P = sm, *R = P + 32 * L, *GZ = R + 32 * L;
  float2 *T3 = reinterpret_cast<float2 *>(GZ + 32 * L);   // T3, double-float
  float2 *LP = T3 + 32 * L;                               // log P3, double-float (set_p2etc's)
  const float2 *tab = M.exp2tab;
  const dfl kap = mconst<dfl>(M, DFC_KAPPA, 0.), lp0 = mconst<dfl>(M, DFC_LOG_P0, 0.), p0_inv = cv<dfl>(1. / M.press0);
  const dfl mu_over_r = cv<dfl>(M.mu_dry / 8.314472e+3);   // return_density: p mu / (R T)
  const float cpf = d2f(M.cp);
  auto level = [&](int k, double theta, double p, double pr, double th2, float2 lpk) {
    const long long x = c.base + k * n2;
    const dfl Pk = cv<dfl>(p);
    const dfl pi = exp_df(kap * (dfl(lpk.x, lpk.y) - lp0), tab);   // (p/p0)^kappa
    const double t3d = H2 ? hydrogen_temp(M, to_d(cv<dfl>(theta) * pi)) : 0.;
    CT(LP, k) = lpk;
    const dfl t3 = H2 ? cv<dfl>(t3d) : cv<dfl>(theta) * pi;
    const double rho = to_d(Pk * mu_over_r / t3);
    if (FULL) {
      M.t3[x] = to_d(t3);
      M.exner3[x] = H2 ? M.cp * t3d / theta : f2d(cpf * pi.hi);
      M.rho3[x] = rho;
    }
    CT(P, k) = p;
    CT(R, k) = rho;
    CT(T3, k) = make_float2(t3.hi, t3.lo);
    if (FULL && k >= 1) {   // the layer's T2, RHO2: read by the Richardson number only
      if (H2) {   // T2 from the binary32 power, as the ideal gas's
        const double t2 = hydrogen_temp(M, f2d(d2f(th2) * powf(d2f(pr) * p0_inv.hi, kap.hi)));
        M.t2[x] = t2;
        const double r2 = return_density(pr, t2, M.mu_dry);
        M.rho2[x] = r2;
        if (k == 1) s_rho2_1[c.lane] = r2;
        return;
      }
      const float t2f = d2f(th2) * powf(d2f(pr) * p0_inv.hi, kap.hi);
      M.t2[x] = f2d(t2f);
      const double r2 = f2d(d2f(pr) * mu_over_r.hi / t2f);
      M.rho2[x] = r2;
      if (k == 1) s_rho2_1[c.lane] = r2;
    }
  };
  if (c.valid) {
    double v[TILE_SLOTS][4];
    float2 vl[TILE_SLOTS];
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++) {
      const long long x = c.base + min(c.warp + r * CT_WARPS, nk) * n2;
      v[r][0] = __ldg(M.theta + x); v[r][1] = __ldg(M.p3 + x);
      v[r][2] = FULL ? __ldg(M.p2 + x) : 0.;
      v[r][3] = FULL ? __ldg(M.theta2 + x) : 0.;
      vl[r] = M.lp3[x];
    }
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++)
      if (c.warp + r * CT_WARPS <= nk) level(c.warp + r * CT_WARPS, v[r][0], v[r][1], v[r][2], v[r][3], vl[r]);
    for (int k = c.warp + TILE_SLOTS * CT_WARPS; k <= nk; k += CT_WARPS) {
      const long long x = c.base + k * n2;
      level(k, M.theta[x], M.p3[x], FULL ? M.p2[x] : 0., FULL ? M.theta2[x] : 0., M.lp3[x]);
    }
  }
  __syncthreads();
  if (FULL && c.valid && c.warp == CT_WARPS - 1) {
    M.rho2[c.base] = CT(R, 0) * CT(R, 0) / s_rho2_1[c.lane];
    M.theta2[c.base] = M.sgth[0];
    M.t2[c.base] = f2d(CT(T3, 0).x) + f2d(CT(T3, 0).y);
  }
  // log(P3(k+1)/P3(k)) as the difference of the interfaces' logarithms
  auto lgd = [&](int k) { const float2 a = CT(LP, k + 1), b = CT(LP, k); return dfl(a.x, a.y) - dfl(b.x, b.y); };
  auto t3df = [&](int k) { const float2 v = CT(T3, k); return dfl(v.x, v.y); };
  const dfl r_over_mu = one_df() / mu_over_r;   // p/rho = R T / mu
  // the geopotential increments of every layer: the Leslie-Purser ones inside, the short
  // centred ones at the two ends; then GZ3 from the surface up by every warp
  if (c.valid) {
    if (c.warp == 0) CT(GZ, nk) = M.topo_scale * M.gz_surface[M.at2(c.j, c.i)];
    if (c.warp == CT_WARPS - 1) {
      CT(GZ, nk - 1) = ((CT(P, nk) + CT(P, nk - 1)) / (CT(R, nk) + CT(R, nk - 1))) * to_d(lgd(nk - 1));
      CT(GZ, 0) = ((CT(P, 1) + CT(P, 0)) / (CT(R, 1) + CT(R, 0))) * to_d(lgd(0));
    }
    for (int k = 2 + c.warp; k <= nk - 1; k += CT_WARPS) {   // Leslie-Purser increments
      const dfl dz10 = lgd(k), dz21 = lgd(k - 1), dz32 = lgd(k - 2);
      const dfl dz20 = dz21 + dz10, dz30 = dz32 + dz20, dz31 = dz32 + dz21;
      const dfl df0 = r_over_mu * t3df(k + 1), df1 = r_over_mu * t3df(k);
      const dfl df2 = r_over_mu * t3df(k - 1), df3 = r_over_mu * t3df(k - 2);
      const dfl two(2.), six(6.);
      const dfl s = df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                    df1 * (dz21 * (dz21 * (dz21 + two * (dz10 - dz31)) - six * dz10 * dz31)) / (dz10 * dz31) +
                    df2 * (dz21 * (dz21 * (dz21 + two * (dz32 - dz20)) - six * dz20 * dz32)) / (dz20 * dz32) +
                    df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32);
      CT(GZ, k - 1) = -to_d(s / dfl(12.));
    }
  }
  __syncthreads();
  ct_running_sum_up(GZ, nk, c.lane, c.warp);
  if (!c.valid) return;
  const bool interior = c.i >= 1 && c.i <= M.ni;
  const long long itime = M.ctl->itime;
  // MONT3 and DZDT3: diagnostics no later kernel of the step reads (k_pgrad_vars_column_mixed)
  const float dtg_inv = -1.f / (d2f(M.dt) * d2f(M.grav[2 * c.j + 1]));
  const float cprf = d2f(M.cpr), rgasf = d2f(M.rgas);
  auto level_out = [&](int k, double old, double w, double h) {
    const long long x = c.base + k * n2;
    const double gzk = CT(GZ, k);
    M.gz3[x] = gzk;
    if (FULL) {
      put_split(M.work1, x, gzk);
      if (H2) M.mont3[x] = gzk + return_enthalpy(M, to_d(t3df(k)));
      else M.mont3[x] = f2d(d2f(gzk) + cprf * CT(T3, k).x * rgasf);
    }
    if (interior && k >= 1) {
      if (FULL) {
        float dz = 0.f;
        if (itime > 1) dz = d2f(old - gzk) * dtg_inv;
        dz += d2f(w) * d2f(h) / d2f(CT(R, k));
        M.dzdt3[x] = f2d(dz);
      }
      if (gzk >= CT(GZ, k - 1)) flag_error(M.ctl, ERR_GZ_MONOTONE, k, c.j, c.i, gzk);
    }
  };
  if (!FULL) {
    for (int k = c.warp; k <= nk; k += CT_WARPS) level_out(k, 0., 0., 0.);
    return;
  }
  double v[TILE_SLOTS][3];   // the loads of this warp's first levels issued together
#pragma unroll
  for (int r = 0; r < TILE_SLOTS; r++) {
    const long long x = c.base + min(c.warp + r * CT_WARPS, nk) * n2;
    v[r][0] = M.gz3[x]; v[r][1] = __ldg(M.w3 + x); v[r][2] = __ldg(M.h3 + x);
  }
#pragma unroll
  for (int r = 0; r < TILE_SLOTS; r++)
    if (c.warp + r * CT_WARPS <= nk) level_out(c.warp + r * CT_WARPS, v[r][0], v[r][1], v[r][2]);
  for (int k = c.warp + TILE_SLOTS * CT_WARPS; k <= nk; k += CT_WARPS) {
    const long long x = c.base + k * n2;
    level_out(k, M.gz3[x], M.w3[x], M.h3[x]);
  }
}

__global__ void __launch_bounds__(CT_THREADS, 4) k_pgrad_vars_column_acc(DevModel M) {
  if (epic_member(M)) return;
  pgrad_vars_column_acc<true, false>(M);
}
__global__ void __launch_bounds__(CT_THREADS, 4) k_gz3_column_acc(DevModel M) {
  if (epic_member(M)) return;
  pgrad_vars_column_acc<false, false>(M);
}
// the same with hydrogen thermodynamics (their binary64 table interpolation needs more registers)
__global__ void __launch_bounds__(CT_THREADS) k_pgrad_vars_column_acc_h2(DevModel M) {
  if (epic_member(M)) return;
  pgrad_vars_column_acc<true, true>(M);
}
__global__ void __launch_bounds__(CT_THREADS) k_gz3_column_acc_h2(DevModel M) {
  if (epic_member(M)) return;
  pgrad_vars_column_acc<false, true>(M);
}

int column_acc_kernels_init() {
  const int big = (int)(5 * 32 * (EPIC_MAX_NK + 1) * sizeof(double));
  if (cudaFuncSetAttribute(k_set_p2etc_acc, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_pgrad_vars_column_acc, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_gz3_column_acc, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_pgrad_vars_column_acc_h2, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_gz3_column_acc_h2, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess)
    return -1;
  return 0;
}

}  // namespace epic
