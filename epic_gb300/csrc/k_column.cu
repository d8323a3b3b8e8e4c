// Column (vertical) kernels: one thread per (j,i) column, marching in k.
// Each kernel restates the reference routine named in its comment.
#include "device_common.cuh"
#include "column_tile.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

// Columns j = 0..nj, i = 0..ni+1 (JLOPAD..JHIPAD, ILOPAD..IHIPAD); thread -> (j, i).
__device__ __forceinline__ bool col_index(const DevModel &M, int &j, int &i) {
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int w = M.ni + 2;
  if (t >= (M.nj + 1) * w) return false;
  j = t / w;
  i = t - j * w;
  return true;
}

// source_sink: THETA += dt*HEAT3/EXNER3 for k >= k_sigma-1, epic_funcs_diag.c:4768-4778
__global__ void k_source_sink(DevModel M) {
  if (epic_member(M)) return;
  int j, i;
  if (!col_index(M, j, i)) return;
  for (int k = M.k_sigma - 1; k <= M.nk; k++) {
    const long long x = M.at(k, j, i);
    M.theta[x] += M.dt * M.heat3[x] / M.exner3[x];
  }
}

// calc_w, epic_flux.c:123-335.  The Leslie-Purser summed divergence keeps SUM_DIV = 0 at
// k = 1 and k = nk in every real column (the reference assigns those entries outside its
// column loops, epic_flux.c:224-226, :259-261), so the dF/dpbot term vanishes.
// Shared arrays: P (pressure), LG (log of successive pressure ratios), DS (SUM_DIV increments),
// W (heating term), DF (dF/dp).
// In the mixed form (R = float) the pointwise terms are FP32, SUM_DIV is accumulated in FP64, and
// the dF/dp difference step is cbrt(FLT_EPSILON) relative instead of cbrt(DBL_EPSILON).
// source_sink = 1: the step's source_sink (k_source_sink) first, in the same pass over the
// columns: THETA(k >= k_sigma-1) += dt*HEAT3/EXNER3 in binary64, written back and then used.
template <class R>
__global__ void __launch_bounds__(CT_THREADS, 3) k_calc_w(DevModel M, int source_sink) {
  if (epic_member(M)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sm = reinterpret_cast<R *>(smraw);
  __shared__ R s_lp[32];
  const ColTile c = col_tile(M);
  const int nk = M.nk, ks = M.k_sigma, L = nk + 1;
  const long long n2 = M.n2;
  R *P = sm, *LG = P + 32 * L, *DS = LG + 32 * L, *W = DS + 32 * L, *DF = W + 32 * L, *DV = DF + 32 * L;
  // Stage P3 and DIV_UV3 of every level, and THETA, HEAT3 and EXNER3 in the DS, W and DF rows
  // that the pointwise pass reads before it overwrites them.  The loads of the first
  // TILE_SLOTS levels of each warp are issued together so that their latencies overlap.
  auto stage = [&](int k, double p3, double dv, double th, double ht, double ex) {
    if (source_sink && k >= ks - 1) {   // epic_funcs_diag.c:4768-4778
      th += M.dt * ht / ex;
      M.theta[c.base + k * n2] = th;
    }
    CT(P, k) = cv<R>(p3); CT(DV, k) = cv<R>(dv); CT(DS, k) = cv<R>(th); CT(W, k) = cv<R>(ht); CT(DF, k) = cv<R>(ex);
  };
  if (c.valid) {
    double v[TILE_SLOTS][5];
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++) {
      const long long x = c.base + min(c.warp + r * CT_WARPS, nk) * n2;
      v[r][0] = __ldg(M.p3 + x); v[r][1] = __ldg(M.div_uv3 + x); v[r][2] = __ldg(M.theta + x);
      v[r][3] = __ldg(M.heat3 + x); v[r][4] = __ldg(M.exner3 + x);
    }
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++)
      if (c.warp + r * CT_WARPS <= nk) stage(c.warp + r * CT_WARPS, v[r][0], v[r][1], v[r][2], v[r][3], v[r][4]);
    for (int k = c.warp + TILE_SLOTS * CT_WARPS; k <= nk; k += CT_WARPS) {
      const long long x = c.base + k * n2;
      stage(k, M.p3[x], M.div_uv3[x], M.theta[x], M.heat3[x], M.exner3[x]);
    }
  }
  __syncthreads();
  const R ptop = CT(P, 0), pbot = CT(P, nk), psigma = CT(P, ks - 1);
  if (c.valid) {
    for (int k = c.warp; k < nk; k += CT_WARPS) CT(LG, k) = RMath<R>::log(M, CT(P, k + 1) / CT(P, k));
    if (c.warp == CT_WARPS - 1) s_lp[c.lane] = RMath<R>::log(M, ptop / pbot);
  }
  __syncthreads();
  const R lp = s_lp[c.lane];
  if (c.valid)
    for (int k = 1 + c.warp; k < nk; k += CT_WARPS) {
      const R p3 = CT(P, k);
      const R theta3 = CT(DS, k), heat = CT(W, k), exner = CT(DF, k);
      R w = R(0.);
      if (k < ks - 1) {
        const R sigma = RMath<R>::log(M, p3 / pbot) / lp;
        R g;
        f_and_g_sigma_r<R>(M, sigma, g);
        w = g * heat / exner;
      }
      if (k >= 2) {
        const R P0 = CT(P, k - 2), P1 = CT(P, k - 1), P2 = p3, P3 = CT(P, k + 1);
        const R dz10 = CT(LG, k - 2), dz21 = CT(LG, k - 1), dz32 = CT(LG, k);
        const R dz20 = dz21 + dz10, dz30 = dz32 + dz20, dz31 = dz32 + dz21;
        const R df0 = P0 * CT(DV, k - 2);
        const R df1 = P1 * CT(DV, k - 1);
        const R df2 = P2 * CT(DV, k);
        const R df3 = P3 * CT(DV, k + 1);
        CT(DS, k) = -(df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                      df1 * (dz21 * (dz21 * (dz21 + R(2.) * (dz10 - dz31)) - R(6.) * dz10 * dz31)) / (dz10 * dz31) +
                      df2 * (dz21 * (dz21 * (dz21 + R(2.) * (dz32 - dz20)) - R(6.) * dz20 * dz32)) / (dz20 * dz32) +
                      df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32)) /
                    R(12.);
      }
      if constexpr (std::is_same_v<R, double>) {
        // dF/dp by a centred difference of return_sigmatheta at fixed theta and pbot
        const R dp = p3 * M.eps13;
        R p2 = rmax(p3 - dp * R(.5), ptop);
        const R p4 = rmin(p3 + dp * R(.5), pbot);
        if (p2 < psigma && p4 >= psigma) p2 = p3;
        if (!(p2 < p4)) flag_error(M.ctl, ERR_CALC_W_P, k, c.j, c.i, p2);
        CT(DF, k) = (sigmatheta_lp<R>(M, theta3, p2, pbot, ptop, lp) - sigmatheta_lp<R>(M, theta3, p4, pbot, ptop, lp)) / (p2 - p4);
      } else {
        // The mixed forms differentiate return_sigmatheta analytically: in binary32 the centred
        // difference loses ~1e-5 of the derivative to rounding and truncation, and W3's error
        // then dominates the mixed form's error after a day (0.5e-3 in V at 128x64x20; the
        // difference quotient in binary64 agrees with the derivative to ~1e-11).  At the
        // interface where the hybrid coordinate turns to pure sigma, the reference's difference
        // is one-sided into the sigma region, so the sigma-side derivative is taken there.
        CT(DF, k) = dsigmatheta_dp<R>(M, theta3, p3, pbot, lp, k == ks - 1);
      }
      CT(W, k) = w;
    }
  __syncthreads();
  if (c.warp == 0 && c.valid) {
    M.w3[c.base] = 0.;
    M.w3[c.base + nk * n2] = 0.;
    double sum_div = 0.;
    for (int k = 1; k < nk; k++) {
      if (k >= 2) sum_div = sum_div + to_d(CT(DS, k));
      // SUM_DIV(nk) = 0, so the dF/dpbot term contributes nothing.
      M.w3[c.base + k * n2] = to_d(CT(W, k)) - (sum_div * to_d(CT(DF, k)) + 0.);
    }
  }
}

// Held-Suarez boundary-layer drag and the top sponge of uv_drag, epic_timestep.c:1303-1509.
// Columns on the u grid (j = 0..nj) and v grid (j = 1..nj), i = 1..ni.
template <class R>
__global__ void k_uv_drag(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int ni = M.ni, nk = M.nk;
  const int nu = (M.nj + 1) * ni;
  const int isv = t >= nu;
  const int tt = isv ? t - nu : t;
  if (tt >= (isv ? M.nj * ni : nu)) return;
  const int j = (isv ? 1 : 0) + tt / ni;
  const int i = 1 + tt % ni;
  const Ctl *c = M.ctl;
  const double *W = (isv ? M.v : M.u) + (long long)c->it_uv_dis * M.n3;
  double *D = (isv ? M.dvdt : M.dudt) + (long long)c->it_uv_tend * M.n3;
  const int jm = isv ? j - 1 : j, im = isv ? i : i - 1;   // neighbour averaged onto the u or v point
  for (int k = 0; k <= M.k_sponge; k++) {
    const long long x = M.at(k, j, i);
    D[x] = D[x] - to_d(cv<R>(M.t_sponge_inv[k]) * (cv<R>(W[x]) - (isv ? R(0.) : cv<R>(M.u_spinup[x]))));
  }
  if (M.rayleigh_on) {
    // The zonal-mean Rayleigh drag block is not part of the supported configurations
    // (held_suarez sets prandtl = 0 and tau_drag = 1e20); epic_model_create rejects it.
  }
  const R pbot = R(0.5) * (cv<R>(M.p3[M.at(nk, j, i)]) + cv<R>(M.p3[M.at(nk, jm, im)]));
  for (int k = nk - 1; k >= 1; k--) {
    const R p3 = R(.5) * (cv<R>(M.p3[M.at(k, j, i)]) + cv<R>(M.p3[M.at(k, jm, im)]));
    const R amp = (p3 / pbot - R(0.7)) / (R(1.) - R(0.7));
    if (amp < R(0.)) break;
    const R nu0 = cv<R>(M.hs_kf) * amp;
    const long long x = M.at(k, j, i);
    D[x] = D[x] - to_d(nu0 * cv<R>(W[x]));
  }
}

// Vertical pass of hsu_advection, epic_flux.c:717-1052.  kind: 0 = unity (P3_INDEX),
// 1 = THETA, 2 = HDRY, 3 = NU_TURB (loaded, moved by the interface velocities and updated as an
// interface variable, with the layer variables' predictor and corrector, :876-960, and the floor
// NU_TURB_MIN).  A column tile (32 columns j = 0..nj, i = 0..ni+1 per block): every pass
// of the predictor-corrector is pointwise in k given the previous pass, so the levels are
// spread over the warps with a barrier between passes; d1, d2 and the smoothness weights are
// recomputed where used (the same expressions, so the same values).  Shared arrays [k][lane]:
// WA (the field), WM, WP (the split vertical velocity), PR (the predictor), FF (the fluxes).
template <class R>
__global__ void __launch_bounds__(CT_THREADS) k_hsu_vertical(DevModel M, double *buff, int kind) {
  if (epic_member(M, buff)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sm = reinterpret_cast<R *>(smraw);
  const ColTile c = col_tile(M);
  const int nk = M.nk, L = nk + 2;
  const long long n2 = M.n2;
  const bool layer = kind == 2, nuk = kind == 3;
  const int kf = kind == 1 ? M.k_sigma - 1 : 1;
  const R ep = R(1.e-10), DT = cv<R>(M.dt);
  R *WA = sm, *WM = WA + 32 * L, *WP = WM + 32 * L, *PR = WP + 32 * L, *FF = PR + 32 * L;
  auto amin = [&](int k) { return layer ? cv<R>(M.h_min[k]) : (nuk && k >= 1 ? cv<R>(1.e-3 * M.kinvisc) : R(0.)); };
  auto dsi = [&](int kk) { return cv<R>(M.dsgth_inv[kk]); };
  auto wa = [&](int k) { return CT(WA, k); };
  if (c.valid)
    for (int k = (layer ? kf : kf - 1) + c.warp; k <= nk; k += CT_WARPS) CT(WA, k) = cv<R>(buff[c.base + k * n2]);
  if (layer || nuk) {
    if (c.valid && layer)
      for (int k = kf - 1 + c.warp; k <= nk; k += CT_WARPS) {
        const R w = cv<R>(M.w3[c.base + k * n2]);
        CT(WM, k) = rmin(R(0.), w);
        CT(WP, k) = rmax(R(0.), w);
      }
    if (c.valid && nuk) {
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const R w = (k == 1 || k == nk) ? R(0.) : R(.5) * (cv<R>(M.w3[c.base + k * n2]) + cv<R>(M.w3[c.base + (k - 1) * n2]));
        CT(WM, k) = rmin(R(0.), w);
        CT(WP, k) = rmax(R(0.), w);
      }
      // entry 0 is never loaded for NU_TURB; the corrector reads it only against d2(1) = 0
      if (c.warp == 0) { CT(WM, 0) = R(0.); CT(WP, 0) = R(0.); }
    }
    __syncthreads();
    if (c.valid)
      for (int k = kf - 1 + c.warp; k <= nk; k += CT_WARPS)
        CT(FF, k) = (k == kf - 1 || k == nk) ? R(0.) : CT(WP, k) * wa(k + 1) + CT(WM, k) * wa(k);
    __syncthreads();
    if (c.valid)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) CT(PR, k) = wa(k) + (CT(FF, k) - CT(FF, k - 1)) * dsi(2 * k) * DT;
    __syncthreads();
    // d1, d2 and the smoothness weight aa of level k (epic_flux.c's first corrector loop)
    auto d1 = [&](int k) { return k == nk ? R(0.) : CT(PR, k) - wa(k + 1); };
    auto d2 = [&](int k) { return k == 1 ? R(0.) : CT(PR, k) - wa(k - 1); };
    auto aa = [&](int k) {
      R tmp;
      if (k == 1) tmp = fabs(wa(k + 1) - wa(k)) + ep;
      else if (k == nk) tmp = fabs(-wa(k) + wa(k - 1)) + ep;
      else tmp = fabs(wa(k + 1) - R(2.) * wa(k) + wa(k - 1)) + ep;
      return tmp * tmp;
    };
    // the corrector reads PR, WA, WM and WP only, so it rewrites FF in place
    if (c.valid)
      for (int k = kf + c.warp; k < nk; k += CT_WARPS) {
        const R wpk = CT(WP, k), wmk = CT(WM, k);
        R f = R(.5) * (wpk * (CT(PR, k) + wa(k + 1)) + wmk * (CT(PR, k + 1) + wa(k)));
        const R whatp = sqrt(wpk * CT(WP, k + 1));
        const R whatm = -sqrt(wmk * CT(WM, k - 1));
        const R mu = (wpk - wmk) * dsi(2 * k + 1) * DT;
        const R al = (R(1.) + mu) / R(6.);
        const R prod = (wa(k + 1) - amin(k + 1)) * (wa(k) - amin(k));
        const R aap = aa(k + 1), aak = aa(k);
        R gap = aap / (aap + prod); gap = gap * gap;
        R gam = aak / (aak + prod); gam = gam * gam;
        const R bep = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gap;
        const R bem = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gam;
        f += -al * (wpk * bep * d1(k) - whatp * (R(1.) - gap) * d1(k + 1) + wmk * bem * d2(k + 1) - whatm * (R(1.) - gam) * d2(k));
        CT(FF, k) = f;
      }
    __syncthreads();
    if (c.valid && layer)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const long long x = c.base + k * n2;
        buff[x] = buff[x] + to_d((CT(FF, k) - CT(FF, k - 1)) * dsi(2 * k) * DT);
      }
    if (c.valid && nuk)   // the interface update; w_ff[nk+1] is the 0 the THETA call left there
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const long long x = c.base + k * n2;
        const R ffk1 = k == nk ? R(0.) : CT(FF, k + 1);
        buff[x] = buff[x] + to_d((ffk1 - CT(FF, k)) * dsi(2 * k + 1) * DT);
      }
  } else {
    if (c.valid)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const R w = (k == 1 || k == nk) ? R(0.) : R(.5) * (cv<R>(M.w3[c.base + k * n2]) + cv<R>(M.w3[c.base + (k - 1) * n2]));
        CT(WM, k) = rmin(R(0.), w);
        CT(WP, k) = rmax(R(0.), w);
      }
    __syncthreads();
    if (c.valid)
      for (int k = kf + c.warp; k <= nk + 1; k += CT_WARPS)
        CT(FF, k) = k == nk + 1 ? R(0.) : CT(WP, k) * wa(k) + CT(WM, k) * wa(k - 1);
    __syncthreads();
    if (c.valid)
      for (int k = kf - 1 + c.warp; k <= nk; k += CT_WARPS)
        CT(PR, k) = k == kf - 1 ? wa(kf - 1) : wa(k) + (CT(FF, k + 1) - CT(FF, k)) * dsi(2 * k + 1) * DT;
    __syncthreads();
    // For THETA (kf > 1) the entry below the first loaded one is the value the reference's
    // static column buffer keeps from the preceding unity advection: 1.0 (epic_flux.c:866-877).
    auto aa = [&](int k) {
      const R wkm1 = k >= 1 ? (k - 1 < kf - 1 ? R(1.0) : wa(k - 1)) : R(0.);
      R tmp;
      if (k == 0) tmp = fabs(wa(k + 1) - wa(k)) + ep;
      else if (k == nk) tmp = fabs(-wa(k) + wkm1) + ep;
      else tmp = fabs(wa(k + 1) - R(2.) * wa(k) + wkm1) + ep;
      return tmp * tmp;
    };
    auto d1 = [&](int k) { return CT(PR, k - 1) - wa(k); };
    auto d2 = [&](int k) { return k == kf - 1 ? R(0.) : CT(PR, k) - wa(k - 1); };
    if (c.valid)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const R wpk = CT(WP, k), wmk = CT(WM, k);
        R f = R(.5) * (wpk * (CT(PR, k - 1) + wa(k)) + wmk * (CT(PR, k) + wa(k - 1)));
        const R whatm = (k == 1 || k - 1 < kf) ? R(0.) : -sqrt(wmk * CT(WM, k - 1));
        const R whatp = (k == nk) ? R(0.) : sqrt(wpk * CT(WP, k + 1));
        const R mu = (wpk - wmk) * dsi(2 * k) * DT;
        const R al = (R(1.) + mu) / R(6.);
        const R prod = (wa(k) - amin(k)) * (wa(k - 1) - amin(k - 1));
        const R aak = aa(k), aam = aa(k - 1);
        R gap = aak / (aak + prod); gap = gap * gap;
        R gam = aam / (aam + prod); gam = gam * gam;
        const R bep = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gap;
        const R bem = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gam;
        R g;
        if (k < nk) g = -al * (wpk * bep * d1(k) - whatp * (R(1.) - gap) * d1(k + 1) + wmk * bem * d2(k) - whatm * (R(1.) - gam) * d2(k - 1));
        else g = -al * (wpk * bep * d1(k) + wmk * bem * d2(k) - whatm * (R(1.) - gam) * d2(k - 1));
        CT(FF, k) = f + g;
      }
    __syncthreads();
    if (c.valid)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const long long x = c.base + k * n2;
        const R ffk1 = k == nk ? R(0.) : CT(FF, k + 1);
        buff[x] = buff[x] + to_d((ffk1 - CT(FF, k)) * dsi(2 * k + 1) * DT);
      }
  }
}

// Akima's harmonic mean of like-signed differences (akima_advection's dela)
template <class R>
__device__ __forceinline__ R akima_dela(R d0, R d1) {
  const R tmp = d0 * d1;
  return (tmp > R(0.)) ? R(2.) * tmp / (d0 + d1) : R(0.);
}

// Vertical pass of akima_advection, epic_flux.c:1549-1744 (mass fluxes through the model top
// and bottom are 0 for Held-Suarez, :47-115).  kind: 0 = unity (P3_INDEX), 1 = THETA,
// 2 = HDRY.  A column tile (32 columns j = 0..nj, i = 0..ni+1 per block), the levels spread over
// the warps; shared arrays [k][lane]: WA (the field), W (the vertical velocity at the flux
// points), DL (dela), FF (the fluxes).
template <class R>
__global__ void __launch_bounds__(CT_THREADS) k_akima_vertical(DevModel M, double *buff, int kind) {
  if (epic_member(M, buff)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sm = reinterpret_cast<R *>(smraw);
  const ColTile c = col_tile(M);
  const int nk = M.nk, L = nk + 2;
  const long long n2 = M.n2;
  const bool layer = kind == 2, nuk = kind == 3;   // NU_TURB: the layer form of the flux (:1687-1706)
  const int kf = kind == 1 ? M.k_sigma - 1 : 1;
  const R DT = cv<R>(M.dt);
  R *WA = sm, *W = WA + 32 * L, *DL = W + 32 * L, *FF = DL + 32 * L;
  auto wa = [&](int k) { return CT(WA, k); };
  if (c.valid) {
    for (int k = (layer ? kf : kf - 1) + c.warp; k <= nk; k += CT_WARPS) CT(WA, k) = cv<R>(buff[c.base + k * n2]);
    if (layer)
      for (int k = kf - 1 + c.warp; k <= nk; k += CT_WARPS) CT(W, k) = cv<R>(M.w3[c.base + k * n2]);
    else
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS)
        CT(W, k) = (k == 1 || k == nk) ? R(0.) : R(.5) * (cv<R>(M.w3[c.base + k * n2]) + cv<R>(M.w3[c.base + (k - 1) * n2]));
  }
  __syncthreads();
  if (layer || nuk) {
    // deltaa(k) = a(k) - a(k+1) for kf <= k < nk, 0 at kf-1 and nk
    auto deltaa = [&](int k) { return (k < kf || k >= nk) ? R(0.) : wa(k) - wa(k + 1); };
    if (c.valid)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) CT(DL, k) = akima_dela<R>(deltaa(k), deltaa(k - 1));
    __syncthreads();
    if (c.valid)
      for (int k = kf - 1 + c.warp; k <= nk; k += CT_WARPS) {
        if (k == kf - 1 || k == nk) { CT(FF, k) = R(0.); continue; }   // mass_flux_top, mass_flux_bot
        const R aval = R(.5) * (wa(k) + wa(k + 1)) - (CT(DL, k) - CT(DL, k + 1)) / R(6.);
        CT(FF, k) = CT(W, k) * aval;
      }
    __syncthreads();
    if (c.valid && layer)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const long long x = c.base + k * n2;
        buff[x] = buff[x] + to_d((CT(FF, k) - CT(FF, k - 1)) * cv<R>(M.dsgth_inv[2 * k]) * DT);
      }
    if (c.valid && nuk)   // the interface update; w_ff[nk+1] is the 0 the THETA call left there
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const long long x = c.base + k * n2;
        const R ffk1 = k == nk ? R(0.) : CT(FF, k + 1);
        buff[x] = buff[x] + to_d((ffk1 - CT(FF, k)) * cv<R>(M.dsgth_inv[2 * k + 1]) * DT);
      }
  } else {
    // deltaa(k) = a(k-1) - a(k) for kf <= k <= nk
    auto deltaa = [&](int k) { return wa(k - 1) - wa(k); };
    if (c.valid)
      for (int k = kf - 1 + c.warp; k <= nk; k += CT_WARPS)
        CT(DL, k) = (k == kf - 1 || k == nk) ? R(0.) : akima_dela<R>(deltaa(k), deltaa(k + 1));
    __syncthreads();
    if (c.valid)
      for (int k = kf + c.warp; k <= nk + 1; k += CT_WARPS) {
        if (k == nk + 1) { CT(FF, k) = R(0.); continue; }
        const R aval = R(.5) * (wa(k - 1) + wa(k)) - (CT(DL, k - 1) - CT(DL, k)) / R(6.);
        CT(FF, k) = CT(W, k) * aval;
      }
    __syncthreads();
    if (c.valid)
      for (int k = kf + c.warp; k <= nk; k += CT_WARPS) {
        const long long x = c.base + k * n2;
        buff[x] = buff[x] + to_d((CT(FF, k + 1) - CT(FF, k)) * cv<R>(M.dsgth_inv[2 * k + 1]) * DT);
      }
  }
}

// restore_mass(HDRY_INDEX), epic_adjust.c:45-96
// Pointwise: one thread per cell of layers 1..nk, rows 0..nj, all columns.
__global__ void k_restore_mass(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int per_k = (M.nj + 1) * (M.ni + 2);
  if (t >= M.nk * per_k) return;
  const int k = 1 + t / per_k;
  const int x = M.at(k, 0, 0) + (t - (k - 1) * per_k);
  M.hdry[x] = dmaxr(M.h_min[k], M.hdry[x]);
}

// set_p2etc, epic_funcs_diag.c:3352-3569 (nq = 0: H2 is HDRY, PDRY3 is P3, HDRY3 is H3).
// Shared arrays: P (interface pressure), HL (get_h at the layers), TH (THETA), PP (P^(kappa+1),
// each interface's power computed once for the two layers that share it).
__global__ void __launch_bounds__(CT_THREADS) k_set_p2etc(DevModel M, int update_theta) {
  if (epic_member(M)) return;
  extern __shared__ double sm[];
  __shared__ double s_lp[32];
  const ColTile c = col_tile(M);
  const int nk = M.nk, ks = M.k_sigma, L = nk + 1;
  const long long n2 = M.n2;
  double *P = sm, *HL = P + 32 * L, *TH = HL + 32 * L, *PP = TH + 32 * L;
  __shared__ int s_kay[EPIC_MAX_NK + 1];
  if (update_theta) theta2_intervals(M, s_kay, nullptr);
  const double g = M.grav[2 * c.j + 1];
  if (c.valid)   // stage H2 (in HL until the prefix sum is done) and THETA
    for (int k = c.warp; k <= nk; k += CT_WARPS) {
      CT(TH, k) = M.theta[c.base + k * n2];
      if (k >= 1) CT(HL, k) = M.hdry[c.base + k * n2];
    }
  __syncthreads();
  if (c.warp == 0 && c.valid) {   // P3 top-down: P3(K) = P3(K-1) + dsgth*g*H2
    double p = M.p3[c.base];
    CT(P, 0) = p;
    for (int k = 1; k <= nk; k++) {
      p = p + M.dsgth[2 * k] * g * CT(HL, k);
      CT(P, k) = p;
    }
    s_lp[c.lane] = xlog(M, CT(P, 0) / p);   // log(ptop/pbot)
  }
  __syncthreads();
  const double ptop = CT(P, 0), pbot = CT(P, nk), lp = s_lp[c.lane];
  if (c.valid)   // pure-sigma interfaces: get_p_sigma
    for (int k = ks - 1 + c.warp; k < nk; k += CT_WARPS) {
      const double sigma = (M.sgth[2 * k + 1] - M.zeta0) / (M.zeta1 - M.zeta0);
      CT(P, k) = pbot * xexp(M, sigma * lp);
    }
  __syncthreads();
  const double kp1 = M.kappa + 1.;
  if (c.valid)
    for (int k = c.warp; k <= nk; k += CT_WARPS) {
      const double pk = CT(P, k);
      if (k >= 1) {
        const long long x = c.base + k * n2;
        M.p3[x] = pk;
        const double hl = (pk - CT(P, k - 1)) / (g * M.dsgth[2 * k]);
        CT(HL, k) = hl;
        M.hdry[x] = dmaxr(M.h_min[k], hl);
      }
      CT(PP, k) = xpow(M, pk, kp1);
      if (update_theta && k < ks - 1) {   // the diagnostic THETA above k_sigma-1
        const double sigma = xlog(M, pk / pbot) / lp;
        double gs;
        const double fs = f_and_g_sigma(M, sigma, gs);
        const double th = (M.sgth[2 * k + 1] - fs) / gs;
        CT(TH, k) = th;
        M.theta[c.base + k * n2] = th;
      }
    }
  __syncthreads();
  if (!c.valid) return;
  for (int k = 1 + c.warp; k <= nk; k += CT_WARPS) {
    const long long x = c.base + k * n2;
    const double top = CT(P, k - 1), bot = CT(P, k);
    double p2;   // onto_kk(P2_INDEX) at the layer, epic_funcs_diag.c:2601-2618
    if (fcmp(bot, top) == 0) p2 = .5 * (bot + top);
    else p2 = xpow(M, (CT(PP, k) - CT(PP, k - 1)) / (kp1 * (bot - top)), 1. / M.kappa);
    M.p2[x] = p2;
    if (k == 1) M.p2[c.base] = top * top / p2;
    double h;
    if (k == nk) h = CT(HL, nk);
    else {
      const double topwt = M.dsgth[2 * k], botwt = M.dsgth[2 * k + 2];
      h = (topwt * CT(HL, k) + botwt * CT(HL, k + 1)) / (topwt + botwt);
    }
    M.h3[x] = h;
    if (k == 1) M.h3[c.base] = h;
    if (!update_theta) continue;
    double t2;
    if (k < ks - 1) {
      const double sigma = xlog(M, p2 / pbot) / lp;
      double gs;
      const double fs = f_and_g_sigma(M, sigma, gs);
      t2 = (M.sgth[2 * k] - fs) / gs;
    } else if (k == ks - 1) {
      t2 = .5 * (CT(TH, ks - 1) + CT(TH, ks - 2));
    } else {
      // linint on the table (sigmatheta[2K+1], THETA(K)), K = nk down to k_sigma-1, in the
      // interval theta2_intervals found for this level
      const double sg = M.sgth[2 * k];
      auto X = [&](int kay) { return M.sgth[2 * (nk - kay) + 1]; };
      auto Y = [&](int kay) { return CT(TH, nk - kay); };
      const int kay = s_kay[k];
      const double dx = X(kay + 1) - X(kay);
      t2 = Y(kay) + (Y(kay + 1) - Y(kay)) * (sg - X(kay)) / dx;
    }
    M.theta2[x] = t2;
  }
}

// store_pgrad_vars, column part (epic_funcs_diag.c:3595-3895): T3, EXNER3, RHO3, T2, RHO2,
// the k = 0 extrapolations, GZ3 and MONT3 from the surface up, the monotone-GZ check, and
// the first DZDT3 terms.  Shared arrays: P, R (RHO3), T3, LG (log of successive pressure
// ratios), GZ (the Leslie-Purser increments, then the running sum in place).
__global__ void __launch_bounds__(CT_THREADS) k_pgrad_vars_column(DevModel M) {
  if (epic_member(M)) return;
  extern __shared__ double sm[];
  __shared__ double s_rho2_1[32];
  const ColTile c = col_tile(M);
  const int nk = M.nk, L = nk + 1;
  const long long n2 = M.n2;
  const double mu = M.mu_dry;
  double *P = sm, *R = P + 32 * L, *T3 = R + 32 * L, *LG = T3 + 32 * L, *GZ = LG + 32 * L;
  if (c.valid)
    for (int k = c.warp; k <= nk; k += CT_WARPS) {
      const long long x = c.base + k * n2;
      const double theta = M.theta[x], p = M.p3[x];
      const double t3 = return_temp(M, p, theta);
      M.t3[x] = t3;
      M.exner3[x] = M.cp * t3 / theta;
      const double rho = return_density(p, t3, mu);
      M.rho3[x] = rho;
      CT(P, k) = p;
      CT(R, k) = rho;
      CT(T3, k) = t3;
      if (k >= 1) {
        const double pr = M.p2[x];
        const double t2 = return_temp(M, pr, M.theta2[x]);
        M.t2[x] = t2;
        const double r2 = return_density(pr, t2, mu);
        M.rho2[x] = r2;
        if (k == 1) s_rho2_1[c.lane] = r2;
      }
    }
  __syncthreads();
  if (c.valid) {
    for (int k = c.warp; k < nk; k += CT_WARPS) CT(LG, k) = xlog(M, CT(P, k + 1) / CT(P, k));
    if (c.warp == CT_WARPS - 1) {
      M.rho2[c.base] = CT(R, 0) * CT(R, 0) / s_rho2_1[c.lane];
      M.theta2[c.base] = M.sgth[0];
      M.t2[c.base] = CT(T3, 0);
    }
  }
  __syncthreads();
  if (c.valid)
    for (int k = 2 + c.warp; k <= nk - 1; k += CT_WARPS) {
      const double dz10 = CT(LG, k), dz21 = CT(LG, k - 1), dz32 = CT(LG, k - 2);
      const double dz20 = dz21 + dz10, dz30 = dz32 + dz20, dz31 = dz32 + dz21;
      const double df0 = CT(P, k + 1) / CT(R, k + 1), df1 = CT(P, k) / CT(R, k), df2 = CT(P, k - 1) / CT(R, k - 1),
                   df3 = CT(P, k - 2) / CT(R, k - 2);
      CT(GZ, k - 1) = -(df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                        df1 * (dz21 * (dz21 * (dz21 + 2. * (dz10 - dz31)) - 6. * dz10 * dz31)) / (dz10 * dz31) +
                        df2 * (dz21 * (dz21 * (dz21 + 2. * (dz32 - dz20)) - 6. * dz20 * dz32)) / (dz20 * dz32) +
                        df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32)) /
                      12.;
    }
  __syncthreads();
  if (c.warp == 0 && c.valid) {   // GZ3 from the surface up
    double gz = M.topo_scale * M.gz_surface[M.at2(c.j, c.i)];
    CT(GZ, nk) = gz;
    gz = gz + ((CT(P, nk) + CT(P, nk - 1)) / (CT(R, nk) + CT(R, nk - 1))) * CT(LG, nk - 1);
    CT(GZ, nk - 1) = gz;
    for (int k = nk - 1; k >= 2; k--) {
      gz = gz + CT(GZ, k - 1);
      CT(GZ, k - 1) = gz;
    }
    CT(GZ, 0) = gz + ((CT(P, 1) + CT(P, 0)) / (CT(R, 1) + CT(R, 0))) * CT(LG, 0);
  }
  __syncthreads();
  if (!c.valid) return;
  const bool interior = c.i >= 1 && c.i <= M.ni;
  const long long itime = M.ctl->itime;
  for (int k = c.warp; k <= nk; k += CT_WARPS) {
    const long long x = c.base + k * n2;
    const double gzk = CT(GZ, k);
    const double old = M.gz3[x];
    M.gz3[x] = gzk;
    M.mont3[x] = gzk + return_enthalpy(M, CT(T3, k));
    if (interior && k >= 1) {
      // DZDT3 = -(GZ3_new - GZ3_old)/(dt*g) from the third step on, 0 before (:3679-3693, :3897-3909)
      double dz = 0.;
      if (itime > 1) {
        const double dtg_inv = -1. / (M.dt * M.grav[2 * c.j + 1]);
        dz = (old - gzk) * dtg_inv;
      }
      dz += M.w3[x] * M.h3[x] / CT(R, k);
      M.dzdt3[x] = dz;
      if (gzk >= CT(GZ, k - 1)) flag_error(M.ctl, ERR_GZ_MONOTONE, k, c.j, c.i, gzk);
    }
  }
}

// ---- the mixed form of the two hydrostatic column routines ----
//
// The interface pressures P3 (prefix sum of the layer masses) and GZ3 (the surface-up sum of
// Leslie-Purser increments) are accumulated in FP64, as are HDRY, H3 and every stored state
// value; the pointwise transcendentals feeding them (the layer-mean pressure P2, T3 and T2,
// the logarithms of successive pressure ratios, the diagnostic theta above k_sigma-1) are
// evaluated in FP32 from FP64 differences (log1p/expm1 of small ratios), which keeps their
// relative error near 1e-7.


// onto_kk(P2_INDEX) at a layer: ((bot^(k+1) - top^(k+1)) / ((k+1)(bot - top)))^(1/k), written as
// bot * q^(1/kappa), q = (1 - r^(kappa+1)) / ((kappa+1)(1 - r)), r = top/bot.  The FP32
// expression stays accurate as eps = 1 - r goes to zero (log1p/expm1), so only eps = 0 needs
// the reference's equal-pressure branch.
__device__ __forceinline__ double layer_p_mixed(const DevModel &M, double top, double bot) {
  const float kap = d2f(M.kappa), kp1 = kap + 1.f;
  const float eps = d2f(bot - top) / d2f(bot);
  if (eps == 0.f) return .5 * (bot + top);
  const float num = -expm1f(kp1 * log1pf(-eps));
  const float q = num / (kp1 * eps);
  return bot * f2d(expf(log1pf(q - 1.f) / kap));
}

// layers = 0: P3 and HDRY only (the call inside advection, whose P2 and H3 stage 11 rewrites
// before anything reads them)
__global__ void __launch_bounds__(CT_THREADS, 4) k_set_p2etc_mixed(DevModel M, int update_theta, int layers) {
  if (epic_member(M)) return;
  extern __shared__ double sm[];
  __shared__ int s_kay[EPIC_MAX_NK + 1];
  __shared__ float s_w[EPIC_MAX_NK + 1];
  if (update_theta && layers) theta2_intervals(M, s_kay, s_w);
  const ColTile c = col_tile(M);
  const int nk = M.nk, ks = M.k_sigma, L = nk + 1;
  const long long n2 = M.n2;
  double *P = sm, *HL = P + 32 * L, *TH = HL + 32 * L;
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
  if (c.valid)
    for (int k = c.warp; k <= nk; k += CT_WARPS) {
      const double pk = CT(P, k);
      if (k >= 1) {
        const long long x = c.base + k * n2;
        M.p3[x] = pk;
        // above the pure-sigma interfaces the layer's dp is the one just summed, so its mass is
        // the input HDRY (to the rounding of the sum); only layers next to a rescaled interface
        // are recomputed from the pressures
        double hl = CT(HL, k);
        if (k >= ks - 1) {
          hl = (pk - CT(P, k - 1)) * (ginv * M.dsgth_inv[2 * k]);
          CT(HL, k) = hl;
        }
        M.hdry[x] = dmaxr(M.h_min[k], hl);
      }
      if (update_theta && k < ks - 1) {
        const float sigma = log_ratio_f(pbot, pk) / lpf;
        float gs;
        const float fs = f_and_g_sigma_r<float>(M, sigma, gs);
        const double th = f2d((d2f(M.sgth[2 * k + 1]) - fs) / gs);
        CT(TH, k) = th;
        M.theta[c.base + k * n2] = th;
      }
    }
  __syncthreads();
  if (!c.valid || !layers) return;
  for (int k = 1 + c.warp; k <= nk; k += CT_WARPS) {
    const long long x = c.base + k * n2;
    const double top = CT(P, k - 1), bot = CT(P, k);
    const double p2 = layer_p_mixed(M, top, bot);
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
    } else {   // linint in binary32 with the block's interval and weight of this level
      const float y0 = d2f(CT(TH, nk - s_kay[k])), y1 = d2f(CT(TH, nk - s_kay[k] - 1));
      t2 = f2d(y0 + (y1 - y0) * s_w[k]);
    }
    M.theta2[x] = t2;
  }
}

// FULL = false: GZ3 alone (and its monotonicity check), for the call before the filtered-GZ
// copy; that call's T3, EXNER3, RHO3, T2, RHO2, MONT3 and DZDT3 are rewritten by the call after
// set_p2etc (stage 19) before anything reads them, and that call reads this GZ3 as the old one.
// H2: the hydrogen thermodynamics (x_h2 > 0): T3, T2 and MONT3's enthalpy from thermo_setup's
// tables in binary64, EXNER3 = cp T3 / THETA (epic_funcs_diag.c:3698, :3717).
template <bool FULL, bool H2>
__global__ void __launch_bounds__(CT_THREADS, 4) k_pgrad_vars_column_mixed(DevModel M) {
  if (epic_member(M)) return;
  extern __shared__ double sm[];
  __shared__ double s_rho2_1[32];
  const ColTile c = col_tile(M);
  const int nk = M.nk, L = nk + 1;
  const long long n2 = M.n2;
  const double mu = M.mu_dry;
  double *P = sm, *R = P + 32 * L, *T3 = R + 32 * L, *GZ = T3 + 32 * L;
  float *LG = reinterpret_cast<float *>(GZ + 32 * L);
  const float kap = d2f(M.kappa);
  const float p0_inv = d2f(1. / M.press0);
  const float mu_over_r = d2f(mu / 8.314472e+3);   // return_density: p mu / (R T)
  const float cpf = d2f(M.cp);
  // T3 = theta (p/p0)^kappa, EXNER3, RHO3 and the layer T2, RHO2 in FP32 (their relative error
  // is that of the FP32 power, 1e-7, either way), stored in binary64
  auto level = [&](int k, double theta, double p, double pr, double th2) {
      const long long x = c.base + k * n2;
      float pf = 0.f;
      double t3, rho;
      pf = powf(d2f(p) * p0_inv, kap);
      if (H2) {   // the table at the binary32 ideal-gas temperature
        t3 = hydrogen_temp(M, f2d(d2f(theta) * pf));
        rho = return_density(p, t3, mu);
      } else {
        const float t3f = d2f(theta) * pf;
        t3 = f2d(t3f);
        rho = f2d(d2f(p) * mu_over_r / t3f);
      }
      CT(P, k) = p;
      CT(R, k) = rho;
      CT(T3, k) = t3;
      if (!FULL) return;
      M.t3[x] = t3;
      M.exner3[x] = H2 ? M.cp * t3 / theta : f2d(cpf * pf);
      M.rho3[x] = rho;
      if (k >= 1) {
        double r2;
        if (H2) {
          const double t2 = hydrogen_temp(M, f2d(d2f(th2) * powf(d2f(pr) * p0_inv, kap)));
          M.t2[x] = t2;
          r2 = return_density(pr, t2, mu);
        } else {
          const float t2f = d2f(th2) * powf(d2f(pr) * p0_inv, kap);
          M.t2[x] = f2d(t2f);
          r2 = f2d(d2f(pr) * mu_over_r / t2f);
        }
        M.rho2[x] = r2;
        if (k == 1) s_rho2_1[c.lane] = r2;
      }
  };
  if (c.valid) {
    // the loads of the first TILE_SLOTS levels of this warp are issued together (their
    // latencies overlap); level 0's P2 and THETA2 are loaded but not used
    double v[TILE_SLOTS][4];
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++) {
      const long long x = c.base + min(c.warp + r * CT_WARPS, nk) * n2;
      v[r][0] = __ldg(M.theta + x); v[r][1] = __ldg(M.p3 + x);
      if (FULL) { v[r][2] = __ldg(M.p2 + x); v[r][3] = __ldg(M.theta2 + x); }
      else v[r][2] = v[r][3] = 0.;
    }
#pragma unroll
    for (int r = 0; r < TILE_SLOTS; r++)
      if (c.warp + r * CT_WARPS <= nk) level(c.warp + r * CT_WARPS, v[r][0], v[r][1], v[r][2], v[r][3]);
    for (int k = c.warp + TILE_SLOTS * CT_WARPS; k <= nk; k += CT_WARPS) {
      const long long x = c.base + k * n2;
      level(k, M.theta[x], M.p3[x], FULL ? M.p2[x] : 0., FULL ? M.theta2[x] : 0.);
    }
  }
  __syncthreads();
  if (c.valid) {
    for (int k = c.warp; k < nk; k += CT_WARPS) CT(LG, k) = log_ratio_f(CT(P, k), CT(P, k + 1));
    if (FULL && c.warp == CT_WARPS - 1) {
      M.rho2[c.base] = CT(R, 0) * CT(R, 0) / s_rho2_1[c.lane];
      M.theta2[c.base] = M.sgth[0];
      M.t2[c.base] = CT(T3, 0);
    }
  }
  __syncthreads();
  // the geopotential increments of every layer (Leslie-Purser inside, short centred at the two
  // ends; the differences of P and RHO in FP64), then GZ3 from the surface up by every warp
  if (c.valid) {
    if (c.warp == 0) CT(GZ, nk) = M.topo_scale * M.gz_surface[M.at2(c.j, c.i)];
    if (c.warp == CT_WARPS - 1) {
      CT(GZ, nk - 1) = ((CT(P, nk) + CT(P, nk - 1)) / (CT(R, nk) + CT(R, nk - 1))) * f2d(CT(LG, nk - 1));
      CT(GZ, 0) = ((CT(P, 1) + CT(P, 0)) / (CT(R, 1) + CT(R, 0))) * f2d(CT(LG, 0));
    }
    for (int k = 2 + c.warp; k <= nk - 1; k += CT_WARPS) {
      const float dz10 = CT(LG, k), dz21 = CT(LG, k - 1), dz32 = CT(LG, k - 2);
      const float dz20 = dz21 + dz10, dz30 = dz32 + dz20, dz31 = dz32 + dz21;
      // p/rho = R T / mu
      const float r_over_mu = 1.f / mu_over_r;
      const float df0 = r_over_mu * d2f(CT(T3, k + 1)), df1 = r_over_mu * d2f(CT(T3, k));
      const float df2 = r_over_mu * d2f(CT(T3, k - 1)), df3 = r_over_mu * d2f(CT(T3, k - 2));
      CT(GZ, k - 1) = f2d(-(df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                                 df1 * (dz21 * (dz21 * (dz21 + 2.f * (dz10 - dz31)) - 6.f * dz10 * dz31)) / (dz10 * dz31) +
                                 df2 * (dz21 * (dz21 * (dz21 + 2.f * (dz32 - dz20)) - 6.f * dz20 * dz32)) / (dz20 * dz32) +
                                 df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32)) /
                               12.f);
    }
  }
  __syncthreads();
  ct_running_sum_up(GZ, nk, c.lane, c.warp);
  if (!c.valid) return;
  const bool interior = c.i >= 1 && c.i <= M.ni;
  const long long itime = M.ctl->itime;
  // MONT3 and DZDT3 are diagnostics that no later kernel of the step reads: FP32 arithmetic on
  // the FP64 change of GZ3 (the difference itself stays FP64: it cancels)
  const float dtg_inv = -1.f / (d2f(M.dt) * d2f(M.grav[2 * c.j + 1]));
  const float cprf = d2f(M.cpr), rgasf = d2f(M.rgas);
  if (!FULL) {
    for (int k = c.warp; k <= nk; k += CT_WARPS) {
      const double gzk = CT(GZ, k);
      M.gz3[c.base + k * n2] = gzk;
      if (interior && k >= 1 && gzk >= CT(GZ, k - 1)) flag_error(M.ctl, ERR_GZ_MONOTONE, k, c.j, c.i, gzk);
    }
    return;
  }
  auto level_out = [&](int k, double old, double w, double h) {
    const long long x = c.base + k * n2;
    const double gzk = CT(GZ, k);
    M.gz3[x] = gzk;
    put_split(M.work1, x, gzk);
    if (H2) M.mont3[x] = gzk + return_enthalpy(M, CT(T3, k));
    else M.mont3[x] = f2d(d2f(gzk) + cprf * d2f(CT(T3, k)) * rgasf);   // GZ3 + return_enthalpy
    if (interior && k >= 1) {
      float dz = 0.f;
      if (itime > 1) dz = d2f(old - gzk) * dtg_inv;
      dz += d2f(w) * d2f(h) / d2f(CT(R, k));
      M.dzdt3[x] = f2d(dz);
      if (gzk >= CT(GZ, k - 1)) flag_error(M.ctl, ERR_GZ_MONOTONE, k, c.j, c.i, gzk);
    }
  };
  double v[TILE_SLOTS][3];
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

// store_pgrad_vars, horizontal part of DZDT3 (epic_funcs_diag.c:3924-3945) plus bc_lateral.
template <class R>
__global__ void k_pgrad_dzdt(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int ni = M.ni, nk = M.nk;
  if (t >= nk * (M.nj + 1) * ni) return;
  const int i = 1 + t % ni;
  const int j = (t / ni) % (M.nj + 1);
  const int k = 1 + t / (ni * (M.nj + 1));
  const int jj = 2 * j;
  const Ctl *c = M.ctl;
  const double *U = M.u + (long long)c->it_uv * M.n3, *V = M.v + (long long)c->it_uv * M.n3;
  const R gdx_inv3 = R(.5) * cv<R>(M.m[jj + 1]) / cv<R>(M.grav[jj + 1]);
  const R gdy_inv2 = R(.5) * cv<R>(M.n[jj]) / cv<R>(M.grav[jj]);
  const R gdy_inv4 = R(.5) * cv<R>(M.n[jj + 2]) / cv<R>(M.grav[jj + 2]);
  const double *G = M.gz3;
  const long long x = M.at(k, j, i);
  // geopotential differences are formed in FP64 in both forms
  const R add = cv<R>(V[x]) * cv<R>(G[x] - G[M.at(k, j - 1, i)]) * gdy_inv2 + cv<R>(V[M.at(k, j + 1, i)]) * cv<R>(G[M.at(k, j + 1, i)] - G[x]) * gdy_inv4 +
                cv<R>(U[x]) * cv<R>(G[x] - G[M.at(k, j, i - 1)]) * gdx_inv3 + cv<R>(U[M.at(k, j, i + 1)]) * cv<R>(G[M.at(k, j, i + 1)] - G[x]) * gdx_inv3;
  write_with_pads(M.dzdt3, M, M.at(k, j, 0), i, M.dzdt3[x] + to_d(add));
}

// Monotone fix of the filtered GZ copy, epic_timestep.c:182-195 (the zonal filter of planes
// 0..nk-1 has already run; each plane's fix only needs the finished plane below it).
__global__ void k_gz_monotone(DevModel M) {
  if (epic_member(M)) return;
  int j, i;
  if (!col_index(M, j, i)) return;
  double below = M.gz[M.at(M.nk, j, i)];
  for (int k = M.nk - 1; k >= 0; k--) {
    const long long x = M.at(k, j, i);
    double g;
    // fcmp(below, 0.) == 0 holds exactly when below is +-0 or NaN (for any other value the
    // tolerance, DBL_EPSILON times 2^exponent, is below |below|): tested without frexp/ldexp,
    // which cost ten FP64 instructions a level
    if (below == 0. || below != below) g = 1.e-3;
    else g = dmaxr(M.gz[x], below + fabs(below) * 1.e-5);
    M.gz[x] = g;
    below = g;
  }
}

// calc_heating -> newtonian_cooling for held_suarez (epic_funcs_diag.c:4793-4869,
// epic_sensible_heating.c:51-180, t_rad :217-314, temp_eq :325-463).  Writes every HEAT3 cell:
// 0 outside k = 1..nk, j = 0..nj, i = 1..ni, with periodic pads.
template <class R>
__global__ void k_calc_heating(DevModel M) {
  if (epic_member(M)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;   // n3 < 2^31
  if (t >= (unsigned)M.n3) return;
  const unsigned r = t / (unsigned)M.iadim, q = r / (unsigned)M.jadim;
  const int i = (int)(t - r * (unsigned)M.iadim);
  const int j = (int)(r - q * (unsigned)M.jadim) - 1;
  const int k = (int)q;
  R val = R(0.);
  int ii = i == 0 ? M.ni : (i == M.ni + 1 ? 1 : i);
  if (k >= 1 && k <= M.nk && j >= 0 && j <= M.nj && M.newt_cool_on) {
    const long long x = M.at(k, j, ii);
    const R ka = R(1.) / (R(40.) * R(60.) * R(60.) * R(24.)), ks = R(1.) / (R(4.) * R(60.) * R(60.) * R(24.));
    const R pressure = cv<R>(M.p3[x]);
    const R pbot = cv<R>(M.p3[M.at(M.nk, j, ii)]);
    const R amp = (pressure / pbot - R(0.7)) / (R(1.) - R(0.7));
    R kt = ka;
    if (amp > R(0.)) kt += (ks - ka) * RMath<R>::cos4(M, j) * amp;   // pow(cos(lat), 4.), per row
    const R cp_over_time = R(1004.) / (R(1.) / kt);
    R c2 = cv<R>(M.coslat[j]);
    c2 *= c2;
    const R s2 = R(1.) - c2;
    const R p_p0 = pressure / (R(1000.) * R(100.));
    R lg;
    const R pw = RMath<R>::log_pow(M, p_p0, cv<R>(M.kappa), lg);
    R teq = (R(315.) - R(60.) * s2 - R(10.) * lg * c2) * pw;
    teq = rmax(R(200.), teq);
    val = -cp_over_time * (cv<R>(M.t3[x]) - teq);
  }
  M.heat3[t] = val;
}

// advection() bookkeeping around hsu_advection, epic_flux.c:377-435:
// phase 0: UNITY = 1 over k = 0..nk+1, j = 0..nj, all i;  phase 1: OLD = THETA for k >= k_sigma-1;
// phase 2: THETA -= OLD*(UNITY-1) for k >= k_sigma-1.
__global__ void k_advection_prep(DevModel M, int phase) {
  if (epic_member(M)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;   // fewer than n3 < 2^31 cells
  const unsigned w = (unsigned)(M.nj + 1) * (unsigned)M.iadim;
  if (t >= w * (unsigned)(M.nk + 2)) return;
  const unsigned q = t / w;
  const int k = (int)q;
  const long long x = M.at(k, 0, 0) + (t - q * w);
  if (phase == 0) M.unity[x] = 1.;
  else if (phase == 3) M.old[x] = M.nu_turb[x];   // NU_TURB, epic_flux.c:569-600
  else if (phase == 4) M.nu_turb[x] = dmaxr(1.e-4 * M.kinvisc, M.nu_turb[x] - M.old[x] * (M.unity[x] - 1.));
  else if (k >= M.k_sigma - 1) {
    if (phase == 1) M.old[x] = M.theta[x];
    else M.theta[x] -= M.old[x] * (M.unity[x] - 1.);
  }
}

// ---- launchers ----

static inline unsigned ncol_blocks(const DevModel &M, int th) { return epic_blocks((long long)(M.nj + 1) * (M.ni + 2), th); }

int launch_source_sink(const DevModel &M, cudaStream_t s) { k_source_sink<<<zg(ncol_blocks(M, TB(M, TB_COLUMN)), M), TB(M, TB_COLUMN), 0, s>>>(M); return 0; }
static inline unsigned ntile_blocks(const DevModel &M) { return epic_blocks((long long)(M.nj + 1) * (M.ni + 2), 32); }
static inline size_t tile_smem(const DevModel &M, int arrays) { return (size_t)arrays * 32 * (M.nk + 1) * sizeof(double); }
int launch_calc_w(const DevModel &M, cudaStream_t s, bool with_source_sink) {
  EPIC_LAUNCH_R(M.mixed, k_calc_w, ntile_blocks(M), CT_THREADS, tile_smem(M, 6), s, M, (int)with_source_sink);
  return 0;
}
int launch_uv_drag(const DevModel &M, cudaStream_t s) {
  const long long n = (long long)(M.nj + 1) * M.ni + (long long)M.nj * M.ni;
  EPIC_LAUNCH_R(M.mixed, k_uv_drag, epic_blocks(n, TB(M, TB_COLUMN)), TB(M, TB_COLUMN), 0, s, M);
  return 0;
}
int launch_hsu_vertical(const DevModel &M, double *buff, int kind, cudaStream_t s) {
  EPIC_LAUNCH_R(M.mixed, k_hsu_vertical, ntile_blocks(M), CT_THREADS,
                (size_t)5 * 32 * (M.nk + 2) * (M.mixed ? sizeof(float) : sizeof(double)), s, M, buff, kind);
  return 0;
}
int launch_akima_vertical(const DevModel &M, double *buff, int kind, cudaStream_t s) {
  EPIC_LAUNCH_R(M.mixed, k_akima_vertical, ntile_blocks(M), CT_THREADS,
                (size_t)4 * 32 * (M.nk + 2) * (M.mixed ? sizeof(float) : sizeof(double)), s, M, buff, kind);
  return 0;
}
int launch_restore_mass(const DevModel &M, cudaStream_t s) {
  k_restore_mass<<<zg(epic_blocks((long long)M.nk * (M.nj + 1) * (M.ni + 2), TB(M, TB_POINT)), M), TB(M, TB_POINT), 0, s>>>(M);
  return 0;
}
int launch_set_p2etc(const DevModel &M, int update_theta, cudaStream_t s, bool early) {
  if (M.col64) k_set_p2etc_acc<<<zg(ntile_blocks(M), M), CT_THREADS, tile_smem(M, 4), s>>>(M, update_theta, !early);
  else if (M.mixed) k_set_p2etc_mixed<<<zg(ntile_blocks(M), M), CT_THREADS, tile_smem(M, 3), s>>>(M, update_theta, !early);
  else k_set_p2etc<<<zg(ntile_blocks(M), M), CT_THREADS, tile_smem(M, 4), s>>>(M, update_theta);
  return 0;
}
// The gas-giant lower boundary of store_pgrad_vars (epic_funcs_diag.c:3779-3811) with gz_from_u
// (:4460-4612): GZ_SURFACE in gradient balance with the zonal means of the bottom layer's U and of
// P3 and RHO3 at K = nk, zero (gz0) at J = jtp.  One block per member, in binary64 in every form
// and in the reference's order: the rows' zonal means (k_gz_means below, RHO3 evaluated as the
// column kernel of store_pgrad_vars evaluates it, which the reference has just stored when it
// takes the means); the absolute vorticity of the zonally symmetric wind (vorticity(ON_SIGMATHETA,
// ABSOLUTE), :4131-4444, v = 0), written into PV3(nk+1) as the reference does (its PV averages
// read it there, and store_diag leaves that level alone); each row's increment of the Bernoulli
// function, (zeta+f) u dy (the Sadourney averages of include/epic_pv_schemes.h:55-61 around the v
// point) plus dp/rho, and its get_kin; then one thread sums the increments from J = jtp.  Every
// row of the reference's arrays is uniform in I, so each row's values are computed once and
// written across it.
//
// The zonal means come first (k_gz_means, one block per row: RHO3 evaluated one thread per cell
// -- the binary64 power is costly on this GPU's FP64 unit -- and each mean summed from shared
// memory by one thread in the reference's order); they wait in the first three columns of
// PV3(nk+1), which k_gz_from_u then rewrites whole.
__global__ void __launch_bounds__(256) k_gz_means(DevModel M) {
  if (epic_member(M)) return;
  extern __shared__ double gm[];
  const int J = (int)blockIdx.x, ni = M.ni, K = M.nk;
  if (J > M.nj) return;   // a member with fewer rows than the launch
  const double *U = M.u + plane_offset(M, PL_UV);
  for (int I = 1 + (int)threadIdx.x; I <= ni; I += (int)blockDim.x) {
    const int x = M.at(K, J, I);
    const double p = M.p3[x];
    gm[I - 1] = U[x];
    gm[ni + I - 1] = p;
    gm[2 * ni + I - 1] = return_density(p, return_temp(M, p, M.theta[x]), M.mu_dry);
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const double *v = gm + threadIdx.x * ni;
    double sum = 0.;
    for (int I = 0; I < ni; I++) sum += v[I];
    M.pv3[(long long)(K + 1) * M.n2 + M.at2(J, (int)threadIdx.x)] = sum / ni;
  }
}

__global__ void __launch_bounds__(256) k_gz_from_u(DevModel M) {
  if (epic_member(M)) return;
  extern __shared__ double gg[];
  const int nj = M.nj, ni = M.ni, K = M.nk, j0 = M.jtp;
  double *u1d = gg, *p1d = u1d + (nj + 1), *rho1d = p1d + (nj + 1), *pvr = rho1d + (nj + 1), *gz = pvr + (nj + 2);
  double *kin = gz + (nj + 1), *pvh = kin + (nj + 1);
  const double *means = M.pv3 + (long long)(K + 1) * M.n2;   // k_gz_means
  for (int J = (int)threadIdx.x; J <= nj; J += (int)blockDim.x) {
    u1d[J] = means[M.at2(J, 0)];
    p1d[J] = means[M.at2(J, 1)];
    rho1d[J] = means[M.at2(J, 2)];
  }
  __syncthreads();
  const double zero = 0.;   // v: the reference's zero array, its operations kept
  for (int J = (int)threadIdx.x; J <= nj + 1; J += (int)blockDim.x) {
    double ze, pv;
    if (J >= 1 && J <= nj) {
      const double m_m1_inv = 1. / M.m[2 * J - 1], m_p1_inv = 1. / M.m[2 * J + 1];
      ze = M.m[2 * J] * ((zero - zero) + M.n[2 * J] * (u1d[J - 1] * m_m1_inv - u1d[J] * m_p1_inv));
      pv = (ze + M.f[2 * J]);
    } else if (J == 0) {   // south pole
      ze = 0.;
      for (int I = 1; I <= ni; I++) ze -= u1d[0];
      ze *= M.mn[0] / ((M.m[1]) * (double)ni);
      pv = ze + M.f[0];
    } else {               // north pole
      ze = 0.;
      for (int I = 1; I <= ni; I++) ze += u1d[nj];
      ze *= M.mn[2 * (nj + 1)] / ((M.m[2 * nj + 1]) * (double)ni);
      pv = ze + M.f[2 * (nj + 1)];
    }
    pvr[J] = pv;
  }
  __syncthreads();
  // get_kin (Sadourney 1975 with the Suarez-Takacs blend, epic_funcs_diag.c:2694-2846) of the
  // zonally symmetric wind at every row, v = 0, and the increments of the Bernoulli function,
  // (zeta+f) u dy plus the pressure term, one row per thread
  for (int J = (int)threadIdx.x; J <= nj; J += (int)blockDim.x) {
    const int jj = 2 * J;
    double u2 = u1d[J], u4 = u1d[J], v2 = zero, v4 = zero;
    const double kin_c = (u2 * u2 + u4 * u4 + M.mn[jj + 1] * (v2 * v2 * M.mn_inv[jj] + v4 * v4 * M.mn_inv[jj + 2])) * .25;
    if (J == 0 || J == nj) {
      kin[J] = kin_c;
    } else {
      u2 = .5 * (u1d[J + 1] + u1d[J - 1]);
      u4 = .5 * (u1d[J + 1] + u1d[J - 1]);
      v2 = .5 * (zero + zero);
      v4 = .5 * (zero + zero);
      const double kin_s = (u2 * u2 + u4 * u4 + M.mn[jj + 1] * (v2 * v2 * M.mn_inv[jj] + v4 * v4 * M.mn_inv[jj + 2])) * .25;
      kin[J] = (5. / 6.) * kin_c + (1. / 6.) * kin_s;
    }
    if (J >= 1) {
      const double udy = u1d[J] / M.n[2 * J + 1], udym = u1d[J - 1] / M.n[2 * J - 1];
      const double al = (pvr[J - 1] + pvr[J] + pvr[J]), be = (pvr[J] + pvr[J] + pvr[J - 1]);
      const double ga = (pvr[J] + pvr[J] + pvr[J + 1]), de = (pvr[J] + pvr[J + 1] + pvr[J]);
      double v = (ga * udy + de * udy + al * udym + be * udym) * (1. / 12.);
      v += (p1d[J] - p1d[J - 1]) * 2. / (rho1d[J] + rho1d[J - 1]);
      pvh[J] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {   // the integral from J = jtp, in the reference's order
    gz[j0] = 0. + kin[j0];
    for (int J = j0 + 1; J <= nj; J++) gz[J] = gz[J - 1] - pvh[J];
    for (int J = j0 - 1; J >= 0; J--) gz[J] = gz[J + 1] + pvh[J + 1];
  }
  __syncthreads();
  for (int J = (int)threadIdx.x; J <= nj; J += (int)blockDim.x) gz[J] = gz[J] - kin[J];
  __syncthreads();
  double *pv3 = M.pv3 + (long long)(K + 1) * M.n2;
  for (int t = (int)threadIdx.x; t < (nj + 2) * (ni + 2); t += (int)blockDim.x) {
    const int J = t / (ni + 2), I = t - J * (ni + 2);
    pv3[M.at2(J, I)] = pvr[J];
    if (J <= nj) M.gz_surface[M.at2(J, I)] = gz[J];
  }
}

int launch_store_pgrad_vars(const DevModel &M, cudaStream_t s, bool early) {
  if (M.gas_giant) {
    k_gz_means<<<zg(M.nj + 1, M), 256, (size_t)3 * M.ni * sizeof(double), s>>>(M);
    k_gz_from_u<<<zg(1, M), 256, (size_t)(7 * M.nj + 8) * sizeof(double), s>>>(M);
  }
  const dim3 grid = zg(ntile_blocks(M), M);
  const size_t smem = tile_smem(M, 5);
  const bool h2 = M.x_h2 != 0.;
  if (M.mixed && early) {   // GZ3 alone: no DZDT3, so no horizontal part either
    if (M.col64) (h2 ? k_gz3_column_acc_h2 : k_gz3_column_acc)<<<grid, CT_THREADS, smem, s>>>(M);
    else (h2 ? k_pgrad_vars_column_mixed<false, true> : k_pgrad_vars_column_mixed<false, false>)<<<grid, CT_THREADS, smem, s>>>(M);
    return 0;
  }
  if (M.col64) (h2 ? k_pgrad_vars_column_acc_h2 : k_pgrad_vars_column_acc)<<<grid, CT_THREADS, smem, s>>>(M);
  else if (M.mixed) (h2 ? k_pgrad_vars_column_mixed<true, true> : k_pgrad_vars_column_mixed<true, false>)<<<grid, CT_THREADS, smem, s>>>(M);
  else k_pgrad_vars_column<<<grid, CT_THREADS, smem, s>>>(M);
  EPIC_LAUNCH_R(M.mixed, k_pgrad_dzdt, epic_blocks((long long)M.nk * (M.nj + 1) * M.ni, TB(M, TB_UPDATE)), TB(M, TB_UPDATE), 0, s, M);
  return 0;
}
int launch_gz_monotone(const DevModel &M, cudaStream_t s) { k_gz_monotone<<<zg(ncol_blocks(M, TB(M, TB_COLUMN)), M), TB(M, TB_COLUMN), 0, s>>>(M); return 0; }
int launch_calc_heating(const DevModel &M, cudaStream_t s) {
  EPIC_LAUNCH_R(M.mixed, k_calc_heating, epic_blocks(M.n3, TB(M, TB_POINT)), TB(M, TB_POINT), 0, s, M);
  return 0;
}
int launch_advection_prep(const DevModel &M, int phase, cudaStream_t s) {
  k_advection_prep<<<zg(epic_blocks((long long)(M.nj + 1) * M.iadim * (M.nk + 2), TB(M, TB_POINT)), M), TB(M, TB_POINT), 0, s>>>(M, phase);
  return 0;
}

// The tile kernels take (arrays x 32 x (nk+1)) doubles of dynamic shared memory: up to 162 KB
// at nk = EPIC_MAX_NK, above the 48 KB default.  The limit is raised once to that maximum, so
// models of different sizes in one process never lower it for one another.
int column_kernels_init(int) {
  const int big = (int)(6 * 32 * (EPIC_MAX_NK + 1) * sizeof(double));
  const int hv = (int)(5 * 32 * (EPIC_MAX_NK + 2) * sizeof(double));
  if (cudaFuncSetAttribute(k_calc_w<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_calc_w<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_set_p2etc, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_pgrad_vars_column, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_set_p2etc_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_pgrad_vars_column_mixed<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_pgrad_vars_column_mixed<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_pgrad_vars_column_mixed<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_pgrad_vars_column_mixed<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(k_hsu_vertical<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, hv) != cudaSuccess ||
      cudaFuncSetAttribute(k_hsu_vertical<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, hv) != cudaSuccess ||
      cudaFuncSetAttribute(k_akima_vertical<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, hv) != cudaSuccess ||
      cudaFuncSetAttribute(k_akima_vertical<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, hv) != cudaSuccess)
    return -1;
  return 0;
}

}  // namespace epic
