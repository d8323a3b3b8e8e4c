// Column (vertical) kernels: one thread per (j,i) column, marching in k.
// Each kernel restates the reference routine named in its comment.
#include "device_common.cuh"
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
__global__ void k_calc_w(DevModel M) {
  int j, i;
  if (!col_index(M, j, i)) return;
  const int nk = M.nk, ks = M.k_sigma;
  const double ptop = M.p3[M.at(0, j, i)], pbot = M.p3[M.at(nk, j, i)];
  const double psigma = M.p3[M.at(ks - 1, j, i)];
  M.w3[M.at(0, j, i)] = 0.;
  M.w3[M.at(nk, j, i)] = 0.;
  double sum_div = 0.;   // SUM_DIV(k) for the current k
  for (int k = 1; k < nk; k++) {
    const long long x = M.at(k, j, i);
    double w;
    if (k < ks - 1) {
      const double sigma = get_sigma(M, pbot, M.p3[x], ptop);
      w = g_sigma(M, sigma) * M.heat3[x] / M.exner3[x];
    } else {
      w = 0.;
    }
    if (k >= 2) {
      const double P0 = M.p3[M.at(k - 2, j, i)], P1 = M.p3[M.at(k - 1, j, i)], P2 = M.p3[x], P3 = M.p3[M.at(k + 1, j, i)];
      const double dz10 = xlog(M, P1 / P0), dz21 = xlog(M, P2 / P1), dz32 = xlog(M, P3 / P2);
      const double dz20 = dz21 + dz10, dz30 = dz32 + dz20, dz31 = dz32 + dz21;
      const double df0 = P0 * M.div_uv3[M.at(k - 2, j, i)];
      const double df1 = P1 * M.div_uv3[M.at(k - 1, j, i)];
      const double df2 = P2 * M.div_uv3[x];
      const double df3 = P3 * M.div_uv3[M.at(k + 1, j, i)];
      const double dsumdiv = -(df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                               df1 * (dz21 * (dz21 * (dz21 + 2. * (dz10 - dz31)) - 6. * dz10 * dz31)) / (dz10 * dz31) +
                               df2 * (dz21 * (dz21 * (dz21 + 2. * (dz32 - dz20)) - 6. * dz20 * dz32)) / (dz20 * dz32) +
                               df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32)) /
                             12.;
      sum_div = sum_div + dsumdiv;
    }
    // dF/dp by a centred difference of return_sigmatheta at fixed theta and pbot
    const double theta3 = M.theta[x], p3 = M.p3[x];
    const double dp = p3 * M.eps13;
    double p2 = dmaxr(p3 - dp * .5, ptop);
    const double p4 = dminr(p3 + dp * .5, pbot);
    if (p2 < psigma && p4 >= psigma) p2 = p3;
    if (!(p2 < p4)) flag_error(M.ctl, ERR_CALC_W_P, k, j, i, p2);
    const double dFdp = (return_sigmatheta(M, theta3, p2, pbot, ptop) - return_sigmatheta(M, theta3, p4, pbot, ptop)) / (p2 - p4);
    // SUM_DIV(nk) = 0, so the dF/dpbot term contributes nothing.
    M.w3[x] = w - (sum_div * dFdp + 0.);
  }
}

// Held-Suarez boundary-layer drag and the top sponge of uv_drag, epic_timestep.c:1303-1509.
// Columns on the u grid (j = 0..nj) and v grid (j = 1..nj), i = 1..ni.
__global__ void k_uv_drag(DevModel M) {
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
    D[x] -= (M.t_sponge_inv[k]) * (W[x] - (isv ? 0. : M.u_spinup[x]));
  }
  if (M.rayleigh_on) {
    // The zonal-mean Rayleigh drag block is not part of the supported configurations
    // (held_suarez sets prandtl = 0 and tau_drag = 1e20); epic_model_create rejects it.
  }
  const double pbot = 0.5 * (M.p3[M.at(nk, j, i)] + M.p3[M.at(nk, jm, im)]);
  for (int k = nk - 1; k >= 1; k--) {
    const double p3 = .5 * (M.p3[M.at(k, j, i)] + M.p3[M.at(k, jm, im)]);
    const double amp = (p3 / pbot - 0.7) / (1. - 0.7);
    if (amp < 0.) break;
    const double nu0 = M.hs_kf * amp;
    const long long x = M.at(k, j, i);
    D[x] -= nu0 * W[x];
  }
}

// Vertical pass of hsu_advection, epic_flux.c:717-1052.  kind: 0 = unity (P3_INDEX),
// 1 = THETA, 2 = HDRY.  One thread per column j = 0..nj, i = 0..ni+1.
__global__ void k_hsu_vertical(DevModel M, double *buff, int kind) {
  int j, i;
  if (!col_index(M, j, i)) return;
  const int nk = M.nk;
  const bool layer = kind == 2;
  const int kf = kind == 1 ? M.k_sigma - 1 : 1;
  const double ep = 1.e-10, DT = M.dt;
  double wm[EPIC_MAX_NK + 2], wp[EPIC_MAX_NK + 2], wa[EPIC_MAX_NK + 2], pred[EPIC_MAX_NK + 2];
  double ff[EPIC_MAX_NK + 2], d1[EPIC_MAX_NK + 2], d2[EPIC_MAX_NK + 2], aa[EPIC_MAX_NK + 2];
  auto amin = [&](int k) { return layer ? M.h_min[k] : 0.; };
  for (int k = layer ? kf : kf - 1; k <= nk; k++) wa[k] = buff[M.at(k, j, i)];
  if (layer) {
    for (int k = kf - 1; k <= nk; k++) {
      const double w = M.w3[M.at(k, j, i)];
      wm[k] = dminr(0., w);
      wp[k] = dmaxr(0., w);
    }
    ff[kf - 1] = 0.;
    ff[nk] = 0.;
    for (int k = kf; k < nk; k++) ff[k] = wp[k] * wa[k + 1] + wm[k] * wa[k];
    for (int k = kf; k <= nk; k++) pred[k] = wa[k] + (ff[k] - ff[k - 1]) * M.dsgth_inv[2 * k] * DT;
    for (int k = kf; k < nk; k++) ff[k] = .5 * (wp[k] * (pred[k] + wa[k + 1]) + wm[k] * (pred[k + 1] + wa[k]));
    for (int k = kf; k <= nk; k++) {
      double tmp;
      if (k == 1) { d1[k] = pred[k] - wa[k + 1]; d2[k] = 0.; tmp = fabs(wa[k + 1] - wa[k]) + ep; }
      else if (k == nk) { d1[k] = 0.; d2[k] = pred[k] - wa[k - 1]; tmp = fabs(-wa[k] + wa[k - 1]) + ep; }
      else { d1[k] = pred[k] - wa[k + 1]; d2[k] = pred[k] - wa[k - 1]; tmp = fabs(wa[k + 1] - 2. * wa[k] + wa[k - 1]) + ep; }
      aa[k] = tmp * tmp;
    }
    for (int k = kf; k < nk; k++) {
      const double whatp = sqrt(wp[k] * wp[k + 1]);
      const double whatm = -sqrt(wm[k] * wm[k - 1]);
      const double mu = (wp[k] - wm[k]) * M.dsgth_inv[2 * k + 1] * DT;
      const double al = (1. + mu) / 6.;
      const double prod = (wa[k + 1] - amin(k + 1)) * (wa[k] - amin(k));
      double gap = aa[k + 1] / (aa[k + 1] + prod); gap = gap * gap;
      double gam = aa[k] / (aa[k] + prod); gam = gam * gam;
      const double bep = 1. + (1. / (2. * al) - 1.) * gap;
      const double bem = 1. + (1. / (2. * al) - 1.) * gam;
      ff[k] += -al * (wp[k] * bep * d1[k] - whatp * (1. - gap) * d1[k + 1] + wm[k] * bem * d2[k + 1] - whatm * (1. - gam) * d2[k]);
    }
    for (int k = kf; k <= nk; k++) buff[M.at(k, j, i)] += (ff[k] - ff[k - 1]) * M.dsgth_inv[2 * k] * DT;
  } else {
    for (int k = kf; k <= nk; k++) {
      const double w = (k == 1 || k == nk) ? 0. : .5 * (M.w3[M.at(k, j, i)] + M.w3[M.at(k - 1, j, i)]);
      wm[k] = dminr(0., w);
      wp[k] = dmaxr(0., w);
    }
    for (int k = kf; k <= nk; k++) ff[k] = wp[k] * wa[k] + wm[k] * wa[k - 1];
    ff[nk + 1] = 0.;
    pred[kf - 1] = wa[kf - 1];
    for (int k = kf; k <= nk; k++) pred[k] = wa[k] + (ff[k + 1] - ff[k]) * M.dsgth_inv[2 * k + 1] * DT;
    for (int k = kf; k <= nk; k++) ff[k] = .5 * (wp[k] * (pred[k - 1] + wa[k]) + wm[k] * (pred[k] + wa[k - 1]));
    for (int k = kf - 1; k <= nk; k++) {
      // For THETA (kf > 1) the entry below the first loaded one is the value the reference's
      // static column buffer keeps from the preceding unity advection: 1.0 (epic_flux.c:866-877).
      const double wkm1 = k >= 1 ? (k - 1 < kf - 1 ? 1.0 : wa[k - 1]) : 0.;
      double tmp;
      if (k == 0) tmp = fabs(wa[k + 1] - wa[k]) + ep;
      else if (k == nk) tmp = fabs(-wa[k] + wkm1) + ep;
      else tmp = fabs(wa[k + 1] - 2. * wa[k] + wkm1) + ep;
      aa[k] = tmp * tmp;
    }
    d2[kf - 1] = 0.;
    for (int k = kf; k <= nk; k++) {
      d1[k] = pred[k - 1] - wa[k];
      d2[k] = pred[k] - wa[k - 1];
    }
    for (int k = kf; k <= nk; k++) {
      const double whatm = (k == 1 || k - 1 < kf) ? 0. : -sqrt(wm[k] * wm[k - 1]);
      const double whatp = (k == nk) ? 0. : sqrt(wp[k] * wp[k + 1]);
      const double mu = (wp[k] - wm[k]) * M.dsgth_inv[2 * k] * DT;
      const double al = (1. + mu) / 6.;
      const double prod = (wa[k] - amin(k)) * (wa[k - 1] - amin(k - 1));
      double gap = aa[k] / (aa[k] + prod); gap = gap * gap;
      double gam = aa[k - 1] / (aa[k - 1] + prod); gam = gam * gam;
      const double bep = 1. + (1. / (2. * al) - 1.) * gap;
      const double bem = 1. + (1. / (2. * al) - 1.) * gam;
      double g;
      if (k < nk) g = -al * (wp[k] * bep * d1[k] - whatp * (1. - gap) * d1[k + 1] + wm[k] * bem * d2[k] - whatm * (1. - gam) * d2[k - 1]);
      else g = -al * (wp[k] * bep * d1[k] + wm[k] * bem * d2[k] - whatm * (1. - gam) * d2[k - 1]);
      ff[k] += g;
    }
    ff[nk + 1] = 0.;
    for (int k = kf; k <= nk; k++) buff[M.at(k, j, i)] += (ff[k + 1] - ff[k]) * M.dsgth_inv[2 * k + 1] * DT;
  }
}

// restore_mass(HDRY_INDEX), epic_adjust.c:45-96
__global__ void k_restore_mass(DevModel M) {
  int j, i;
  if (!col_index(M, j, i)) return;
  for (int k = 1; k <= M.nk; k++) {
    const long long x = M.at(k, j, i);
    M.hdry[x] = dmaxr(M.h_min[k], M.hdry[x]);
  }
}

// set_p2etc, epic_funcs_diag.c:3352-3569 (nq = 0: H2 is HDRY, PDRY3 is P3, HDRY3 is H3)
__global__ void k_set_p2etc(DevModel M, int update_theta) {
  int j, i;
  if (!col_index(M, j, i)) return;
  const int nk = M.nk, ks = M.k_sigma;
  const double g = M.grav[2 * j + 1];
  double p[EPIC_MAX_NK + 2];
  p[0] = M.p3[M.at(0, j, i)];
  for (int k = 1; k <= nk; k++) p[k] = p[k - 1] + M.dsgth[2 * k] * g * M.hdry[M.at(k, j, i)];
  const double ptop = p[0], pbot = p[nk];
  for (int k = ks - 1; k < nk; k++) {
    const double sigma = (M.sgth[2 * k + 1] - M.zeta0) / (M.zeta1 - M.zeta0);
    p[k] = get_p_sigma(M, pbot, sigma, ptop);
  }
  double hl[EPIC_MAX_NK + 2];   // get_h at the layers, from the final P3
  for (int k = 1; k <= nk; k++) {
    M.p3[M.at(k, j, i)] = p[k];
    hl[k] = (p[k] - p[k - 1]) / (g * M.dsgth[2 * k]);
    M.hdry[M.at(k, j, i)] = dmaxr(M.h_min[k], hl[k]);
  }
  double th[EPIC_MAX_NK + 2];
  for (int k = 0; k <= nk; k++) th[k] = M.theta[M.at(k, j, i)];
  if (update_theta) {
    for (int k = 0; k < ks - 1; k++) {
      const double sigma = get_sigma(M, pbot, p[k], ptop);
      th[k] = (M.sgth[2 * k + 1] - f_sigma(M, sigma)) / g_sigma(M, sigma);
      M.theta[M.at(k, j, i)] = th[k];
    }
  }
  double p2[EPIC_MAX_NK + 2];
  for (int k = 1; k <= nk; k++) {
    p2[k] = layer_p(M, p[k - 1], p[k]);
    M.p2[M.at(k, j, i)] = p2[k];
  }
  M.p2[M.at(0, j, i)] = p[0] * p[0] / p2[1];
  for (int k = 1; k <= nk; k++) {
    double h;
    if (k == nk) h = hl[nk];
    else {
      const double topwt = M.dsgth[2 * k], botwt = M.dsgth[2 * k + 2];
      h = (topwt * hl[k] + botwt * hl[k + 1]) / (topwt + botwt);
    }
    M.h3[M.at(k, j, i)] = h;
    if (k == 1) M.h3[M.at(0, j, i)] = h;
  }
  if (update_theta) {
    for (int k = 1; k < ks - 1; k++) {
      const double sigma = get_sigma(M, pbot, p2[k], ptop);
      M.theta2[M.at(k, j, i)] = (M.sgth[2 * k] - f_sigma(M, sigma)) / g_sigma(M, sigma);
    }
    M.theta2[M.at(ks - 1, j, i)] = .5 * (th[ks - 1] + th[ks - 2]);
    // linint on the table (sigmatheta[2K+1], THETA(K)), K = nk down to k_sigma-1
    const int nkay = nk - (ks - 1) + 1;
    for (int k = ks; k <= nk; k++) {
      const double sg = M.sgth[2 * k];
      // find_place_in_table on ascending x = sigmatheta[2(nk-kay)+1]
      auto X = [&](int kay) { return M.sgth[2 * (nk - kay) + 1]; };
      auto Y = [&](int kay) { return th[nk - kay]; };
      int kay;
      if (fcmp(sg, X(0)) <= 0) kay = 0;
      else if (fcmp(sg, X(nkay - 1)) >= 0) kay = nkay - 2;
      else {
        int il = -1, iu = nkay;
        while (iu - il > 1) {
          const int im = (iu + il) >> 1;
          if (fcmp(sg, X(im)) >= 0) il = im; else iu = im;
        }
        kay = il;
      }
      const double dx = X(kay + 1) - X(kay);
      M.theta2[M.at(k, j, i)] = Y(kay) + (Y(kay + 1) - Y(kay)) * (sg - X(kay)) / dx;
    }
  }
}

// store_pgrad_vars, column part (epic_funcs_diag.c:3595-3895): T3, EXNER3, RHO3, T2, RHO2,
// the k = 0 extrapolations, GZ3 and MONT3 from the surface up, the monotone-GZ check, and
// the first DZDT3 terms.
__global__ void k_pgrad_vars_column(DevModel M) {
  int j, i;
  if (!col_index(M, j, i)) return;
  const int nk = M.nk;
  const double mu = M.mu_dry;
  const long long itime = M.ctl->itime;
  double p[EPIC_MAX_NK + 2], rho[EPIC_MAX_NK + 2], t3[EPIC_MAX_NK + 2];
  for (int k = 0; k <= nk; k++) {
    const long long x = M.at(k, j, i);
    const double theta = M.theta[x];
    p[k] = M.p3[x];
    t3[k] = return_temp(M, p[k], theta);
    M.t3[x] = t3[k];
    M.exner3[x] = M.cp * t3[k] / theta;
    rho[k] = return_density(p[k], t3[k], mu);
    M.rho3[x] = rho[k];
  }
  double rho2_1 = 0.;
  for (int k = 1; k <= nk; k++) {
    const long long x = M.at(k, j, i);
    const double pr = M.p2[x];
    const double t2 = return_temp(M, pr, M.theta2[x]);
    M.t2[x] = t2;
    const double r2 = return_density(pr, t2, mu);
    M.rho2[x] = r2;
    if (k == 1) rho2_1 = r2;
  }
  {
    const long long x = M.at(0, j, i);
    M.rho2[x] = rho[0] * rho[0] / rho2_1;
    M.theta2[x] = M.sgth[0];
    M.t2[x] = t3[0];
  }
  double gz[EPIC_MAX_NK + 2];
  gz[nk] = M.topo_scale * M.gz_surface[M.at2(j, i)];
  gz[nk - 1] = gz[nk] + ((p[nk] + p[nk - 1]) / (rho[nk] + rho[nk - 1])) * xlog(M, p[nk] / p[nk - 1]);
  for (int k = nk - 1; k >= 2; k--) {
    const double dz10 = xlog(M, p[k + 1] / p[k]), dz21 = xlog(M, p[k] / p[k - 1]), dz32 = xlog(M, p[k - 1] / p[k - 2]);
    const double dz20 = dz21 + dz10, dz30 = dz32 + dz20, dz31 = dz32 + dz21;
    const double df0 = p[k + 1] / rho[k + 1], df1 = p[k] / rho[k], df2 = p[k - 1] / rho[k - 1], df3 = p[k - 2] / rho[k - 2];
    const double dgz = -(df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                         df1 * (dz21 * (dz21 * (dz21 + 2. * (dz10 - dz31)) - 6. * dz10 * dz31)) / (dz10 * dz31) +
                         df2 * (dz21 * (dz21 * (dz21 + 2. * (dz32 - dz20)) - 6. * dz20 * dz32)) / (dz20 * dz32) +
                         df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32)) /
                       12.;
    gz[k - 1] = gz[k] + dgz;
  }
  gz[0] = gz[1] + ((p[1] + p[0]) / (rho[1] + rho[0])) * xlog(M, p[1] / p[0]);
  const bool interior = i >= 1 && i <= M.ni;
  for (int k = 0; k <= nk; k++) {
    const long long x = M.at(k, j, i);
    const double old = M.gz3[x];
    M.gz3[x] = gz[k];
    M.mont3[x] = gz[k] + return_enthalpy(M, t3[k]);
    if (interior && k >= 1) {
      // DZDT3 = -(GZ3_new - GZ3_old)/(dt*g) from the third step on, 0 before (:3679-3693, :3897-3909)
      double dz = 0.;
      if (itime > 1) {
        const double dtg_inv = -1. / (M.dt * M.grav[2 * j + 1]);
        dz = (old - gz[k]) * dtg_inv;
      }
      dz += M.w3[x] * M.h3[x] / M.rho3[x];
      M.dzdt3[x] = dz;
      if (gz[k] >= gz[k - 1]) flag_error(M.ctl, ERR_GZ_MONOTONE, k, j, i, gz[k]);
    }
  }
}

// store_pgrad_vars, horizontal part of DZDT3 (epic_funcs_diag.c:3924-3945) plus bc_lateral.
__global__ void k_pgrad_dzdt(DevModel M) {
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int ni = M.ni, nk = M.nk;
  if (t >= nk * (M.nj + 1) * ni) return;
  const int i = 1 + t % ni;
  const int j = (t / ni) % (M.nj + 1);
  const int k = 1 + t / (ni * (M.nj + 1));
  const int jj = 2 * j;
  const Ctl *c = M.ctl;
  const double *U = M.u + (long long)c->it_uv * M.n3, *V = M.v + (long long)c->it_uv * M.n3;
  const double gdx_inv3 = .5 * M.m[jj + 1] / M.grav[jj + 1];
  const double gdy_inv2 = .5 * M.n[jj] / M.grav[jj];
  const double gdy_inv4 = .5 * M.n[jj + 2] / M.grav[jj + 2];
  const double *G = M.gz3;
  const long long x = M.at(k, j, i);
  const double add = V[x] * (G[x] - G[M.at(k, j - 1, i)]) * gdy_inv2 + V[M.at(k, j + 1, i)] * (G[M.at(k, j + 1, i)] - G[x]) * gdy_inv4 +
                     U[x] * (G[x] - G[M.at(k, j, i - 1)]) * gdx_inv3 + U[M.at(k, j, i + 1)] * (G[M.at(k, j, i + 1)] - G[x]) * gdx_inv3;
  write_with_pads(M.dzdt3, M, M.at(k, j, 0), i, M.dzdt3[x] + add);
}

// Monotone fix of the filtered GZ copy, epic_timestep.c:182-195 (the zonal filter of planes
// 0..nk-1 has already run; each plane's fix only needs the finished plane below it).
__global__ void k_gz_monotone(DevModel M) {
  int j, i;
  if (!col_index(M, j, i)) return;
  double below = M.gz[M.at(M.nk, j, i)];
  for (int k = M.nk - 1; k >= 0; k--) {
    const long long x = M.at(k, j, i);
    double g;
    if (fcmp(below, 0.) == 0) g = 1.e-3;
    else g = dmaxr(M.gz[x], below + fabs(below) * 1.e-5);
    M.gz[x] = g;
    below = g;
  }
}

// calc_heating -> newtonian_cooling for held_suarez (epic_funcs_diag.c:4793-4869,
// epic_sensible_heating.c:51-180, t_rad :217-314, temp_eq :325-463).  Writes every HEAT3 cell:
// 0 outside k = 1..nk, j = 0..nj, i = 1..ni, with periodic pads.
__global__ void k_calc_heating(DevModel M) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.n3) return;
  const int i = (int)(t % M.iadim);
  const int j = (int)((t / M.iadim) % M.jadim) - 1;
  const int k = (int)(t / M.n2);
  double val = 0.;
  int ii = i == 0 ? M.ni : (i == M.ni + 1 ? 1 : i);
  if (k >= 1 && k <= M.nk && j >= 0 && j <= M.nj && M.newt_cool_on) {
    const long long x = M.at(k, j, ii);
    const double ka = 1. / (40. * 60. * 60. * 24.), ks = 1. / (4. * 60. * 60. * 24.);
    const double pressure = M.p3[x];
    const double pbot = M.p3[M.at(M.nk, j, ii)];
    const double amp = (pressure / pbot - 0.7) / (1. - 0.7);
    double kt = ka;
    if (amp > 0.) kt += (ks - ka) * xpow(M, M.coslat[j], 4.) * amp;
    const double cp_over_time = 1004. / (1. / kt);
    double c2 = M.coslat[j];
    c2 *= c2;
    const double s2 = 1. - c2;
    const double p_p0 = pressure / (1000. * 100.);
    double teq = (315. - 60. * s2 - 10. * xlog(M, p_p0) * c2) * xpow(M, p_p0, M.kappa);
    teq = dmaxr(200., teq);
    val = -cp_over_time * (M.t3[x] - teq);
  }
  M.heat3[t] = val;
}

// advection() bookkeeping around hsu_advection, epic_flux.c:377-435:
// phase 0: UNITY = 1 over k = 0..nk+1, j = 0..nj, all i;  phase 1: OLD = THETA for k >= k_sigma-1;
// phase 2: THETA -= OLD*(UNITY-1) for k >= k_sigma-1.
__global__ void k_advection_prep(DevModel M, int phase) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long w = (long long)(M.nj + 1) * M.iadim;
  if (t >= w * (M.nk + 2)) return;
  const int k = (int)(t / w);
  const long long x = M.at(k, 0, 0) + t % w;
  if (phase == 0) M.unity[x] = 1.;
  else if (k >= M.k_sigma - 1) {
    if (phase == 1) M.old[x] = M.theta[x];
    else M.theta[x] -= M.old[x] * (M.unity[x] - 1.);
  }
}

// ---- launchers ----

static inline unsigned ncol_blocks(const DevModel &M, int th) { return epic_blocks((long long)(M.nj + 1) * (M.ni + 2), th); }

int launch_source_sink(const DevModel &M, cudaStream_t s) { k_source_sink<<<ncol_blocks(M, 128), 128, 0, s>>>(M); return 0; }
int launch_calc_w(const DevModel &M, cudaStream_t s) { k_calc_w<<<ncol_blocks(M, 128), 128, 0, s>>>(M); return 0; }
int launch_uv_drag(const DevModel &M, cudaStream_t s) {
  const long long n = (long long)(M.nj + 1) * M.ni + (long long)M.nj * M.ni;
  k_uv_drag<<<epic_blocks(n, 128), 128, 0, s>>>(M);
  return 0;
}
int launch_hsu_vertical(const DevModel &M, double *buff, int kind, cudaStream_t s) {
  k_hsu_vertical<<<ncol_blocks(M, 64), 64, 0, s>>>(M, buff, kind);
  return 0;
}
int launch_restore_mass(const DevModel &M, cudaStream_t s) { k_restore_mass<<<ncol_blocks(M, 128), 128, 0, s>>>(M); return 0; }
int launch_set_p2etc(const DevModel &M, int update_theta, cudaStream_t s) {
  k_set_p2etc<<<ncol_blocks(M, 64), 64, 0, s>>>(M, update_theta);
  return 0;
}
int launch_store_pgrad_vars(const DevModel &M, cudaStream_t s) {
  k_pgrad_vars_column<<<ncol_blocks(M, 64), 64, 0, s>>>(M);
  k_pgrad_dzdt<<<epic_blocks((long long)M.nk * (M.nj + 1) * M.ni, 128), 128, 0, s>>>(M);
  return 0;
}
int launch_gz_monotone(const DevModel &M, cudaStream_t s) { k_gz_monotone<<<ncol_blocks(M, 128), 128, 0, s>>>(M); return 0; }
int launch_calc_heating(const DevModel &M, cudaStream_t s) { k_calc_heating<<<epic_blocks(M.n3, 128), 128, 0, s>>>(M); return 0; }
int launch_advection_prep(const DevModel &M, int phase, cudaStream_t s) {
  k_advection_prep<<<epic_blocks((long long)(M.nj + 1) * M.iadim * (M.nk + 2), 128), 128, 0, s>>>(M, phase);
  return 0;
}

}  // namespace epic
