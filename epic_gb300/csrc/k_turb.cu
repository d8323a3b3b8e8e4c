// The Spalart-Allmaras DES turbulence closure of the FP64 form: source_sink_turb, the horizontal
// and vertical subgrid diffusion of THETA, NU_TURB and the winds, and set_diffusion_coef
// (src/shared/epic_subgrid.c), with crank_nicolson's banded solve (src/shared/epic_funcs_util.c).
// Every expression is the reference's, in its order, in binary64 with the correctly rounded
// log/exp/pow/atan/cos of dd_math.cuh, so each kernel's output equals the CPU restatement's bit
// for bit.  The parallel decomposition is this file's own:
//   - source_sink_SA updates NU_TURB in place in K, J, I order (each point reads the new values of
//     its K-1, J-1 and I-1 neighbours, the old ones of K+1, J+1, I+1).  Its NU_TURB-free part
//     (strain, wall distance, Brunt-Vaisala frequency) is one pointwise pass; the rest runs as
//     wavefronts K + J + I = d, one launch each, every point of a front independent of the others;
//   - the Laplacians of laplacian_h are three pointwise passes around the row filter, all layers
//     at once (each layer's Laplacian reads only its own plane);
//   - the implicit vertical diffusions are one thread per column (crank_nicolson and the band
//     solver with partial pivoting in registers and local memory);
//   - uv_horizontal_diffusion's stresses are recomputed where the wind updates read them.
#include "device_common.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

namespace {

constexpr double SA_CV1_3 = 7.1 * 7.1 * 7.1;   // cv1^3, epic_subgrid.c:2186-2187
constexpr int TN = EPIC_TURB_MAX_NK + 4;        // crank_nicolson's column arrays (n + 2 <= nk + 3)
enum { WALL_U, WALL_V, WALL_H };               // law_of_the_wall's grids: U_INDEX, V_INDEX, the h-grid

__device__ __forceinline__ double nu_floor(const DevModel &M) { return 1.e-4 * M.kinvisc; }

// D_WALL as dwall_SA sets it before each use (:2716-2770): the height above the surface, or
// FLOAT_MAX on a gas giant
__device__ __forceinline__ double d_wall(const DevModel &M, int k, int j, int i) {
  if (M.gas_giant) return DBL_MAX;
  return (M.gz3[M.at(k, j, i)] - M.topo_scale * M.gz_surface[M.at2(j, i)]) / M.grav[2 * j + 1];
}

__device__ __forceinline__ double limit_range(double lo, double x, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

// func_utau, :3112-3165
__device__ double func_utau(const DevModel &M, double u_tau, double u_tan, double dwall, int j, int i) {
  const double C = 5., const1 = 0.127, const2 = 1. / .41, const3 = 0.41 * 1.43e-3, one_third = 1. / 3., pi_six = M_PI / 6.;
  const double sqrt_one_third = sqrt(1. / 3.);
  const MathTable &T = *M.lt;
  double u_plus = 0.;
  if (u_tau != 0.) u_plus = u_tan / u_tau;
  else flag_error(M.ctl, ERR_TURB, -1, j, i, u_tau);
  const double y_plus = fabs(u_tau * dwall / M.kinvisc);
  if (u_plus < 0.1) return 1.e+20;
  if (y_plus < 5.) return y_plus - u_plus;
  if (y_plus < 70.) {
    const double yy = const1 * y_plus;
    return (one_third * cr_log((1. + yy) / (sqrt(yy * (yy - 1.) + 1.)), T) +
            sqrt_one_third * (cr_atan(sqrt_one_third * (2. * yy - 1.), T) + pi_six)) / const1 +
           .25 * const2 * cr_log(1. + const3 * cr_pow(y_plus, 4., T), T) - u_plus;
  }
  return const2 * cr_log(y_plus, T) + C - u_plus;
}

// law_of_the_wall, :2995-3105: secant iterations on the wall law for the friction velocity
// (the reference scales its t_vis argument by fv1 and leaves it unused)
__device__ double law_of_the_wall(const DevModel &M, int k, int j, int i, int index, double u_tan) {
  const double kinvisc = M.kinvisc, tol = 1.e-6;
  if (M.gas_giant) return 1.0e-4 * kinvisc;
  double dwall;
  if (index == WALL_U) dwall = 0.5 * (d_wall(M, k, j, i) + d_wall(M, k, j, i - 1));
  else if (index == WALL_V) dwall = 0.5 * M.m[2 * j] * (d_wall(M, k, j, i) / M.m[2 * j + 1] + d_wall(M, k, j - 1, i) / M.m[2 * j - 1]);
  else dwall = d_wall(M, k, j, i);
  if (dwall * u_tan < 0.00023) return 0.01 * kinvisc;
  double dwall_inv = 0.;
  if (dwall > 0.) dwall_inv = 1. / dwall;
  else flag_error(M.ctl, ERR_TURB, k, j, i, dwall);
  const double x1 = sqrt(kinvisc * (1. + 0.01) * u_tan * dwall_inv);
  const double x2 = sqrt(kinvisc * (1. + 20.) * u_tan * dwall_inv);
  double fl = func_utau(M, x1, u_tan, dwall, j, i), f = func_utau(M, x2, u_tan, dwall, j, i), rts, xl;
  if (fabs(fl) < fabs(f)) {
    rts = x1; xl = x2;
    const double sw = fl; fl = f; f = sw;
  } else {
    xl = x1; rts = x2;
  }
  double u_tau = 0.;
  int iter;
  for (iter = 0; iter < 30; iter++) {
    const double dx = (xl - rts) * f / (f - fl);
    xl = rts;
    fl = f;
    rts += dx;
    f = func_utau(M, rts, u_tan, dwall, j, i);
    if (f > .99e+20) return 0.01 * kinvisc;
    if (fabs(dx) < tol || f == 0.0) {
      u_tau = rts;
      break;
    }
  }
  if (iter < 30) return dmaxr((u_tau * u_tau * dwall / u_tan) - kinvisc, 0.01 * kinvisc);
  return 20. * kinvisc;
}

// invert_fv1, :3172-3226
__device__ double invert_fv1(const DevModel &M, double t_vis, int j, int i) {
  const double pi_factor = M_PI * 0.5 / 30.0;
  if (t_vis < 0.) flag_error(M.ctl, ERR_TURB, -1, j, i, t_vis);
  const double chi = t_vis / M.kinvisc;
  if (chi > 30) return t_vis;
  if (chi < 0.4) return M.kinvisc * cr_pow(chi * SA_CV1_3, .25, *M.lt);
  double fv1 = cr_cos(pi_factor * cr_pow(chi, 0.35, *M.lt), *M.lt);
  fv1 = 1.0 - fv1 * fv1;
  return M.kinvisc * chi / fv1;
}

// get_kin at h-point (j, i) of layer k of the wind time plane `sel`; i = 0 is the pad (bc_lateral)
__device__ __forceinline__ double kin_plane(const DevModel &M, int sel, int k, int j, int i) {
  if (i == 0) i = M.ni;
  const long long off = plane_offset(M, sel) + (long long)k * M.n2;
  return kin_at<double>(M, M.u + off, M.v + off, j, i);
}

// The wall stress of tau_surface (:2819-2988) under the wind component `index` at (j, i), from
// layer K = nk-1 and the winds of plane it_uv
__device__ double tau_wall(const DevModel &M, int index, int j, int i) {
  if (M.gas_giant) return 0.;
  const int k = M.nk - 1;
  const double *U = M.u + plane_offset(M, PL_UV), *V = M.v + plane_offset(M, PL_UV);
  auto rho3 = [&](int jj, int ii) { return M.rho3[M.at(k, jj, ii)]; };
  auto gz = [&](int kk, int jj, int ii) { return M.gz3[M.at(kk, jj, ii)]; };
  if (index == WALL_U) {
    const double rho = .5 * (rho3(j, i) + rho3(j, i - 1));
    const double dz = .5 * (gz(k, j, i) + gz(k, j, i - 1) - gz(k + 1, j, i) - gz(k + 1, j, i - 1)) / M.grav[2 * j + 1];
    const double kin = .5 * (kin_plane(M, PL_UV, k, j, i) + kin_plane(M, PL_UV, k, j, i - 1));
    const double u_tan = sqrt(2. * kin);
    const double dc = law_of_the_wall(M, k, j, i, WALL_U, u_tan);
    return (M.dynvisc + rho * dc) * (U[M.at(k, j, i)] - 0.) / dz;
  }
  if (index == WALL_V) {
    const double rho = .5 * (rho3(j, i) + rho3(j - 1, i));
    const double dz = .5 * (gz(k, j, i) + gz(k, j - 1, i) - gz(k + 1, j, i) - gz(k + 1, j - 1, i)) / M.grav[2 * j];
    const double kin = .5 * (kin_plane(M, PL_UV, k, j, i) + kin_plane(M, PL_UV, k, j - 1, i));
    const double u_tan = sqrt(2. * kin);
    const double dc = law_of_the_wall(M, k, j, i, WALL_V, u_tan);
    return (M.dynvisc + rho * dc) * (V[M.at(k, j, i)] - 0.) / dz;
  }
  const double rho = rho3(j, i);
  const double dz = (gz(k, j, i) - gz(k + 1, j, i)) / M.grav[2 * j + 1];
  const double kin = kin_plane(M, PL_UV, k, j, i);
  const double u_tan = sqrt(2. * kin);
  const double dc = law_of_the_wall(M, k, j, i, WALL_H, u_tan);
  const double nu = invert_fv1(M, dc, j, i);
  return (M.dynvisc + rho * nu) * (u_tan - 0.) / dz;
}

// stability_factor (:2309-2415) of column (j, i) at the layers, sf[K] = stab_factor[2K], K = 0..nk
// (the only entries the diffusions read).  The slope limiter runs over kk = 1..2nk in order, each
// step reading the entry the one before may have zeroed.
__device__ void stability_layers(const DevModel &M, int j, int i, double *sf) {
  const int nk = M.nk;
  if (!M.stab) {
    for (int k = 0; k <= nk; k++) sf[k] = 1.;
    return;
  }
  const double max_ri = 100.;
  auto ri2 = [&](int k) { return M.ri2[M.at(k, j, i)]; };
  auto raw = [&](int kk) -> double {   // Ri[kk] before the limiter
    if (kk == 1) return limit_range(-max_ri, ri2(1), max_ri);
    if (kk == 2 * nk + 1) return limit_range(-max_ri, ri2(nk), max_ri);
    const int k = kk / 2;
    if ((kk & 1) == 0) return limit_range(-max_ri, ri2(k), max_ri);
    return limit_range(-max_ri, .5 * (ri2(k) + ri2(k + 1)), max_ri);
  };
  auto factor = [&](double r) { return r > 0. ? 1. / (1. + 10. * r * (1. + 8. * r)) : sqrt(1. - 18. * r); };
  double cur = raw(1);
  sf[0] = 0.;
  for (int kk = 1; kk <= 2 * nk; kk++) {
    double nxt = raw(kk + 1);
    if (-(nxt - cur) > .9 * max_ri) nxt = 0.;
    if (((kk + 1) & 1) == 0) sf[(kk + 1) / 2] = factor(nxt);
    cur = nxt;
  }
}

// band_decomp / band_back_sub for m1 = m2 = 1 (Numerical Recipes' bandec/banbks with partial
// pivoting, zero-based, epic_funcs_util.c:3130-3260): A[i][0..2] holds row i's band
__device__ void band_decomp3(int n, double (*A)[3], double *al, int *index) {
  int l = 1;
  A[0][0] = A[0][1]; A[0][1] = A[0][2]; A[0][2] = 0.;
  for (int k = 0; k < n; k++) {
    double tmp = A[k][0];
    int i = k;
    if (l < n) l++;
    for (int j = k + 1; j < l; j++)
      if (fabs(A[j][0]) > fabs(tmp)) { tmp = A[j][0]; i = j; }
    index[k] = i;
    if (tmp == 0.) A[k][0] = 1.e-20;
    if (i != k)
      for (int j = 0; j < 3; j++) { const double t = A[k][j]; A[k][j] = A[i][j]; A[i][j] = t; }
    for (i = k + 1; i < l; i++) {
      tmp = A[i][0] / A[k][0];
      al[k] = tmp;
      for (int j = 1; j < 3; j++) A[i][j - 1] = A[i][j] - tmp * A[k][j];
      A[i][2] = 0.;
    }
  }
}
__device__ void band_back_sub3(int n, double (*A)[3], const double *al, const int *index, double *b) {
  int l = 1;
  for (int k = 0; k < n; k++) {
    const int i = index[k];
    if (i != k) { const double t = b[k]; b[k] = b[i]; b[i] = t; }
    if (l < n) l++;
    for (int q = k + 1; q < l; q++) b[q] -= al[k] * b[k];
  }
  l = 1;
  for (int i = n - 1; i >= 0; i--) {
    double tmp = b[i];
    for (int k = 1; k < l; k++) tmp -= A[i][k] * b[k + i];
    b[i] = tmp / A[i][0];
    if (l < 3) l++;
  }
}

// crank_nicolson (epic_funcs_util.c:3643-3787) with tridiag(WITH_PIVOTING): band_decomp,
// band_back_sub and one band_improve pass (:2994-3120, :3330-3400).  z, A, mu, rho (may be null)
// and ans are indexed 0..n+1; A[0] or A[n+1] above .99e20 marks a no-flux end.  Returns 0, or the
// first index j where z does not increase (z[j] <= z[j-1]; the reference exits there).
// Kept out of line: inlined into the column kernels (nvcc 13.0, sm_103a), the callers' store of
// the no-flux marker A[0] = 1e20 into their local array was not seen by the solver's read of it
// (measured: every column then took the flux branch); a call makes the arrays' stores complete.
__device__ __noinline__ int crank_nicolson(int n, double dt, const double *z, const double *A, const double *mu, const double *rho, double *ans) {
  double a[TN], b[TN], c[TN], r[TN], Ab[TN][3], al[TN];
  int idx[TN];
  const int jstart = A[0] > .99e+20 ? 2 : 1, jend = A[n + 1] > .99e+20 ? n : n + 1;
  for (int j = jstart; j <= jend; j++)
    if (z[j] <= z[j - 1]) return j;
  double coeff3 = (A[0] > .99e+20) ? 0. : mu[0] / (z[1] - z[0]), coeff1, factor;
  a[0] = 0.;
  c[n - 1] = 0.;
  for (int j = 1; j <= n; j++) {
    coeff1 = coeff3;
    if (j == 1) {
      coeff3 = mu[j] / (z[j + 1] - z[j]);
      factor = rho ? dt / (rho[j] * (z[j + 1] - z[j - 1])) : dt / (z[j + 1] - z[j - 1]);
      b[j - 1] = 1. + (coeff1 + coeff3) * factor;
      c[j - 1] = -coeff3 * factor;
      r[j - 1] = 2. * A[j - 1] * coeff1 * factor + A[j] * (1. - (coeff1 + coeff3) * factor) + A[j + 1] * coeff3 * factor;
    } else if (j == n) {
      coeff3 = (A[n + 1] > .99e+20) ? 0. : mu[j] / (z[j + 1] - z[j]);
      factor = rho ? dt / (rho[j] * (z[j + 1] - z[j - 1])) : dt / (z[j + 1] - z[j - 1]);
      a[j - 1] = -coeff1 * factor;
      b[j - 1] = 1. + (coeff1 + coeff3) * factor;
      r[j - 1] = A[j - 1] * coeff1 * factor + A[j] * (1. - (coeff1 + coeff3) * factor) + 2. * A[j + 1] * coeff3 * factor;
    } else {
      coeff3 = mu[j] / (z[j + 1] - z[j]);
      factor = rho ? dt / (rho[j] * (z[j + 1] - z[j - 1])) : dt / (z[j + 1] - z[j - 1]);
      a[j - 1] = -coeff1 * factor;
      b[j - 1] = 1. + (coeff1 + coeff3) * factor;
      c[j - 1] = -coeff3 * factor;
      r[j - 1] = A[j - 1] * coeff1 * factor + A[j] * (1. - (coeff1 + coeff3) * factor) + A[j + 1] * coeff3 * factor;
    }
  }
  for (int j = 0; j < n; j++) {
    Ab[j][0] = a[j];
    Ab[j][1] = b[j];
    Ab[j][2] = c[j];
  }
  band_decomp3(n, Ab, al, idx);
  for (int j = 0; j < n; j++) ans[j + 1] = r[j];
  band_back_sub3(n, Ab, al, idx, ans + 1);
  // band_improve: the residual of the original band (a, b, c) in binary64, one correction
  double res[TN];
  for (int i = 0; i < n; i++) {
    double sdp = -r[i];
    if (i > 0) sdp += a[i] * ans[i];
    sdp += b[i] * ans[i + 1];
    if (i < n - 1) sdp += c[i] * ans[i + 2];
    res[i] = sdp;
  }
  band_back_sub3(n, Ab, al, idx, res);
  for (int i = 0; i < n; i++) ans[i + 1] -= res[i];
  return 0;
}

// ---------------------------------------------------------------------------------------------
// source_sink_SA, :2434-2711
// ---------------------------------------------------------------------------------------------

// get_brunt2 on the interface kk = 2k+1, 1 <= k < nk (np = 1, fpara off, Held-Suarez cp),
// epic_funcs_diag.c:2885-3075
__device__ double brunt2_iface(const DevModel &M, int k, int j, int i) {
  const long long x = M.at(k, j, i);
  const double pressure = M.p3[x], temperature = M.t3[x], density = M.rho3[x];
  const double cp = 1004., mu = M.mu_dry;
  const double deltap = 0.001 * pressure, deltaT = 0.001 * temperature;
  auto dens = [&](double p, double t) { return p * mu / (8.314472e+3 * t); };   // return_density
  const double drho_dp_T = (dens(pressure + deltap, temperature) - dens(pressure - deltap, temperature)) / (2. * deltap);
  const double drho_dT_p = (dens(pressure, temperature + deltaT) - dens(pressure, temperature - deltaT)) / (2. * deltaT);
  const double Drho_Dp = (M.rho2[M.at(k + 1, j, i)] - M.rho2[x]) / (M.p2[M.at(k + 1, j, i)] - M.p2[x]);
  const double g = M.grav[2 * j + 1];
  return g * g * (Drho_Dp - drho_dp_T + temperature / (cp * density * density) * drho_dT_p * drho_dT_p);
}

// Everything of a point's update but the three gradient terms, at every point k = 1..nk-1,
// j = 0..nj, i = 1..ni: the terms that read only the point's own NU_TURB (which the sweep has not
// changed when it reaches the point) and the NU_TURB-free strain, wall distance and buoyancy.
// work0 = the production cb1 S~ NU, work1 = the destruction cw1 fw (NU/d~)^2, work3 = the buoyancy
// term (0 where N^2 >= 0, which subtracts nothing), work2 = 1/dz.
__global__ void k_sa_prep(DevModel M) {
  if (epic_member(M)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)(M.nj + 1);
  if (t >= (unsigned)(M.nk - 1) * nr * ni) return;
  const unsigned r = t / ni, q = r / nr;
  const int i = 1 + (int)(t - r * ni), j = (int)(r - q * nr), k = 1 + (int)q;
  const double cw2 = 0.3, cw3_6 = 64., cb1 = 0.1355, cb2 = 0.622, sigma = 2. / 3., kappa = 0.41;
  const double kappa_2 = kappa * kappa, cw1 = (cb1 / kappa_2) + ((1. + cb2) / sigma), nu_turb_limiter = 3000.;
  const MathTable &T = *M.lt;
  const long long off = plane_offset(M, PL_UV_DIS);
  const double *U = M.u + off, *V = M.v + off;
  auto u = [&](int kk, int jj, int ii) { return U[M.at(kk, jj, ii)]; };
  auto v = [&](int kk, int jj, int ii) { return V[M.at(kk, jj, ii)]; };
  auto w3 = [&](int kk, int jj, int ii) { return M.w3[M.at(kk, jj, ii)]; };
  auto gz3 = [&](int kk) { return M.gz3[M.at(kk, j, i)]; };
  const int jj = 2 * j, kk = 2 * k + 1;
  const double m_2jp1 = M.m[jj + 1], n_2jp1 = M.n[jj + 1];
  // delta_SA (:2774-2808), for k < nk
  const double dx = 1. / M.m[jj + 1], dy = 1. / M.n[jj + 1];
  const double dz = (gz3(k - 1) - gz3(k + 1)) / M.grav[jj + 1];
  double delta = dminr(dx, dy);
  delta = dminr(delta, dz);
  const double d_tilda = dminr(d_wall(M, k, j, i), 0.65 * delta);
  const double dz_inv = M.grav[jj + 1] / (gz3(k - 1) - gz3(k + 1));
  // U on the v-grid (zero on the polar rows) and V on the u-grid, layer k
  auto u2d = [&](int J) -> double {
    if (J == 0 || J == M.nj + 1) return 0.;
    const int JJ = 2 * J;
    const double mn_v = .5 / (1. / M.mn[JJ - 1] + 1. / M.mn[JJ + 1]);
    return ((u(k, J, i) + u(k, J, i + 1)) * (1. / M.mn[JJ + 1]) + (u(k, J - 1, i) + u(k, J - 1, i + 1)) * (1. / M.mn[JJ - 1])) * mn_v;
  };
  auto v2d = [&](int I) -> double {
    if (I == M.ni + 1) I = 1;
    const double mn_u = .5 / (1. / M.mn[jj] + 1. / M.mn[jj + 2]);
    return ((v(k, j, I) + v(k, j, I - 1)) * (1. / M.mn[jj]) + (v(k, j + 1, I) + v(k, j + 1, I - 1)) * (1. / M.mn[jj + 2])) * mn_u;
  };
  const double s11 = (u(k, j, i + 1) - u(k, j, i)) * m_2jp1;
  const double s22 = (v(k, j + 1, i) - v(k, j, i)) * n_2jp1;
  const double s33 = (w3(k - 1, j, i) - w3(k + 1, j, i)) / (M.sgth[kk - 2] - M.sgth[kk + 2]);
  const double s12 = .5 * ((u2d(j + 1) - u2d(j)) * n_2jp1 + (v2d(i + 1) - v2d(i)) * m_2jp1);
  const double u_var3 = 0.5 * (u(k + 1, j, i) + u(k + 1, j, i + 1));
  const double u_var1 = 0.5 * (u(k - 1, j, i) + u(k - 1, j, i + 1));
  double w_var3 = 0.5 * (w3(k, j, i) + w3(k, j, i + 1));
  double w_var1 = 0.5 * (w3(k, j, i) + w3(k, j, i - 1));
  const long long x = M.at(k, j, i);
  const double h_rho = M.h3[x] / M.rho3[x];
  const double s13 = .5 * ((u_var1 - u_var3) * dz_inv + h_rho * (w_var3 - w_var1) * m_2jp1);
  const double v_var3 = 0.5 * (v(k + 1, j, i) + v(k + 1, j + 1, i));
  const double v_var1 = 0.5 * (v(k - 1, j, i) + v(k - 1, j + 1, i));
  w_var3 = 0.5 * (w3(k, j, i) + w3(k, j + 1, i));
  w_var1 = 0.5 * (w3(k, j, i) + w3(k, j - 1, i));
  const double s23 = .5 * ((v_var1 - v_var3) * dz_inv + h_rho * (w_var3 - w_var1) * n_2jp1);
  const double S = sqrt(2. * (s11 * s11 + s22 * s22 + s33 * s33 + 2. * (s12 * s12 + s13 * s13 + s23 * s23)));
  // the point's own NU_TURB terms
  const double nu = M.nu_turb[x];
  const double chi = nu / M.kinvisc;
  const double chi3 = cr_pow(chi, 3., T);
  const double fv1 = chi3 / (chi3 + SA_CV1_3);
  const double fv2 = 1. - (chi / (1. + chi * fv1));
  const double tmp1 = kappa_2 * d_tilda * d_tilda;
  const double S_tilda = S + (nu * fv2) / tmp1;
  const double tmp2 = S_tilda * tmp1;
  double fw = 1.;
  if (tmp2 != 0.) {
    const double r_sa = nu / tmp2;
    if (r_sa < 0.) flag_error(M.ctl, ERR_TURB, k, j, i, r_sa);
    else if (r_sa < 10.) {
      const double g_sa = r_sa + cw2 * (cr_pow(r_sa, 6., T) - r_sa);
      fw = g_sa * cr_pow(((1. + cw3_6) / (cr_pow(g_sa, 6., T) + cw3_6)), (1. / 6.), T);
    }
  }
  const double brunt2 = brunt2_iface(M, k, j, i);
  const double brunt = sqrt(fabs(brunt2));
  M.work0[x] = cb1 * S_tilda * nu;
  M.work1[x] = cw1 * fw * cr_pow((nu / d_tilda), 2., T);
  M.work2[x] = dz_inv;
  M.work3[x] = brunt2 < 0. ? nu * cr_exp(-nu / nu_turb_limiter, T) * brunt2 / brunt : 0.;
}

// One wavefront k + j + i = d of the in-place NU_TURB update: the three gradient terms from the
// neighbours (new at k-1, j-1, i-1; old at k+1, j+1, i+1), summed in the reference's order between
// the point's own terms
__global__ void k_sa_wave(DevModel M, int d) {
  if (epic_member(M)) return;
  const int nr = M.nj + 1;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (M.nk - 1) * nr) return;
  const int k = 1 + t / nr, j = t - (k - 1) * nr, i = d - k - j;
  if (i < 1 || i > M.ni) return;
  const double cb2 = 0.622, sigma = 2. / 3.;
  double *NU = M.nu_turb;
  auto nut = [&](int kk, int jj, int ii) { return NU[M.at(kk, jj, ii)]; };
  const long long x = M.at(k, j, i);
  const int jj = 2 * j;
  const double m_2jp1 = M.m[jj + 1], n_2jp2 = M.n[jj + 2], n_2j = M.n[jj];
  const double nu = NU[x];
  const double g1 = (nut(k, j, i + 1) - nut(k, j, i - 1)) * m_2jp1 * .5;
  const double g2 = .5 * ((nut(k, j + 1, i) - nu) * n_2jp2 + (nu - nut(k, j - 1, i)) * n_2j);
  const double g3 = (nut(k - 1, j, i) - nut(k + 1, j, i)) * M.work2[x];
  double dnudt = M.work0[x];
  dnudt += (cb2 / sigma) * (g1 * g1);   // pow(g, 2.), the correctly rounded square
  dnudt += (cb2 / sigma) * (g2 * g2);
  dnudt += (cb2 / sigma) * (g3 * g3);
  dnudt -= M.work1[x];
  dnudt -= M.work3[x];
  NU[x] = dmaxr(1.e-4 * M.kinvisc, nu + M.dt * dnudt);
}

// The solid-surface block (:2690-2704): NU_TURB(nk) = MAX(1e-4 kinvisc, NU_TURB(nk-1)) (the
// reference computes law_of_the_wall and invert_fv1 there first and then overwrites their result)
__global__ void k_sa_bottom(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (M.nj + 1) * M.ni) return;
  const int j = t / M.ni, i = 1 + t - j * M.ni;
  M.nu_turb[M.at(M.nk, j, i)] = dmaxr(nu_floor(M), M.nu_turb[M.at(M.nk - 1, j, i)]);
}

// bc_lateral of layers k0..k1, rows 0..nj+1 (src/single/s_epic_functions.c:39-87)
__global__ void k_pads(DevModel M, double *a, int k0, int k1) {
  if (epic_member(M, a)) return;
  const int nr = M.nj + 2;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (k1 - k0 + 1) * nr) return;
  const int k = k0 + t / nr, j = t - (k - k0) * nr;
  const long long b = M.at(k, j, 0);
  a[b] = a[b + M.ni];
  a[b + M.ni + 1] = a[b + 1];
}

// restore_mass(NU_TURB_INDEX), epic_adjust.c:80-88: layers 0..nk+1, rows 0..nj, every column
__global__ void k_restore_nu(DevModel M) {
  if (epic_member(M)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned w = (unsigned)(M.nj + 1) * (unsigned)M.iadim;
  if (t >= w * (unsigned)(M.nk + 2)) return;
  const unsigned q = t / w;
  const long long x = M.at((int)q, 0, 0) + (t - q * w);
  M.nu_turb[x] = dmaxr(nu_floor(M), M.nu_turb[x]);
}

// ---------------------------------------------------------------------------------------------
// laplacian_h (:423-583) for the layers k0..nk of `var`, with DIFF_COEF = dc (nu_coef = 0) or
// 3/2 (kinvisc + NU_TURB) (nu_coef = 1); bf = the zonally filtered copy of var
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ double diff_coef(const DevModel &M, const double *dc, int nu_coef, long long x) {
  return nu_coef ? 3. / 2. * (M.kinvisc + M.nu_turb[x]) : dc[x];
}

// GH1 (the x-flux, rows 0..nj, with pads) and GH2 (the y-flux, rows 0..nj+1; 0 on the polar rows)
__global__ void k_lap_fluxes(DevModel M, const double *var, const double *bf, const double *dc, int nu_coef, int k0,
                             double *gh1, double *gh2) {
  if (epic_member(M, var, bf, dc, gh1, gh2)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)(M.nj + 2);
  if (t >= (unsigned)(M.nk - k0 + 1) * nr * ni) return;
  const unsigned r = t / ni, q = r / nr;
  const int i = 1 + (int)(t - r * ni), j = (int)(r - q * nr), k = k0 + (int)q;
  const long long x = M.at(k, j, i);
  if (j <= M.nj) {
    const double g1 = M.m[2 * j + 1] * (bf[x] - bf[x - 1]);
    write_with_pads(gh1, M, M.at(k, j, 0), i, g1 * (.5 * (diff_coef(M, dc, nu_coef, x) + diff_coef(M, dc, nu_coef, x - 1))));
  }
  double g2 = 0.;
  if (j >= 1 && j <= M.nj) {
    const long long xs = M.at(k, j - 1, i);
    g2 = M.n[2 * j] * (var[x] - var[xs]);
    g2 *= .5 * (diff_coef(M, dc, nu_coef, x) + diff_coef(M, dc, nu_coef, xs));
  }
  gh2[x] = g2;
}

// var += dt LPH, rows 0..nj (with pads), from the filtered GH1 and GH2
__global__ void k_lap_apply(DevModel M, double *var, int k0, const double *gh1, const double *gh2) {
  if (epic_member(M, var, gh1, gh2)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)(M.nj + 1);
  if (t >= (unsigned)(M.nk - k0 + 1) * nr * ni) return;
  const unsigned r = t / ni, q = r / nr;
  const int i = 1 + (int)(t - r * ni), j = (int)(r - q * nr), k = k0 + (int)q;
  const double m_2jp1 = M.m[2 * j + 1], n_2jp1 = M.n[2 * j + 1];
  const double m_2j_inv = (j == 0) ? 0. : 1. / M.m[2 * j];
  const double m_2jp2_inv = (j == M.nj) ? 0. : 1. / M.m[2 * j + 2];
  const long long x = M.at(k, j, i);
  const double lph = m_2jp1 * ((gh1[x + 1] - gh1[x]) + n_2jp1 * (gh2[M.at(k, j + 1, i)] * m_2jp2_inv - gh2[x] * m_2j_inv));
  write_with_pads(var, M, M.at(k, j, 0), i, var[x] + M.dt * lph);
}

// ---------------------------------------------------------------------------------------------
// scalar_vertical_diffusion (:1273-1488), one thread per column j = 0..nj, i = 1..ni
// ---------------------------------------------------------------------------------------------

__global__ void __launch_bounds__(64) k_theta_vdiff(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (M.nj + 1) * M.ni) return;
  const int j = t / M.ni, i = 1 + t - j * M.ni;
  const int nk = M.nk, ks = M.k_sigma;
  const double gi = M.grav[2 * j + 1];
  double sf[TN], z[TN], A[TN], dee[TN], ans[TN];
  stability_layers(M, j, i, sf);
  A[0] = 1.e+20;
  z[0] = M.gz3[M.at(nk, j, i)] / gi;
  for (int k = nk; k >= ks - 2; k--) {
    const int kay = nk - k + 1;
    A[kay] = M.theta[M.at(k, j, i)];
    z[kay] = M.gz3[M.at(k, j, i)] / gi;
  }
  for (int k = nk; k > ks - 2; k--)
    dee[nk - k + 1] = sf[k] * .5 * (M.dc_theta[M.at(k, j, i)] + M.dc_theta[M.at(k - 1, j, i)]);
  if (const int bad = crank_nicolson(nk - ks + 2, M.dt, z, A, dee, nullptr, ans)) {   // THETA: z[bad] - z[bad-1] recorded
    flag_error(M.ctl, ERR_TURB, nk - bad + 1, j, i, z[bad] - z[bad - 1]);
    return;
  }
  for (int k = nk; k >= ks - 1; k--) write_with_pads(M.theta, M, M.at(k, j, 0), i, ans[nk - k + 1]);
}

__global__ void __launch_bounds__(64) k_nu_vdiff(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (M.nj + 1) * M.ni) return;
  const int j = t / M.ni, i = 1 + t - j * M.ni;
  const int nk = M.nk;
  const double gi = M.grav[2 * j + 1], sigma_inv = 3. / 2.;
  const double tw = tau_wall(M, WALL_H, j, i);
  double z[TN], A[TN], dee[TN], ans[TN];
  auto gz = [&](int k) { return M.gz3[M.at(k, j, i)]; };
  auto nu = [&](int k) { return M.nu_turb[M.at(k, j, i)]; };
  A[nk + 2] = 1.e+20;
  z[nk + 2] = (gz(0) + (gz(0) - gz(1))) / gi;
  for (int k = nk; k >= 0; k--) {
    A[nk - k + 1] = nu(k);
    z[nk - k + 1] = gz(k) / gi;
  }
  for (int k = nk; k > 0; k--) dee[nk - k + 1] = sigma_inv * (M.kinvisc + .5 * (nu(k) + nu(k - 1)));
  z[0] = (gz(nk) - (gz(nk - 1) - gz(nk))) / gi;
  dee[0] = dee[1];
  A[0] = A[1] - tw * (z[1] - z[0]) / dee[0];
  if (const int bad = crank_nicolson(nk + 1, M.dt, z, A, dee, nullptr, ans)) {
    flag_error(M.ctl, ERR_TURB, nk - bad + 1, j, i, z[bad] - z[bad - 1]);
    return;
  }
  for (int k = nk; k >= 0; k--) write_with_pads(M.nu_turb, M, M.at(k, j, 0), i, ans[nk - k + 1]);
}

// ---------------------------------------------------------------------------------------------
// uv_vertical_diffusion (:1940-2075): the wall stresses of all columns first (tau_surface reads
// the neighbours' bottom winds, which the columns' solves then change), then one thread per column
// ---------------------------------------------------------------------------------------------

__global__ void k_tau_wall(DevModel M, int comp, double *tw) {
  if (epic_member(M, tw)) return;
  const int j0 = comp == 0 ? 0 : 1;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (M.nj + 1 - j0) * M.ni) return;
  const int j = j0 + t / M.ni, i = 1 + t - (j - j0) * M.ni;
  tw[M.at2(j, i)] = tau_wall(M, comp == 0 ? WALL_U : WALL_V, j, i);
}

__global__ void __launch_bounds__(64) k_wind_vdiff(DevModel M, int comp, const double *tw) {
  if (epic_member(M, tw)) return;
  const int j0 = comp == 0 ? 0 : 1;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (M.nj + 1 - j0) * M.ni) return;
  const int j = j0 + t / M.ni, i = 1 + t - (j - j0) * M.ni;
  const int nk = M.nk;
  // the neighbouring column of the stencil: (j, i-1) for U, (j-1, i) for V
  const int jn = comp == 0 ? j : j - 1, in = comp == 0 ? i - 1 : i;
  const double gi = comp == 0 ? M.grav[2 * j + 1] : M.grav[2 * j];
  double *W = (comp == 0 ? M.u : M.v) + plane_offset(M, PL_UV);
  double sf2[TN], sf0[TN], z[TN], A[TN], mu[TN], rho[TN], ans[TN];
  stability_layers(M, j, i, sf2);
  stability_layers(M, jn, in, sf0);
  auto gzm = [&](int k) { return .5 * (M.gz3[M.at(k, j, i)] + M.gz3[M.at(k, jn, in)]); };
  A[nk] = 1.e+20;
  z[nk] = gzm(0) / gi;
  for (int k = nk - 1; k >= 1; k--) {
    const int kay = nk - k;
    A[kay] = W[M.at(k, j, i)];
    z[kay] = gzm(k) / gi;
    rho[kay] = .5 * (M.rho3[M.at(k, j, i)] + M.rho3[M.at(k, jn, in)]);
  }
  for (int k = nk - 1; k >= 1; k--)
    mu[nk - k] = M.dynvisc + .5 * (sf2[k] * M.rho2[M.at(k, j, i)] * .5 * (M.dc_uv[M.at(k - 1, j, i)] + M.dc_uv[M.at(k, j, i)]) +
                                   sf0[k] * M.rho2[M.at(k, jn, in)] * .5 * (M.dc_uv[M.at(k - 1, jn, in)] + M.dc_uv[M.at(k, jn, in)]));
  z[0] = gzm(nk) / gi;
  mu[0] = mu[1];
  A[0] = A[1] - tw[M.at2(j, i)] * (z[1] - z[0]) / mu[0];
  if (const int bad = crank_nicolson(nk - 1, M.dt, z, A, mu, rho, ans)) {
    flag_error(M.ctl, ERR_TURB, nk - bad, j, i, z[bad] - z[bad - 1]);
    return;
  }
  for (int k = nk - 1; k >= 1; k--) write_with_pads(W, M, M.at(k, j, 0), i, ans[nk - k]);
}

// ---------------------------------------------------------------------------------------------
// uv_horizontal_diffusion (:1571-1787).  work0 = COEFFD, work1 = H_RHO, work2 = UU, work3 = VV
// (layers 1..nk-1, zonally filtered); the stresses are recomputed where the updates read them.
// ---------------------------------------------------------------------------------------------

__global__ void k_uvh_coef(DevModel M) {
  if (epic_member(M)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned w = (unsigned)(M.nj + 1) * (unsigned)M.iadim;
  if (t >= w * (unsigned)(M.nk - 1)) return;
  const unsigned q = t / w;
  const long long x = M.at(1 + (int)q, 0, 0) + (t - q * w);
  M.work0[x] = M.dynvisc + M.rho3[x] * M.dc_uv[x];
  M.work1[x] = M.h3[x] / M.rho3[x];
}

// TAU12 on the polar rows, per layer: vorticity(ON_SIGMATHETA, RELATIVE) there (epic_funcs_diag.c:
// 4279-4290, 4357-4379) times minus the row mean of COEFFD H_RHO, the sums in the reference's order
__global__ void k_uvh_poles(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= 2 * (M.nk - 1)) return;
  const int k = 1 + t / 2, north = t & 1;
  const double *uu = M.work2, *cd = M.work0, *hr = M.work1;
  const int ni = M.ni, jr = north ? M.nj : 0;
  double ze = 0., coeff = 0.;
  for (int i = 1; i <= ni; i++) {
    if (north) ze += uu[M.at(k, jr, i)];
    else ze -= uu[M.at(k, jr, i)];
  }
  if (north) ze *= M.mn[2 * (M.nj + 1)] / (M.m[2 * M.nj + 1] * (double)ni);
  else ze *= M.mn[0] / ((M.m[1]) * (double)ni);
  for (int i = 1; i <= ni; i++) coeff += cd[M.at(k, jr, i)] * hr[M.at(k, jr, i)];
  coeff /= ni;
  M.turb_pole[2 * k + north] = ze * -coeff;
}

struct Stress { double t11, t22, t33; };

__device__ __forceinline__ Stress stress_h(const DevModel &M, int k, int j, int i) {
  if (i == 0) i = M.ni;   // bc_lateral
  const double *cd = M.work0, *hr = M.work1, *uu = M.work2, *vv = M.work3;
  auto U = [&](int jj, int ii) { return uu[M.at(k, jj, ii)]; };
  auto Vv = [&](int jj, int ii) { return vv[M.at(k, jj, ii)]; };
  auto H = [&](int jj, int ii) { return hr[M.at(k, jj, ii)]; };
  const int jj = 2 * j;
  const double rln_inv = 1. / M.rln[jj + 1], m_2jp1 = M.m[jj + 1], n_2jp2 = M.n[jj + 2], n_2jp1 = M.n[jj + 1], n_2j = M.n[jj];
  const double e11 = (U(j, i + 1) - U(j, i)) * m_2jp1 + .5 * (Vv(j, i) + Vv(j + 1, i)) * rln_inv * (M.rln[jj + 2] - M.rln[jj]) * n_2jp1;
  const double e22 = (Vv(j + 1, i) - Vv(j, i)) * n_2jp1;
  double coeff = .5 / H(j, i);
  double e33 = coeff * (U(j, i + 1) * (H(j, i + 1) - H(j, i)) * m_2jp1 + U(j, i) * (H(j, i) - H(j, i - 1)) * m_2jp1);
  if (Vv(j + 1, i) != 0.) e33 += coeff * Vv(j + 1, i) * (H(j + 1, i) - H(j, i)) * n_2jp2;
  if (Vv(j, i) != 0.) e33 += coeff * Vv(j, i) * (H(j, i) - H(j - 1, i)) * n_2j;
  coeff = H(j, i) * (2. / 3.) * cd[M.at(k, j, i)];
  Stress s;
  s.t11 = coeff * (2. * e11 - e22 - e33);
  s.t22 = coeff * (2. * e22 - e11 - e33);
  s.t33 = (coeff / H(j, i)) * (2. * e33 - e11 - e22);
  return s;
}

__device__ __forceinline__ double stress_12(const DevModel &M, int k, int j, int i) {
  if (j == 0) return M.turb_pole[2 * k];
  if (j == M.nj + 1) return M.turb_pole[2 * k + 1];
  if (i == 0) i = M.ni;   // bc_lateral
  const double *cd = M.work0, *hr = M.work1, *uu = M.work2, *vv = M.work3;
  auto c = [&](int jj, int ii) { return cd[M.at(k, jj, ii)] * hr[M.at(k, jj, ii)]; };
  const int jj = 2 * j;
  const double e12 = (vv[M.at(k, j, i)] - vv[M.at(k, j, i - 1)]) * M.m[jj] +
                     M.rln[jj] * (uu[M.at(k, j, i)] / M.rln[jj + 1] - uu[M.at(k, j - 1, i)] / M.rln[jj - 1]) * M.n[jj];
  const double coeff = .25 * (c(j, i) + c(j, i - 1) + c(j - 1, i) + c(j - 1, i - 1));
  return coeff * e12;
}

__global__ void k_uvh_apply(DevModel M) {
  if (epic_member(M)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)(M.nj + 1);
  if (t >= (unsigned)(M.nk - 1) * nr * ni) return;
  const unsigned r = t / ni, q = r / nr;
  const int i = 1 + (int)(t - r * ni), j = (int)(r - q * nr), k = 1 + (int)q;
  const double *hr = M.work1;
  auto H = [&](int jj, int ii) { return hr[M.at(k, jj, ii == 0 ? M.ni : ii)]; };
  const long long tend = plane_offset(M, PL_UV_TEND);
  const Stress s = stress_h(M, k, j, i), sw = stress_h(M, k, j, i - 1);
  {
    const int jj = 2 * j;
    const double rln_inv = 1. / M.rln[jj + 1], m_2jp1 = M.m[jj + 1], n_2jp1 = M.n[jj + 1];
    const double h_inv = 2. / (M.hdry[M.at(k, j, i)] + M.hdry[M.at(k, j, i - 1)]);
    const double t12n = stress_12(M, k, j + 1, i), t12 = stress_12(M, k, j, i);
    const long long x = tend + M.at(k, j, i);
    M.dudt[x] += h_inv * (m_2jp1 * (s.t11 - sw.t11) +
                          n_2jp1 * rln_inv * (M.rln[jj + 2] * t12n - M.rln[jj] * t12 + .5 * (t12n + t12) * (M.rln[jj + 2] - M.rln[jj])) -
                          .5 * (s.t33 + sw.t33) * m_2jp1 * (H(j, i) - H(j, i - 1)));
  }
  if (j >= 1) {
    const Stress ss = stress_h(M, k, j - 1, i);
    const int jj = 2 * j;
    const double rln_inv = 1. / M.rln[jj], m_2j = M.m[jj], n_2j = M.n[jj];
    const double h_inv = 2. / (M.hdry[M.at(k, j, i)] + M.hdry[M.at(k, j - 1, i)]);
    const long long x = tend + M.at(k, j, i);
    M.dvdt[x] += h_inv * (m_2j * (stress_12(M, k, j, i) - stress_12(M, k, j, i - 1)) -
                          n_2j * rln_inv * (M.rln[jj + 1] * s.t22 - M.rln[jj - 1] * ss.t22 - .5 * (s.t11 + ss.t11) * (M.rln[jj + 1] - M.rln[jj - 1])) -
                          .5 * (s.t33 + ss.t33) * n_2j * (H(j, i) - H(j - 1, i)));
  }
}

// ---------------------------------------------------------------------------------------------
// set_diffusion_coef (:2171-2302), inside store_diag.  DIFFUSION_COEF_UV stays as it is above the
// bottom layer (the reference never sets it there).
// ---------------------------------------------------------------------------------------------

__global__ void k_dc_layers(DevModel M) {
  if (epic_member(M)) return;
  const int kend = M.gas_giant ? M.nk : M.nk - 1;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)(M.nj + 1);
  if (t >= (unsigned)kend * nr * ni) return;
  const unsigned r = t / ni, q = r / nr;
  const int i = 1 + (int)(t - r * ni), j = (int)(r - q * nr), k = 1 + (int)q;
  const long long x = M.at(k, j, i), row = M.at(k, j, 0);
  const double nu = M.nu_turb[x];
  double chi3 = nu / M.kinvisc;
  chi3 *= chi3 * chi3;
  const double fv1 = chi3 / (chi3 + SA_CV1_3);
  const double turb = fv1 * nu;
  const double v = limit_range(0., turb, M.turb_maxnu2[j]);
  write_with_pads(M.dc_theta, M, row, i, v);
  write_with_pads(M.dc_mass, M, row, i, v);
}

__global__ void k_dc_bottom(DevModel M) {
  if (epic_member(M)) return;
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= (M.nj + 1) * M.ni) return;
  const int j = t / M.ni, i = 1 + t - j * M.ni;
  const int k = M.nk - 1;
  const double kin = kin_plane(M, PL_UV_DIS, k, j, i);
  const double u_tan = sqrt(2. * kin);
  const double turb = law_of_the_wall(M, k, j, i, WALL_H, u_tan);
  const long long row = M.at(M.nk, j, 0);
  write_with_pads(M.dc_uv, M, row, i, limit_range(0., turb + M.kinvisc, M.turb_maxnu2[j]));
  const double v = limit_range(0., turb, M.turb_maxnu2[j]);
  write_with_pads(M.dc_theta, M, row, i, v);
  write_with_pads(M.dc_mass, M, row, i, v);
}

inline unsigned nblk(long long n, int th) { return (unsigned)((n + th - 1) / th); }

// cfl_dt (epic_funcs_diag.c:4884-5022): the minimum of each direction's limit over the grid, by
// an atomic minimum on the bits of the positive binary64 limits (their order is the integers');
// a minimum does not depend on the order of its operands, so the result is the reference's
__global__ void k_cfl(DevModel M, unsigned long long *lim) {
  if (epic_member(M, lim)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)(M.nj + 1);
  double cx = DBL_MAX, cy = DBL_MAX, cz = DBL_MAX;
  if (t < (unsigned)M.nk * nr * ni) {
    const unsigned r = t / ni, q = r / nr;
    const int i = 1 + (int)(t - r * ni), j = (int)(r - q * nr), k = 1 + (int)q;
    const long long off = plane_offset(M, PL_UV);
    const double *U = M.u + off, *V = M.v + off;
    const double dz = M.dsgth[2 * k];
    double w = M.w3[M.at(k - 1, j, i)];
    if (w > 0.) cz = dminr(cz, dz / w);
    w = M.w3[M.at(k, j, i)];
    if (w < 0.) cz = dminr(cz, -dz / w);
    if (j >= 1) {
      const double dy = 1. / M.n[2 * j + 1];
      const double cs = sqrt(M.rgas * .5 * (M.t3[M.at(k, j, i)] + M.t3[M.at(k, j - 1, i)]) / (1. - M.kappa));
      double v = V[M.at(k, j + 1, i)] + cs;
      if (v > 0.) cy = dminr(cy, dy / v);
      v = V[M.at(k, j, i)] - cs;
      if (v < 0.) cy = dminr(cy, -dy / v);
    }
    if (fabs(M.lat[2 * j + 1]) <= M.lat0) {
      const double dx = 1. / M.m[2 * j + 1];
      const double cs = sqrt(M.rgas * .5 * (M.t3[M.at(k, j, i)] + M.t3[M.at(k, j, i - 1)]) / (1. - M.kappa));
      double u = U[M.at(k, j, i + 1)] + cs;
      if (u > 0.) cx = dminr(cx, dx / u);
      u = U[M.at(k, j, i)] - cs;
      if (u < 0.) cx = dminr(cx, -dx / u);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cx = dminr(cx, __shfl_xor_sync(0xffffffffu, cx, o));
    cy = dminr(cy, __shfl_xor_sync(0xffffffffu, cy, o));
    cz = dminr(cz, __shfl_xor_sync(0xffffffffu, cz, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&lim[0], (unsigned long long)__double_as_longlong(cx));
    atomicMin(&lim[1], (unsigned long long)__double_as_longlong(cy));
    atomicMin(&lim[2], (unsigned long long)__double_as_longlong(cz));
  }
}

}  // namespace

int launch_cfl_dt(const DevModel &M, unsigned long long *lim, cudaStream_t s) {
  k_cfl<<<zg(nblk((long long)M.nk * (M.nj + 1) * M.ni, 128), M), 128, 0, s>>>(M, lim);
  return 0;
}

// ---- launchers ----

int launch_restore_nu(const DevModel &M, cudaStream_t s) {
  k_restore_nu<<<zg(nblk((long long)(M.nj + 1) * M.iadim * (M.nk + 2), 256), M), 256, 0, s>>>(M);
  return 0;
}

static int launch_pads(const DevModel &M, double *a, int k0, int k1, cudaStream_t s) {
  k_pads<<<zg(nblk((long long)(k1 - k0 + 1) * (M.nj + 2), 128), M), 128, 0, s>>>(M, a, k0, k1);
  return 0;
}

int launch_source_sink_turb(const DevModel &M, cudaStream_t s) {
  const long long cells = (long long)(M.nk - 1) * (M.nj + 1) * M.ni;
  k_sa_prep<<<zg(nblk(cells, 128), M), 128, 0, s>>>(M);
  const int fronts_lo = 1 + 0 + 1, fronts_hi = (M.nk - 1) + M.nj + M.ni;
  const unsigned blocks = nblk((long long)(M.nk - 1) * (M.nj + 1), 128);
  for (int d = fronts_lo; d <= fronts_hi; d++) k_sa_wave<<<zg(blocks, M), 128, 0, s>>>(M, d);
  if (!M.gas_giant) k_sa_bottom<<<zg(nblk((long long)(M.nj + 1) * M.ni, 128), M), 128, 0, s>>>(M);
  return launch_pads(M, M.nu_turb, 0, M.nk + 1, s);
}

// laplacian_h of layers k0..nk of var, then var += dt LPH (scratch work0..2)
static int laplacian_step(const DevModel &M, double *var, const double *dc, int nu_coef, int k0, cudaStream_t s) {
  const int n = M.nk - k0 + 1;
  launch_filter_planes(M, var, PL_NONE, M.work0, k0, n, 0, s);   // zonal_filter(H2_INDEX) of a copy
  k_lap_fluxes<<<zg(nblk((long long)n * (M.nj + 2) * M.ni, 128), M), 128, 0, s>>>(M, var, M.work0, dc, nu_coef, k0, M.work1, M.work2);
  launch_filter_planes(M, M.work1, PL_NONE, M.work1, k0, n, 0, s);   // zonal_filter(U_INDEX) of GH1
  k_lap_apply<<<zg(nblk((long long)n * (M.nj + 1) * M.ni, 128), M), 128, 0, s>>>(M, var, k0, M.work1, M.work2);
  return 0;
}

int launch_scalar_hdiff(const DevModel &M, cudaStream_t s) {
  laplacian_step(M, M.theta, M.dc_theta, 0, M.k_sigma - 1, s);
  launch_set_p2etc(M, 1, s);
  laplacian_step(M, M.nu_turb, nullptr, 1, 1, s);
  return launch_restore_nu(M, s);
}

int launch_scalar_vdiff(const DevModel &M, cudaStream_t s) {
  const unsigned blocks = nblk((long long)(M.nj + 1) * M.ni, 64);
  k_theta_vdiff<<<zg(blocks, M), 64, 0, s>>>(M);
  launch_set_p2etc(M, 1, s);
  k_nu_vdiff<<<zg(blocks, M), 64, 0, s>>>(M);
  return launch_restore_nu(M, s);
}

int launch_uv_hdiff(const DevModel &M, cudaStream_t s) {
  k_uvh_coef<<<zg(nblk((long long)(M.nj + 1) * M.iadim * (M.nk - 1), 256), M), 256, 0, s>>>(M);
  launch_filter_planes(M, M.work0, PL_NONE, M.work0, 1, M.nk - 1, 0, s);
  launch_filter_planes(M, M.work1, PL_NONE, M.work1, 1, M.nk - 1, 0, s);
  launch_filter_planes(M, M.u, PL_UV_DIS, M.work2, 1, M.nk - 1, 0, s);
  launch_filter_planes(M, M.v, PL_UV_DIS, M.work3, 1, M.nk - 1, 1, s);
  k_uvh_poles<<<zg(nblk(2LL * (M.nk - 1), 64), M), 64, 0, s>>>(M);
  k_uvh_apply<<<zg(nblk((long long)(M.nk - 1) * (M.nj + 1) * M.ni, 128), M), 128, 0, s>>>(M);
  return 0;
}

int launch_uv_vdiff(const DevModel &M, cudaStream_t s) {
  for (int comp = 0; comp < 2; comp++) {
    const unsigned blocks = nblk((long long)(M.nj + 1 - comp) * M.ni, 64);
    k_tau_wall<<<zg(blocks, M), 64, 0, s>>>(M, comp, M.work0);
    k_wind_vdiff<<<zg(blocks, M), 64, 0, s>>>(M, comp, M.work0);
  }
  return 0;
}

int launch_set_diffusion_coef(const DevModel &M, cudaStream_t s) {
  const int kend = M.gas_giant ? M.nk : M.nk - 1;
  k_dc_layers<<<zg(nblk((long long)kend * (M.nj + 1) * M.ni, 128), M), 128, 0, s>>>(M);
  if (!M.gas_giant) k_dc_bottom<<<zg(nblk((long long)(M.nj + 1) * M.ni, 64), M), 64, 0, s>>>(M);
  launch_pads(M, M.dc_uv, 0, M.nk + 1, s);
  launch_pads(M, M.dc_theta, 0, M.nk + 1, s);
  return launch_pads(M, M.dc_mass, 0, M.nk + 1, s);
}

}  // namespace epic
