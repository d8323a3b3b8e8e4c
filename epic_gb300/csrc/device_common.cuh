// Device-side model description and the pointwise helpers every kernel shares.
//
// All device arrays keep the reference layout X(k,j,i) = base[i + (j+1)*iadim + k*n2]
// (include/epic.h:407-449), so host upload/download are plain copies.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cfloat>
#include <type_traits>
#include "dd_math.cuh"
#include "df.cuh"

// kernel groups whose block size the autotuner picks (DevModel::tb)
enum TuneGroup { TB_UV_CORE = 0, TB_PGRAD, TB_HSU, TB_VISC, TB_DIAG, TB_UPDATE, TB_COLUMN, TB_POINT, TB_ROW,
                 TB_HSU_MERID_VARIANT,   // not a block size: 0 automatic, 1 fused march, 2 four passes
                 TB_COUNT };
#define TB(M, g) ((M).tb[g] > 0 ? (M).tb[g] : 128)

#define EPIC_MAX_NK 126      // column kernels keep per-column arrays of nk+2 entries
#define EPIC_MAX_NI 1024     // row kernels keep one row of ni entries in shared memory
#define EPIC_TURB_MAX_NK 64  // the turbulence closure's column solves keep nk+3 entries per array

namespace epic {

// Time-plane indices and step counters live on the device so that one captured CUDA graph
// serves every step (the reference rotates IT_ZERO/IT_MINUS1/IT_MINUS2 on the host,
// src/shared/epic_timestep.c:257-274).
struct Ctl {
  int it_zero, it_minus1, it_minus2;
  int it_uv, it_uv_dis, it_uv_tend;
  long long itime, model_time;
  int err_code, err_k, err_j, err_i;   // first model error (0 = none)
  double err_val;
  double ab[2][3];                     // Adams-Bashforth coefficients chosen for u, v this step
  float2 abf[2][3];                    // the same as double-floats (the mixed forms' update)
  int lf_first[2];                     // leapfrog: forward (Euler) first step for u, v
  int halted;                          // set between steps once err_code is set: every kernel of the
                                       // model then returns at entry (the reference stops the run at
                                       // its first epic_error); cleared by an upload
};

enum ErrCode { ERR_NONE = 0, ERR_GZ_MONOTONE = 1, ERR_CALC_W_P = 2, ERR_PCHIP_X = 3, ERR_NONFINITE = 4, ERR_TIMEOUT = 5,
               ERR_TURB = 6 };

// double-float constants of the mixed form (DevModel::dfc), split on the host
enum { DFC_KAPPA, DFC_KAPPA_INV, DFC_KAPPA1, DFC_SIGMA_SIGMA, DFC_ZETA0, DFC_ZETA1, DFC_G_COEFF, DFC_ALPHA, DFC_LOG_P0,
       DFC_COUNT };

struct DevModel {
  // sizes
  int ni, nj, nk, iadim, jadim, kadim;
  long long n2, n3;
  int nvp, ntp;
  // scalars
  int uv_scheme, k_sigma, k_sponge, newt_cool_on, drag_v, drag_zonal_avg, rayleigh_on;
  int akima;   // advection scheme: 0 Hsu-Konor-Arakawa predictor-corrector, 1 Akima
  double dt, press0, topo_scale, prandtl, tau_drag, nudiv;
  double zeta0, zeta1, alpha, sigma_sigma, g_coeff;   // g_coeff = 1/(1-exp(-alpha*(1-sigma_sigma)))
  double kappa, cp, cpr, rgas, mu_dry, hs_kf, lat0, m0, eps13;
  double coef[9], nu[9];
  // 1-D grid arrays (device copies)
  const double *lon, *lat, *rln, *rlt, *f, *m, *n, *mn, *grav, *mn_inv;
  const double *sgth, *dsgth, *dsgth_inv, *h_min, *t_sponge_inv;
  const double *high_lat_h, *high_lat_pv;   // [(nj+3)*(ni+2)] 2-D like the reference
  const double *h_coef, *v_coef;            // d2dy2 coefficients, 3 per row
  const double *tw;                         // realft/four1 twiddles (see k_filter.cu)
  const double *coslat;                     // cos(lat[2j+1] deg), j = 0..nj, from the host libm
  const double *coslat4;                    // pow(coslat[j], 4.) correctly rounded (t_rad's cos^4)
  const MathTable *lt;                      // double-double tables for cr_log/cr_exp/cr_pow
  const float *twf;                         // the twiddles rounded to float (mixed form)
  const void *fop_map;                      // tensor-core filter (mixed form): the TMA tensor map of the
                                            // operator tiles of the filtered rows (k_filter_gemm.cu), or null
  const int *fop_slot;                      // their slot of each row j = -1..nj+1, h rows then v rows; -1
                                            // where the row is not filtered
  const float2 *exp2tab;                    // 2^(j/32), j = 0..31, as double-floats (exp_df)
  float2 dfc[DFC_COUNT];                    // kappa, 1/kappa, kappa+1, the hybrid-coordinate constants
                                            // and log(press0) as double-floats (hi, lo)
  double x_h2, x_he, x_3;                   // hydrogen thermodynamics when x_h2 > 0 (FP64 form)
  const double *thermo;                     // thermo_setup's tables (thermo_tables in epic_model.cu)
  int gas_giant;                            // planet->type "gas-giant": GZ_SURFACE from gz_from_u in store_pgrad_vars
  int jtp;                                  // grid.jtp: the row where gz_from_u puts GZ_SURFACE's zero
  // the Spalart-Allmaras DES turbulence closure (FP64 form; k_turb.cu)
  int turb;                                 // epic_grid.turbulence on
  int turb_h, turb_v;                       // horizontal / vertical subgrid diffusion (grid.diffusion_direction)
  int stab;                                 // grid.stability_factor "Collins et al. (2004)" (else "off")
  double kinvisc, dynvisc, max_nu2;         // planet->kinvisc, planet->dynvisc, set_max_nu's max_nu[2]
  double *nu_turb, *dc_uv, *dc_theta, *dc_mass;   // NU_TURB and DIFFUSION_COEF_UV, _THETA, _MASS
  double *turb_pole;                        // scratch: the polar TAU12 rows of uv_horizontal_diffusion
  const double *turb_maxnu2;                // set_diffusion_coef's taper max_nu[2] MIN(1, (dy0 m)^-2), j = 0..nj
  int mixed;                                // FP32 stencils, advection, hyperviscosity, filter, physics
  int col64;                                // mixed, with the vertical pressure/geopotential integration
                                            // (set_p2etc, store_pgrad_vars) and the pressure gradient in FP64
  int cr;                                   // binary64 log/exp/pow correctly rounded (the drop-in form);
                                            // else the libdevice functions
  // state
  double *u, *v, *dudt, *dvdt, *hdry, *theta, *p3, *h3, *p2, *theta2, *t2, *t3, *rho2, *rho3, *exner3;
  double *gz3, *mont3, *heat3, *pv3, *ri2, *div_uv3, *w3, *dzdt3, *u_spinup, *gz_surface;
  // scratch
  double *gz, *unity, *old, *work0, *work1, *work2, *work3, *ptable;
  float2 *lp3;   // log P3 at every interface as a double-float: written by set_p2etc of the mixed
                 // form (stage 11), read by its store_pgrad_vars (stage 19); P3 does not change
                 // between the two
  Ctl *ctl;
  // batch: the members' descriptions on the device (nullptr for a single model); kernels
  // launched over a batch take member blockIdx.z's description on entry (EPIC_MEMBER)
  const DevModel *batch;
  int nbatch;
  int hetero;          // batch launch over members of different ni / nj (epic_member relocates
                       // pointer arguments field by field); the launch description then carries
                       // the largest sizes of its members, and member 0's arrays
  long long reloc_n3;  // a launch description's field size of member 0 (whose arrays it carries)
  int fop_shared;      // a batch whose members all filter with member 0's operator tiles (same grid)
  char *pool_base;   // start of the model's device pool (state, scratch and tables)
  // launch shapes (host side only): threads per block of each kernel group, set by the
  // autotuner; they change no result (every tuned kernel is pointwise or per row)
  int tb[TB_COUNT];

  // Offsets within one 3-D field of one model: 32-bit arithmetic (epic_model_create rejects
  // grids whose wind arrays, up to three time planes, reach 2^31 elements).
  __host__ __device__ __forceinline__ int at(int k, int j, int i) const { return i + (j + 1) * iadim + k * (int)n2; }
  __host__ __device__ __forceinline__ int at2(int j, int i) const { return i + (j + 1) * iadim; }
};

// A pointer into member 0's arrays, moved to the same place in member `to`'s arrays.  The pool of
// a model (epic_model_create) packs the state arrays back to back as planes of n3 values (u and v
// value planes, the tendency planes, then the single fields), and carves the scratch volumes gz,
// unity, old, work0..3 one after another, each rounded up to 256 bytes (and, with the turbulence
// closure, NU_TURB and the three diffusivities the same way); so the plane (or volume) index and
// the offset inside it follow from the address by integer arithmetic, and map to the member's
// pool with its own n3.  A pointer outside these regions (a table) is returned as is.
__host__ __device__ __forceinline__ long long scratch_stride(long long n3) { return ((n3 * 8 + 255) / 256) * 256; }
template <class P>
__device__ __forceinline__ P *relocate_field(const DevModel &from, const DevModel &to, P *p) {
  const char *c = reinterpret_cast<const char *>(p);
  const long long n3 = from.reloc_n3;
  const char *s0 = reinterpret_cast<const char *>(from.gz);
  const long long st0 = scratch_stride(n3);
  if (c >= s0 && c < s0 + 7 * st0) {
    const long long o = c - s0, q = o / st0;
    return reinterpret_cast<P *>(reinterpret_cast<char *>(to.gz) + q * scratch_stride(to.n3) + (o - q * st0));
  }
  if (from.nu_turb) {   // the turbulence closure's four volumes (NU_TURB, the diffusivities), one stride apart
    const char *t0 = reinterpret_cast<const char *>(from.nu_turb);
    if (c >= t0 && c < t0 + 4 * st0) {
      const long long o = c - t0, q = o / st0;
      return reinterpret_cast<P *>(reinterpret_cast<char *>(to.nu_turb) + q * scratch_stride(to.n3) + (o - q * st0));
    }
  }
  const char *b0 = reinterpret_cast<const char *>(from.u);
  const long long planes = 2LL * from.nvp + 2LL * from.ntp + 20;
  if (c >= b0 && c < b0 + planes * n3 * 8) {
    const long long o = (c - b0) / 8, q = o / n3;
    return reinterpret_cast<P *>(to.u + q * to.n3 + (o - q * n3));
  }
  return p;
}

// Entry of every kernel: in a batch launch, take member blockIdx.z's description and move the
// state pointers passed as arguments (addresses in the launch description's arrays) to the same
// places in the member's arrays: by offset when the members share the pool layout (same sizes),
// array by array when they do not.  Returns true when the model is halted (a step found a fatal
// error): the kernel then returns at once.  Ctl::halted changes only in k_itime_advance, between
// steps, so every thread of a launch reads the same value.
template <class P>
__device__ __forceinline__ P *member_ptr(const DevModel &M, const DevModel &mem, P *p) {
  if (!p) return p;
  if (M.hetero) return relocate_field(M, mem, p);
  return (P *)(mem.pool_base + ((const char *)p - M.pool_base));
}
template <class... P>
__device__ __forceinline__ bool epic_member(DevModel &M, P *&...ptrs) {
  if (M.batch) {
    const DevModel &mem = M.batch[blockIdx.z];
    ((ptrs = member_ptr(M, mem, ptrs)), ...);
    M = mem;
  }
  return M.ctl->halted != 0;
}

// ---- pointwise helpers: restatements of the reference routines named beside each ----

__device__ __forceinline__ double dmaxr(double x, double y) { return x > y ? x : y; }   // MAX, include/epic.h:144
__device__ __forceinline__ double dminr(double x, double y) { return x < y ? x : y; }   // MIN, include/epic.h:138

// fcmp, src/shared/epic_funcs_util.c:4275-4330
__device__ __forceinline__ int fcmp(double x1, double x2) {
  int e;
  frexp(fabs(x1) > fabs(x2) ? x1 : x2, &e);
  const double delta = ldexp(DBL_EPSILON, e);
  const double d = x1 - x2;
  return d > delta ? 1 : (d < -delta ? -1 : 0);
}

// THETA2 at an isentropic layer (set_p2etc, K > k_sigma-1) interpolates linearly in the table
// (sigmatheta[2K+1], THETA(K)), K = nk down to k_sigma-1, at sigmatheta[2K] (linint after
// find_place_in_table, epic_funcs_diag.c:3553-3561, epic_funcs_util.c:636-648,2908-2976).  The interval
// found depends on the vertical grid alone: a column kernel finds it once per level for the whole
// block (theta2_intervals, before its first barrier) instead of once per column -- the search's
// fcmp calls are binary64 operations.  kay indexes the ascending table x = sigmatheta[2(nk-kay)+1].
__device__ __forceinline__ int theta2_interval(const DevModel &M, int k) {
  const int nk = M.nk, nkay = nk - (M.k_sigma - 1) + 1;
  const double sg = M.sgth[2 * k];
  auto X = [&](int kay) { return M.sgth[2 * (nk - kay) + 1]; };
  if (fcmp(sg, X(0)) <= 0) return 0;
  if (fcmp(sg, X(nkay - 1)) >= 0) return nkay - 2;
  int il = -1, iu = nkay;
  while (iu - il > 1) {
    const int im = (iu + il) >> 1;
    if (fcmp(sg, X(im)) >= 0) il = im; else iu = im;
  }
  return il;
}
// the intervals of levels k_sigma..nk, and for the binary32 forms (w != nullptr) the weights
// (sigmatheta[2k] - x0) / (x1 - x0) rounded to binary32
__device__ __forceinline__ void theta2_intervals(const DevModel &M, int *kay, float *w) {
  for (int k = M.k_sigma + (int)threadIdx.x; k <= M.nk; k += (int)blockDim.x) {
    const int q = theta2_interval(M, k);
    kay[k] = q;
    if (w) {
      const double x0 = M.sgth[2 * (M.nk - q) + 1], x1 = M.sgth[2 * (M.nk - q - 1) + 1];
      w[k] = (float)((M.sgth[2 * k] - x0) / (x1 - x0));
    }
  }
}

// get_sigma / get_p_sigma / g_sigma / f_sigma / return_sigmatheta, epic_funcs_diag.c:1238-1314,1751-1770
// In the drop-in form the transcendentals are correctly rounded (dd_math.cuh) so that they agree
// with the reference's libm; the mixed form's binary64 kernels take the libdevice functions.
__device__ __forceinline__ double xlog(const DevModel &M, double x) { return M.cr ? cr_log(x, *M.lt) : ::log(x); }
__device__ __forceinline__ double xexp(const DevModel &M, double x) { return M.cr ? cr_exp(x, *M.lt) : ::exp(x); }
__device__ __forceinline__ double xpow(const DevModel &M, double x, double y) { return M.cr ? cr_pow(x, y, *M.lt) : ::pow(x, y); }
__device__ __forceinline__ double get_sigma(const DevModel &M, double pbot, double p, double ptop) {
  return xlog(M, p / pbot) / xlog(M, ptop / pbot);
}
__device__ __forceinline__ double get_p_sigma(const DevModel &M, double pbot, double sigma, double ptop) {
  return pbot * xexp(M, sigma * xlog(M, ptop / pbot));
}
__device__ __forceinline__ double g_sigma(const DevModel &M, double s) {
  if (s <= M.sigma_sigma) return 0.;
  if (s >= 1.) return 1.;
  return M.g_coeff * (1. - xexp(M, -M.alpha * (s - M.sigma_sigma)));
}
__device__ __forceinline__ double f_sigma(const DevModel &M, double s) {
  if (s < 0.) return M.zeta0;
  if (s <= M.sigma_sigma) return M.zeta0 + s * (M.zeta1 - M.zeta0);
  if (s < 1.) return (1. - g_sigma(M, s)) * (M.zeta0 + s * (M.zeta1 - M.zeta0));
  return 0.;
}
// f_sigma(s), with g_sigma(s) returned in g: one exponential serves both.
__device__ __forceinline__ double f_and_g_sigma(const DevModel &M, double s, double &g) {
  g = g_sigma(M, s);
  if (s < 0.) return M.zeta0;
  if (s <= M.sigma_sigma) return M.zeta0 + s * (M.zeta1 - M.zeta0);
  if (s < 1.) return (1. - g) * (M.zeta0 + s * (M.zeta1 - M.zeta0));
  return 0.;
}
__device__ __forceinline__ double return_sigmatheta(const DevModel &M, double theta, double p, double pbot, double ptop) {
  if (p <= ptop) return theta;
  const double s = get_sigma(M, pbot, p, ptop);
  return f_sigma(M, s) + g_sigma(M, s) * theta;
}
// return_density (ideal gas); return_temp and return_enthalpy below (the ideal gas, or hydrogen)
// The hydrogen thermodynamics of thermo_setup's tables (x_h2 > 0; normal hydrogen, fpara = 0.25,
// the para fraction the reference takes when the fpara tracer is off, epic_funcs_diag.c:3709;
// ideal equation of state).  Layout of DevModel::thermo: T(fp, theta_mean) [16][128], the ortho
// and para enthalpies [2][128], the temperature grid [128], the mean potential temperature grid
// [128], the para fractions [16].
constexpr int TH_M = 128, TH_N = 16;
constexpr double TH_FP = 0.25;
__device__ __forceinline__ const double *th_t(const DevModel &M) { return M.thermo; }
__device__ __forceinline__ const double *th_h(const DevModel &M, int q) { return M.thermo + TH_N * TH_M + q * TH_M; }
__device__ __forceinline__ const double *th_tgrid(const DevModel &M) { return M.thermo + TH_N * TH_M + 2 * TH_M; }
__device__ __forceinline__ const double *th_thgrid(const DevModel &M) { return M.thermo + TH_N * TH_M + 3 * TH_M; }
__device__ __forceinline__ const double *th_fpdat(const DevModel &M) { return M.thermo + TH_N * TH_M + 4 * TH_M; }

// return_temp, epic_funcs_diag.c:6112-6210: the ideal relation, or with hydrogen the table of
// temperature against para fraction and mean potential temperature (bilinear).  The hydrogen
// part, from the ideal-gas temperature theta1 = theta (p/p0)^kappa (which the mixed forms' column
// kernels evaluate with their own power):
__device__ __forceinline__ double hydrogen_temp(const DevModel &M, double theta1) {
  if (theta1 <= 20.) return theta1;
  if (theta1 >= 600.)
    return xexp(M, (M.cpr * xlog(M, theta1) - 2.5 * M.x_h2 * ((1. - TH_FP) * -2.105769 + TH_FP * -1.666421)) /
                       (2.5 * M.x_he + 3.5 * (1. - M.x_he)));
  const double *fpdat = th_fpdat(M), *thg = th_thgrid(M), *t = th_t(M);
  const double en = (double)(TH_N - 1) * (TH_FP - fpdat[0]) / (fpdat[TH_N - 1] - fpdat[0]);
  int n = (int)en;
  double ffp, fth;
  if (n > TH_N - 2) { n = TH_N - 2; ffp = 1.; }
  else if (n < 0) { n = 0; ffp = 0.; }
  else ffp = fmod(en, 1.);
  const double em = (double)(TH_M - 1) * (theta1 - thg[0]) / (thg[TH_M - 1] - thg[0]);
  int m = (int)em;
  if (m > TH_M - 2) { m = TH_M - 2; fth = 1.; }
  else if (m < 0) { m = 0; fth = 0.; }
  else fth = fmod(em, 1.);
  return t[n * TH_M + m] * (1. - fth) * (1. - ffp) + t[(n + 1) * TH_M + m] * (1. - fth) * (ffp) +
         t[n * TH_M + m + 1] * (fth) * (1. - ffp) + t[(n + 1) * TH_M + m + 1] * (fth) * (ffp);
}
__device__ __forceinline__ double return_temp(const DevModel &M, double p, double theta) {
  if (M.x_h2 == 0.) return theta * xpow(M, p / M.press0, M.kappa);
  return hydrogen_temp(M, theta * xpow(M, p / M.press0, M.kappa));
}
__device__ __forceinline__ double return_density(double p, double t, double mu) { return p * mu / (8.314472e+3 * t); }
__device__ __forceinline__ double return_enthalpy(const DevModel &M, double t) {
  if (M.x_h2 == 0. || t <= 20.) return (M.cpr * t) * M.rgas;
  double enthalpy;
  if (t > 500.) {   // hydrogen above the table, epic_funcs_diag.c:6699-6712
    const double ho = 1545.3790 + 3.5 * (t - 500.), hp = 1720.3776 + 3.5 * (t - 500.);
    enthalpy = (M.x_h2) * ((1. - TH_FP) * ho + TH_FP * hp) + (M.x_he * 2.5 + M.x_3 * 3.5) * t;
  } else {          // :6713-6735
    const double *tg = th_tgrid(M), *ho = th_h(M, 0), *hp = th_h(M, 1);
    const double em = (double)(TH_M - 1) * (t - tg[0]) / (tg[TH_M - 1] - tg[0]);
    int m = (int)em;
    double fract;
    if (m == TH_M - 1) { m--; fract = 1.; }
    else fract = fmod(em, 1.);
    const double h0 = (1. - fract) * ho[m] + (fract) * ho[m + 1], h1 = (1. - fract) * hp[m] + (fract) * hp[m + 1];
    enthalpy = (M.x_h2) * ((1. - TH_FP) * h0 + (TH_FP) * h1) + (M.x_he * 2.5 + M.x_3 * 3.5) * t;
  }
  return enthalpy * M.rgas;
}
// onto_kk(P2_INDEX) at a layer, epic_funcs_diag.c:2601-2618
__device__ __forceinline__ double layer_p(const DevModel &M, double top, double bot) {
  if (fcmp(bot, top) == 0) return .5 * (bot + top);
  const double kp1 = M.kappa + 1.;
  return xpow(M, (xpow(M, bot, kp1) - xpow(M, top, kp1)) / (kp1 * (bot - top)), 1. / M.kappa);
}

// ---- binary64 <-> binary32 conversions on the integer pipe ----
//
// GB300 executes FP64 arithmetic and the F64<->F32 conversion instructions on the same narrow
// FP64 unit, about 1.7 operations per clock per SM against ~114 for FP32 adds (measured).  The
// mixed form reads its binary64 state in every kernel, so it converts with a few integer
// operations and selects instead (no branch).  For every normal binary32 result, zero,
// infinity and overflow the bits are those of the hardware's round-to-nearest-even conversion;
// a NaN stays a NaN; binary32 subnormals (magnitudes below 1.2e-38, which the model's fields
// never hold except as exact zeros) are flushed to signed zero in both directions.
__device__ __forceinline__ float d2f(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned a = hi & 0x7fffffffu;
  // round the 64-bit pattern to nearest-even at bit 29 (a carry may bump the exponent), then
  // take the 8 low exponent bits and the 23 leading mantissa bits and rebias the exponent
  const unsigned long long v = (((unsigned long long)hi << 32) | lo) + (0x0fffffffull + ((lo >> 29) & 1u));
  unsigned u = (__funnelshift_l((unsigned)v, (unsigned)(v >> 32), 3) - (896u << 23)) | (hi & 0x80000000u);
  if (a - 0x38100000u >= 0x0fe00000u)   // |x| < FLT_MIN (to signed zero), or beyond FLT_MAX, inf, NaN
    u = (hi & 0x80000000u) | (a < 0x38100000u ? 0u : ((a | (lo != 0u)) > 0x7ff00000u ? 0x7fc00000u : 0x7f800000u));
  return __uint_as_float(u);
}
__device__ __forceinline__ double f2d(float f) {
  const unsigned w = __float_as_uint(f), a = w & 0x7fffffffu;
  unsigned hi = (a >> 3) + (896u << 20), lo = a << 29;
  hi = a >= 0x7f800000u ? hi + (896u << 20) : hi;            // infinity, NaN: exponent 2047
  hi = a < 0x00800000u ? 0u : hi;
  lo = a < 0x00800000u ? 0u : lo;
  return __hiloint2double((int)(hi | (w & 0x80000000u)), (int)lo);
}

// ---- binary64 <-> double-float without the FP64 unit ----
//
// The double-float form of x is (hi, lo) = (RN32(x), RN32(x - hi)) and its binary64 value is
// RN64(hi + lo): one FP64 subtraction or addition each, at the FP64 unit's rate.  The mixed
// form's column kernels convert several values per level, so both are computed on the integer
// and FP32 pipes instead, with the same bits: the residual x - hi is the part of x's 53-bit
// significand below hi's rounding point, an integer r (|r| <= 2^28) in units of x's last place,
// rounded to binary32 by one fused multiply-add of two exact halves; hi + lo moves hi's binary64
// significand by lo in units of its last place, rounded to nearest-even by the conversion to
// integer (in the binade below a power of two when lo takes hi towards zero, whose unit is half
// as large; a normalised lo, |lo| <= ulp32(hi)/2, never takes the sum out of those binades).
// Magnitudes below 2^-74 (5e-23, far below any value of the model's fields but exact zeros) keep
// binary32 precision: lo is zero there, and a hi that small converts without its lo.
__device__ __forceinline__ dfl d2df(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned a = hi & 0x7fffffffu;
  const unsigned half = 0x0fffffffu + ((lo >> 29) & 1u);   // d2f's rounding increment
  const unsigned long long v = (((unsigned long long)hi << 32) | lo) + half;
  unsigned u = (__funnelshift_l((unsigned)v, (unsigned)(v >> 32), 3) - (896u << 23)) | (hi & 0x80000000u);
  if (a - 0x38100000u >= 0x0fe00000u)
    u = (hi & 0x80000000u) | (a < 0x38100000u ? 0u : ((a | (lo != 0u)) > 0x7ff00000u ? 0x7fc00000u : 0x7f800000u));
  // x - hi in units of x's last place: the 29 bits below the rounding point, less the carry
  const int r = (int)((unsigned)v & 0x1fffffffu) - (int)half;
  const int rs = (int)hi < 0 ? -r : r;
  // rs = 64 q + b with |q| <= 2^22 and 0 <= b < 64, both exact in binary32 by the 1.5 2^23 and
  // 2^23 shifts; lo = RN32(rs 2^(E-1075)), E the binary64 exponent field, normal for E >= 949
  const float fq = __uint_as_float(0x4B400000u + (unsigned)(rs >> 6)) - 12582912.f;
  const float fb = __uint_as_float(0x4B000000u + ((unsigned)rs & 63u)) - 8388608.f;
  const unsigned e = a >> 20;
  const float sc = e - 949u < 202u ? __uint_as_float((e - 948u) << 23) : 0.f;
  return dfl(__uint_as_float(u), fmaf(fq, 64.f * sc, fb * sc));
}
__device__ __forceinline__ double df2d(dfl x) {
  const unsigned wh = __float_as_uint(x.hi), wl = __float_as_uint(x.lo), ah = wh & 0x7fffffffu, eh = ah >> 23;
  // lo towards zero from a power of two: the binade below, its unit half as large
  const unsigned down = (ah & 0x007fffffu) == 0u && ((wl ^ wh) & 0x80000000u) && (wl & 0x7fffffffu) ? 1u : 0u;
  const bool ok = eh - 52u - down < 202u - down;   // 2^-74 <= |hi| (2^-73 going down), finite
  // lo in units of the last place of hi's binary64 significand: lo 2^(52 - (eh - 127) + down)
  const float sc = __uint_as_float(((ok ? 306u - eh : 127u) + down) << 23);
  const int k = ok ? __float2int_rn(x.lo * sc) : 0;
  unsigned long long mag = ((unsigned long long)ah << 29) + (896ull << 52);
  mag = ah >= 0x7f800000u ? mag + (896ull << 52) : (ah < 0x00800000u ? 0ull : mag);   // f2d's cases
  mag += (long long)((int)wh < 0 ? -k : k);
  return __longlong_as_double((long long)(mag | ((unsigned long long)(wh & 0x80000000u) << 32)));
}

// ---- compute-type helpers for kernels instantiated in FP64 (R = double: the drop-in form,
// bit-identical to the reference's arithmetic) and FP32 (R = float: the mixed form) ----

// a binary64 value in the compute type, and a compute-type value back in binary64
template <class R> __device__ __forceinline__ R cv(double x);
template <> __device__ __forceinline__ double cv<double>(double x) { return x; }
template <> __device__ __forceinline__ float cv<float>(double x) { return d2f(x); }
template <> __device__ __forceinline__ dfl cv<dfl>(double x) { return d2df(x); }
// a model constant in the compute type: the double-float ones come split from the host (the
// same bits as cv<dfl> of the binary64 value), the others by cv
template <class R> __device__ __forceinline__ R mconst(const DevModel &, int, double v) { return cv<R>(v); }
template <> __device__ __forceinline__ dfl mconst<dfl>(const DevModel &M, int q, double) { return dfl(M.dfc[q].x, M.dfc[q].y); }
__device__ __forceinline__ double to_d(double x) { return x; }
__device__ __forceinline__ double to_d(float x) { return f2d(x); }
__device__ __forceinline__ double to_d(dfl x) { return df2d(x); }

template <class R> __device__ __forceinline__ R rmax(R x, R y) { return x > y ? x : y; }
template <class R> __device__ __forceinline__ R rmin(R x, R y) { return x < y ? x : y; }
template <class R> struct RMath;
template <> struct RMath<double> {
  static __device__ __forceinline__ double log(const DevModel &M, double x) { return xlog(M, x); }
  static __device__ __forceinline__ double exp(const DevModel &M, double x) { return xexp(M, x); }
  static __device__ __forceinline__ double pow(const DevModel &M, double x, double y) { return xpow(M, x, y); }
  static __device__ __forceinline__ int cmp(double x1, double x2) { return fcmp(x1, x2); }
  static __device__ __forceinline__ double log_pow(const DevModel &M, double x, double y, double &lg) {
    if (!M.cr) { lg = ::log(x); return ::pow(x, y); }
    return cr_log_pow(x, y, *M.lt, lg);
  }
  static __device__ __forceinline__ double cos4(const DevModel &M, int j) { return M.coslat4[j]; }
};
template <> struct RMath<dfl> {
  static __device__ __forceinline__ dfl log(const DevModel &M, dfl x) { return log_df(x, M.exp2tab); }
  static __device__ __forceinline__ dfl exp(const DevModel &M, dfl x) { return exp_df(x, M.exp2tab); }
  static __device__ __forceinline__ dfl pow(const DevModel &M, dfl x, dfl y) { return exp_df(y * log_df(x, M.exp2tab), M.exp2tab); }
};
template <> struct RMath<float> {
  static __device__ __forceinline__ float log(const DevModel &, float x) { return logf(x); }
  static __device__ __forceinline__ float exp(const DevModel &, float x) { return expf(x); }
  static __device__ __forceinline__ float pow(const DevModel &, float x, float y) { return powf(x, y); }
  static __device__ __forceinline__ float log_pow(const DevModel &, float x, float y, float &lg) {
    lg = logf(x);
    return powf(x, y);
  }
  static __device__ __forceinline__ float cos4(const DevModel &M, int j) { return (float)M.coslat4[j]; }
  // fcmp with the float epsilon
  static __device__ __forceinline__ int cmp(float x1, float x2) {
    int e;
    frexpf(fabsf(x1) > fabsf(x2) ? x1 : x2, &e);
    const float delta = ldexpf(FLT_EPSILON, e);
    const float d = x1 - x2;
    return d > delta ? 1 : (d < -delta ? -1 : 0);
  }
};

struct Trip { double x, y, z; };

__device__ __forceinline__ double pchst(double a, double b) {
  if (a == 0.0) return 0.0;
  if (a < 0.0) return b < 0.0 ? 1.0 : (b == 0.0 ? 0.0 : -1.0);
  return b < 0.0 ? -1.0 : (b == 0.0 ? 0.0 : 1.0);
}
// spline_pchip (Fritsch-Carlson PCHIM slopes), epic_funcs_util.c:721-845; returns false if x not increasing
__device__ __forceinline__ bool spline_pchip(int n, Trip *t) {
  for (int i = 1; i < n; i++)
    if (t[i].x <= t[i - 1].x) return false;
  double h1 = t[1].x - t[0].x;
  double del1 = (t[1].y - t[0].y) / h1;
  if (n == 2) { t[0].z = del1; t[1].z = del1; return true; }
  double h2 = t[2].x - t[1].x;
  double del2 = (t[2].y - t[1].y) / h2;
  double hsum = h1 + h2;
  double w1 = (h1 + hsum) / hsum, w2 = -h1 / hsum;
  t[0].z = w1 * del1 + w2 * del2;
  if (pchst(t[0].z, del1) <= 0.0) t[0].z = 0.0;
  else if (pchst(del1, del2) < 0.0) {
    const double dmx = 3.0 * del1;
    if (fabs(dmx) < fabs(t[0].z)) t[0].z = dmx;
  }
  for (int i = 2; i <= n - 1; i++) {
    if (2 < i) {
      h1 = h2;
      h2 = t[i].x - t[i - 1].x;
      hsum = h1 + h2;
      del1 = del2;
      del2 = (t[i].y - t[i - 1].y) / h2;
    }
    t[i - 1].z = 0.0;
    if (pchst(del1, del2) > 0.0) {
      const double hsumt3 = 3.0 * hsum;
      w1 = (hsum + h1) / hsumt3;
      w2 = (hsum + h2) / hsumt3;
      const double dmx = dmaxr(fabs(del1), fabs(del2)), dmn = dminr(fabs(del1), fabs(del2));
      t[i - 1].z = dmn / (w1 * (del1 / dmx) + w2 * (del2 / dmx));
    }
  }
  w1 = -h2 / hsum;
  w2 = (h2 + hsum) / hsum;
  t[n - 1].z = w1 * del1 + w2 * del2;
  if (pchst(t[n - 1].z, del2) <= 0.0) t[n - 1].z = 0.0;
  else if (pchst(del1, del2) < 0.0) {
    const double dmx = 3.0 * del2;
    if (fabs(dmx) < fabs(t[n - 1].z)) t[n - 1].z = dmx;
  }
  return true;
}
// splint_pchip, epic_funcs_util.c:926-946
__device__ __forceinline__ double splint_pchip(double xx, const Trip *t, double h) {
  const double delta = (t[1].y - t[0].y) / h;
  const double del1 = (t[0].z - delta) / h;
  const double del2 = (t[1].z - delta) / h;
  const double c3 = (del1 + del2) / h;
  const double c2 = -(del1 + del1 + del2);
  const double x = xx - t[0].x;
  return t[0].y + x * (t[0].z + x * (c2 + x * c3));
}
// find_place_in_table (ascending tables only), epic_funcs_util.c:2908-2967
__device__ __forceinline__ int find_place_in_table(int n, const Trip *t, double x, double *dx) {
  if (fcmp(x, t[0].x) <= 0) { *dx = t[1].x - t[0].x; return 0; }
  if (fcmp(x, t[n - 1].x) >= 0) { *dx = t[n - 1].x - t[n - 2].x; return n - 2; }
  int il = -1, iu = n;
  while (iu - il > 1) {
    const int im = (iu + il) >> 1;
    if (fcmp(x, t[im].x) >= 0) il = im; else iu = im;
  }
  *dx = t[il + 1].x - t[il].x;
  return il;
}

// get_kin (the Suarez-Takacs blend for the Sadourney scheme, epic_funcs_diag.c:2694-2847) at h-point
// (j, i) of the layer planes Uk, Vk
template <class R>
__device__ __forceinline__ R kin_at(const DevModel &M, const double *Uk, const double *Vk, int j, int i) {
  const int jj = 2 * j;
  const R mn1 = cv<R>(M.mn[jj + 1]), mni0 = cv<R>(M.mn_inv[jj]), mni2 = cv<R>(M.mn_inv[jj + 2]);
  R u2 = cv<R>(Uk[M.at2(j, i)]), u4 = cv<R>(Uk[M.at2(j, i + 1)]), v2 = cv<R>(Vk[M.at2(j, i)]), v4 = cv<R>(Vk[M.at2(j + 1, i)]);
  const R kin_c = (u2 * u2 + u4 * u4 + mn1 * (v2 * v2 * mni0 + v4 * v4 * mni2)) * R(.25);
  if (j == 0 || j == M.nj) return kin_c;
  u2 = R(.5) * (cv<R>(Uk[M.at2(j + 1, i)]) + cv<R>(Uk[M.at2(j - 1, i)]));
  u4 = R(.5) * (cv<R>(Uk[M.at2(j + 1, i + 1)]) + cv<R>(Uk[M.at2(j - 1, i + 1)]));
  v2 = R(.5) * (cv<R>(Vk[M.at2(j, i + 1)]) + cv<R>(Vk[M.at2(j, i - 1)]));
  v4 = R(.5) * (cv<R>(Vk[M.at2(j + 1, i + 1)]) + cv<R>(Vk[M.at2(j + 1, i - 1)]));
  const R kin_s = (u2 * u2 + u4 * u4 + mn1 * (v2 * v2 * mni0 + v4 * v4 * mni2)) * R(.25);
  return (R(5.) / R(6.)) * kin_c + (R(1.) / R(6.)) * kin_s;
}
// Record the first model error (the reference would epic_error() and exit).
__device__ __forceinline__ void flag_error(Ctl *c, int code, int k, int j, int i, double v) {
  if (atomicCAS(&c->err_code, 0, code) == 0) {
    c->err_k = k; c->err_j = j; c->err_i = i; c->err_val = v;
  }
}

// The mixed forms' pressure gradient reads GZ3 and P2 as (hi, lo) binary32 splits, hi = float(x),
// lo = float(x - hi), kept in the scratch volumes work1 (GZ3) and work2 (P2) from the kernels that
// write the two fields before it (store_pgrad_vars and set_p2etc of stages 19 and 11, and the
// polar rows of GZ3 in uv_pgrad itself) to the pressure gradient.
__device__ __forceinline__ void put_split(double *work, long long x, double v) {
  const dfl d = d2df(v);
  reinterpret_cast<float2 *>(work)[x] = make_float2(d.hi, d.lo);
}

// Zonal periodicity of one row: pads i = 0 and i = ni+1 (bc_lateral, src/single/s_epic_functions.c:55-59).
// Called by the thread that owns interior cell i after it wrote the final value.
__device__ __forceinline__ void write_with_pads(double *a, const DevModel &M, long long rowbase, int i, double val) {
  a[rowbase + i] = val;
  if (i == M.ni) a[rowbase] = val;
  if (i == 1) a[rowbase + M.ni + 1] = val;
}

}  // namespace epic

// Kernel launch helpers.
#define EPIC_CUDA_CHECK(x)                                                     \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) return epic::set_error(EPIC_ERR_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

inline unsigned epic_blocks(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }
