/*
 * CPU restatement of the reference EPIC Held-Suarez step -- the oracle (test infrastructure).
 *
 * Only tests, the smoke check and the CPU-baseline leg of bench.py load this library.  It
 * restates the reference functions with the same operation order, so that compiled with
 * -O2 -ffp-contract=off on x86-64 it reproduces the reference build bit for bit.  Reference
 * quirks that change results are reproduced and marked QUIRK.
 *
 * Layout: X(k,j,i) = base[i + (j+1)*iadim + k*n2] (include/epic.h:407-449).
 */
#include "epic_port.h"

#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define DEG (M_PI / 180.)
#define R_GAS 8.314472e+3                 /* include/epic.h:188 */
#define EP_EPS_HSU 1.e-10                 /* ep in hsu_advection, epic_flux.c:711 */
#define DLOGZ_TOL 1.e-2                   /* epic_timestep.c:907 */
#define GAMMA_ASSELIN 0.06                /* epic_timestep.c:512 */

typedef struct { double x, y, z; } trip;  /* float_triplet */

struct ep_model {
  epic_grid g;
  int ni, nj, nk, iadim, jadim, kadim;
  long n2, n3;
  int nvp, ntp;             /* wind value / tendency planes */
  /* copies of the grid arrays */
  double *lon, *lat, *rln, *rlt, *f, *m, *n, *mn, *grav, *sgth, *dsgth, *dsgth_inv, *h_min, *t_sponge_inv;
  /* state (reference layout) */
  double *u, *v, *dudt, *dvdt, *hdry, *theta, *p3, *h3, *p2, *theta2, *t2, *t3, *rho2, *rho3, *exner3;
  double *gz3, *mont3, *heat3, *pv3, *ri2, *div_uv3, *w3, *dzdt3, *u_spinup, *gz_surface;
  /* scratch */
  double *gz, *sum_div, *unity, *old, *varz;
  double *b2d[8];
  double *data;             /* [ni+1], 1-based */
  trip *table;              /* [nk+2] */
  double *high_lat_h, *high_lat_pv;
  trip *h_coef, *v_coef;
  double *mn_inv;
  /* hsu_advection column buffers (static in the reference) */
  double *wm, *wp, *w_a, *w_a_pred, *w_a_min, *w_ff, *w_a_diff1, *w_a_diff2, *w_aaa;
  double coef[9], max_nu[9], m0, n0, mu_dry, eps13;
  /* turbulence closure (g.turbulence): NU_TURB, the eddy diffusivities, column buffers of
   * crank_nicolson and the band solver, and the first error a wall function meets */
  double *nu_turb, *dc_uv, *dc_theta, *dc_mass;
  double *cz, *ca, *cd, *crho, *cans, *sf0, *sf2, *ri, *tb, *tl, *tr, *taorig, *tal;
  int *tindex;
  char turb_err[160];
  /* hydrogen thermodynamics (x_h2 > 0): thermo_setup's tables */
  double th_t[16][128], th_array[5][128], th_tgrid[128], th_thetagrid[128], th_fpdat[16];
  int it_zero, it_minus1, it_minus2, it_uv, it_uv_dis, it_uv_tend;
  long itime, model_time;
  int uploaded;
  char err[256];
};

static char create_err[256];

static int fail(ep_model *M, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(M->err, sizeof(M->err), fmt, ap);
  va_end(ap);
  return -4;
}

#define IX(M, k, j, i) ((long)(i) + (long)((j) + 1) * (M)->iadim + (long)(k) * (M)->n2)
#define IX2(M, j, i) ((long)(i) + (long)((j) + 1) * (M)->iadim)
#define A3(a, k, j, i) (a)[IX(M, k, j, i)]
#define A2(a, j, i) (a)[IX2(M, j, i)]
#define DT ((double)M->g.dt)
#define KHI (M->nk)
#define NJ (M->nj)
#define NI (M->ni)
#define LAT0 (M->g.lat0)
/* the turbulence closure (epic_grid.turbulence, grid.diffusion_direction) */
#define KINVISC (M->g.kinvisc)
#define SA_CV1_3 (7.1 * 7.1 * 7.1)
#define TURB_ON(M) ((M)->g.turbulence == EPIC_TURB_SA_DES)
#define DIFF_HORIZONTAL(M) ((M)->g.diffusion_direction == EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL || \
                            (M)->g.diffusion_direction == EPIC_DIFFUSION_JUST_HORIZONTAL)
#define DIFF_VERTICAL(M) ((M)->g.diffusion_direction == EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL || \
                          (M)->g.diffusion_direction == EPIC_DIFFUSION_JUST_VERTICAL)

static inline double dmax(double x, double y) { return x > y ? x : y; }  /* MAX, include/epic.h:144 */
static inline double dmin(double x, double y) { return x < y ? x : y; }  /* MIN, include/epic.h:138 */

/* ---------------------------------------------------------------------------------------- */
/* Numerical utilities (src/shared/epic_funcs_util.c)                                        */
/* ---------------------------------------------------------------------------------------- */

/* fcmp, epic_funcs_util.c:4275-4330 */
static int fcmp(double x1, double x2) {
  int exponent;
  double delta, difference;
  frexp(fabs(x1) > fabs(x2) ? x1 : x2, &exponent);
  delta = ldexp(DBL_EPSILON, exponent);
  difference = x1 - x2;
  if (difference > delta) return 1;
  if (difference < -delta) return -1;
  return 0;
}

/* pchst (sign of a*b without the product), epic_funcs_util.c:1000-1030 */
static double pchst(double a, double b) {
  if (a == 0.0) return 0.0;
  if (a < 0.0) return b < 0.0 ? 1.0 : (b == 0.0 ? 0.0 : -1.0);
  return b < 0.0 ? -1.0 : (b == 0.0 ? 0.0 : 1.0);
}

/* spline_pchip (Fritsch-Carlson monotone slopes, PCHIM), epic_funcs_util.c:721-845 */
static int spline_pchip(int n, trip *t) {
  int i;
  double del1, del2, dmx, dmn, drat1, drat2, h1, h2, hsum, hsumt3, w1, w2;
  if (n < 2) return -1;
  for (i = 1; i < n; i++)
    if (t[i].x <= t[i - 1].x) return -3;
  h1 = t[1].x - t[0].x;
  del1 = (t[1].y - t[0].y) / h1;
  if (n == 2) { t[0].z = del1; t[1].z = del1; return 0; }
  h2 = t[2].x - t[1].x;
  del2 = (t[2].y - t[1].y) / h2;
  hsum = h1 + h2;
  w1 = (h1 + hsum) / hsum;
  w2 = -h1 / hsum;
  t[0].z = w1 * del1 + w2 * del2;
  if (pchst(t[0].z, del1) <= 0.0) t[0].z = 0.0;
  else if (pchst(del1, del2) < 0.0) {
    dmx = 3.0 * del1;
    if (fabs(dmx) < fabs(t[0].z)) t[0].z = dmx;
  }
  for (i = 2; i <= n - 1; i++) {
    if (2 < i) {
      h1 = h2;
      h2 = t[i].x - t[i - 1].x;
      hsum = h1 + h2;
      del1 = del2;
      del2 = (t[i].y - t[i - 1].y) / h2;
    }
    t[i - 1].z = 0.0;
    if (pchst(del1, del2) > 0.0) {
      hsumt3 = 3.0 * hsum;
      w1 = (hsum + h1) / hsumt3;
      w2 = (hsum + h2) / hsumt3;
      dmx = dmax(fabs(del1), fabs(del2));
      dmn = dmin(fabs(del1), fabs(del2));
      drat1 = del1 / dmx;
      drat2 = del2 / dmx;
      t[i - 1].z = dmn / (w1 * drat1 + w2 * drat2);
    }
  }
  w1 = -h2 / hsum;
  w2 = (h2 + hsum) / hsum;
  t[n - 1].z = w1 * del1 + w2 * del2;
  if (pchst(t[n - 1].z, del2) <= 0.0) t[n - 1].z = 0.0;
  else if (pchst(del1, del2) < 0.0) {
    dmx = 3.0 * del2;
    if (fabs(dmx) < fabs(t[n - 1].z)) t[n - 1].z = dmx;
  }
  return 0;
}

/* splint_pchip (cubic Hermite evaluation, CHFEV), epic_funcs_util.c:926-946 */
static double splint_pchip(double xx, const trip *t, double h) {
  double c2, c3, del1, del2, delta, x;
  delta = (t[1].y - t[0].y) / h;
  del1 = (t[0].z - delta) / h;
  del2 = (t[1].z - delta) / h;
  c3 = (del1 + del2) / h;
  c2 = -(del1 + del1 + del2);
  x = xx - t[0].x;
  return t[0].y + x * (t[0].z + x * (c2 + x * c3));
}

/* linint, epic_funcs_util.c:636-646 */
static double linint(double xx, const trip *t, double dx) { return t->y + ((t + 1)->y - t->y) * (xx - t->x) / dx; }

/* find_place_in_table (bisection), epic_funcs_util.c:2908-2967 */
static int find_place_in_table(int n, const trip *t, double x, double *dx) {
  int il = -1, iu = n, im, ascend, cmplo, cmphi;
  ascend = (t[n - 1].x >= t[0].x);
  cmplo = fcmp(x, t[0].x);
  cmphi = fcmp(x, t[n - 1].x);
  if (ascend) {
    if (cmplo <= 0) { *dx = t[1].x - t[0].x; return 0; }
    if (cmphi >= 0) { *dx = t[n - 1].x - t[n - 2].x; return n - 2; }
  } else {
    if (cmplo >= 0) { *dx = t[1].x - t[0].x; return 0; }
    if (cmphi <= 0) { *dx = t[n - 1].x - t[n - 2].x; return n - 2; }
  }
  while (iu - il > 1) {
    im = (iu + il) >> 1;
    if ((fcmp(x, t[im].x) >= 0) == ascend) il = im;
    else iu = im;
  }
  *dx = t[il + 1].x - t[il].x;
  return il;
}

/* four1: radix-2 complex FFT of Numerical Recipes in C (2nd ed., p. 507), as restated by
 * epic_funcs_util.c:4023-4076; data is 1-based, nn complex points. */
static void four1(double *data, unsigned long nn, int isign) {
  unsigned long n, mmax, m, j, istep, i;
  double tempr, tempi, wtemp, wr, wpr, wpi, wi, theta;
  n = nn << 1;
  j = 1;
  for (i = 1; i < n; i += 2) {
    if (j > i) {
      tempr = data[j]; data[j] = data[i]; data[i] = tempr;
      tempr = data[j + 1]; data[j + 1] = data[i + 1]; data[i + 1] = tempr;
    }
    m = n >> 1;
    while (m >= 2 && j > m) { j -= m; m >>= 1; }
    j += m;
  }
  mmax = 2;
  while (n > mmax) {
    istep = mmax << 1;
    theta = isign * (2 * M_PI / mmax);
    wtemp = sin(0.5 * theta);
    wpr = -2.0 * wtemp * wtemp;
    wpi = sin(theta);
    wr = 1.0;
    wi = 0.0;
    for (m = 1; m < mmax; m += 2) {
      for (i = m; i <= n; i += istep) {
        j = i + mmax;
        tempr = wr * data[j] - wi * data[j + 1];
        tempi = wr * data[j + 1] + wi * data[j];
        data[j] = data[i] - tempr;
        data[j + 1] = data[i + 1] - tempi;
        data[i] += tempr;
        data[i + 1] += tempi;
      }
      wr = (wtemp = wr) * wpr - wi * wpi + wr;
      wi = wi * wpr + wtemp * wpi + wi;
    }
    mmax = istep;
  }
}

/* realft: real FFT of Numerical Recipes in C (2nd ed., p. 513), as restated by
 * epic_funcs_util.c:4084-4132; the inverse must be scaled by 2/n by the caller. */
static void realft(double *data, unsigned long n, int isign) {
  unsigned long i, i1, i2, i3, i4, np3;
  double c1 = 0.5, c2, h1r, h1i, h2r, h2i, wr, wi, wpr, wpi, wtemp, theta;
  theta = M_PI / (double)(n >> 1);
  if (isign == 1) {
    c2 = -0.5;
    four1(data, n >> 1, 1);
  } else {
    c2 = 0.5;
    theta = -theta;
  }
  wtemp = sin(0.5 * theta);
  wpr = -2.0 * wtemp * wtemp;
  wpi = sin(theta);
  wr = 1.0 + wpr;
  wi = wpi;
  np3 = n + 3;
  for (i = 2; i <= (n >> 2); i++) {
    i1 = i + i - 1;
    i2 = 1 + i1;
    i3 = np3 - i2;
    i4 = 1 + i3;
    h1r = c1 * (data[i1] + data[i3]);
    h1i = c1 * (data[i2] - data[i4]);
    h2r = -c2 * (data[i2] + data[i4]);
    h2i = c2 * (data[i1] - data[i3]);
    data[i1] = h1r + wr * h2r - wi * h2i;
    data[i2] = h1i + wr * h2i + wi * h2r;
    data[i3] = h1r - wr * h2r + wi * h2i;
    data[i4] = -h1i + wr * h2i + wi * h2r;
    wr = (wtemp = wr) * wpr - wi * wpi + wr;
    wi = wi * wpr + wtemp * wpi + wi;
  }
  if (isign == 1) {
    data[1] = (h1r = data[1]) + data[2];
    data[2] = h1r - data[2];
  } else {
    data[1] = c1 * ((h1r = data[1]) + data[2]);
    data[2] = c1 * (h1r - data[2]);
    four1(data, n >> 1, -1);
  }
}

/* ---------------------------------------------------------------------------------------- */
/* Coordinate and thermodynamic helpers (src/shared/epic_funcs_diag.c), HS: x_h2 = 0, nq = 0  */
/* ---------------------------------------------------------------------------------------- */

static double get_sigma(double pbot, double p, double ptop) { return log(p / pbot) / log(ptop / pbot); } /* :1751 */
static double get_p_sigma(double pbot, double sigma, double ptop) { return pbot * exp(sigma * log(ptop / pbot)); } /* :1765 */
static double g_sigma(const ep_model *M, double sigma) { /* :1300-1314 */
  const double coeff = 1. / (1 - exp(-M->g.hybrid_alpha * (1. - M->g.sigma_sigma)));
  if (sigma <= M->g.sigma_sigma) return 0.;
  if (sigma >= 1.) return 1.;
  return coeff * (1. - exp(-M->g.hybrid_alpha * (sigma - M->g.sigma_sigma)));
}
static double f_sigma(const ep_model *M, double sigma) { /* :1271-1289 */
  if (sigma < 0.) return M->g.zeta0;
  if (sigma <= M->g.sigma_sigma) return M->g.zeta0 + sigma * (M->g.zeta1 - M->g.zeta0);
  if (sigma < 1.) return (1. - g_sigma(M, sigma)) * (M->g.zeta0 + sigma * (M->g.zeta1 - M->g.zeta0));
  return 0.;
}
static double return_sigmatheta(const ep_model *M, double theta, double p, double pbot, double ptop) { /* :1238-1260 */
  double sigma;
  if (p <= ptop) return theta;
  sigma = get_sigma(pbot, p, ptop);
  return f_sigma(M, sigma) + g_sigma(M, sigma) * theta;
}
/* Hydrogen thermodynamics (x_h2 > 0), after thermo_setup (epic_funcs_diag.c:5864-6105): per
 * temperature T_i = 500 (i+1)/128 K the rotational partition sums of ortho and para H2 (Dowling et
 * al. 1998, appendix A), their enthalpies, curly F, the equilibrium para fraction and the ortho and
 * para potential temperatures; then, for 16 para fractions, the temperature on a grid of mean
 * potential temperatures 20..600 K by linear interpolation of the inverted relation.  Where the
 * reference's inversion search does not find a bracketing entry it reads one past its arrays; here
 * the last interval extrapolates (those entries belong to mean potential temperatures the runs never
 * reach). */
#define MDIM_TH 128
#define NDIM_TH 16
#define THLO_TH 20.
#define THHI_TH 600.
#define CCOLN_TH -2.105769
#define CCPLN_TH -1.666421
#define CPRH2 2.5
#define CPRHE 2.5
#define CPR3 3.5
#define FPARA_NORMAL 0.25   /* the para fraction when the fpara tracer is off, epic_funcs_diag.c:3709 */
static void thermo_setup(ep_model *M) {
  const double xh2 = M->g.x_h2, xhe = M->g.x_he, x3 = M->g.x_3;
  const double cpr = (CPRH2 * xh2 + CPRHE * xhe + CPR3 * x3) / (xh2 + xhe + x3);
  const double t0 = 1., p0 = 1.e+5, theta = 87.567, ndeg[2] = {3., 1.};
  const double c1 = log(1.3806503e-23 * t0 / p0 * pow(2. * M_PI * (1.67262158e-27 / 6.62606876e-34) * (1.3806503e-23 * t0 / 6.62606876e-34), 1.5));
  const double c2 = log(9.);
  const double p = p0;
  double temp[MDIM_TH], tho[MDIM_TH], thp[MDIM_TH], tvec[MDIM_TH], thvec[MDIM_TH], aa[MDIM_TH];
  int i, j, m, n;
  for (i = 0; i < MDIM_TH; i++) {
    const double temperature = 500. * (double)(i + 1) / (double)MDIM_TH;
    double ho, hp, pottempo, pottempp, ff, a[8];
    if (temperature < 10.) {
      ho = CPRH2 * temperature;
      hp = CPRH2 * temperature;
      pottempo = temperature;
      pottempp = temperature;
      a[0] = 1.; a[1] = 175.1340; a[2] = 0.; a[3] = 0.; a[4] = 0.; a[5] = 0.; a[6] = 0.; a[7] = 0.;
      ff = 0.;
    } else {
      double y = theta / temperature, z[3][2], term = 0., den, so, sp;
      int jn[2];
      y = dmin(y, 30.);
      for (n = 0; n < 2; n++)
        for (m = 0; m < 3; m++) z[m][n] = 0.;
      for (j = 1; j <= 50; j++) {
        jn[0] = 2 * j - 1;
        jn[1] = jn[0] - 1;
        for (n = 0; n < 2; n++) {
          term = ndeg[n] * (2 * jn[n] + 1) * exp(-jn[n] * (jn[n] + 1) * y);
          for (m = 0; m < 3; m++) {
            z[m][n] += term;
            if (m < 2) term *= jn[n] * (jn[n] + 1);
          }
        }
        if (j > 1 && term < 1.e-20) break;
      }
      den = z[0][0] + z[0][1];
      a[0] = z[0][1] / den;
      for (n = 0; n < 2; n++) {
        a[n + 1] = theta * z[1][n] / z[0][n];
        a[n + 3] = y * y * (z[0][n] * z[2][n] - z[1][n] * z[1][n]) / (z[0][n] * z[0][n]);
        a[n + 5] = log(z[0][n]);
      }
      a[7] = (1. - a[0]) * a[3] + a[0] * a[4] + (a[2] - a[1]) * y / temperature * (z[1][1] * z[0][0] - z[0][1] * z[1][0]) / (den * den);
      ho = a[1] + CPRH2 * temperature - 2. * theta;
      hp = a[2] + CPRH2 * temperature;
      so = -log(p / p0) + 2.5 * log(temperature) + 1.5 * M_LN2 + c1 + (ho + 2. * theta) / temperature + a[5];
      sp = -log(p / p0) + 2.5 * log(temperature) + 1.5 * M_LN2 + c1 + hp / temperature + a[6];
      pottempo = exp(0.4 * (so - c2 - 1.5 * M_LN2 - c1 - 2.5));
      pottempp = exp(0.4 * (sp - 1.5 * M_LN2 - c1 - 2.5));
      ff = -(so - c2 - 1.5 * M_LN2 - c1 - 2.5 - ho / temperature) + (sp - 1.5 * M_LN2 - c1 - 2.5 - hp / temperature);
      ff *= temperature;
    }
    temp[i] = temperature;
    tho[i] = pottempo;
    thp[i] = pottempp;
    M->th_array[0][i] = ho;
    M->th_array[1][i] = hp;
    M->th_array[2][i] = ff;
    M->th_array[3][i] = a[0];
    M->th_array[4][i] = a[1] - a[2];
    M->th_tgrid[i] = temperature;
  }
  for (m = 0; m < MDIM_TH; m++)
    M->th_thetagrid[m] = (THLO_TH * (double)(MDIM_TH - (m + 1)) + THHI_TH * (double)(m)) / (double)(MDIM_TH - 1);
  for (n = 0; n < NDIM_TH; n++) {
    M->th_fpdat[n] = ((double)(n)) / (double)(NDIM_TH - 1);
    for (i = 0; i < MDIM_TH; i++) {
      const double thetaln = (xh2 * CPRH2 * ((1. - M->th_fpdat[n]) * log(tho[i]) + (M->th_fpdat[n]) * log(thp[i])) +
                              (xhe * CPRHE + x3 * CPR3) * log(temp[i])) / cpr;
      thvec[i] = exp(thetaln);
      tvec[i] = temp[i];
    }
    for (j = 0; j < MDIM_TH; j++) aa[j] = tvec[j];
    tvec[MDIM_TH - 1] = aa[MDIM_TH - 1];
    for (i = 0; i < MDIM_TH; i++) {
      for (j = 1; j < MDIM_TH; j++)
        if (thvec[j] >= M->th_thetagrid[i]) break;
      if (j == MDIM_TH) j = MDIM_TH - 1;
      tvec[i] = aa[j - 1] + (aa[j] - aa[j - 1]) * (M->th_thetagrid[i] - thvec[j - 1]) / (thvec[j] - thvec[j - 1]);
    }
    for (m = 0; m < MDIM_TH; m++) M->th_t[n][m] = tvec[m];
  }
}

/* return_temp, :6112-6210: x_h2 = 0 the ideal relation; x_h2 > 0 the table of thermo_setup at
 * fp = 0.25 (bilinear in fp and the mean potential temperature), ideal equation of state */
static double return_temp(const ep_model *M, double p, double theta) {
  double theta1, en, em, fract_fp, fract_theta;
  int n, m;
  if (M->g.x_h2 == 0.) return theta * pow(p / M->g.press0, M->g.kappa);
  theta1 = theta * pow(p / M->g.press0, M->g.kappa);
  if (theta1 <= THLO_TH) return theta1;
  if (theta1 >= THHI_TH)
    return exp((M->g.cpr * log(theta1) - CPRH2 * M->g.x_h2 * ((1. - FPARA_NORMAL) * CCOLN_TH + FPARA_NORMAL * CCPLN_TH)) /
               (CPRHE * M->g.x_he + CPR3 * (1. - M->g.x_he)));
  en = (double)(NDIM_TH - 1) * (FPARA_NORMAL - M->th_fpdat[0]) / (M->th_fpdat[NDIM_TH - 1] - M->th_fpdat[0]);
  n = (int)en;
  if (n > NDIM_TH - 2) { n = NDIM_TH - 2; fract_fp = 1.; }
  else if (n < 0) { n = 0; fract_fp = 0.; }
  else fract_fp = fmod(en, 1.);
  em = (double)(MDIM_TH - 1) * (theta1 - M->th_thetagrid[0]) / (M->th_thetagrid[MDIM_TH - 1] - M->th_thetagrid[0]);
  m = (int)em;
  if (m > MDIM_TH - 2) { m = MDIM_TH - 2; fract_theta = 1.; }
  else if (m < 0) { m = 0; fract_theta = 0.; }
  else fract_theta = fmod(em, 1.);
  return M->th_t[n][m] * (1. - fract_theta) * (1. - fract_fp) + M->th_t[n + 1][m] * (1. - fract_theta) * (fract_fp) +
         M->th_t[n][m + 1] * (fract_theta) * (1. - fract_fp) + M->th_t[n + 1][m + 1] * (fract_theta) * (fract_fp);
}
/* return_density, ideal gas, :6353-6385 */
static double return_density(double p, double temperature, double mu) { return p * mu / (R_GAS * temperature); }
/* return_enthalpy, :6652-6746: x_h2 = 0 cpr*T*rgas; x_h2 > 0 the ortho/para enthalpies of
 * thermo_setup's table at fp = 0.25, ideal equation of state */
static double return_enthalpy(const ep_model *M, double temperature) {
  double enthalpy;
  if (M->g.x_h2 == 0.) {
    enthalpy = M->g.cpr * temperature;
  } else if (temperature <= 20.) {   /* hydrogen, :6692-6740, fp = 0.25, ideal */
    enthalpy = M->g.cpr * temperature;
  } else if (temperature > 500.) {
    const double ho = 1545.3790 + 3.5 * (temperature - 500.), hp = 1720.3776 + 3.5 * (temperature - 500.);
    enthalpy = (M->g.x_h2) * ((1. - FPARA_NORMAL) * ho + FPARA_NORMAL * hp) + (M->g.x_he * 2.5 + M->g.x_3 * 3.5) * temperature;
  } else {
    const double em = (double)(MDIM_TH - 1) * (temperature - M->th_tgrid[0]) / (M->th_tgrid[MDIM_TH - 1] - M->th_tgrid[0]);
    int m = (int)em;
    double fract, h0, h1;
    if (m == MDIM_TH - 1) { m--; fract = 1.; }
    else fract = fmod(em, 1.);
    h0 = (1. - fract) * M->th_array[0][m] + (fract) * M->th_array[0][m + 1];
    h1 = (1. - fract) * M->th_array[1][m] + (fract) * M->th_array[1][m + 1];
    enthalpy = (M->g.x_h2) * ((1. - FPARA_NORMAL) * h0 + (FPARA_NORMAL) * h1) + (M->g.x_he * 2.5 + M->g.x_3 * 3.5) * temperature;
  }
  return enthalpy * M->g.rgas;
}
/* onto_kk for P2_INDEX at a layer, :2601-2618 */
static double layer_p(const ep_model *M, double topval, double botval) {
  double kappap1;
  if (fcmp(botval, topval) == 0) return .5 * (botval + topval);
  kappap1 = M->g.kappa + 1.;
  return pow((pow(botval, kappap1) - pow(topval, kappap1)) / (kappap1 * (botval - topval)), 1. / M->g.kappa);
}
/* get_h at a layer (kk = 2K), :1802-1815 */
static double get_h_layer(const ep_model *M, int K, int J, int I) {
  return (A3(M->p3, K, J, I) - A3(M->p3, K - 1, J, I)) / (M->grav[2 * J + 1] * M->dsgth[2 * K]);
}
/* get_h at an interface (kk = 2K+1), :1816-1833 with onto_kk's default weighting, :2661-2677 */
static double get_h_iface(const ep_model *M, int K, int J, int I) {
  int kk = 2 * K + 1;
  double topwt, botwt;
  if (K == 0) return get_h_layer(M, 1, J, I);
  if (K == KHI) return get_h_layer(M, KHI, J, I);
  topwt = M->dsgth[kk - 1];
  botwt = M->dsgth[kk + 1];
  return (topwt * get_h_layer(M, K, J, I) + botwt * get_h_layer(M, K + 1, J, I)) / (topwt + botwt);
}

/* bc_lateral, src/single/s_epic_functions.c:39-87 */
static void bc2(const ep_model *M, double *a) {
  int J;
  for (J = 0; J <= NJ + 1; J++) {
    A2(a, J, 0) = A2(a, J, NI);
    A2(a, J, NI + 1) = A2(a, J, 1);
  }
}
static void bc3(const ep_model *M, double *a) {
  int K;
  for (K = 0; K <= KHI + 1; K++) bc2(M, a + K * M->n2);
}

/* ---------------------------------------------------------------------------------------- */
/* Zonal filter, src/shared/epic_adjust.c:102-480                                            */
/* ---------------------------------------------------------------------------------------- */

enum { IDX_U = 0, IDX_V = 1, IDX_HDRY = 2, IDX_THETA = 3, IDX_OTHER = 4, IDX_NU = 5 };

static void filter_tables(ep_model *M) { /* the initialisation block, epic_adjust.c:132-241 */
  double lat0 = M->g.lat0 * DEG, rln0, rlt0, r, tmp0, tmp1, re = M->g.re, rp = M->g.rp;
  int J, I;
  rln0 = re / sqrt(1. + pow(rp / re * tan(lat0), 2.));
  rlt0 = rln0 / (cos(lat0) * (pow(sin(lat0), 2.) + pow(re / rp * cos(lat0), 2.)));
  M->m0 = 1. / (rln0 * M->g.dln * DEG);
  M->n0 = 1. / (rlt0 * M->g.dlt * DEG);
  for (J = 0; J <= NJ; J++) {
    A2(M->high_lat_h, J, 1) = 1.;
    r = M->mn[2 * J + 1] / (M->m[2 * J + 1] * M->n[2 * J + 1]);
    tmp0 = (M->n[2 * J + 1] / M->n0) / (M->m[2 * J + 1] / M->m0);
    tmp0 = pow(tmp0, 2.);
    for (I = 2; I <= NI / 2 + 1; I++) {
      tmp1 = sin((I - 1) * (M->g.dln) * DEG / 2.);
      tmp1 = pow(tmp1, -2.);
      tmp1 *= r * tmp0;
      tmp1 = (tmp1 < 1.) ? tmp1 : 1.;
      A2(M->high_lat_h, J, I) = tmp1;
    }
  }
  for (J = 1; J <= NJ; J++) {
    A2(M->high_lat_pv, J, 1) = 1.;
    r = M->mn[2 * J] / (M->m[2 * J] * M->n[2 * J]);
    tmp0 = (M->n[2 * J] / M->n0) / (M->m[2 * J] / M->m0);
    tmp0 = pow(tmp0, 2.);
    for (I = 2; I <= NI / 2 + 1; I++) {
      tmp1 = sin((I - 1) * (M->g.dln) * DEG / 2.);
      tmp1 = pow(tmp1, -2.);
      tmp1 *= r * tmp0;
      tmp1 = (tmp1 < 1.) ? tmp1 : 1.;
      A2(M->high_lat_pv, J, I) = tmp1;
    }
  }
}

/* Filter one row of plane `a` in place (the realft block of epic_adjust.c:412-431). */
static void filter_row(ep_model *M, double *a, int J, const double *hl) {
  double *data = M->data;
  int I;
  for (I = 1; I <= NI; I++) data[I] = A2(a, J, I);
  realft(data, NI, 1);
  data[1] *= A2(hl, J, 1);
  for (I = 2; I <= NI / 2; I++) {
    data[2 * I - 1] *= A2(hl, J, I);
    data[2 * I] *= A2(hl, J, I);
  }
  data[2] *= A2(hl, J, NI / 2 + 1);
  realft(data, NI, -1);
  for (I = 1; I <= NI; I++) A2(a, J, I) = data[I] * (2. / (NI));
}

/* Rows of one plane: v/pv grid (index V) or h/u grid (everything else). */
static void filter_plane_rows(ep_model *M, double *a, int vgrid) {
  int J;
  if (vgrid) {
    for (J = 1; J <= NJ; J++) {
      if (fabs(M->lat[2 * J]) < LAT0) continue;
      filter_row(M, a, J, M->high_lat_pv);
    }
  } else {
    for (J = 0; J <= NJ; J++) {
      if (fabs(M->lat[2 * J + 1]) < LAT0) continue;
      filter_row(M, a, J, M->high_lat_h);
    }
  }
}

/* zonal_filter(index, plane, NULL, TWODIM) */
static void zonal_filter_2d(ep_model *M, int index, double *a) {
  filter_plane_rows(M, a, index == IDX_V);
  bc2(M, a);
}

/* zonal_filter(index, buff3d, gz, THREEDIM), epic_adjust.c:270-480 */
static int zonal_filter_3d(ep_model *M, int index, double *buff) {
  const double *gz = M->gz;
  double *varz = M->varz;
  trip *table = M->table;
  int K, J, I, Imin = 1, kstart = 1, kend = KHI, kay, jstart, n;
  double gzmin, geezee, dgz;
  jstart = (index == IDX_V) ? 1 : 0;
  for (J = jstart; J <= NJ; J++) {
    K = KHI;
    gzmin = DBL_MAX;
    for (I = 1; I <= NI; I++) {
      if (A3(gz, K, J, I) < gzmin) { Imin = I; gzmin = A3(gz, K, J, I); }
    }
    I = Imin;
    switch (index) {
      case IDX_U:
        kstart = 1; kend = KHI;
        for (K = kend; K >= kstart; K--) {
          kay = kend - K;
          table[kay].x = .5 * (A3(gz, K, J, I) + A3(gz, K, J, I - 1));
          table[kay].y = A3(buff, K, J, I);
        }
        break;
      case IDX_V:
        kstart = 1; kend = KHI;
        for (K = kend; K >= kstart; K--) {
          kay = kend - K;
          table[kay].x = .5 * (A3(gz, K, J, I) + A3(gz, K, J - 1, I));
          table[kay].y = A3(buff, K, J, I);
        }
        break;
      case IDX_HDRY:
        kstart = 1; kend = KHI;
        for (K = kend; K >= kstart; K--) {
          kay = kend - K;
          table[kay].x = .5 * (A3(gz, K, J, I) + A3(gz, K - 1, J, I));
          table[kay].y = log(A3(buff, K, J, I));
        }
        break;
      case IDX_THETA:
        kstart = M->g.k_sigma - 1; kend = KHI;
        for (K = kend; K >= kstart; K--) {
          kay = kend - K;
          table[kay].x = A3(gz, K, J, I);
          table[kay].y = A3(buff, K, J, I);
        }
        break;
      default:   /* NU_TURB and the other interface variables, epic_adjust.c:369-387 */
        kstart = 0; kend = KHI;
        for (K = kend; K >= kstart; K--) {
          kay = kend - K;
          table[kay].x = A3(gz, K, J, I);
          table[kay].y = A3(buff, K, J, I);
        }
        break;
    }
    n = kend - kstart + 1;
    if (spline_pchip(n, table) != 0) return fail(M, "spline_pchip: x not increasing (J=%d)", J);
    for (I = 1; I <= NI; I++) {
      for (K = kstart; K <= kend; K++) {
        switch (index) {
          case IDX_U: geezee = .5 * (A3(gz, K, J, I) + A3(gz, K, J, I - 1)); break;
          case IDX_V: geezee = .5 * (A3(gz, K, J, I) + A3(gz, K, J - 1, I)); break;
          case IDX_HDRY: geezee = .5 * (A3(gz, K, J, I) + A3(gz, K - 1, J, I)); break;
          default: geezee = A3(gz, K, J, I); break;
        }
        kay = find_place_in_table(n, table, geezee, &dgz);
        if (index == IDX_HDRY) A3(varz, K, J, I) = exp(splint_pchip(geezee, table + kay, dgz));
        else A3(varz, K, J, I) = splint_pchip(geezee, table + kay, dgz);
        A3(buff, K, J, I) -= A3(varz, K, J, I);
      }
    }
  }
  for (K = kstart; K <= kend; K++) filter_plane_rows(M, buff + K * M->n2, index == IDX_V);
  for (K = kstart; K <= kend; K++)
    for (J = jstart; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A3(buff, K, J, I) += A3(varz, K, J, I);
  bc3(M, buff);
  return 0;
}

/* restore_mass(HDRY_INDEX), epic_adjust.c:45-96 */
static void restore_mass(ep_model *M) {
  int K, J, I;
  for (K = 1; K <= KHI; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) A3(M->hdry, K, J, I) = dmax(M->h_min[K], A3(M->hdry, K, J, I));
}

/* ---------------------------------------------------------------------------------------- */
/* Hyperviscosity, src/shared/epic_subgrid.c:590-1232                                        */
/* ---------------------------------------------------------------------------------------- */

static void visc_tables(ep_model *M) {
  int itmp, itmp2, J;
  double r2_inv, lat[3];
  /* coef[] factoring of the hyperviscosity init blocks, :651-668 and :879-895 (nu[2] forced to 0). */
  M->g.nu[2] = 0.;
  for (itmp2 = 2; itmp2 <= 8; itmp2 += 2) {
    M->coef[itmp2] = M->g.nu[itmp2] > 0. ? M->g.nu[itmp2] : 0.01 * M->max_nu[itmp2];
    for (itmp = 2; itmp < itmp2; itmp += 2) M->coef[itmp2] /= M->coef[itmp];
  }
  /* d2dy2 coefficients, :1049-1141 (Legendre fit to a 3-point stencil). */
#define SETC(c, l0, l1, l2, first, last)                                                                     \
  do {                                                                                                       \
    lat[0] = (l0) * DEG; lat[1] = (l1) * DEG; lat[2] = (l2) * DEG;                                           \
    if (first) {                                                                                             \
      (c).x = r2_inv * (1. + sin(lat[0]) * (-3. * sin(lat[0]) + sin(lat[1]) + sin(lat[2]))) /                 \
              ((sin(lat[1]) - sin(lat[0])) * .5 * (sin(lat[2]) - sin(lat[0])));                              \
      (c).y = -r2_inv * 2. * (cos(2. * lat[0]) + sin(lat[0]) * sin(lat[2])) /                                 \
              ((sin(lat[1]) - sin(lat[0])) * (sin(lat[2]) - sin(lat[1])));                                   \
      (c).z = r2_inv * (cos(2. * lat[0]) + sin(lat[0]) * sin(lat[1])) /                                       \
              (.5 * (sin(lat[2]) - sin(lat[0])) * (sin(lat[2]) - sin(lat[1])));                              \
    } else if (last) {                                                                                       \
      (c).x = r2_inv * (cos(2. * lat[2]) + sin(lat[1]) * sin(lat[2])) /                                       \
              ((sin(lat[1]) - sin(lat[0])) * .5 * (sin(lat[2]) - sin(lat[0])));                              \
      (c).y = -r2_inv * 2. * (cos(2. * lat[2]) + sin(lat[0]) * sin(lat[2])) /                                 \
              ((sin(lat[1]) - sin(lat[0])) * (sin(lat[2]) - sin(lat[1])));                                   \
      (c).z = r2_inv * (1. + sin(lat[2]) * (sin(lat[0]) + sin(lat[1]) - 3. * sin(lat[2]))) /                  \
              (.5 * (sin(lat[2]) - sin(lat[0])) * (sin(lat[2]) - sin(lat[1])));                              \
    } else {                                                                                                 \
      (c).x = r2_inv * (cos(2. * lat[1]) + sin(lat[1]) * sin(lat[2])) /                                       \
              ((sin(lat[1]) - sin(lat[0])) * .5 * (sin(lat[2]) - sin(lat[0])));                              \
      (c).y = -r2_inv * 2. * (1. + sin(lat[1]) * (sin(lat[0]) - 3. * sin(lat[1]) + sin(lat[2]))) /            \
              ((sin(lat[1]) - sin(lat[0])) * (sin(lat[2]) - sin(lat[1])));                                   \
      (c).z = r2_inv * (cos(2. * lat[1]) + sin(lat[0]) * sin(lat[1])) /                                       \
              (.5 * (sin(lat[2]) - sin(lat[0])) * (sin(lat[2]) - sin(lat[1])));                              \
    }                                                                                                        \
  } while (0)
  J = 0;
  r2_inv = M->rlt[2 * J + 1]; r2_inv = 1. / (r2_inv * r2_inv);
  SETC(M->h_coef[J], M->lat[2 * J + 1], M->lat[2 * J + 3], M->lat[2 * J + 5], 1, 0);
  for (J = 1; J < NJ; J++) {
    r2_inv = M->rlt[2 * J + 1]; r2_inv = 1. / (r2_inv * r2_inv);
    SETC(M->h_coef[J], M->lat[2 * J - 1], M->lat[2 * J + 1], M->lat[2 * J + 3], 0, 0);
  }
  J = NJ;
  r2_inv = M->rlt[2 * J + 1]; r2_inv = 1. / (r2_inv * r2_inv);
  SETC(M->h_coef[J], M->lat[2 * J - 3], M->lat[2 * J - 1], M->lat[2 * J + 1], 0, 1);
  J = 0;
  r2_inv = M->rlt[2 * J]; r2_inv = 1. / (r2_inv * r2_inv);
  SETC(M->v_coef[J], M->lat[2 * J], M->lat[2 * J + 2], M->lat[2 * J + 4], 1, 0);
  for (J = 1; J <= NJ; J++) {
    r2_inv = M->rlt[2 * J]; r2_inv = 1. / (r2_inv * r2_inv);
    SETC(M->v_coef[J], M->lat[2 * J - 2], M->lat[2 * J], M->lat[2 * J + 2], 0, 0);
  }
  J = NJ + 1;
  r2_inv = M->rlt[2 * J]; r2_inv = 1. / (r2_inv * r2_inv);
  SETC(M->v_coef[J], M->lat[2 * J - 4], M->lat[2 * J - 2], M->lat[2 * J], 0, 1);
#undef SETC
}

/* d2dy2, epic_subgrid.c:1023-1232 (after initialisation) */
static void d2dy2(ep_model *M, int index, const double *hh, double diff_coef, double *d) {
  int J, I;
  double a0, a1, a2;
  if (index == IDX_V) {
    J = 0;
    for (I = 1; I <= NI; I++) {
      a0 = diff_coef * M->v_coef[J].x; a1 = diff_coef * M->v_coef[J].y; a2 = diff_coef * M->v_coef[J].z;
      A2(d, J, I) = a0 * A2(hh, J, I) + a1 * A2(hh, J + 1, I) + a2 * A2(hh, J + 2, I);
    }
    for (J = 1; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        a0 = diff_coef * M->v_coef[J].x; a1 = diff_coef * M->v_coef[J].y; a2 = diff_coef * M->v_coef[J].z;
        A2(d, J, I) = a0 * A2(hh, J - 1, I) + a1 * A2(hh, J, I) + a2 * A2(hh, J + 1, I);
      }
    J = NJ + 1;
    for (I = 1; I <= NI; I++) {
      a0 = diff_coef * M->v_coef[J].x; a1 = diff_coef * M->v_coef[J].y; a2 = diff_coef * M->v_coef[J].z;
      A2(d, J, I) = a0 * A2(hh, J - 2, I) + a1 * A2(hh, J - 1, I) + a2 * A2(hh, J, I);
    }
  } else {
    for (J = 0; J <= NJ; J++) {
      for (I = 1; I <= NI; I++) {
        a0 = diff_coef * M->h_coef[J].x; a1 = diff_coef * M->h_coef[J].y; a2 = diff_coef * M->h_coef[J].z;
        if (J == 0) A2(d, J, I) = a0 * A2(hh, J, I) + a1 * A2(hh, J + 1, I) + a2 * A2(hh, J + 2, I);
        else if (J == NJ) A2(d, J, I) = a0 * A2(hh, J - 2, I) + a1 * A2(hh, J - 1, I) + a2 * A2(hh, J, I);
        else A2(d, J, I) = a0 * A2(hh, J - 1, I) + a1 * A2(hh, J, I) + a2 * A2(hh, J + 1, I);
      }
    }
  }
  bc2(M, d);
}

static int nu_rest_positive(const ep_model *M, int from) {
  double tmp = 0.;
  int i;
  for (i = from; i <= 8; i += 2) tmp += M->g.nu[i];
  return tmp > 0.;
}

static void krange(const ep_model *M, int index, int *kstart, int *kend) {
  *kstart = 1; *kend = KHI;
  if (index == IDX_U || index == IDX_V) *kend = KHI - 1;
  if (index == IDX_THETA) *kstart = M->g.k_sigma - 1;
}

/* meridional_hyperviscosity(index, variable, THREEDIM), epic_subgrid.c:829-1006 */
static void meridional_hyperviscosity(ep_model *M, int index, double *var3) {
  int K, J, I, kstart, kend, itmp, sign, jlo;
  double *a, *hh, *d, *p;
  if (!nu_rest_positive(M, 4)) return;
  krange(M, index, &kstart, &kend);
  jlo = (index == IDX_V) ? 1 : 0;
  for (K = kstart; K <= kend; K++) {
    a = var3 + K * M->n2;
    hh = M->b2d[0];
    d = M->b2d[1];
    for (J = 0; J <= NJ + 1; J++)
      for (I = 0; I <= NI + 1; I++) A2(hh, J, I) = A2(a, J, I);
    sign = 1;
    itmp = 2;
    while (1) {
      d2dy2(M, index, hh, M->coef[itmp], d);
      if (M->g.nu[itmp] > 0.) {
        zonal_filter_2d(M, index == IDX_V ? IDX_V : IDX_OTHER, d);
        for (J = jlo; J <= NJ; J++)
          for (I = 1; I <= NI; I++) A2(a, J, I) += DT * (double)sign * A2(d, J, I);
        bc2(M, a);
      }
      sign *= -1;
      itmp += 2;
      p = hh; hh = d; d = p;
      if (!nu_rest_positive(M, itmp)) break;
    }
  }
}

/* zonal_hyperviscosity(index, variable, THREEDIM), epic_subgrid.c:590-818 */
static void zonal_hyperviscosity(ep_model *M, int index, double *var3) {
  int K, J, I, kstart, kend, itmp, sign, jbot, jhalf;
  double *a, *hh, *d, *p, diff_coef, false_mean, mm;
  if (NI < 2 || !nu_rest_positive(M, 4)) return;
  krange(M, index, &kstart, &kend);
  jbot = (index == IDX_V) ? 1 : 0;
  jhalf = (index == IDX_V) ? 0 : 1;
  for (K = kstart; K <= kend; K++) {
    a = var3 + K * M->n2;
    hh = M->b2d[0];
    d = M->b2d[1];
    for (J = 0; J <= NJ + 1; J++)
      for (I = 0; I <= NI + 1; I++) A2(hh, J, I) = A2(a, J, I);
    sign = 1;
    itmp = 2;
    while (1) {
      for (J = jbot; J <= NJ; J++) {
        if (fabs(M->lat[2 * J + jhalf]) > LAT0) diff_coef = M->coef[itmp] * M->m0 * M->m0;
        else {
          mm = M->m[2 * J + jhalf];
          diff_coef = M->coef[itmp] * mm * mm;
        }
        for (I = 1; I <= NI; I++)
          A2(d, J, I) = diff_coef * (A2(hh, J, I - 1) - 2. * A2(hh, J, I) + A2(hh, J, I + 1));
        A2(d, J, NI + 1) = A2(d, J, 1);
        A2(d, J, 0) = A2(d, J, NI);
        false_mean = 0.;
        for (I = 1; I <= NI; I++) false_mean += A2(d, J, I);
        false_mean /= NI;
        for (I = 0; I <= NI + 1; I++) A2(d, J, I) -= false_mean;
        if (M->g.nu[itmp] > 0.)
          for (I = 1; I <= NI; I++) A2(a, J, I) += DT * (double)sign * A2(d, J, I);
      }
      if (M->g.nu[itmp] > 0.) bc2(M, a);
      sign *= -1;
      itmp += 2;
      p = hh; hh = d; d = p;
      if (!nu_rest_positive(M, itmp)) break;
    }
  }
}

/* ---------------------------------------------------------------------------------------- */
/* Diagnostics: set_p2etc, store_pgrad_vars, store_diag, calc_heating                       */
/* ---------------------------------------------------------------------------------------- */

/* set_p2etc, epic_funcs_diag.c:3352-3569 (nq = 0: H2 is HDRY, PDRY3 is P3, HDRY3 is H3) */
static void set_p2etc(ep_model *M, int update_theta) {
  int K, J, I, kay, nkay, ks = M->g.k_sigma;
  double g, ptop, pbot, sigma, sg, h;
  trip *table = M->table;
  for (J = 0; J <= NJ; J++) {
    g = M->grav[2 * J + 1];
    for (I = 0; I <= NI + 1; I++) {
      for (K = 1; K <= KHI; K++) A3(M->p3, K, J, I) = A3(M->p3, K - 1, J, I) + M->dsgth[2 * K] * g * A3(M->hdry, K, J, I);
      ptop = A3(M->p3, 0, J, I);
      pbot = A3(M->p3, KHI, J, I);
      for (K = ks - 1; K < KHI; K++) {
        sigma = (M->sgth[2 * K + 1] - M->g.zeta0) / (M->g.zeta1 - M->g.zeta0);
        A3(M->p3, K, J, I) = get_p_sigma(pbot, sigma, ptop);
      }
      for (K = 1; K <= KHI; K++) A3(M->hdry, K, J, I) = dmax(M->h_min[K], get_h_layer(M, K, J, I));
    }
  }
  if (update_theta) {
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        ptop = A3(M->p3, 0, J, I);
        pbot = A3(M->p3, KHI, J, I);
        for (K = 0; K < ks - 1; K++) {
          sigma = get_sigma(pbot, A3(M->p3, K, J, I), ptop);
          A3(M->theta, K, J, I) = (M->sgth[2 * K + 1] - f_sigma(M, sigma)) / g_sigma(M, sigma);
        }
      }
  }
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      for (K = 1; K <= KHI; K++) A3(M->p2, K, J, I) = layer_p(M, A3(M->p3, K - 1, J, I), A3(M->p3, K, J, I));
      A3(M->p2, 0, J, I) = A3(M->p3, 0, J, I) * A3(M->p3, 0, J, I) / A3(M->p2, 1, J, I);
      for (K = 1; K <= KHI; K++) A3(M->h3, K, J, I) = get_h_iface(M, K, J, I);
      A3(M->h3, 0, J, I) = A3(M->h3, 1, J, I);
    }
  if (update_theta) {
    nkay = KHI - (ks - 1) + 1;
    for (K = KHI; K >= ks - 1; K--) table[KHI - K].x = M->sgth[2 * K + 1];
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        ptop = A3(M->p3, 0, J, I);
        pbot = A3(M->p3, KHI, J, I);
        for (K = 1; K < ks - 1; K++) {
          sigma = get_sigma(pbot, A3(M->p2, K, J, I), ptop);
          A3(M->theta2, K, J, I) = (M->sgth[2 * K] - f_sigma(M, sigma)) / g_sigma(M, sigma);
        }
        K = ks - 1;
        A3(M->theta2, K, J, I) = .5 * (A3(M->theta, K, J, I) + A3(M->theta, K - 1, J, I));
        for (K = KHI; K >= ks - 1; K--) table[KHI - K].y = A3(M->theta, K, J, I);
        for (K = ks; K <= KHI; K++) {
          sg = M->sgth[2 * K];
          kay = find_place_in_table(nkay, table, sg, &h);
          A3(M->theta2, K, J, I) = linint(sg, table + kay, h);
        }
      }
  }
}

/* store_pgrad_vars, epic_funcs_diag.c:3595-3950 (terrestrial, fpara off) */
/* get_kin (Sadourney 1975 with the Suarez-Takacs blend), epic_funcs_diag.c:2694-2846 */
static double get_kin(const ep_model *M, const double *u2d, const double *v2d, int J, int I) {
  const int jj = 2 * J;
  double u2 = A2(u2d, J, I), u4 = A2(u2d, J, I + 1), v2 = A2(v2d, J, I), v4 = A2(v2d, J + 1, I), kin_c, kin_s;
  kin_c = (u2 * u2 + u4 * u4 + M->mn[jj + 1] * (v2 * v2 * M->mn_inv[jj] + v4 * v4 * M->mn_inv[jj + 2])) * .25;
  if (J == 0 || J == NJ) return kin_c;
  u2 = .5 * (A2(u2d, J + 1, I) + A2(u2d, J - 1, I));
  u4 = .5 * (A2(u2d, J + 1, I + 1) + A2(u2d, J - 1, I + 1));
  v2 = .5 * (A2(v2d, J, I + 1) + A2(v2d, J, I - 1));
  v4 = .5 * (A2(v2d, J + 1, I + 1) + A2(v2d, J + 1, I - 1));
  kin_s = (u2 * u2 + u4 * u4 + M->mn[jj + 1] * (v2 * v2 * M->mn_inv[jj] + v4 * v4 * M->mn_inv[jj + 2])) * .25;
  return (5. / 6.) * kin_c + (1. / 6.) * kin_s;
}

/* The gas-giant lower boundary of store_pgrad_vars (epic_funcs_diag.c:3779-3811): zonal means of U,
 * P3 and RHO3 at K = nk, then gz_from_u (:4460-4612) with gz0 = 0 at J = grid.jtp: the absolute
 * vorticity of the zonally symmetric bottom wind (vorticity(ON_SIGMATHETA, ABSOLUTE), :4131-4444,
 * written into PV3(nk+1) as the reference does, where its PV macros read it), the meridional
 * integral of -(zeta+f) u dy - dp/rho, and GZ_SURFACE = Bernoulli function - kinetic energy on
 * every row 0..nj. */
static void gas_giant_gz_surface(ep_model *M) {
  int J, I;
  const int K = KHI, j0 = M->g.jtp;
  const double *U = M->u + (long)M->it_uv * M->n3;
  double *u1d = calloc(NJ + 1, sizeof(double)), *p1d = calloc(NJ + 1, sizeof(double)), *rho1d = calloc(NJ + 1, sizeof(double));
  double *udy = calloc(NJ + 1, sizeof(double)), *pvhudy = calloc(NJ + 1, sizeof(double)), *bern = calloc(NJ + 1, sizeof(double));
  double *u2d = calloc(M->n2, sizeof(double)), *v2d = calloc(M->n2, sizeof(double));
  double *pv = M->pv3 + (long)(K + 1) * M->n2;
  double ze, pv_pole, kin0;
  for (J = 0; J <= NJ; J++) {
    for (I = 1; I <= NI; I++) {
      u1d[J] += A3(U, K, J, I);
      p1d[J] += A3(M->p3, K, J, I);
      rho1d[J] += A3(M->rho3, K, J, I);
    }
    u1d[J] /= NI;
    p1d[J] /= NI;
    rho1d[J] /= NI;
  }
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) A2(u2d, J, I) = u1d[J];
  for (J = 1; J <= NJ; J++) {
    const double f2j = M->f[2 * J], m2j = M->m[2 * J], n2j = M->n[2 * J];
    const double m_m1_inv = 1. / M->m[2 * J - 1], m_p1_inv = 1. / M->m[2 * J + 1];
    for (I = 1; I <= NI; I++) {
      ze = m2j * ((A2(v2d, J, I) - A2(v2d, J, I - 1)) + n2j * (A2(u2d, J - 1, I) * m_m1_inv - A2(u2d, J, I) * m_p1_inv));
      A2(pv, J, I) = (ze + f2j);
    }
  }
  ze = 0.;
  for (I = 1; I <= NI; I++) ze -= A2(u2d, 0, I);
  ze *= M->mn[0] / ((M->m[1]) * (double)(NI));
  pv_pole = ze + M->f[0];
  for (I = 1; I <= NI; I++) A2(pv, 0, I) = pv_pole;
  ze = 0.;
  for (I = 1; I <= NI; I++) ze += A2(u2d, NJ, I);
  ze *= M->mn[2 * (NJ + 1)] / ((M->m[2 * NJ + 1]) * (double)(NI));
  pv_pole = ze + M->f[2 * (NJ + 1)];
  for (I = 1; I <= NI; I++) A2(pv, NJ + 1, I) = pv_pole;
  bc2(M, pv);
  I = 1;
  for (J = 0; J <= NJ; J++) udy[J] = A2(u2d, J, I) / M->n[2 * J + 1];
  for (J = 1; J <= NJ; J++) {
    /* the Sadourney PV averages of include/epic_pv_schemes.h:55-61 around the v point */
    const double al = (A2(pv, J - 1, I) + A2(pv, J, I) + A2(pv, J, I + 1));
    const double be = (A2(pv, J, I) + A2(pv, J, I + 1) + A2(pv, J - 1, I + 1));
    const double ga = (A2(pv, J, I) + A2(pv, J, I + 1) + A2(pv, J + 1, I + 1));
    const double de = (A2(pv, J, I) + A2(pv, J + 1, I) + A2(pv, J, I + 1));
    pvhudy[J] = (ga * udy[J] + de * udy[J] + al * udy[J - 1] + be * udy[J - 1]) * (1. / 12.);
    pvhudy[J] += (p1d[J] - p1d[J - 1]) * 2. / (rho1d[J] + rho1d[J - 1]);
  }
  kin0 = 0.;
  if (j0 >= 0 && j0 <= NJ) kin0 = get_kin(M, u2d, v2d, j0, 1);
  bern[j0] = 0. + kin0;
  for (J = j0 + 1; J <= NJ; J++) bern[J] = bern[J - 1] - pvhudy[J];
  for (J = j0 - 1; J >= 0; J--) bern[J] = bern[J + 1] + pvhudy[J + 1];
  for (J = 0; J <= NJ; J++) {
    const double gz = bern[J] - get_kin(M, u2d, v2d, J, 1);
    for (I = 0; I <= NI + 1; I++) A2(M->gz_surface, J, I) = gz;
  }
  free(u1d); free(p1d); free(rho1d); free(udy); free(pvhudy); free(bern); free(u2d); free(v2d);
}

static int store_pgrad_vars(ep_model *M) {
  int K, J, I, jj;
  double theta, pressure, temperature, mu = M->mu_dry, dtg_inv, gdx_inv3, gdy_inv2, gdy_inv4;
  double dz10, dz21, dz32, dz20, dz30, dz31, df0, df1, df2, df3, dgz;
  if (M->itime > 1) {
    for (K = 1; K <= KHI; K++)
      for (J = 0; J <= NJ; J++)
        for (I = 1; I <= NI; I++) A3(M->dzdt3, K, J, I) = A3(M->gz3, K, J, I);
  } else {
    memset(M->dzdt3, 0, M->n3 * sizeof(double));
  }
  for (K = 0; K <= KHI; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        theta = A3(M->theta, K, J, I);
        pressure = A3(M->p3, K, J, I);
        A3(M->t3, K, J, I) = temperature = return_temp(M, pressure, theta);
        A3(M->exner3, K, J, I) = M->g.cp * A3(M->t3, K, J, I) / theta;
        A3(M->rho3, K, J, I) = return_density(pressure, temperature, mu);
      }
  for (K = 1; K <= KHI; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        pressure = A3(M->p2, K, J, I);
        theta = A3(M->theta2, K, J, I);
        A3(M->t2, K, J, I) = temperature = return_temp(M, pressure, theta);
        A3(M->rho2, K, J, I) = return_density(pressure, temperature, mu);
      }
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      A3(M->rho2, 0, J, I) = A3(M->rho3, 0, J, I) * A3(M->rho3, 0, J, I) / A3(M->rho2, 1, J, I);
      A3(M->theta2, 0, J, I) = M->sgth[0];
      A3(M->t2, 0, J, I) = A3(M->t3, 0, J, I);
    }
  if (M->g.gas_giant) gas_giant_gz_surface(M);
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      A3(M->gz3, KHI, J, I) = M->g.topo_scale * A2(M->gz_surface, J, I);
      A3(M->mont3, KHI, J, I) = A3(M->gz3, KHI, J, I) + return_enthalpy(M, A3(M->t3, KHI, J, I));
    }
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
#define P(k) A3(M->p3, k, J, I)
#define R(k) A3(M->rho3, k, J, I)
      K = KHI;
      A3(M->gz3, K - 1, J, I) = A3(M->gz3, K, J, I) + ((P(K) + P(K - 1)) / (R(K) + R(K - 1))) * log(P(K) / P(K - 1));
      A3(M->mont3, K - 1, J, I) = A3(M->gz3, K - 1, J, I) + return_enthalpy(M, A3(M->t3, K - 1, J, I));
      for (K = KHI - 1; K >= 2; K--) {
        dz10 = log(P(K + 1) / P(K));
        dz21 = log(P(K) / P(K - 1));
        dz32 = log(P(K - 1) / P(K - 2));
        dz20 = dz21 + dz10;
        dz30 = dz32 + dz20;
        dz31 = dz32 + dz21;
        df0 = P(K + 1) / R(K + 1);
        df1 = P(K) / R(K);
        df2 = P(K - 1) / R(K - 1);
        df3 = P(K - 2) / R(K - 2);
        dgz = -(df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                df1 * (dz21 * (dz21 * (dz21 + 2. * (dz10 - dz31)) - 6. * dz10 * dz31)) / (dz10 * dz31) +
                df2 * (dz21 * (dz21 * (dz21 + 2. * (dz32 - dz20)) - 6. * dz20 * dz32)) / (dz20 * dz32) +
                df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32)) /
              12.;
        A3(M->gz3, K - 1, J, I) = A3(M->gz3, K, J, I) + dgz;
        A3(M->mont3, K - 1, J, I) = A3(M->gz3, K - 1, J, I) + return_enthalpy(M, A3(M->t3, K - 1, J, I));
      }
      K = 1;
      A3(M->gz3, K - 1, J, I) = A3(M->gz3, K, J, I) + ((P(K) + P(K - 1)) / (R(K) + R(K - 1))) * log(P(K) / P(K - 1));
      A3(M->mont3, K - 1, J, I) = A3(M->gz3, K - 1, J, I) + return_enthalpy(M, A3(M->t3, K - 1, J, I));
#undef P
#undef R
    }
  for (K = 1; K <= KHI; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++)
        if (A3(M->gz3, K, J, I) >= A3(M->gz3, K - 1, J, I))
          return fail(M, "store_pgrad_vars: GZ3(%d,%d,%d)=%g >= GZ3(%d,%d,%d)=%g", K, J, I, A3(M->gz3, K, J, I), K - 1, J,
                      I, A3(M->gz3, K - 1, J, I));
  if (M->itime > 1) {
    for (K = 1; K <= KHI; K++)
      for (J = 0; J <= NJ; J++) {
        dtg_inv = -1. / (DT * M->grav[2 * J + 1]);
        for (I = 1; I <= NI; I++) {
          A3(M->dzdt3, K, J, I) -= A3(M->gz3, K, J, I);
          A3(M->dzdt3, K, J, I) *= dtg_inv;
        }
      }
  }
  for (K = 1; K <= KHI; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A3(M->dzdt3, K, J, I) += A3(M->w3, K, J, I) * A3(M->h3, K, J, I) / A3(M->rho3, K, J, I);
  {
    const double *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3;
    for (K = 1; K <= KHI; K++)
      for (J = 0; J <= NJ; J++) {
        jj = 2 * J;
        gdx_inv3 = .5 * M->m[jj + 1] / M->grav[jj + 1];
        gdy_inv2 = .5 * M->n[jj] / M->grav[jj];
        gdy_inv4 = .5 * M->n[jj + 2] / M->grav[jj + 2];
        for (I = 1; I <= NI; I++)
          A3(M->dzdt3, K, J, I) += A3(V, K, J, I) * (A3(M->gz3, K, J, I) - A3(M->gz3, K, J - 1, I)) * gdy_inv2 +
                                   A3(V, K, J + 1, I) * (A3(M->gz3, K, J + 1, I) - A3(M->gz3, K, J, I)) * gdy_inv4 +
                                   A3(U, K, J, I) * (A3(M->gz3, K, J, I) - A3(M->gz3, K, J, I - 1)) * gdx_inv3 +
                                   A3(U, K, J, I + 1) * (A3(M->gz3, K, J, I + 1) - A3(M->gz3, K, J, I)) * gdx_inv3;
      }
  }
  bc3(M, M->dzdt3);
  return 0;
}

/* divergence, epic_funcs_diag.c:4064-4117 */
static void divergence(ep_model *M, const double *uu, const double *vv, double *di) {
  int J, I, jj;
  double n_inv, mn1, m_2j_inv, m_2jp2_inv;
  for (J = 0; J <= NJ; J++) {
    jj = 2 * J + 1;
    n_inv = 1. / M->n[jj];
    mn1 = M->mn[jj];
    m_2j_inv = (J == 0) ? 0. : 1. / M->m[jj - 1];
    m_2jp2_inv = (J == NJ) ? 0. : 1. / M->m[jj + 1];
    for (I = 1; I <= NI; I++)
      A2(di, J, I) = mn1 * ((A2(uu, J, I + 1) * n_inv - A2(uu, J, I) * n_inv) +
                            (A2(vv, J + 1, I) * m_2jp2_inv - A2(vv, J, I) * m_2j_inv));
  }
  bc2(M, di);
}

/* vorticity(ON_SIGMATHETA, POTENTIAL, ...) on the globe with both poles, epic_funcs_diag.c:4131-4445 */
static void potential_vorticity(ep_model *M, const double *uu, const double *vv, const double *hh, double *pv) {
  int J, I;
  double f2j, m2j, n2j, m_m1_inv, m_p1_inv, mn_m1_inv, mn_p1_inv, mn_pv, ze, h_pv, pv_pole;
  for (J = 1; J <= NJ; J++) {
    f2j = M->f[2 * J];
    m2j = M->m[2 * J];
    n2j = M->n[2 * J];
    m_m1_inv = 1. / M->m[2 * J - 1];
    m_p1_inv = 1. / M->m[2 * J + 1];
    mn_m1_inv = 1. / M->mn[2 * J - 1];
    mn_p1_inv = 1. / M->mn[2 * J + 1];
    mn_pv = .5 / (mn_m1_inv + mn_p1_inv);
    for (I = 1; I <= NI; I++) {
      ze = m2j * ((A2(vv, J, I) - A2(vv, J, I - 1)) + n2j * (A2(uu, J - 1, I) * m_m1_inv - A2(uu, J, I) * m_p1_inv));
      A2(pv, J, I) = (ze + f2j);
    }
    for (I = 1; I <= NI; I++) {
      h_pv = ((A2(hh, J, I) + A2(hh, J, I - 1)) * mn_p1_inv + (A2(hh, J - 1, I) + A2(hh, J - 1, I - 1)) * mn_m1_inv) * mn_pv;
      A2(pv, J, I) /= h_pv;
    }
  }
  /* south pole */
  J = 0;
  ze = 0.;
  for (I = 1; I <= NI; I++) ze -= A2(uu, J, I);
  ze *= M->mn[0] / ((M->m[1]) * (double)(NI));
  h_pv = 0.;
  for (I = 1; I <= NI; I++) h_pv += A2(hh, J, I);
  h_pv /= (double)(NI);
  pv_pole = (ze + M->f[0]) / h_pv;
  for (I = 1; I <= NI; I++) A2(pv, J, I) = pv_pole;
  /* north pole */
  J = NJ;
  ze = 0.;
  for (I = 1; I <= NI; I++) ze += A2(uu, J, I);
  ze *= M->mn[2 * (J + 1)] / (M->m[2 * J + 1] * (double)(NI));
  h_pv = 0.;
  for (I = 1; I <= NI; I++) h_pv += A2(hh, J, I);
  h_pv /= (double)(NI);
  pv_pole = (ze + M->f[2 * (J + 1)]) / h_pv;
  for (I = 1; I <= NI; I++) A2(pv, NJ + 1, I) = pv_pole;
  bc2(M, pv);
}

/* get_brunt2 for a layer (np = 1, fpara off, HS cp = 1004), epic_funcs_diag.c:2885-3075 */
static double brunt2_layer(const ep_model *M, int K, int J, int I) {
  double pressure = A3(M->p2, K, J, I), temperature = A3(M->t2, K, J, I), density = A3(M->rho2, K, J, I);
  double cp = 1004., mu = M->mu_dry, deltap, deltaT, drho_dp_T, drho_dT_p, Drho_Dp, g;
  deltap = 0.001 * pressure;
  deltaT = 0.001 * temperature;
  drho_dp_T = (return_density(pressure + deltap, temperature, mu) - return_density(pressure - deltap, temperature, mu)) /
              (2. * deltap);
  drho_dT_p = (return_density(pressure, temperature + deltaT, mu) - return_density(pressure, temperature - deltaT, mu)) /
              (2. * deltaT);
  Drho_Dp = (A3(M->rho3, K, J, I) - A3(M->rho3, K - 1, J, I)) / (A3(M->p3, K, J, I) - A3(M->p3, K - 1, J, I));
  g = M->grav[2 * J + 1];
  return g * g * (Drho_Dp - drho_dp_T + temperature / (cp * density * density) * drho_dT_p * drho_dT_p);
}

/* store_diag, epic_funcs_diag.c:3963-4053 */
static void store_diag(ep_model *M) {
  int K, J, I;
  double *buff = M->b2d[7], dudz2, dvdz2;
  const double *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3;
  for (K = 0; K <= KHI; K++) {
    memcpy(buff, V + K * M->n2, M->n2 * sizeof(double));
    zonal_filter_2d(M, IDX_V, buff);
    potential_vorticity(M, U + K * M->n2, buff, M->h3 + K * M->n2, M->pv3 + K * M->n2);
  }
  for (K = 0; K <= KHI; K++) {
    memcpy(buff, U + K * M->n2, M->n2 * sizeof(double));
    zonal_filter_2d(M, IDX_U, buff);
    divergence(M, buff, V + K * M->n2, M->div_uv3 + K * M->n2);
  }
  /* get_richardson for layers, :3079-3156 (QUIRK: the V term of dvdz2 has a sign slip, :3127-3128) */
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++)
      for (K = 1; K <= KHI; K++) {
        dudz2 = .5 * (A3(U, K - 1, J, I) + A3(U, K - 1, J, I + 1) - A3(U, K, J, I) - A3(U, K, J, I + 1));
        dvdz2 = .5 * (A3(V, K - 1, J, I) + A3(V, K - 1, J + 1, I) - A3(V, K, J, I) + A3(V, K, J + 1, I));
        dudz2 *= dudz2;
        dvdz2 *= dvdz2;
        if (fcmp(dudz2, 0.) != 0) A3(M->ri2, K, J, I) = brunt2_layer(M, K, J, I) / (dudz2 + dvdz2);
        else A3(M->ri2, K, J, I) = 1.e+6;
      }
  bc3(M, M->ri2);
}

/* t_rad for held_suarez, epic_sensible_heating.c:217-314 */
static double t_rad(const ep_model *M, int K, int J, int I) {
  const double ka = 1. / (40. * 60. * 60. * 24.), ks = 1. / (4. * 60. * 60. * 24.);
  double pressure = A3(M->p3, K, J, I), kt = ka, pbot, amp, cos_lat;
  pbot = A3(M->p3, KHI, J, I);
  amp = (pressure / pbot - 0.7) / (1. - 0.7);
  if (amp > 0.) {
    cos_lat = cos(M->lat[2 * J + 1] * DEG);
    kt += (ks - ka) * pow(cos_lat, 4.) * amp;
  }
  return 1. / kt;
}

/* temp_eq for held_suarez, epic_sensible_heating.c:394-406 */
static double temp_eq(const ep_model *M, double latitude, double pressure) {
  double cos2_lat, sin2_lat, p_p0, ans;
  cos2_lat = cos(latitude * DEG);
  cos2_lat *= cos2_lat;
  sin2_lat = 1. - cos2_lat;
  p_p0 = pressure / (1000. * 100.);
  ans = (315. - 60. * sin2_lat - 10. * log(p_p0) * cos2_lat) * pow(p_p0, M->g.kappa);
  return dmax(200., ans);
}

/* calc_heating -> newtonian_cooling, epic_funcs_diag.c:4793-4869, epic_sensible_heating.c:51-180 */
static void calc_heating(ep_model *M) {
  int K, J, I;
  double *buffji = M->b2d[7], lat, cp_over_time, t_eq, area, heat_area, da, heat_avg;
  memset(M->heat3, 0, M->n3 * sizeof(double));
  if (M->g.newt_cool_on) {
    for (K = 1; K <= KHI; K++) {
      for (J = 0; J <= NJ; J++) {
        lat = M->lat[2 * J + 1];
        for (I = 1; I <= NI; I++) {
          cp_over_time = 1004. / t_rad(M, K, J, I);
          t_eq = temp_eq(M, lat, A3(M->p3, K, J, I));
          A2(buffji, J, I) = -cp_over_time * (A3(M->t3, K, J, I) - t_eq);
        }
      }
      if (K <= M->g.k_sponge || M->g.newt_cool_adjust) {
        area = 0.;
        heat_area = 0.;
        for (J = 0; J <= NJ; J++) {
          da = 1. / M->mn[2 * J + 1];
          for (I = 1; I <= NI; I++) {
            area += da;
            heat_area += A2(buffji, J, I) * da;
          }
        }
        heat_avg = heat_area / area;
        for (J = 0; J <= NJ; J++)
          for (I = 1; I <= NI; I++) A2(buffji, J, I) -= heat_avg;
      }
      for (J = 0; J <= NJ; J++)
        for (I = 1; I <= NI; I++) A3(M->heat3, K, J, I) += A2(buffji, J, I);
    }
  }
  bc3(M, M->heat3);
}

/* ---------------------------------------------------------------------------------------- */
/* Prognostic pieces                                                                        */
/* ---------------------------------------------------------------------------------------- */

/* source_sink: THETA += dt*HEAT3/EXNER3 where theta is prognostic, epic_funcs_diag.c:4768-4778 */
static void source_sink(ep_model *M) {
  int K, J, I;
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++)
      for (K = M->g.k_sigma - 1; K <= KHI; K++)
        A3(M->theta, K, J, I) += DT * A3(M->heat3, K, J, I) / A3(M->exner3, K, J, I);
}

/* calc_w, epic_flux.c:123-335 */
static int calc_w(ep_model *M) {
  int K, J, I, ks = M->g.k_sigma;
  double ptop, pbot, psigma, sigma, theta3, p2, p3, p4, dp, pbot2, pbot3, pbot4, dpbot, dFdp, dFdpbot;
  double dz10, dz21, dz32, dz20, dz30, dz31, df0, df1, df2, df3, dsumdiv;
  double *sd = M->sum_div;
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      A3(M->w3, 0, J, I) = 0.;
      A3(M->w3, KHI, J, I) = 0.;
    }
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      ptop = A3(M->p3, 0, J, I);
      pbot = A3(M->p3, KHI, J, I);
      for (K = 1; K < ks - 1; K++) {
        sigma = get_sigma(pbot, A3(M->p3, K, J, I), ptop);
        A3(M->w3, K, J, I) = g_sigma(M, sigma) * A3(M->heat3, K, J, I) / A3(M->exner3, K, J, I);
      }
      for (K = ks - 1; K < KHI; K++) A3(M->w3, K, J, I) = 0.;
    }
  /* Leslie-Purser summed divergence.  QUIRK: the reference assigns the K = KLO and K = KHI
   * entries outside the J,I loops (epic_flux.c:224-226, :259-261), at a pad cell of another
   * plane, so every real column keeps SUM_DIV(KLO) = SUM_DIV(KHI) = 0 from the memset. */
  memset(sd, 0, M->n3 * sizeof(double));
  for (K = 2; K < KHI; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
#define P(k) A3(M->p3, k, J, I)
#define D(k) A3(M->div_uv3, k, J, I)
        dz10 = log(P(K - 1) / P(K - 2));
        dz21 = log(P(K) / P(K - 1));
        dz32 = log(P(K + 1) / P(K));
        dz20 = dz21 + dz10;
        dz30 = dz32 + dz20;
        dz31 = dz32 + dz21;
        df0 = P(K - 2) * D(K - 2);
        df1 = P(K - 1) * D(K - 1);
        df2 = P(K) * D(K);
        df3 = P(K + 1) * D(K + 1);
#undef P
#undef D
        dsumdiv = -(df0 * (dz21 * dz21 * dz21 * (dz31 + dz32)) / (dz10 * dz20 * dz30) +
                    df1 * (dz21 * (dz21 * (dz21 + 2. * (dz10 - dz31)) - 6. * dz10 * dz31)) / (dz10 * dz31) +
                    df2 * (dz21 * (dz21 * (dz21 + 2. * (dz32 - dz20)) - 6. * dz20 * dz32)) / (dz20 * dz32) +
                    df3 * (dz21 * dz21 * dz21 * (dz10 + dz20)) / (dz30 * dz31 * dz32)) /
                  12.;
        A3(sd, K, J, I) = A3(sd, K - 1, J, I) + dsumdiv;
      }
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      ptop = A3(M->p3, 0, J, I);
      psigma = A3(M->p3, ks - 1, J, I);
      pbot = A3(M->p3, KHI, J, I);
      for (K = 1; K < KHI; K++) {
        theta3 = A3(M->theta, K, J, I);
        p3 = A3(M->p3, K, J, I);
        pbot3 = pbot;
        dp = p3 * M->eps13;
        dpbot = pbot3 * M->eps13;
        p2 = dmax(p3 - dp * .5, ptop);
        p4 = dmin(p3 + dp * .5, pbot);
        if (p2 < psigma && p4 >= psigma) p2 = p3;
        pbot2 = dmax(pbot3 - dpbot * .5, p3);
        pbot4 = dmax(pbot3 + dpbot * .5, p3);
        if (get_sigma(pbot4, p3, ptop) > M->g.sigma_sigma && get_sigma(pbot2, p3, ptop) <= M->g.sigma_sigma) pbot4 = pbot3;
        if (!(p2 < p4)) return fail(M, "calc_w: p2=%g p4=%g", p2, p4);
        dFdp = (return_sigmatheta(M, theta3, p2, pbot3, ptop) - return_sigmatheta(M, theta3, p4, pbot3, ptop)) / (p2 - p4);
        if (!(pbot2 < pbot4)) return fail(M, "calc_w: pbot2=%g pbot4=%g", pbot2, pbot4);
        dFdpbot = (return_sigmatheta(M, theta3, p3, pbot2, ptop) - return_sigmatheta(M, theta3, p3, pbot4, ptop)) /
                  (pbot2 - pbot4);
        A3(M->w3, K, J, I) -= A3(sd, K, J, I) * dFdp + A3(sd, KHI, J, I) * dFdpbot;
      }
    }
  return 0;
}

/* uv_core with get_kin (Sadourney 1975 PV averaging), epic_timestep.c:628-762,
 * epic_funcs_diag.c:2694-2847, include/epic_pv_schemes.h:48-61 */
static void uv_core(ep_model *M) {
  int K, J, I, kk;
  double *uh = M->b2d[0], *vh = M->b2d[1], *kin = M->b2d[2];
  const double *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3;
  double *DU = M->dudt + (long)M->it_uv_tend * M->n3, *DV = M->dvdt + (long)M->it_uv_tend * M->n3;
  double havg, n_inv, m_inv, n2j, m2jp1, u2, u4, v2, v4, kin_c, kin_s, al, be, ga, de;
  const double pv_coef = 1. / 12.;
  for (K = 1; K < KHI; K++) {
    const double *Uk = U + K * M->n2, *Vk = V + K * M->n2;
    memset(uh, 0, M->n2 * sizeof(double));
    memset(vh, 0, M->n2 * sizeof(double));
    memset(kin, 0, M->n2 * sizeof(double));
    for (J = 0; J <= NJ; J++) {
      n_inv = 1. / M->n[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        havg = .5 * (A3(M->h3, K, J, I) + A3(M->h3, K, J, I - 1));
        A2(uh, J, I) = A2(Uk, J, I) * havg * n_inv;
      }
    }
    bc2(M, uh);
    for (J = 1; J <= NJ; J++) {
      m_inv = 1. / M->m[2 * J];
      for (I = 1; I <= NI; I++) {
        havg = .5 * (A3(M->h3, K, J, I) + A3(M->h3, K, J - 1, I));
        A2(vh, J, I) = A2(Vk, J, I) * havg * m_inv;
      }
    }
    bc2(M, vh);
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        int jj = 2 * J;
        u2 = A2(Uk, J, I); u4 = A2(Uk, J, I + 1); v2 = A2(Vk, J, I); v4 = A2(Vk, J + 1, I);
        kin_c = (u2 * u2 + u4 * u4 + M->mn[jj + 1] * (v2 * v2 * M->mn_inv[jj] + v4 * v4 * M->mn_inv[jj + 2])) * .25;
        if (J == 0 || J == NJ) A2(kin, J, I) = kin_c;
        else {
          u2 = .5 * (A2(Uk, J + 1, I) + A2(Uk, J - 1, I));
          u4 = .5 * (A2(Uk, J + 1, I + 1) + A2(Uk, J - 1, I + 1));
          v2 = .5 * (A2(Vk, J, I + 1) + A2(Vk, J, I - 1));
          v4 = .5 * (A2(Vk, J + 1, I + 1) + A2(Vk, J + 1, I - 1));
          kin_s = (u2 * u2 + u4 * u4 + M->mn[jj + 1] * (v2 * v2 * M->mn_inv[jj] + v4 * v4 * M->mn_inv[jj + 2])) * .25;
          A2(kin, J, I) = (5. / 6.) * kin_c + (1. / 6.) * kin_s;
        }
      }
    bc2(M, kin);
#define PV(j, i) A3(M->pv3, K, j, i)
    for (J = 1; J <= NJ; J++) {
      n2j = M->n[2 * J];
      for (I = 1; I <= NI; I++) {
        ga = (PV(J, I) + PV(J, I + 1) + PV(J + 1, I + 1));
        de = (PV(J, I) + PV(J + 1, I) + PV(J, I + 1));
        al = (PV(J - 1, I) + PV(J, I) + PV(J, I + 1));
        be = (PV(J, I) + PV(J, I + 1) + PV(J - 1, I + 1));
        A3(DV, K, J, I) += ((-ga * A2(uh, J, I + 1) - de * A2(uh, J, I) - al * A2(uh, J - 1, I) - be * A2(uh, J - 1, I + 1) +
                             0. * A2(vh, J - 1, I) - 0. * A2(vh, J + 1, I)) * pv_coef +
                            A2(kin, J - 1, I) - A2(kin, J, I)) * n2j;
      }
    }
    zonal_filter_2d(M, IDX_HDRY, kin);
    for (J = 0; J <= NJ; J++) {
      m2jp1 = M->m[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        al = (PV(J, I) + PV(J + 1, I) + PV(J + 1, I + 1));
        be = (PV(J + 1, I - 1) + PV(J + 1, I) + PV(J, I));
        ga = (PV(J, I - 1) + PV(J, I) + PV(J + 1, I));
        de = (PV(J, I) + PV(J + 1, I) + PV(J, I + 1));
        A3(DU, K, J, I) += ((al * A2(vh, J + 1, I) + be * A2(vh, J + 1, I - 1) + ga * A2(vh, J, I - 1) + de * A2(vh, J, I) +
                             0. * A2(uh, J, I - 1) - 0. * A2(uh, J, I + 1)) * pv_coef +
                            A2(kin, J, I - 1) - A2(kin, J, I)) * m2jp1;
      }
    }
#undef PV
  }
  for (K = 1; K < KHI; K++) {
    kk = 2 * K + 1;
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++)
        A3(DU, K, J, I) -= .5 * (A3(M->w3, K, J, I) + A3(M->w3, K, J, I - 1)) * (A3(U, K - 1, J, I) - A3(U, K + 1, J, I)) /
                           (M->sgth[kk - 2] - M->sgth[kk + 2]);
    for (J = 1; J <= NJ; J++)
      for (I = 1; I <= NI; I++)
        A3(DV, K, J, I) -= .5 * (A3(M->w3, K, J, I) + A3(M->w3, K, J - 1, I)) * (A3(V, K - 1, J, I) - A3(V, K + 1, J, I)) /
                           (M->sgth[kk - 2] - M->sgth[kk + 2]);
  }
}

/* uv_drag, epic_timestep.c:1303-1509 (LATERAL_SPONGE_DEPTH = -1) */
static void uv_drag(ep_model *M) {
  int K, J, I;
  const double *U = M->u + (long)M->it_uv_dis * M->n3, *V = M->v + (long)M->it_uv_dis * M->n3;
  double *DU = M->dudt + (long)M->it_uv_tend * M->n3, *DV = M->dvdt + (long)M->it_uv_tend * M->n3;
  double uavg, vavg, uray, vray, tmp, nu0, pbot, p3, amp;
  for (K = 0; K <= M->g.k_sponge; K++) {
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A3(DU, K, J, I) -= (M->t_sponge_inv[K]) * (A3(U, K, J, I) - A3(M->u_spinup, K, J, I));
    for (J = 1; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A3(DV, K, J, I) -= (M->t_sponge_inv[K]) * (A3(V, K, J, I) - 0.);
  }
  if ((M->g.newt_cool_on && M->g.prandtl > 0.) || (M->g.tau_drag > 0. && M->g.tau_drag < 1.e+20)) {
    for (K = M->g.k_sponge + 1; K < KHI; K++) {
      for (J = 0; J <= NJ; J++) {
        uavg = 0.;
        for (I = 1; I <= NI; I++) uavg += A3(U, K, J, I);
        uavg /= (NI);
        for (I = 1; I <= NI; I++) {
          uray = (M->g.drag_zonal_avg) * uavg + (1 - M->g.drag_zonal_avg) * A3(U, K, J, I);
          if (M->g.newt_cool_on) {
            tmp = .5 * (t_rad(M, K, J, I) + t_rad(M, K, J, I - 1));
            nu0 = M->g.prandtl / tmp;
          } else nu0 = 1. / M->g.tau_drag;
          A3(DU, K, J, I) -= nu0 * (uray - A3(M->u_spinup, K, J, I));
        }
      }
      if (M->g.drag_v) {
        for (J = 1; J <= NJ; J++) {
          vavg = 0.;
          for (I = 1; I <= NI; I++) vavg += A3(V, K, J, I);
          vavg /= NI;
          for (I = 1; I <= NI; I++) {
            vray = (M->g.drag_zonal_avg) * vavg + (1 - M->g.drag_zonal_avg) * A3(V, K, J, I);
            if (M->g.newt_cool_on) {
              tmp = .5 * (t_rad(M, K, J, I) + t_rad(M, K, J - 1, I));
              nu0 = M->g.prandtl / tmp;
            } else nu0 = 1. / M->g.tau_drag;
            A3(DV, K, J, I) -= nu0 * vray;
          }
        }
      }
    }
  }
  /* Held-Suarez boundary-layer drag, :1473-1506 */
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++) {
      pbot = 0.5 * (A3(M->p3, KHI, J, I) + A3(M->p3, KHI, J, I - 1));
      for (K = KHI - 1; K >= 1; K--) {
        p3 = .5 * (A3(M->p3, K, J, I) + A3(M->p3, K, J, I - 1));
        amp = (p3 / pbot - 0.7) / (1. - 0.7);
        if (amp < 0.) break;
        nu0 = M->g.hs_kf * amp;
        A3(DU, K, J, I) -= nu0 * A3(U, K, J, I);
      }
    }
  for (J = 1; J <= NJ; J++)
    for (I = 1; I <= NI; I++) {
      pbot = 0.5 * (A3(M->p3, KHI, J, I) + A3(M->p3, KHI, J - 1, I));
      for (K = KHI - 1; K >= 1; K--) {
        p3 = .5 * (A3(M->p3, K, J, I) + A3(M->p3, K, J - 1, I));
        amp = (p3 / pbot - 0.7) / (1. - 0.7);
        if (amp < 0.) break;
        nu0 = M->g.hs_kf * amp;
        A3(DV, K, J, I) -= nu0 * A3(V, K, J, I);
      }
    }
}

/* hsu_advection(is, buff3d, HORIZONTAL_AND_VERTICAL), epic_flux.c:652-1488.
 * kind: IDX_OTHER = P3_INDEX (unity), IDX_THETA, IDX_HDRY, IDX_NU = NU_TURB_INDEX.  NU_TURB is
 * loaded, moved by the interface velocities and updated as an interface variable, but its
 * predictor and corrector fluxes take the layer variables' form (the reference's
 * `is == HDRY_INDEX || is == NU_TURB_INDEX` branches, :876-960), with floor NU_TURB_MIN. */
static void hsu_advection(ep_model *M, int kind, double *buff) {
  const double ep = EP_EPS_HSU;
  const int layer = (kind == IDX_HDRY), nu = (kind == IDX_NU), layer_flux = layer || nu;
  const double nu_min = 1.e-3 * M->g.kinvisc;   /* NU_TURB_MIN, include/epic_subgrid.h:40 */
  const int k_first = (kind == IDX_THETA) ? M->g.k_sigma - 1 : 1;
  int K, J, I;
  double *wm = M->wm, *wp = M->wp, *w_a = M->w_a, *pred = M->w_a_pred, *amin = M->w_a_min, *w_ff = M->w_ff;
  double *d1 = M->w_a_diff1, *d2 = M->w_a_diff2, *aaa = M->w_aaa;
  double vertvel, da, tmp, whatp, whatm, mu, al, gap, gam, bep, bem, behatp, behatm, g_hsu, a_min;
  const double *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3;

  /* Vertical advection, column by column (:717-1052). */
  if (layer) for (K = k_first; K <= KHI; K++) amin[K] = M->h_min[K];
  else for (K = k_first - 1; K <= KHI; K++) amin[K] = 0.;
  /* NU_TURB sets entries 1 .. nk; entry 0 keeps the 0 of the calls before it */
  if (nu) for (K = k_first; K <= KHI; K++) amin[K] = nu_min;
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      if (layer) for (K = k_first; K <= KHI; K++) w_a[K] = A3(buff, K, J, I);
      else for (K = k_first - 1; K <= KHI; K++) w_a[K] = A3(buff, K, J, I);
      if (layer) {
        for (K = k_first - 1; K <= KHI; K++) {
          vertvel = A3(M->w3, K, J, I);
          wm[K] = dmin(0., vertvel);
          wp[K] = dmax(0., vertvel);
        }
      } else {
        for (K = k_first; K <= KHI; K++) {
          if (K == 1 || K == KHI) vertvel = 0.;
          else vertvel = .5 * (A3(M->w3, K, J, I) + A3(M->w3, K - 1, J, I));
          wm[K] = dmin(0., vertvel);
          wp[K] = dmax(0., vertvel);
        }
      }
      /* predictor */
      if (layer_flux) {
        w_ff[k_first - 1] = 0.;
        w_ff[KHI] = 0.;
        for (K = k_first; K < KHI; K++) w_ff[K] = wp[K] * w_a[K + 1] + wm[K] * w_a[K];
        for (K = k_first; K <= KHI; K++) {
          da = (w_ff[K] - w_ff[K - 1]) * M->dsgth_inv[2 * K] * DT;
          pred[K] = w_a[K] + da;
        }
      } else {
        for (K = k_first; K <= KHI; K++) w_ff[K] = wp[K] * w_a[K] + wm[K] * w_a[K - 1];
        w_ff[KHI + 1] = 0.;
        pred[k_first - 1] = w_a[k_first - 1];
        for (K = k_first; K <= KHI; K++) {
          da = (w_ff[K + 1] - w_ff[K]) * M->dsgth_inv[2 * K + 1] * DT;
          pred[K] = w_a[K] + da;
        }
      }
      /* corrector */
      if (layer_flux) {
        for (K = k_first; K < KHI; K++) w_ff[K] = .5 * (wp[K] * (pred[K] + w_a[K + 1]) + wm[K] * (pred[K + 1] + w_a[K]));
        for (K = k_first; K <= KHI; K++) {
          if (K == 1) {
            d1[K] = pred[K] - w_a[K + 1];
            d2[K] = 0.;
            tmp = fabs(w_a[K + 1] - w_a[K]) + ep;
          } else if (K == KHI) {
            d1[K] = 0.;
            d2[K] = pred[K] - w_a[K - 1];
            tmp = fabs(-w_a[K] + w_a[K - 1]) + ep;
          } else {
            d1[K] = pred[K] - w_a[K + 1];
            d2[K] = pred[K] - w_a[K - 1];
            tmp = fabs(w_a[K + 1] - 2. * w_a[K] + w_a[K - 1]) + ep;
          }
          aaa[K] = tmp * tmp;
        }
        for (K = k_first; K < KHI; K++) {
          whatp = sqrt(wp[K] * wp[K + 1]);
          whatm = -sqrt(wm[K] * wm[K - 1]);
          mu = (wp[K] - wm[K]) * M->dsgth_inv[2 * K + 1] * DT;
          al = (1. + mu) / 6.;
          gap = aaa[K + 1] / (aaa[K + 1] + (w_a[K + 1] - amin[K + 1]) * (w_a[K] - amin[K]));
          gap = gap * gap;
          gam = aaa[K] / (aaa[K] + (w_a[K + 1] - amin[K + 1]) * (w_a[K] - amin[K]));
          gam = gam * gam;
          bep = 1. + (1. / (2. * al) - 1.) * gap;
          bem = 1. + (1. / (2. * al) - 1.) * gam;
          behatp = 1. - gap;
          behatm = 1. - gam;
          g_hsu = -al * (wp[K] * bep * d1[K] - whatp * behatp * d1[K + 1] + wm[K] * bem * d2[K + 1] - whatm * behatm * d2[K]);
          w_ff[K] += g_hsu;
        }
      } else {
        for (K = k_first; K <= KHI; K++) w_ff[K] = .5 * (wp[K] * (pred[K - 1] + w_a[K]) + wm[K] * (pred[K] + w_a[K - 1]));
        for (K = k_first - 1; K <= KHI; K++) {
          /* QUIRK: for THETA (k_first > 1) the K = k_first-1 entry reads w_a[k_first-2], which this
           * call never loads; the reference's static buffer still holds the value the preceding
           * unity advection loaded there, 1.0 (epic_flux.c:371-384, :866-877). */
          double wkm1 = (K >= 1 && K - 1 < k_first - 1) ? 1.0 : (K >= 1 ? w_a[K - 1] : 0.);
          if (K == 0) tmp = fabs(w_a[K + 1] - w_a[K]) + ep;
          else if (K == KHI) tmp = fabs(-w_a[K] + wkm1) + ep;
          else tmp = fabs(w_a[K + 1] - 2. * w_a[K] + wkm1) + ep;
          aaa[K] = tmp * tmp;
        }
        d2[k_first - 1] = 0.;
        for (K = k_first; K <= KHI; K++) {
          d1[K] = pred[K - 1] - w_a[K];
          d2[K] = pred[K] - w_a[K - 1];
        }
        for (K = k_first; K <= KHI; K++) {
          /* wm[k_first-1] is not loaded for THETA either; its only use multiplies d2[k_first-1] = 0. */
          whatm = (K == 1) ? 0. : (K - 1 < k_first ? 0. : -sqrt(wm[K] * wm[K - 1]));
          whatp = (K == KHI) ? 0. : sqrt(wp[K] * wp[K + 1]);
          mu = (wp[K] - wm[K]) * M->dsgth_inv[2 * K] * DT;
          al = (1. + mu) / 6.;
          gap = aaa[K] / (aaa[K] + (w_a[K] - amin[K]) * (w_a[K - 1] - amin[K - 1]));
          gap = gap * gap;
          gam = aaa[K - 1] / (aaa[K - 1] + (w_a[K] - amin[K]) * (w_a[K - 1] - amin[K - 1]));
          gam = gam * gam;
          bep = 1. + (1. / (2. * al) - 1.) * gap;
          bem = 1. + (1. / (2. * al) - 1.) * gam;
          behatp = 1. - gap;
          behatm = 1. - gam;
          if (K < KHI)
            g_hsu = -al * (wp[K] * bep * d1[K] - whatp * behatp * d1[K + 1] + wm[K] * bem * d2[K] - whatm * behatm * d2[K - 1]);
          else
            g_hsu = -al * (wp[K] * bep * d1[K] + wm[K] * bem * d2[K] - whatm * behatm * d2[K - 1]);
          w_ff[K] += g_hsu;
        }
        w_ff[KHI + 1] = 0.;
      }
      if (nu) w_ff[KHI + 1] = 0.;   /* the reference's static entry, left 0 by the THETA call */
      if (layer) {
        for (K = k_first; K <= KHI; K++) {
          da = (w_ff[K] - w_ff[K - 1]) * M->dsgth_inv[2 * K] * DT;
          A3(buff, K, J, I) += da;
        }
      } else {
        for (K = k_first; K <= KHI; K++) {
          da = (w_ff[K + 1] - w_ff[K]) * M->dsgth_inv[2 * K + 1] * DT;
          A3(buff, K, J, I) += da;
        }
      }
    }

  /* Meridional advection, plane by plane (:1060-1310). */
  for (K = 1; K <= KHI; K++) {
    double *a, *vm = M->b2d[0], *vp = M->b2d[1], *v2d = M->b2d[2], *ff = M->b2d[4], *ap = M->b2d[5];
    double *ad1, *ad2, *aa, mi, mn1, vhatp, vhatm;
    if (kind == IDX_THETA && K <= M->g.k_sigma - 2) continue;
    a_min = layer ? M->h_min[K] : (nu ? nu_min : 0.);
    a = buff + K * M->n2;
    memset(vm, 0, M->n2 * sizeof(double));
    memset(vp, 0, M->n2 * sizeof(double));
    memset(v2d, 0, M->n2 * sizeof(double));
    if (layer) {
      for (J = 1; J <= NJ; J++)
        for (I = 1; I <= NI; I++) A2(v2d, J, I) = .5 * (A3(V, K, J, I) + A3(V, K - 1, J, I));
      bc2(M, v2d);
    } else {
      for (J = 0; J <= NJ + 1; J++)
        for (I = 0; I <= NI + 1; I++) A2(v2d, J, I) = A3(V, K, J, I);
    }
    for (J = 0; J <= NJ + 1; J++) {
      mi = (fabs(M->lat[2 * J]) == 90.) ? 0. : 1. / M->m[2 * J];
      for (I = 1; I <= NI; I++) {
        A2(vm, J, I) = dmin(0., A2(v2d, J, I) * mi);
        A2(vp, J, I) = dmax(0., A2(v2d, J, I) * mi);
      }
    }
    memset(ff, 0, M->n2 * sizeof(double));
    for (J = 1; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A2(ff, J, I) = A2(vp, J, I) * A2(a, J - 1, I) + A2(vm, J, I) * A2(a, J, I);
    bc2(M, ff);
    memset(ap, 0, M->n2 * sizeof(double));
    for (J = 0; J <= NJ; J++) {
      mn1 = M->mn[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        da = (A2(ff, J, I) - A2(ff, J + 1, I)) * mn1 * DT;
        A2(ap, J, I) = A2(a, J, I) + da;
      }
    }
    bc2(M, ap);
    for (J = 1; J <= NJ; J++)
      for (I = 1; I <= NI; I++)
        A2(ff, J, I) = .5 * (A2(vp, J, I) * (A2(ap, J, I) + A2(a, J - 1, I)) + A2(vm, J, I) * (A2(ap, J - 1, I) + A2(a, J, I)));
    ad1 = M->b2d[2];
    ad2 = M->b2d[3];
    memset(ad1, 0, M->n2 * sizeof(double));
    memset(ad2, 0, M->n2 * sizeof(double));
    for (J = 1; J < NJ; J++)
      for (I = 1; I <= NI; I++) {
        A2(ad1, J, I) = A2(ap, J, I) - A2(a, J - 1, I);
        A2(ad2, J, I) = A2(ap, J, I) - A2(a, J + 1, I);
      }
    for (I = 1; I <= NI; I++) {
      A2(ad1, 0, I) = 0.;
      A2(ad2, 0, I) = A2(ap, 0, I) - A2(a, 1, I);
      A2(ad1, NJ, I) = A2(ap, NJ, I) - A2(a, NJ - 1, I);
      A2(ad2, NJ, I) = 0.;
    }
    bc2(M, ad1);
    bc2(M, ad2);
    aa = M->b2d[5];
    memset(aa, 0, M->n2 * sizeof(double));
    for (J = 1; J < NJ; J++)
      for (I = 1; I <= NI; I++) {
        tmp = fabs(A2(a, J - 1, I) - 2. * A2(a, J, I) + A2(a, J + 1, I)) + ep;
        A2(aa, J, I) = tmp * tmp;
      }
    for (I = 1; I <= NI; I++) {
      tmp = fabs(-A2(a, 0, I) + A2(a, 1, I)) + ep;
      A2(aa, 0, I) = tmp * tmp;
      tmp = fabs(A2(a, NJ - 1, I) - A2(a, NJ, I)) + ep;
      A2(aa, NJ, I) = tmp * tmp;
    }
    bc2(M, aa);
    for (J = 1; J <= NJ; J++) {
      double mn2 = M->mn[2 * J];
      for (I = 1; I <= NI; I++) {
        vhatp = sqrt(A2(vp, J, I) * A2(vp, J - 1, I));
        vhatm = -sqrt(A2(vm, J, I) * A2(vm, J + 1, I));
        mu = (A2(vp, J, I) - A2(vm, J, I)) * mn2 * DT;
        al = (1. + mu) / 6.;
        gap = A2(aa, J - 1, I) / (A2(aa, J - 1, I) + (A2(a, J - 1, I) - a_min) * (A2(a, J, I) - a_min));
        gap = gap * gap;
        gam = A2(aa, J, I) / (A2(aa, J, I) + (A2(a, J - 1, I) - a_min) * (A2(a, J, I) - a_min));
        gam = gam * gam;
        bep = 1. + (1. / (2. * al) - 1.) * gap;
        bem = 1. + (1. / (2. * al) - 1.) * gam;
        behatp = 1. - gap;
        behatm = 1. - gam;
        g_hsu = -al * (A2(vp, J, I) * bep * A2(ad1, J, I) - vhatp * behatp * A2(ad1, J - 1, I) +
                       A2(vm, J, I) * bem * A2(ad2, J - 1, I) - vhatm * behatm * A2(ad2, J, I));
        A2(ff, J, I) += g_hsu;
      }
    }
    bc2(M, ff);
    for (J = 0; J <= NJ; J++) {
      mn1 = M->mn[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        da = (A2(ff, J, I) - A2(ff, J + 1, I)) * mn1 * DT;
        A2(a, J, I) += da;
      }
    }
    bc2(M, a);
  }

  /* Zonal advection, plane by plane, fluxes from a filtered copy (:1316-1484). */
  for (K = 1; K <= KHI; K++) {
    double *a = M->b2d[6], *um = M->b2d[0], *up = M->b2d[1], *u2d = M->b2d[2], *ff = M->b2d[4], *ap = M->b2d[5];
    double *ad1, *ad2, *aa, n_inv, mn1, uhatp, uhatm;
    if (kind == IDX_THETA && K <= M->g.k_sigma - 2) continue;
    a_min = layer ? M->h_min[K] : (nu ? nu_min : 0.);
    memcpy(a, buff + K * M->n2, M->n2 * sizeof(double));
    zonal_filter_2d(M, IDX_OTHER, a);
    memset(um, 0, M->n2 * sizeof(double));
    memset(up, 0, M->n2 * sizeof(double));
    memset(u2d, 0, M->n2 * sizeof(double));
    if (layer) {
      for (J = 0; J <= NJ; J++)
        for (I = 1; I <= NI; I++) A2(u2d, J, I) = .5 * (A3(U, K, J, I) + A3(U, K - 1, J, I));
      bc2(M, u2d);
    } else {
      for (J = 0; J <= NJ; J++)
        for (I = 0; I <= NI + 1; I++) A2(u2d, J, I) = A3(U, K, J, I);
    }
    for (J = 0; J <= NJ; J++) {
      n_inv = 1. / M->n[2 * J + 1];
      for (I = 0; I <= NI + 1; I++) {
        A2(um, J, I) = dmin(0., A2(u2d, J, I) * n_inv);
        A2(up, J, I) = dmax(0., A2(u2d, J, I) * n_inv);
      }
    }
    memset(ff, 0, M->n2 * sizeof(double));
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A2(ff, J, I) = A2(up, J, I) * A2(a, J, I - 1) + A2(um, J, I) * A2(a, J, I);
    bc2(M, ff);
    memset(ap, 0, M->n2 * sizeof(double));
    for (J = 0; J <= NJ; J++) {
      mn1 = M->mn[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        da = (A2(ff, J, I) - A2(ff, J, I + 1)) * mn1 * DT;
        A2(ap, J, I) = A2(a, J, I) + da;
      }
    }
    bc2(M, ap);
    ad1 = M->b2d[2];
    ad2 = M->b2d[3];
    memset(ad1, 0, M->n2 * sizeof(double));
    memset(ad2, 0, M->n2 * sizeof(double));
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        A2(ff, J, I) = .5 * (A2(up, J, I) * (A2(ap, J, I) + A2(a, J, I - 1)) + A2(um, J, I) * (A2(ap, J, I - 1) + A2(a, J, I)));
        A2(ad1, J, I) = A2(ap, J, I) - A2(a, J, I - 1);
        A2(ad2, J, I) = A2(ap, J, I) - A2(a, J, I + 1);
      }
    bc2(M, ad1);
    bc2(M, ad2);
    aa = M->b2d[5];
    memset(aa, 0, M->n2 * sizeof(double));
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        tmp = fabs(A2(a, J, I - 1) - 2. * A2(a, J, I) + A2(a, J, I + 1)) + ep;
        A2(aa, J, I) = tmp * tmp;
      }
    bc2(M, aa);
    for (J = 0; J <= NJ; J++) {
      mn1 = M->mn[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        uhatp = sqrt(A2(up, J, I) * A2(up, J, I - 1));
        uhatm = -sqrt(A2(um, J, I) * A2(um, J, I + 1));
        mu = (A2(up, J, I) - A2(um, J, I)) * mn1 * DT;
        al = (1. + mu) / 6.;
        gap = A2(aa, J, I - 1) / (A2(aa, J, I - 1) + (A2(a, J, I - 1) - a_min) * (A2(a, J, I) - a_min));
        gap = gap * gap;
        gam = A2(aa, J, I) / (A2(aa, J, I) + (A2(a, J, I - 1) - a_min) * (A2(a, J, I) - a_min));
        gam = gam * gam;
        bep = 1. + (1. / (2. * al) - 1.) * gap;
        bem = 1. + (1. / (2. * al) - 1.) * gam;
        behatp = 1. - gap;
        behatm = 1. - gam;
        g_hsu = -al * (A2(up, J, I) * bep * A2(ad1, J, I) - uhatp * behatp * A2(ad1, J, I - 1) +
                       A2(um, J, I) * bem * A2(ad2, J, I - 1) - uhatm * behatm * A2(ad2, J, I));
        A2(ff, J, I) += g_hsu;
      }
    }
    bc2(M, ff);
    for (J = 0; J <= NJ; J++) {
      mn1 = M->mn[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        da = (A2(ff, J, I) - A2(ff, J, I + 1)) * mn1 * DT;
        A3(buff, K, J, I) += da;
      }
    }
  }
  bc3(M, buff);
}

/* akima_advection(is, buff3d, HORIZONTAL_AND_VERTICAL), epic_flux.c:1502-1940: the monotonized
 * fourth-order centred divergence-form scheme (Shchepetkin and McWilliams 2003, (4.9)-(4.12)).
 * kind: IDX_OTHER = P3_INDEX (unity), IDX_THETA, IDX_HDRY.  mass_flux_top/bot are 0 for
 * Held-Suarez (epic_flux.c:47-115). */
static double akima_dela(double d0, double d1) {   /* harmonic mean of like-signed differences */
  const double tmp = d0 * d1;
  return (tmp > 0.) ? 2. * tmp / (d0 + d1) : 0.;
}
static void akima_advection(ep_model *M, int kind, double *buff) {
  const int layer = (kind == IDX_HDRY), nu = (kind == IDX_NU);
  const int k_first = (kind == IDX_THETA) ? M->g.k_sigma - 1 : 1;
  int K, J, I;
  double *w = M->wm, *w_a = M->w_a, *w_deltaa = M->w_a_diff1, *w_dela = M->w_a_diff2, *w_ff = M->w_ff;
  double aval;
  const double *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3;

  /* Vertical advection, column by column (:1549-1744). */
  for (J = 0; J <= NJ; J++)
    for (I = 0; I <= NI + 1; I++) {
      for (K = layer ? k_first : k_first - 1; K <= KHI; K++) w_a[K] = A3(buff, K, J, I);
      if (layer) {
        for (K = k_first - 1; K <= KHI; K++) w[K] = A3(M->w3, K, J, I);
        w_deltaa[k_first - 1] = 0.;
        for (K = k_first; K < KHI; K++) w_deltaa[K] = w_a[K] - w_a[K + 1];
        w_deltaa[KHI] = 0.;
        for (K = k_first; K <= KHI; K++) w_dela[K] = akima_dela(w_deltaa[K], w_deltaa[K - 1]);
        w_ff[k_first - 1] = 0.;   /* mass_flux_top for k_first = 1, else 0 */
        for (K = k_first; K < KHI; K++) {
          aval = .5 * (w_a[K] + w_a[K + 1]) - (w_dela[K] - w_dela[K + 1]) / 6.;
          w_ff[K] = w[K] * aval;
        }
        w_ff[KHI] = 0.;           /* mass_flux_bot */
        for (K = k_first; K <= KHI; K++) A3(buff, K, J, I) += (w_ff[K] - w_ff[K - 1]) * M->dsgth_inv[2 * K] * DT;
      } else if (nu) {   /* NU_TURB: interface velocities and update, the layer form of the flux (:1687-1706) */
        for (K = k_first; K <= KHI; K++)
          w[K] = (K == 1 || K == KHI) ? 0. : .5 * (A3(M->w3, K, J, I) + A3(M->w3, K - 1, J, I));
        w_deltaa[k_first - 1] = 0.;
        for (K = k_first; K < KHI; K++) w_deltaa[K] = w_a[K] - w_a[K + 1];
        w_deltaa[KHI] = 0.;
        for (K = k_first; K <= KHI; K++) w_dela[K] = akima_dela(w_deltaa[K], w_deltaa[K - 1]);
        w_ff[k_first - 1] = 0.;
        for (K = k_first; K < KHI; K++) {
          aval = .5 * (w_a[K] + w_a[K + 1]) - (w_dela[K] - w_dela[K + 1]) / 6.;
          w_ff[K] = w[K] * aval;
        }
        w_ff[KHI] = 0.;
        w_ff[KHI + 1] = 0.;   /* the reference's static entry, left 0 by the THETA call */
        for (K = k_first; K <= KHI; K++) A3(buff, K, J, I) += (w_ff[K + 1] - w_ff[K]) * M->dsgth_inv[2 * K + 1] * DT;
      } else {
        for (K = k_first; K <= KHI; K++)
          w[K] = (K == 1 || K == KHI) ? 0. : .5 * (A3(M->w3, K, J, I) + A3(M->w3, K - 1, J, I));
        for (K = k_first; K <= KHI; K++) w_deltaa[K] = w_a[K - 1] - w_a[K];
        w_dela[k_first - 1] = 0.;
        for (K = k_first; K < KHI; K++) w_dela[K] = akima_dela(w_deltaa[K], w_deltaa[K + 1]);
        w_dela[KHI] = 0.;
        for (K = k_first; K <= KHI; K++) {
          aval = .5 * (w_a[K - 1] + w_a[K]) - (w_dela[K - 1] - w_dela[K]) / 6.;
          w_ff[K] = w[K] * aval;
        }
        w_ff[KHI + 1] = 0.;
        for (K = k_first; K <= KHI; K++) A3(buff, K, J, I) += (w_ff[K + 1] - w_ff[K]) * M->dsgth_inv[2 * K + 1] * DT;
      }
    }

  /* Meridional advection, plane by plane (:1752-1820). */
  for (K = 1; K <= KHI; K++) {
    double *a = buff + K * M->n2, *v2d = M->b2d[0], *deltaa = M->b2d[1], *dela = M->b2d[2], *ff = M->b2d[3];
    double m_2j_inv, mn_2jp1;
    if (kind == IDX_THETA && K <= M->g.k_sigma - 2) continue;
    memset(v2d, 0, M->n2 * sizeof(double));
    memset(deltaa, 0, M->n2 * sizeof(double));
    memset(dela, 0, M->n2 * sizeof(double));
    memset(ff, 0, M->n2 * sizeof(double));
    if (layer) {
      for (J = 1; J <= NJ; J++)
        for (I = 1; I <= NI; I++) A2(v2d, J, I) = .5 * (A3(V, K, J, I) + A3(V, K - 1, J, I));   /* get_var at kk = 2K */
      bc2(M, v2d);
    } else {
      for (J = 0; J <= NJ + 1; J++)
        for (I = 0; I <= NI + 1; I++) A2(v2d, J, I) = A3(V, K, J, I);
    }
    for (J = 1; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A2(deltaa, J, I) = A2(a, J, I) - A2(a, J - 1, I);
    bc2(M, deltaa);
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A2(dela, J, I) = akima_dela(A2(deltaa, J, I), A2(deltaa, J + 1, I));
    bc2(M, dela);
    for (J = 1; J <= NJ; J++) {
      m_2j_inv = (fabs(M->lat[2 * J]) == 90.) ? 0. : 1. / M->m[2 * J];
      for (I = 1; I <= NI; I++) {
        aval = .5 * (A2(a, J, I) + A2(a, J - 1, I)) - (A2(dela, J, I) - A2(dela, J - 1, I)) / 6.;
        A2(ff, J, I) = A2(v2d, J, I) * aval * m_2j_inv;
      }
    }
    bc2(M, ff);
    for (J = 0; J <= NJ; J++) {
      mn_2jp1 = M->mn[2 * J + 1];
      for (I = 1; I <= NI; I++) A2(a, J, I) += (A2(ff, J, I) - A2(ff, J + 1, I)) * mn_2jp1 * DT;
    }
    bc2(M, a);
  }

  /* Zonal advection, plane by plane, fluxes from a filtered copy (:1826-1932). */
  for (K = 1; K <= KHI; K++) {
    double *a = M->b2d[6], *u2d = M->b2d[0], *deltaa = M->b2d[1], *dela = M->b2d[2], *ff = M->b2d[3];
    double n_2jp1_inv, mn_2jp1;
    if (kind == IDX_THETA && K <= M->g.k_sigma - 2) continue;
    memcpy(a, buff + K * M->n2, M->n2 * sizeof(double));
    zonal_filter_2d(M, IDX_OTHER, a);
    memset(u2d, 0, M->n2 * sizeof(double));
    memset(deltaa, 0, M->n2 * sizeof(double));
    memset(dela, 0, M->n2 * sizeof(double));
    memset(ff, 0, M->n2 * sizeof(double));
    if (layer) {
      for (J = 0; J <= NJ; J++)
        for (I = 1; I <= NI; I++) A2(u2d, J, I) = .5 * (A3(U, K, J, I) + A3(U, K - 1, J, I));   /* get_var at kk = 2K */
      bc2(M, u2d);
    } else {
      for (J = 0; J <= NJ; J++)
        for (I = 0; I <= NI + 1; I++) A2(u2d, J, I) = A3(U, K, J, I);
    }
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A2(deltaa, J, I) = A2(a, J, I) - A2(a, J, I - 1);
    bc2(M, deltaa);
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A2(dela, J, I) = akima_dela(A2(deltaa, J, I), A2(deltaa, J, I + 1));
    bc2(M, dela);
    for (J = 0; J <= NJ; J++) {
      n_2jp1_inv = 1. / M->n[2 * J + 1];
      for (I = 1; I <= NI; I++) {
        aval = .5 * (A2(a, J, I) + A2(a, J, I - 1)) - (A2(dela, J, I) - A2(dela, J, I - 1)) / 6.;
        A2(ff, J, I) = A2(u2d, J, I) * aval * n_2jp1_inv;
      }
    }
    bc2(M, ff);
    for (J = 0; J <= NJ; J++) {
      mn_2jp1 = M->mn[2 * J + 1];
      for (I = 1; I <= NI; I++) A3(buff, K, J, I) += (A2(ff, J, I) - A2(ff, J, I + 1)) * mn_2jp1 * DT;
    }
  }
  bc3(M, buff);
}

/* advection, epic_flux.c:346-637 (theta and hdry, one scheme for both) */
static void advect(ep_model *M, int kind, double *buff) {
  if (M->g.advection_scheme == EPIC_ADV_AKIMA) akima_advection(M, kind, buff);
  else hsu_advection(M, kind, buff);
}
static void advection(ep_model *M) {
  int K, J, I;
  for (K = 0; K <= KHI + 1; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) A3(M->unity, K, J, I) = 1.;
  advect(M, IDX_OTHER, M->unity);
  for (K = M->g.k_sigma - 1; K <= KHI + 1; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) A3(M->old, K, J, I) = A3(M->theta, K, J, I);
  advect(M, IDX_THETA, M->theta);
  for (K = M->g.k_sigma - 1; K <= KHI + 1; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) A3(M->theta, K, J, I) -= A3(M->old, K, J, I) * (A3(M->unity, K, J, I) - 1.);
  if (TURB_ON(M)) {   /* NU_TURB with the same scheme (UNITY stands), before HDRY, epic_flux.c:540-600 */
    for (K = 0; K <= KHI + 1; K++)
      for (J = 0; J <= NJ; J++)
        for (I = 0; I <= NI + 1; I++) A3(M->old, K, J, I) = A3(M->nu_turb, K, J, I);
    advect(M, IDX_NU, M->nu_turb);
    for (K = 0; K <= KHI + 1; K++)
      for (J = 0; J <= NJ; J++)
        for (I = 0; I <= NI + 1; I++) {
          A3(M->nu_turb, K, J, I) -= A3(M->old, K, J, I) * (A3(M->unity, K, J, I) - 1.);
          A3(M->nu_turb, K, J, I) = dmax(1.e-4 * M->g.kinvisc, A3(M->nu_turb, K, J, I));
        }
  }
  advect(M, IDX_HDRY, M->hdry);
  restore_mass(M);
  set_p2etc(M, 0);
}

/* Filtered, monotone copy of GZ3, epic_timestep.c:176-196 */
static void gz_filtered(ep_model *M) {
  int K, J, I;
  double tmp;
  memcpy(M->gz, M->gz3, M->n3 * sizeof(double));
  for (K = KHI - 1; K >= 0; K--) {
    zonal_filter_2d(M, IDX_OTHER, M->gz + K * M->n2);
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        tmp = A3(M->gz, K + 1, J, I);
        if (fcmp(tmp, 0.) == 0) A3(M->gz, K, J, I) = 1.e-3;
        else A3(M->gz, K, J, I) = dmax(A3(M->gz, K, J, I), A3(M->gz, K + 1, J, I) + fabs(A3(M->gz, K + 1, J, I)) * 1.e-5);
      }
  }
}

/* uv_pgrad_finite_volume, epic_timestep.c:909-1273 */
static void uv_pgrad_fv(ep_model *M) {
  int K, J, I;
  double *G = M->gz3, *P2a = M->p2;
  double *DU = M->dudt + (long)M->it_uv_tend * M->n3, *DV = M->dvdt + (long)M->it_uv_tend * M->n3;
  double rho, lnw, lne, lts, ltn, rlt, rlns, rlnn, pgflon, pgflat, zbsw, zbse, zbnw, zbne, zbw, zbe, ztsw, ztse, ztnw, ztne,
      ztw, zte, zbs, zbn, zts, ztn, pbw, pbe, ptw, pte, pbs, pbn, pts, ptn, top, bottom, east, west, north, south, terms1,
      terms2, dzn, dzs, tmp, a1, a2, b1, b2, b3;
#define GZ(k, j, i) A3(G, k, j, i)
#define PP(k, j, i) A3(P2a, k, j, i)
  for (K = 0; K <= KHI; K++) {
    tmp = 0.;
    for (I = 1; I <= NI; I++) tmp += GZ(K, 0, I);
    tmp /= NI;
    for (I = 0; I <= NI + 1; I++) GZ(K, -1, I) = tmp;
  }
  for (K = 0; K <= KHI; K++) {
    tmp = 0.;
    for (I = 1; I <= NI; I++) tmp += GZ(K, NJ, I);
    tmp /= NI;
    for (I = 0; I <= NI + 1; I++) GZ(K, NJ + 1, I) = tmp;
  }
  for (K = 1; K < KHI; K++)
    for (J = 0; J <= NJ; J++) {
      rlt = M->rlt[2 * J + 1];
      (void)rlt;
      rlns = M->rln[2 * J];
      rlnn = M->rln[2 * J + 2];
      I = 0;
      lne = M->lon[2 * I + 1] * DEG;
      zbse = .25 * (GZ(K, J, I) + GZ(K, J - 1, I) + GZ(K + 1, J, I) + GZ(K + 1, J - 1, I));
      zbne = .25 * (GZ(K, J, I) + GZ(K, J + 1, I) + GZ(K + 1, J, I) + GZ(K + 1, J + 1, I));
      ztse = .25 * (GZ(K, J, I) + GZ(K, J - 1, I) + GZ(K - 1, J, I) + GZ(K - 1, J - 1, I));
      ztne = .25 * (GZ(K, J, I) + GZ(K, J + 1, I) + GZ(K - 1, J, I) + GZ(K - 1, J + 1, I));
      zbe = .5 * (GZ(K, J, I) + GZ(K + 1, J, I));
      zte = .5 * (GZ(K, J, I) + GZ(K - 1, J, I));
      pbe = PP(K + 1, J, I);
      pte = PP(K, J, I);
      a1 = ztne + ztse; b1 = ztne * ztse; a2 = zbne + zbse; b2 = zbne * zbse;
      terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
      terms2 = 3. * (a1 - a2);
      east = (-terms1 * (pbe - pte) + terms2 * (zte * pbe - zbe * pte)) / (zte - zbe);
      for (I = 1; I <= NI; I++) {
        rho = .5 * (A3(M->rho3, K, J, I) + A3(M->rho3, K, J, I - 1));
        lnw = lne;
        zbsw = zbse; zbnw = zbne; zbw = zbe; ztsw = ztse; ztnw = ztne; ztw = zte; pbw = pbe; ptw = pte;
        west = east;
        lne = M->lon[2 * I + 1] * DEG;
        zbse = .25 * (GZ(K, J, I) + GZ(K, J - 1, I) + GZ(K + 1, J, I) + GZ(K + 1, J - 1, I));
        zbne = .25 * (GZ(K, J, I) + GZ(K, J + 1, I) + GZ(K + 1, J, I) + GZ(K + 1, J + 1, I));
        ztse = .25 * (GZ(K, J, I) + GZ(K, J - 1, I) + GZ(K - 1, J, I) + GZ(K - 1, J - 1, I));
        ztne = .25 * (GZ(K, J, I) + GZ(K, J + 1, I) + GZ(K - 1, J, I) + GZ(K - 1, J + 1, I));
        zbe = .5 * (GZ(K, J, I) + GZ(K + 1, J, I));
        zte = .5 * (GZ(K, J, I) + GZ(K - 1, J, I));
        pbe = PP(K + 1, J, I);
        pte = PP(K, J, I);
        a1 = ztne + ztse; b1 = ztne * ztse; a2 = zbne + zbse; b2 = zbne * zbse;
        terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
        terms2 = 3. * (a1 - a2);
        east = (-terms1 * (pbe - pte) + terms2 * (zte * pbe - zbe * pte)) / (zte - zbe);
        a1 = ztne + ztse; a2 = ztnw + ztsw;
        terms2 = 3. * (a1 - a2);
        if (fabs(2. * (zte - ztw) / (zte + ztw - zbe - zbw)) > DLOGZ_TOL) {
          b1 = ztne * ztse; b2 = ztnw * ztsw;
          terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
          top = (-terms1 * (ptw - pte) + terms2 * (zte * ptw - ztw * pte)) / (zte - ztw);
        } else top = .5 * (ptw + pte) * terms2;
        a1 = zbne + zbse; a2 = zbnw + zbsw;
        terms2 = 3. * (a1 - a2);
        if (fabs(2. * (zbe - zbw) / (zte + ztw - zbe - zbw)) > DLOGZ_TOL) {
          b1 = zbne * zbse; b2 = zbnw * zbsw;
          terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
          bottom = (-terms1 * (pbw - pbe) + terms2 * (zbe * pbw - zbw * pbe)) / (zbe - zbw);
        } else bottom = .5 * (pbw + pbe) * terms2;
        north = 0.;
        south = 0.;
        pgflon = top - bottom + south - north + west - east;
        dzn = ztne - zbne + ztnw - zbnw;
        dzs = ztse - zbse + ztsw - zbsw;
        pgflon /= (lne - lnw) * rho * (rlns * (dzs + .5 * dzn) + rlnn * (dzn + .5 * dzs));
        A3(DU, K, J, I) += pgflon;
      }
    }
  for (K = 1; K < KHI; K++)
    for (I = 1; I <= NI; I++) {
      J = 0;
      rlnn = M->rln[2 * J + 1];
      ltn = M->lat[2 * J + 1] * DEG;
      zbnw = .25 * (GZ(K, J, I) + GZ(K, J, I - 1) + GZ(K + 1, J, I) + GZ(K + 1, J, I - 1));
      zbne = .25 * (GZ(K, J, I) + GZ(K, J, I + 1) + GZ(K + 1, J, I) + GZ(K + 1, J, I + 1));
      ztnw = .25 * (GZ(K, J, I) + GZ(K, J, I - 1) + GZ(K - 1, J, I) + GZ(K - 1, J, I - 1));
      ztne = .25 * (GZ(K, J, I) + GZ(K, J, I + 1) + GZ(K - 1, J, I) + GZ(K - 1, J, I + 1));
      zbn = .5 * (GZ(K, J, I) + GZ(K + 1, J, I));
      ztn = .5 * (GZ(K, J, I) + GZ(K - 1, J, I));
      pbn = PP(K + 1, J, I);
      ptn = PP(K, J, I);
      a1 = ztne + ztnw; b1 = ztne * ztnw; a2 = zbne + zbnw; b2 = zbne * zbnw;
      terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
      terms2 = 3. * (a1 - a2);
      north = rlnn * (-terms1 * (pbn - ptn) + terms2 * (ztn * pbn - zbn * ptn)) / (ztn - zbn);
      for (J = 1; J <= NJ; J++) {
        rho = .5 * (A3(M->rho3, K, J, I) + A3(M->rho3, K, J - 1, I));
        rlt = M->rlt[2 * J];
        rlns = rlnn; lts = ltn;
        zbsw = zbnw; zbse = zbne; ztsw = ztnw; ztse = ztne;
        south = north;
        zbs = zbn; zts = ztn; pbs = pbn; pts = ptn;
        rlnn = M->rln[2 * J + 1];
        ltn = M->lat[2 * J + 1] * DEG;
        zbnw = .25 * (GZ(K, J, I) + GZ(K, J, I - 1) + GZ(K + 1, J, I) + GZ(K + 1, J, I - 1));
        zbne = .25 * (GZ(K, J, I) + GZ(K, J, I + 1) + GZ(K + 1, J, I) + GZ(K + 1, J, I + 1));
        ztnw = .25 * (GZ(K, J, I) + GZ(K, J, I - 1) + GZ(K - 1, J, I) + GZ(K - 1, J, I - 1));
        ztne = .25 * (GZ(K, J, I) + GZ(K, J, I + 1) + GZ(K - 1, J, I) + GZ(K - 1, J, I + 1));
        zbn = .5 * (GZ(K, J, I) + GZ(K + 1, J, I));
        ztn = .5 * (GZ(K, J, I) + GZ(K - 1, J, I));
        pbn = PP(K + 1, J, I);
        ptn = PP(K, J, I);
        a1 = ztne + ztnw; b1 = ztne * ztnw; a2 = zbne + zbnw; b2 = zbne * zbnw;
        terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
        terms2 = 3. * (a1 - a2);
        north = rlnn * (-terms1 * (pbn - ptn) + terms2 * (ztn * pbn - zbn * ptn)) / (ztn - zbn);
        a1 = ztse + ztsw; b1 = ztse * ztsw; a2 = zbse + zbsw; b2 = zbse * zbsw;
        terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
        terms2 = 3. * (a1 - a2);
        south = rlns * (-terms1 * (pbs - pts) + terms2 * (zts * pbs - zbs * pts)) / (zts - zbs);
        zbe = .125 * (GZ(K, J, I) + GZ(K, J, I + 1) + GZ(K, J - 1, I) + GZ(K, J - 1, I + 1) + GZ(K + 1, J, I) +
                      GZ(K + 1, J, I + 1) + GZ(K + 1, J - 1, I) + GZ(K + 1, J - 1, I + 1));
        zte = .125 * (GZ(K - 1, J, I) + GZ(K - 1, J, I + 1) + GZ(K - 1, J - 1, I) + GZ(K - 1, J - 1, I + 1) + GZ(K, J, I) +
                      GZ(K, J, I + 1) + GZ(K, J - 1, I) + GZ(K, J - 1, I + 1));
        pbe = .25 * (PP(K + 1, J, I) + PP(K + 1, J, I + 1) + PP(K + 1, J - 1, I) + PP(K + 1, J - 1, I + 1));
        pte = .25 * (PP(K, J, I) + PP(K, J, I + 1) + PP(K, J - 1, I) + PP(K, J - 1, I + 1));
        a1 = ztne + ztse; b1 = ztne * ztse; a2 = zbne + zbse; b2 = zbne * zbse;
        terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
        terms2 = 3. * (a1 - a2);
        east = .5 * (rlns - rlnn) * (-terms1 * (pbe - pte) + terms2 * (zte * pbe - zbe * pte)) / (zte - zbe);
        zbw = .125 * (GZ(K, J, I) + GZ(K, J, I - 1) + GZ(K, J - 1, I) + GZ(K, J - 1, I - 1) + GZ(K + 1, J, I) +
                      GZ(K + 1, J, I - 1) + GZ(K + 1, J - 1, I) + GZ(K + 1, J - 1, I - 1));
        ztw = .125 * (GZ(K - 1, J, I) + GZ(K - 1, J, I - 1) + GZ(K - 1, J - 1, I) + GZ(K - 1, J - 1, I - 1) + GZ(K, J, I) +
                      GZ(K, J, I - 1) + GZ(K, J - 1, I) + GZ(K, J - 1, I - 1));
        pbw = .25 * (PP(K + 1, J, I) + PP(K + 1, J, I - 1) + PP(K + 1, J - 1, I) + PP(K + 1, J - 1, I - 1));
        ptw = .25 * (PP(K, J, I) + PP(K, J, I - 1) + PP(K, J - 1, I) + PP(K, J - 1, I - 1));
        a1 = ztnw + ztsw; b1 = ztnw * ztsw; a2 = zbnw + zbsw; b2 = zbnw * zbsw;
        terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
        terms2 = 3. * (a1 - a2);
        west = .5 * (rlns - rlnn) * (-terms1 * (pbw - ptw) + terms2 * (ztw * pbw - zbw * ptw)) / (ztw - zbw);
        a1 = ztne + ztnw; a2 = ztse + ztsw;
        terms2 = 3. * (a1 - a2);
        if (fabs(2. * (ztn - zts) / (ztn + zts - zbn - zbs)) > DLOGZ_TOL) {
          b1 = ztne * ztnw; b2 = ztse * ztsw; b3 = ztne * ztse + ztnw * ztsw;
          terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
          top = .5 * ((ptn - pts) * ((rlnn + rlns) * terms1 + (rlnn - rlns) * (b1 + b2 - b3)) + (rlnn + rlns) * terms2 * (ztn * pts - zts * ptn)) /
                (ztn - zts);
        } else top = .25 * (rlnn + rlns) * (pts + ptn) * terms2;
        a1 = zbne + zbnw; a2 = zbse + zbsw;
        terms2 = 3. * (a1 - a2);
        if (fabs(2. * (zbn - zbs) / (ztn + zts - zbn - zbs)) > DLOGZ_TOL) {
          b1 = zbne * zbnw; b2 = zbse * zbsw; b3 = zbne * zbse + zbnw * zbsw;
          terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
          bottom = .5 * ((pbn - pbs) * ((rlnn + rlns) * terms1 + (rlnn - rlns) * (b1 + b2 - b3)) + (rlnn + rlns) * terms2 * (zbn * pbs - zbs * pbn)) /
                   (zbn - zbs);
        } else bottom = .25 * (rlnn + rlns) * (pbs + pbn) * terms2;
        pgflat = top - bottom + south - (north + west + east);
        dzn = ztne - zbne + ztnw - zbnw;
        dzs = ztse - zbse + ztsw - zbsw;
        pgflat /= (ltn - lts) * rho * rlt * (rlns * (dzs + .5 * dzn) + rlnn * (dzn + .5 * dzs));
        A3(DV, K, J, I) += pgflat;
      }
    }
#undef GZ
#undef PP
}

/* divergence_damping, epic_subgrid.c:1792-1885 (skipped when the coefficient is zero) */
static void divergence_damping(ep_model *M) {
  int K, J, I;
  double nudiv = M->g.nudiv_nondim * M->max_nu[2], coef;
  double *buff = M->b2d[7], *div = M->b2d[6];
  const double *U = M->u + (long)M->it_uv_dis * M->n3, *V = M->v + (long)M->it_uv_dis * M->n3;
  double *DU = M->dudt + (long)M->it_uv_tend * M->n3, *DV = M->dvdt + (long)M->it_uv_tend * M->n3;
  if (nudiv == 0.) return;
  for (K = 1; K < KHI; K++) {
    memcpy(buff, U + K * M->n2, M->n2 * sizeof(double));
    zonal_filter_2d(M, IDX_U, buff);
    divergence(M, buff, V + K * M->n2, div);
    for (J = 0; J <= NJ; J++) {
      coef = (M->lat[2 * J + 1] > LAT0) ? nudiv * M->m0 : nudiv * M->m[2 * J + 1];
      for (I = 1; I <= NI; I++) A3(DU, K, J, I) += coef * (A2(div, J, I) - A2(div, J, I - 1));
    }
    for (J = 1; J <= NJ; J++) {
      coef = nudiv * M->n[2 * J];
      for (I = 1; I <= NI; I++) A3(DV, K, J, I) += coef * (A2(div, J, I) - A2(div, J - 1, I));
    }
  }
}

/* timeplane_bookkeeping, epic_funcs_diag.c:7086-7124 */
static void timeplane_bookkeeping(ep_model *M) {
  if (M->g.uv_scheme == EPIC_UV_AB3) {
    M->it_uv = 0;
    M->it_uv_dis = 0;
    M->it_uv_tend = M->it_zero;
  } else {
    M->it_uv = M->it_zero;
    M->it_uv_dis = (A3(M->u + (long)M->it_minus1 * M->n3, 1, 0, 1) == DBL_MAX) ? M->it_zero : M->it_minus1;
    M->it_uv_tend = 0;
  }
}

/* adams_bashforth_step / leapfrog_step for U and V and the index rotation, epic_timestep.c:242-281, :406-615 */
static void uv_update(ep_model *M) {
  int w, K, J, I, jlo, itmp;
  for (w = 0; w < 2; w++) {
    double *val = w == 0 ? M->u : M->v, *ten = w == 0 ? M->dudt : M->dvdt;
    jlo = w == 0 ? 0 : 1;
    if (M->g.uv_scheme == EPIC_UV_AB3) {
      double ab0, ab1, ab2;
      double *d0 = ten + (long)M->it_zero * M->n3, *dm1 = ten + (long)M->it_minus1 * M->n3, *dm2 = ten + (long)M->it_minus2 * M->n3;
      double *x = val + (long)M->it_uv * M->n3;
      if (A3(dm2, 1, jlo, 1) == DBL_MAX) {
        if (A3(dm1, 1, jlo, 1) == DBL_MAX) { ab0 = 1.; ab1 = 0.; ab2 = 0.; }
        else { ab0 = 3. / 2.; ab1 = -1. / 2.; ab2 = 0.; }
      } else { ab0 = 23. / 12.; ab1 = -16. / 12.; ab2 = 5. / 12.; }
      for (K = 1; K < KHI; K++)
        for (J = jlo; J <= NJ; J++)
          for (I = 1; I <= NI; I++)
            A3(x, K, J, I) += DT * (ab0 * A3(d0, K, J, I) + ab1 * A3(dm1, K, J, I) + ab2 * A3(dm2, K, J, I));
      bc3(M, x);
    } else {
      double *x0 = val + (long)M->it_zero * M->n3, *xm1 = val + (long)M->it_minus1 * M->n3, *d = ten + (long)M->it_uv_tend * M->n3;
      double twodt, old_filtered, present, new_leap;
      if (A3(xm1, 1, jlo, 1) == DBL_MAX) {
        for (K = 1; K < KHI; K++)
          for (J = jlo; J <= NJ; J++)
            for (I = 1; I <= NI; I++) {
              present = A3(x0, K, J, I);
              A3(xm1, K, J, I) = present + DT * A3(d, K, J, I);
            }
        bc3(M, xm1);
      } else {
        twodt = 2. * DT;
        for (K = 1; K < KHI; K++)
          for (J = jlo; J <= NJ; J++)
            for (I = 1; I <= NI; I++) {
              old_filtered = A3(xm1, K, J, I);
              present = A3(x0, K, J, I);
              new_leap = old_filtered + twodt * A3(d, K, J, I);
              A3(xm1, K, J, I) = new_leap;
              A3(x0, K, J, I) = present * (1. - 2. * GAMMA_ASSELIN) + GAMMA_ASSELIN * (old_filtered + new_leap);
            }
        bc3(M, xm1);
        bc3(M, x0);
      }
    }
  }
  if (M->g.uv_scheme == EPIC_UV_AB3) {
    itmp = M->it_minus2;
    M->it_minus2 = M->it_minus1;
    M->it_minus1 = M->it_zero;
    M->it_zero = itmp;
  } else {
    itmp = M->it_minus1;
    M->it_minus1 = M->it_zero;
    M->it_zero = itmp;
  }
  timeplane_bookkeeping(M);
}

/* ---------------------------------------------------------------------------------------- */
/* Turbulence closure, Spalart-Allmaras DES: src/shared/epic_subgrid.c:207-590 (the diffusion */
/* parts), 1236-1488, 1493-1790, 1889-2080, 2127-3228; crank_nicolson and the band solver,   */
/* src/shared/epic_funcs_util.c:2994-3400, 3643-3787                                         */
/* ---------------------------------------------------------------------------------------- */

/* The libepicport_cr.so build routes these two to the correctly rounded ones of the kernels. */
#ifndef EP_TURB_ATAN
#define EP_TURB_ATAN atan
#define EP_TURB_COS cos
#endif
enum { WALL_U, WALL_V, WALL_H };   /* law_of_the_wall's grids: U_INDEX, V_INDEX, the h-grid default */

static double limit_range(double lo, double x, double hi) { return x < lo ? lo : (x > hi ? hi : x); } /* LIMIT_RANGE, include/epic.h:147 */

static void turb_error(ep_model *M, const char *what, int J, int I, double v) {
  if (!M->turb_err[0]) snprintf(M->turb_err, sizeof(M->turb_err), "%s (J=%d, I=%d): %g", what, J, I, v);
}

/* D_WALL as dwall_SA sets it before each use, epic_subgrid.c:2716-2770 */
static double d_wall(const ep_model *M, int K, int J, int I) {
  if (M->g.gas_giant) return DBL_MAX;
  return (A3(M->gz3, K, J, I) - M->g.topo_scale * A2(M->gz_surface, J, I)) / M->grav[2 * J + 1];
}

/* delta_SA, :2774-2808 */
static double delta_sa(const ep_model *M, int K, int J, int I) {
  const int jj = 2 * J + 1;
  double dx = 1. / M->m[jj], dy = 1. / M->n[jj], dz, delta;
  if (K < M->nk) dz = (A3(M->gz3, K - 1, J, I) - A3(M->gz3, K + 1, J, I)) / M->grav[jj];
  else dz = (A3(M->gz3, K - 1, J, I) - A3(M->gz3, M->nk, J, I)) / M->grav[jj];
  delta = dmin(dx, dy);
  return dmin(delta, dz);
}

/* func_utau, :3112-3165: the wall law's residual u+(y+) - u_tan/u_tau */
static double func_utau(ep_model *M, double u_tau, double u_tan, double dwall) {
  const double C = 5., const1 = 0.127, const2 = 1. / .41, const3 = 0.41 * 1.43e-3, one_third = 1. / 3.,
               sqrt_one_third = sqrt(1. / 3.), pi_six = M_PI / 6.;
  double u_plus = 0., y_plus, yy;
  if (u_tau != 0.) u_plus = u_tan / u_tau;
  else turb_error(M, "func_utau: u_tau = 0", -1, -1, u_tau);
  y_plus = fabs(u_tau * dwall / KINVISC);
  if (u_plus < 0.1) return 1.e+20;
  if (y_plus < 5.) return y_plus - u_plus;
  if (y_plus < 70.) {
    yy = const1 * y_plus;
    return (one_third * log((1. + yy) / (sqrt(yy * (yy - 1.) + 1.))) +
            sqrt_one_third * (EP_TURB_ATAN(sqrt_one_third * (2. * yy - 1.)) + pi_six)) / const1 +
           .25 * const2 * log(1. + const3 * pow(y_plus, 4.)) - u_plus;
  }
  return const2 * log(y_plus) + C - u_plus;
}

/* law_of_the_wall, :2995-3105: the eddy viscosity next to the wall from the secant solution of
 * the wall law for the friction velocity (index: WALL_U, WALL_V or the h-grid WALL_H) */
static double law_of_the_wall(ep_model *M, int K, int J, int I, int index, double t_vis, double u_tan) {
  const double tol = 1.e-6;
  double dwall, dwall_inv = 0., u_tau = 0., x1, x2, xl, dx, fl, f, rts, swap;
  int iter;
  (void)t_vis;   /* the reference scales t_vis by fv1 and then leaves it unused */
  if (M->g.gas_giant) return 1.0e-4 * KINVISC;
  if (index == WALL_U) dwall = 0.5 * (d_wall(M, K, J, I) + d_wall(M, K, J, I - 1));
  else if (index == WALL_V)
    dwall = 0.5 * M->m[2 * J] * (d_wall(M, K, J, I) / M->m[2 * J + 1] + d_wall(M, K, J - 1, I) / M->m[2 * J - 1]);
  else dwall = d_wall(M, K, J, I);
  if (dwall * u_tan < 0.00023) return 0.01 * KINVISC;
  if (dwall > 0.) dwall_inv = 1. / dwall;
  else turb_error(M, "law_of_the_wall: dwall <= 0", J, I, dwall);
  x1 = sqrt(KINVISC * (1. + 0.01) * u_tan * dwall_inv);
  x2 = sqrt(KINVISC * (1. + 20.) * u_tan * dwall_inv);
  fl = func_utau(M, x1, u_tan, dwall);
  f = func_utau(M, x2, u_tan, dwall);
  if (fabs(fl) < fabs(f)) {
    rts = x1; xl = x2; swap = fl; fl = f; f = swap;
  } else {
    xl = x1; rts = x2;
  }
  for (iter = 0; iter < 30; iter++) {
    dx = (xl - rts) * f / (f - fl);
    xl = rts;
    fl = f;
    rts += dx;
    f = func_utau(M, rts, u_tan, dwall);
    if (f > .99e+20) return 0.01 * KINVISC;
    if (fabs(dx) < tol || f == 0.0) {
      u_tau = rts;
      break;
    }
  }
  if (iter < 30) return dmax((u_tau * u_tau * dwall / u_tan) - KINVISC, 0.01 * KINVISC);
  return 20. * KINVISC;
}

/* invert_fv1, :3172-3226: the working viscosity nu~ from an eddy viscosity (fitted fv1) */
static double invert_fv1(ep_model *M, double t_vis) {
  const double pi_factor = M_PI * 0.5 / 30.0;
  double chi, fv1;
  if (t_vis < 0.) turb_error(M, "invert_fv1: t_vis < 0", -1, -1, t_vis);
  chi = t_vis / KINVISC;
  if (chi > 30) return t_vis;
  if (chi < 0.4) return KINVISC * pow(chi * SA_CV1_3, .25);
  fv1 = EP_TURB_COS(pi_factor * pow(chi, 0.35));
  fv1 = 1.0 - fv1 * fv1;
  return KINVISC * chi / fv1;
}

/* tau_surface, :2819-2988: the wall stress under the wind component `index` (WALL_U, WALL_V)
 * or for NU_TURB (WALL_H), from layer K = nk-1 */
static void tau_surface(ep_model *M, int index, double *tau_wall) {
  const int K = M->nk - 1;
  const double *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3;
  const double *u2d = U + K * M->n2, *v2d = V + K * M->n2;
  double *kie = M->b2d[1], rho, nu_turb, dz, kin, u_tan, dc;
  int J, I;
  memset(kie, 0, M->n2 * sizeof(double));
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++) A2(kie, J, I) = get_kin(M, u2d, v2d, J, I);
  bc2(M, kie);
  if (M->g.gas_giant) {
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A2(tau_wall, J, I) = 0.;
  } else if (index == WALL_U) {
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        rho = .5 * (A3(M->rho3, K, J, I) + A3(M->rho3, K, J, I - 1));
        nu_turb = .5 * (A3(M->nu_turb, K, J, I) + A3(M->nu_turb, K, J, I - 1));
        dz = .5 * (A3(M->gz3, K, J, I) + A3(M->gz3, K, J, I - 1) - A3(M->gz3, K + 1, J, I) - A3(M->gz3, K + 1, J, I - 1)) /
             M->grav[2 * J + 1];
        kin = .5 * (A2(kie, J, I) + A2(kie, J, I - 1));
        u_tan = sqrt(2. * kin);
        dc = law_of_the_wall(M, K, J, I, WALL_U, nu_turb, u_tan);
        A2(tau_wall, J, I) = (M->g.dynvisc + rho * dc) * (A3(U, K, J, I) - 0.) / dz;
      }
  } else if (index == WALL_V) {
    for (J = 1; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        rho = .5 * (A3(M->rho3, K, J, I) + A3(M->rho3, K, J - 1, I));
        nu_turb = .5 * (A3(M->nu_turb, K, J, I) + A3(M->nu_turb, K, J - 1, I));
        dz = .5 * (A3(M->gz3, K, J, I) + A3(M->gz3, K, J - 1, I) - A3(M->gz3, K + 1, J, I) - A3(M->gz3, K + 1, J - 1, I)) /
             M->grav[2 * J];
        kin = .5 * (A2(kie, J, I) + A2(kie, J - 1, I));
        u_tan = sqrt(2. * kin);
        dc = law_of_the_wall(M, K, J, I, WALL_V, nu_turb, u_tan);
        A2(tau_wall, J, I) = (M->g.dynvisc + rho * dc) * (A3(V, K, J, I) - 0.) / dz;
      }
  } else {
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        rho = A3(M->rho3, K, J, I);
        nu_turb = A3(M->nu_turb, K, J, I);
        dz = (A3(M->gz3, K, J, I) - A3(M->gz3, K + 1, J, I)) / M->grav[2 * J + 1];
        kin = get_kin(M, u2d, v2d, J, I);
        u_tan = sqrt(2. * kin);
        dc = law_of_the_wall(M, K, J, I, WALL_H, nu_turb, u_tan);
        nu_turb = invert_fv1(M, dc);
        A2(tau_wall, J, I) = (M->g.dynvisc + rho * nu_turb) * (u_tan - 0.) / dz;
      }
  }
  bc2(M, tau_wall);
}

/* set_diffusion_coef, :2171-2302 (inside store_diag).  Note that it leaves DIFFUSION_COEF_UV
 * zero above the bottom layer: the winds' turbulent viscosity acts only at K = nk. */
static void set_diffusion_coef(ep_model *M) {
  const int kend = M->g.gas_giant ? KHI : KHI - 1;
  const double *U = M->u + (long)M->it_uv_dis * M->n3, *V = M->v + (long)M->it_uv_dis * M->n3;
  double max_nu2, chi3, fv1, turb, nu_turb, kin, u_tan;
  int K, J, I;
  for (K = 1; K <= kend; K++)
    for (J = 0; J <= NJ; J++) {
      max_nu2 = M->max_nu[2] * dmin(1., pow(M->g.dy0 * M->m[2 * J + 1], -2.));
      for (I = 0; I <= NI + 1; I++) {
        chi3 = A3(M->nu_turb, K, J, I) / KINVISC;
        chi3 *= chi3 * chi3;
        fv1 = chi3 / (chi3 + SA_CV1_3);
        turb = fv1 * A3(M->nu_turb, K, J, I);
        A3(M->dc_theta, K, J, I) = limit_range(0., turb, max_nu2);
        A3(M->dc_mass, K, J, I) = limit_range(0., turb, max_nu2);
      }
    }
  if (!M->g.gas_giant) {
    K = KHI - 1;
    for (J = 0; J <= NJ; J++) {
      max_nu2 = M->max_nu[2] * dmin(1., pow(M->g.dy0 * M->m[2 * J + 1], -2.));
      for (I = 1; I <= NI; I++) {
        nu_turb = A3(M->nu_turb, K, J, I);
        kin = get_kin(M, U + K * M->n2, V + K * M->n2, J, I);
        u_tan = sqrt(2. * kin);
        turb = law_of_the_wall(M, K, J, I, WALL_H, nu_turb, u_tan);
        A3(M->dc_uv, KHI, J, I) = limit_range(0., turb + KINVISC, max_nu2);
        A3(M->dc_theta, KHI, J, I) = limit_range(0., turb, max_nu2);
        A3(M->dc_mass, KHI, J, I) = limit_range(0., turb, max_nu2);
      }
    }
  }
  bc3(M, M->dc_uv);
  bc3(M, M->dc_theta);
  bc3(M, M->dc_mass);
}

/* stability_factor, :2309-2415, over kk = 1 .. 2 nk + 1 */
static void stability_factor(ep_model *M, int J, int I, double *sf) {
  const double max_ri = 100.;
  double *Ri = M->ri, slope;
  int K, kk;
  if (!M->g.stability_factor) {
    for (kk = 1; kk <= 2 * KHI + 1; kk++) sf[kk] = 1.;
    return;
  }
  Ri[1] = limit_range(-max_ri, A3(M->ri2, 1, J, I), max_ri);
  for (K = 1; K < KHI; K++) {
    kk = 2 * K;
    Ri[kk] = limit_range(-max_ri, A3(M->ri2, K, J, I), max_ri);
    Ri[kk + 1] = limit_range(-max_ri, .5 * (A3(M->ri2, K, J, I) + A3(M->ri2, K + 1, J, I)), max_ri);
  }
  kk = 2 * KHI;
  Ri[kk] = limit_range(-max_ri, A3(M->ri2, KHI, J, I), max_ri);
  Ri[kk + 1] = Ri[kk];
  for (kk = 1; kk <= 2 * KHI; kk++) {
    slope = Ri[kk + 1] - Ri[kk];
    if (-slope > .9 * max_ri) Ri[kk + 1] = 0.;
  }
  for (kk = 1; kk <= 2 * KHI + 1; kk++) {
    if (Ri[kk] > 0.) sf[kk] = 1. / (1. + 10. * Ri[kk] * (1. + 8. * Ri[kk]));
    else sf[kk] = sqrt(1. - 18. * Ri[kk]);
  }
}

/* get_brunt2 on the interface kk = 2K+1, 1 <= K < nk (np = 1, fpara off, Held-Suarez cp),
 * epic_funcs_diag.c:2885-3075 */
static double brunt2_iface(const ep_model *M, int K, int J, int I) {
  double pressure = A3(M->p3, K, J, I), temperature = A3(M->t3, K, J, I), density = A3(M->rho3, K, J, I);
  double cp = 1004., mu = M->mu_dry, deltap, deltaT, drho_dp_T, drho_dT_p, Drho_Dp, g;
  deltap = 0.001 * pressure;
  deltaT = 0.001 * temperature;
  drho_dp_T = (return_density(pressure + deltap, temperature, mu) - return_density(pressure - deltap, temperature, mu)) /
              (2. * deltap);
  drho_dT_p = (return_density(pressure, temperature + deltaT, mu) - return_density(pressure, temperature - deltaT, mu)) /
              (2. * deltaT);
  Drho_Dp = (A3(M->rho2, K + 1, J, I) - A3(M->rho2, K, J, I)) / (A3(M->p2, K + 1, J, I) - A3(M->p2, K, J, I));
  g = M->grav[2 * J + 1];
  return g * g * (Drho_Dp - drho_dp_T + temperature / (cp * density * density) * drho_dT_p * drho_dT_p);
}

/* source_sink_SA, :2434-2711: production, gradient, destruction and buoyancy terms of the
 * Spalart-Allmaras equation.  NU_TURB is updated in place in K, J, I order, so each point reads
 * the new values of its K-1, J-1 and I-1 neighbours and the old ones of K+1, J+1, I+1. */
static void source_sink_sa(ep_model *M) {
  const double cw2 = 0.3, cw3_6 = pow(2., 6.), cb1 = 0.1355, cb2 = 0.622, sigma = 2. / 3., kappa = 0.41,
               kappa_2 = kappa * kappa, cw1 = (cb1 / kappa_2) + ((1. + cb2) / sigma), C_DES = 0.65, nu_turb_limiter = 3000.;
  const double *U = M->u + (long)M->it_uv_dis * M->n3, *V = M->v + (long)M->it_uv_dis * M->n3;
  double *u2d = M->b2d[0], *v2d = M->b2d[1], *NU = M->nu_turb;
  double mn_v, mn_u, m_2jp1, n_2jp1, n_2jp2, n_2j, delta, d_tilda, dz_inv, chi, fv1, fv2, s11, s22, s33, s12, s13, s23;
  double u_var1, u_var3, v_var1, v_var3, w_var1, w_var3, h_rho, S, tmp1, tmp2, S_tilda, dnudt, r_sa, g_sa, fw, brunt2, brunt;
  int K, J, I, kk, jj;
  for (K = 1; K < KHI; K++) {
    kk = 2 * K + 1;
    memset(u2d, 0, M->n2 * sizeof(double));
    memset(v2d, 0, M->n2 * sizeof(double));
    /* U onto the v-grid; zero at the poles (the edge rows of the globe) */
    for (J = 1; J <= NJ; J++) {
      jj = 2 * J;
      mn_v = .5 / (1. / M->mn[jj - 1] + 1. / M->mn[jj + 1]);
      for (I = 1; I <= NI; I++)
        A2(u2d, J, I) = ((A3(U, K, J, I) + A3(U, K, J, I + 1)) * (1. / M->mn[jj + 1]) +
                         (A3(U, K, J - 1, I) + A3(U, K, J - 1, I + 1)) * (1. / M->mn[jj - 1])) * mn_v;
    }
    for (I = 1; I <= NI; I++) A2(u2d, 0, I) = 0.;
    for (I = 1; I <= NI; I++) A2(u2d, NJ + 1, I) = 0.;
    bc2(M, u2d);
    /* V onto the u-grid */
    for (J = 0; J <= NJ; J++) {
      jj = 2 * J;
      mn_u = .5 / (1. / M->mn[jj] + 1. / M->mn[jj + 2]);
      for (I = 1; I <= NI; I++)
        A2(v2d, J, I) = ((A3(V, K, J, I) + A3(V, K, J, I - 1)) * (1. / M->mn[jj]) +
                         (A3(V, K, J + 1, I) + A3(V, K, J + 1, I - 1)) * (1. / M->mn[jj + 2])) * mn_u;
    }
    bc2(M, v2d);
    for (J = 0; J <= NJ; J++) {
      jj = 2 * J;
      m_2jp1 = M->m[jj + 1];
      n_2jp1 = M->n[jj + 1];
      n_2jp2 = M->n[jj + 2];
      n_2j = M->n[jj];
      for (I = 1; I <= NI; I++) {
        delta = delta_sa(M, K, J, I);
        d_tilda = dmin(d_wall(M, K, J, I), C_DES * delta);
        dz_inv = M->grav[jj + 1] / (A3(M->gz3, K - 1, J, I) - A3(M->gz3, K + 1, J, I));
        chi = A3(NU, K, J, I) / KINVISC;
        fv1 = pow(chi, 3.) / (pow(chi, 3.) + SA_CV1_3);
        fv2 = 1. - (chi / (1. + chi * fv1));
        s11 = (A3(U, K, J, I + 1) - A3(U, K, J, I)) * m_2jp1;
        s22 = (A3(V, K, J + 1, I) - A3(V, K, J, I)) * n_2jp1;
        s33 = (A3(M->w3, K - 1, J, I) - A3(M->w3, K + 1, J, I)) / (M->sgth[kk - 2] - M->sgth[kk + 2]);
        s12 = .5 * ((A2(u2d, J + 1, I) - A2(u2d, J, I)) * n_2jp1 + (A2(v2d, J, I + 1) - A2(v2d, J, I)) * m_2jp1);
        u_var3 = 0.5 * (A3(U, K + 1, J, I) + A3(U, K + 1, J, I + 1));
        u_var1 = 0.5 * (A3(U, K - 1, J, I) + A3(U, K - 1, J, I + 1));
        w_var3 = 0.5 * (A3(M->w3, K, J, I) + A3(M->w3, K, J, I + 1));
        w_var1 = 0.5 * (A3(M->w3, K, J, I) + A3(M->w3, K, J, I - 1));
        h_rho = A3(M->h3, K, J, I) / A3(M->rho3, K, J, I);
        s13 = .5 * ((u_var1 - u_var3) * dz_inv + h_rho * (w_var3 - w_var1) * m_2jp1);
        v_var3 = 0.5 * (A3(V, K + 1, J, I) + A3(V, K + 1, J + 1, I));
        v_var1 = 0.5 * (A3(V, K - 1, J, I) + A3(V, K - 1, J + 1, I));
        w_var3 = 0.5 * (A3(M->w3, K, J, I) + A3(M->w3, K, J + 1, I));
        w_var1 = 0.5 * (A3(M->w3, K, J, I) + A3(M->w3, K, J - 1, I));
        s23 = .5 * ((v_var1 - v_var3) * dz_inv + h_rho * (w_var3 - w_var1) * n_2jp1);
        S = sqrt(2. * (s11 * s11 + s22 * s22 + s33 * s33 + 2. * (s12 * s12 + s13 * s13 + s23 * s23)));
        tmp1 = kappa_2 * d_tilda * d_tilda;
        S_tilda = S + (A3(NU, K, J, I) * fv2) / tmp1;
        tmp2 = S_tilda * tmp1;
        dnudt = cb1 * S_tilda * A3(NU, K, J, I);
        dnudt += (cb2 / sigma) * pow(((A3(NU, K, J, I + 1) - A3(NU, K, J, I - 1)) * m_2jp1 * .5), 2.);
        dnudt += (cb2 / sigma) * pow(.5 * ((A3(NU, K, J + 1, I) - A3(NU, K, J, I)) * n_2jp2 +
                                           (A3(NU, K, J, I) - A3(NU, K, J - 1, I)) * n_2j), 2.);
        dnudt += (cb2 / sigma) * pow(((A3(NU, K - 1, J, I) - A3(NU, K + 1, J, I)) * dz_inv), 2.);
        fw = 1.;
        if (tmp2 != 0.) {
          r_sa = A3(NU, K, J, I) / tmp2;
          if (r_sa < 0.) turb_error(M, "source_sink_SA: r_sa < 0", J, I, r_sa);
          else if (r_sa < 10.) {
            g_sa = r_sa + cw2 * (pow(r_sa, 6.) - r_sa);
            fw = g_sa * pow(((1. + cw3_6) / (pow(g_sa, 6.) + cw3_6)), (1. / 6.));
          }
        }
        dnudt -= cw1 * fw * pow((A3(NU, K, J, I) / d_tilda), 2.);
        brunt2 = brunt2_iface(M, K, J, I);
        brunt = sqrt(fabs(brunt2));
        if (brunt2 < 0.) dnudt -= A3(NU, K, J, I) * exp(-A3(NU, K, J, I) / nu_turb_limiter) * brunt2 / brunt;
        A3(NU, K, J, I) += DT * dnudt;
        A3(NU, K, J, I) = dmax(1.e-4 * KINVISC, A3(NU, K, J, I));
      }
    }
  }
  /* the solid-surface block: the reference computes law_of_the_wall and invert_fv1 for K = nk-1
   * and then overwrites NU_TURB(nk) with MAX(1e-4 kinvisc, NU_TURB(nk-1)), :2690-2704 */
  if (!M->g.gas_giant)
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) A3(NU, KHI, J, I) = dmax(1.e-4 * KINVISC, A3(NU, KHI - 1, J, I));
  bc3(M, NU);
}

/* restore_mass(NU_TURB_INDEX), epic_adjust.c:80-88 */
static void restore_nu_turb(ep_model *M) {
  int K, J, I;
  for (K = 0; K <= KHI + 1; K++)
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) A3(M->nu_turb, K, J, I) = dmax(1.e-4 * KINVISC, A3(M->nu_turb, K, J, I));
}

/* laplacian_h, epic_subgrid.c:423-583: DIFF_COEF times the Laplacian of an h-grid plane, with the
 * zonal filter on a copy of hh before d/dx and on the x-flux before its divergence */
static void laplacian_h(ep_model *M, const double *hh, const double *diff_coef, double *lph) {
  double *gh1 = M->b2d[3], *gh2 = M->b2d[4], *buffji = M->b2d[5], m_2jp1, n_2jp1, m_2j_inv, m_2jp2_inv;
  int J, I;
  memset(gh1, 0, M->n2 * sizeof(double));
  memset(gh2, 0, M->n2 * sizeof(double));
  memcpy(buffji, hh, M->n2 * sizeof(double));
  zonal_filter_2d(M, IDX_OTHER, buffji);
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++) A2(gh1, J, I) = M->m[2 * J + 1] * (A2(buffji, J, I) - A2(buffji, J, I - 1));
  for (J = 1; J <= NJ; J++)
    for (I = 1; I <= NI; I++) A2(gh2, J, I) = M->n[2 * J] * (A2(hh, J, I) - A2(hh, J - 1, I));
  bc2(M, gh1);
  bc2(M, gh2);
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++) A2(gh1, J, I) *= .5 * (A2(diff_coef, J, I) + A2(diff_coef, J, I - 1));
  bc2(M, gh1);
  for (J = 1; J <= NJ; J++)
    for (I = 1; I <= NI; I++) A2(gh2, J, I) *= .5 * (A2(diff_coef, J, I) + A2(diff_coef, J - 1, I));
  bc2(M, gh2);
  zonal_filter_2d(M, IDX_U, gh1);
  for (J = 0; J <= NJ; J++) {
    m_2jp1 = M->m[2 * J + 1];
    n_2jp1 = M->n[2 * J + 1];
    m_2j_inv = (J == 0) ? 0. : 1. / M->m[2 * J];
    m_2jp2_inv = (J == NJ) ? 0. : 1. / M->m[2 * J + 2];
    for (I = 1; I <= NI; I++)
      A2(lph, J, I) = m_2jp1 * ((A2(gh1, J, I + 1) - A2(gh1, J, I)) +
                                n_2jp1 * (A2(gh2, J + 1, I) * m_2jp2_inv - A2(gh2, J, I) * m_2j_inv));
  }
  bc2(M, lph);
}

/* scalar_horizontal_diffusion, :275-415: THETA (interfaces k_sigma-1 .. nk), set_p2etc, NU_TURB
 * (interfaces 1 .. nk) */
static void scalar_horizontal_diffusion(ep_model *M) {
  const double sigma_inv = 3. / 2., dt = DT;
  double *hh = M->b2d[0], *lph = M->b2d[1], *dc = M->b2d[2];
  int K, J, I;
  for (K = M->g.k_sigma - 1; K <= KHI; K++) {
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        A2(hh, J, I) = A3(M->theta, K, J, I);
        A2(dc, J, I) = A3(M->dc_theta, K, J, I);
      }
    laplacian_h(M, hh, dc, lph);
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) A3(M->theta, K, J, I) += dt * A2(lph, J, I);
  }
  set_p2etc(M, 1);
  for (K = 1; K <= KHI; K++) {
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        A2(hh, J, I) = A3(M->nu_turb, K, J, I);
        A2(dc, J, I) = sigma_inv * (KINVISC + A3(M->nu_turb, K, J, I));
      }
    laplacian_h(M, hh, dc, lph);
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) A3(M->nu_turb, K, J, I) += dt * A2(lph, J, I);
  }
  restore_nu_turb(M);
}

/* band_decomp / band_back_sub for m1 = m2 = 1 (Numerical Recipes' bandec/banbks with partial
 * pivoting, zero-based), epic_funcs_util.c:3130-3260: A[i][0..2] holds row i's band */
static void band_decomp3(int n, double (*A)[3], double *al, int *index) {
  int i, j, k, l = 1;
  double tmp;
  A[0][0] = A[0][1]; A[0][1] = A[0][2]; A[0][2] = 0.;
  for (k = 0; k < n; k++) {
    tmp = A[k][0];
    i = k;
    if (l < n) l++;
    for (j = k + 1; j < l; j++)
      if (fabs(A[j][0]) > fabs(tmp)) { tmp = A[j][0]; i = j; }
    index[k] = i;
    if (tmp == 0.) A[k][0] = 1.e-20;
    if (i != k)
      for (j = 0; j < 3; j++) { tmp = A[k][j]; A[k][j] = A[i][j]; A[i][j] = tmp; }
    for (i = k + 1; i < l; i++) {
      tmp = A[i][0] / A[k][0];
      al[k] = tmp;
      for (j = 1; j < 3; j++) A[i][j - 1] = A[i][j] - tmp * A[k][j];
      A[i][2] = 0.;
    }
  }
}
static void band_back_sub3(int n, double (*A)[3], const double *al, const int *index, double *b) {
  int i, k, l = 1;
  double tmp;
  for (k = 0; k < n; k++) {
    i = index[k];
    if (i != k) { tmp = b[k]; b[k] = b[i]; b[i] = tmp; }
    if (l < n) l++;
    for (i = k + 1; i < l; i++) b[i] -= al[k] * b[k];
  }
  l = 1;
  for (i = n - 1; i >= 0; i--) {
    tmp = b[i];
    for (k = 1; k < l; k++) tmp -= A[i][k] * b[k + i];
    b[i] = tmp / A[i][0];
    if (l < 3) l++;
  }
}

/* crank_nicolson, epic_funcs_util.c:3643-3787, with tridiag(WITH_PIVOTING) (:2994-3120):
 * band_decomp, band_back_sub and one band_improve pass (:3330-3400).  Arrays z, A, mu, rho and
 * ans are indexed 0 .. n+1; A[0] or A[n+1] above .99e20 marks a no-flux end.  Returns nonzero
 * if z is not increasing where it is used. */
static int crank_nicolson(ep_model *M, int n, double dt, const double *z, const double *A, const double *mu,
                          const double *rho, double *ans) {
  double (*Ab)[3] = (double (*)[3])M->tb, (*Ao)[3] = (double (*)[3])M->taorig, *a = M->tl, *b = M->tl + (n + 2),
         *c = M->tl + 2 * (n + 2), *r = M->tr, *al = M->tal, coeff1, coeff3, factor, sdp;
  int j, jstart = A[0] > .99e+20 ? 2 : 1, jend = A[n + 1] > .99e+20 ? n : n + 1, i, k, jj;
  for (j = jstart; j <= jend; j++)
    if (z[j] <= z[j - 1]) return 1;
  coeff3 = (A[0] > .99e+20) ? 0. : mu[0] / (z[1] - z[0]);
  a[0] = 0.;
  c[n - 1] = 0.;
  for (j = 1; j <= n; j++) {
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
  for (j = 0; j < n; j++) {
    Ab[j][2] = Ao[j][2] = c[j];
    Ab[j][1] = Ao[j][1] = b[j];
    Ab[j][0] = Ao[j][0] = a[j];
  }
  band_decomp3(n, Ab, al, M->tindex);
  for (j = 0; j < n; j++) ans[j + 1] = r[j];
  band_back_sub3(n, Ab, al, M->tindex, ans + 1);
  /* band_improve: residual of the original band matrix in double, one correction */
  for (i = 0; i < n; i++) {
    k = i - 1;
    jj = n - k < 3 ? n - k : 3;
    sdp = -r[i];
    for (j = k < 0 ? -k : 0; j < jj; j++) sdp += Ao[i][j] * ans[1 + j + k];
    M->cd[i] = sdp;
  }
  band_back_sub3(n, Ab, al, M->tindex, M->cd);
  for (i = 0; i < n; i++) ans[i + 1] -= M->cd[i];
  return 0;
}

/* scalar_vertical_diffusion, :1273-1488: THETA below k_sigma, set_p2etc, NU_TURB with the wall
 * stress at the bottom (implicit Crank-Nicolson in z = GZ3/g) */
static int scalar_vertical_diffusion(ep_model *M) {
  const double sigma_inv = 3. / 2.;
  double *tau_wall = M->b2d[0], *zee = M->cz, *aaa = M->ca, *dee = M->crho, *ans = M->cans, *sf = M->sf2, gi;
  int K, J, I, kay, n;
  memset(tau_wall, 0, M->n2 * sizeof(double));
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++) {
      gi = M->grav[2 * J + 1];
      stability_factor(M, J, I, sf);
      aaa[0] = 1.e+20;
      zee[0] = A3(M->gz3, KHI, J, I) / gi;
      for (K = KHI; K >= M->g.k_sigma - 2; K--) {
        kay = KHI - K + 1;
        aaa[kay] = A3(M->theta, K, J, I);
        zee[kay] = A3(M->gz3, K, J, I) / gi;
      }
      for (K = KHI; K > M->g.k_sigma - 2; K--) {
        kay = KHI - K + 1;
        dee[kay] = sf[2 * K] * .5 * (A3(M->dc_theta, K, J, I) + A3(M->dc_theta, K - 1, J, I));
      }
      n = KHI - M->g.k_sigma + 2;
      if (crank_nicolson(M, n, DT, zee, aaa, dee, NULL, ans)) return fail(M, "crank_nicolson: z not increasing (THETA, J=%d, I=%d)", J, I);
      for (K = KHI; K >= M->g.k_sigma - 1; K--) A3(M->theta, K, J, I) = ans[KHI - K + 1];
    }
  bc3(M, M->theta);
  set_p2etc(M, 1);
  tau_surface(M, WALL_H, tau_wall);
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++) {
      gi = M->grav[2 * J + 1];
      aaa[KHI + 2] = 1.e+20;
      zee[KHI + 2] = (A3(M->gz3, 0, J, I) + (A3(M->gz3, 0, J, I) - A3(M->gz3, 1, J, I))) / gi;
      for (K = KHI; K >= 0; K--) {
        kay = KHI - K + 1;
        aaa[kay] = A3(M->nu_turb, K, J, I);
        zee[kay] = A3(M->gz3, K, J, I) / gi;
      }
      for (K = KHI; K > 0; K--) {
        kay = KHI - K + 1;
        dee[kay] = sigma_inv * (KINVISC + .5 * (A3(M->nu_turb, K, J, I) + A3(M->nu_turb, K - 1, J, I)));
      }
      zee[0] = (A3(M->gz3, KHI, J, I) - (A3(M->gz3, KHI - 1, J, I) - A3(M->gz3, KHI, J, I))) / gi;
      dee[0] = dee[1];
      aaa[0] = aaa[1] - A2(tau_wall, J, I) * (zee[1] - zee[0]) / dee[0];
      if (crank_nicolson(M, KHI + 1, DT, zee, aaa, dee, NULL, ans)) return fail(M, "crank_nicolson: z not increasing (NU_TURB, J=%d, I=%d)", J, I);
      for (K = KHI; K >= 0; K--) A3(M->nu_turb, K, J, I) = ans[KHI - K + 1];
    }
  bc3(M, M->nu_turb);
  restore_nu_turb(M);
  return 0;
}

/* uv_horizontal_diffusion, :1571-1787: the horizontal-gradient viscous stresses of the winds
 * (Tannehill, Anderson and Pletcher 1997) into DUDT, DVDT */
static void uv_horizontal_diffusion(ep_model *M) {
  double *tau11 = M->b2d[0], *tau22 = M->b2d[1], *tau33 = M->b2d[2], *tau12 = M->b2d[3], *coeffd = M->b2d[4],
         *h_rho = M->b2d[5], *uu = M->b2d[6], *vv = M->b2d[7];
  double *DU = M->dudt + (long)M->it_uv_tend * M->n3, *DV = M->dvdt + (long)M->it_uv_tend * M->n3;
  const double *U = M->u + (long)M->it_uv_dis * M->n3, *V = M->v + (long)M->it_uv_dis * M->n3;
  double rln_inv, m_2jp1, m_2j, n_2jp2, n_2jp1, n_2j, e11, e22, e33, e12, coeff, ze, h_inv;
  int K, J, I, jj;
  for (K = 1; K < KHI; K++) {
    for (J = 0; J <= NJ; J++)
      for (I = 0; I <= NI + 1; I++) {
        A2(coeffd, J, I) = M->g.dynvisc + A3(M->rho3, K, J, I) * A3(M->dc_uv, K, J, I);
        A2(h_rho, J, I) = A3(M->h3, K, J, I) / A3(M->rho3, K, J, I);
      }
    memcpy(uu, U + K * M->n2, M->n2 * sizeof(double));
    memcpy(vv, V + K * M->n2, M->n2 * sizeof(double));
    zonal_filter_2d(M, IDX_OTHER, coeffd);
    zonal_filter_2d(M, IDX_OTHER, h_rho);
    zonal_filter_2d(M, IDX_U, uu);
    zonal_filter_2d(M, IDX_V, vv);
    for (J = 0; J <= NJ; J++) {
      jj = 2 * J;
      rln_inv = 1. / M->rln[jj + 1];
      m_2jp1 = M->m[jj + 1];
      m_2j = M->m[jj];
      n_2jp2 = M->n[jj + 2];
      n_2jp1 = M->n[jj + 1];
      n_2j = M->n[jj];
      (void)m_2j;
      for (I = 1; I <= NI; I++) {
        e11 = (A2(uu, J, I + 1) - A2(uu, J, I)) * m_2jp1 +
              .5 * (A2(vv, J, I) + A2(vv, J + 1, I)) * rln_inv * (M->rln[jj + 2] - M->rln[jj]) * n_2jp1;
        e22 = (A2(vv, J + 1, I) - A2(vv, J, I)) * n_2jp1;
        coeff = .5 / A2(h_rho, J, I);
        e33 = coeff * (A2(uu, J, I + 1) * (A2(h_rho, J, I + 1) - A2(h_rho, J, I)) * m_2jp1 +
                       A2(uu, J, I) * (A2(h_rho, J, I) - A2(h_rho, J, I - 1)) * m_2jp1);
        if (A2(vv, J + 1, I) != 0.) e33 += coeff * A2(vv, J + 1, I) * (A2(h_rho, J + 1, I) - A2(h_rho, J, I)) * n_2jp2;
        if (A2(vv, J, I) != 0.) e33 += coeff * A2(vv, J, I) * (A2(h_rho, J, I) - A2(h_rho, J - 1, I)) * n_2j;
        coeff = A2(h_rho, J, I) * (2. / 3.) * A2(coeffd, J, I);
        A2(tau11, J, I) = coeff * (2. * e11 - e22 - e33);
        A2(tau22, J, I) = coeff * (2. * e22 - e11 - e33);
        A2(tau33, J, I) = (coeff / A2(h_rho, J, I)) * (2. * e33 - e11 - e22);
      }
    }
    bc2(M, tau11);
    bc2(M, tau22);
    bc2(M, tau33);
    /* TAU12 at the poles: vorticity(ON_SIGMATHETA, RELATIVE, uu, vv) there (epic_funcs_diag.c:
     * 4279-4290, 4357-4379), times minus the row's mean of COEFFD H_RHO */
    ze = 0.;
    for (I = 1; I <= NI; I++) ze -= A2(uu, 0, I);
    ze *= M->mn[0] / ((M->m[1]) * (double)(NI));
    for (I = 1; I <= NI; I++) A2(tau12, 0, I) = ze;
    ze = 0.;
    for (I = 1; I <= NI; I++) ze += A2(uu, NJ, I);
    ze *= M->mn[2 * (NJ + 1)] / (M->m[2 * NJ + 1] * (double)(NI));
    for (I = 1; I <= NI; I++) A2(tau12, NJ + 1, I) = ze;
    coeff = 0.;
    for (I = 1; I <= NI; I++) coeff += A2(coeffd, NJ, I) * A2(h_rho, NJ, I);
    coeff /= NI;
    for (I = 1; I <= NI; I++) A2(tau12, NJ + 1, I) *= -coeff;
    coeff = 0.;
    for (I = 1; I <= NI; I++) coeff += A2(coeffd, 0, I) * A2(h_rho, 0, I);
    coeff /= NI;
    for (I = 1; I <= NI; I++) A2(tau12, 0, I) *= -coeff;
    for (J = 1; J <= NJ; J++) {
      jj = 2 * J;
      m_2j = M->m[jj];
      n_2j = M->n[jj];
      for (I = 1; I <= NI; I++) {
        e12 = (A2(vv, J, I) - A2(vv, J, I - 1)) * m_2j +
              M->rln[jj] * (A2(uu, J, I) / M->rln[jj + 1] - A2(uu, J - 1, I) / M->rln[jj - 1]) * n_2j;
        coeff = .25 * (A2(coeffd, J, I) * A2(h_rho, J, I) + A2(coeffd, J, I - 1) * A2(h_rho, J, I - 1) +
                       A2(coeffd, J - 1, I) * A2(h_rho, J - 1, I) + A2(coeffd, J - 1, I - 1) * A2(h_rho, J - 1, I - 1));
        A2(tau12, J, I) = coeff * e12;
      }
    }
    bc2(M, tau12);
    for (J = 0; J <= NJ; J++) {
      jj = 2 * J;
      rln_inv = 1. / M->rln[jj + 1];
      m_2jp1 = M->m[jj + 1];
      n_2jp1 = M->n[jj + 1];
      for (I = 1; I <= NI; I++) {
        h_inv = 2. / (A3(M->hdry, K, J, I) + A3(M->hdry, K, J, I - 1));
        A3(DU, K, J, I) += h_inv * (m_2jp1 * (A2(tau11, J, I) - A2(tau11, J, I - 1)) +
                                    n_2jp1 * rln_inv * (M->rln[jj + 2] * A2(tau12, J + 1, I) - M->rln[jj] * A2(tau12, J, I) +
                                                        .5 * (A2(tau12, J + 1, I) + A2(tau12, J, I)) * (M->rln[jj + 2] - M->rln[jj])) -
                                    .5 * (A2(tau33, J, I) + A2(tau33, J, I - 1)) * m_2jp1 * (A2(h_rho, J, I) - A2(h_rho, J, I - 1)));
      }
    }
    for (J = 1; J <= NJ; J++) {
      jj = 2 * J;
      rln_inv = 1. / M->rln[jj];
      m_2j = M->m[jj];
      n_2j = M->n[jj];
      for (I = 1; I <= NI; I++) {
        h_inv = 2. / (A3(M->hdry, K, J, I) + A3(M->hdry, K, J - 1, I));
        A3(DV, K, J, I) += h_inv * (m_2j * (A2(tau12, J, I) - A2(tau12, J, I - 1)) -
                                    n_2j * rln_inv * (M->rln[jj + 1] * A2(tau22, J, I) - M->rln[jj - 1] * A2(tau22, J - 1, I) -
                                                      .5 * (A2(tau11, J, I) + A2(tau11, J - 1, I)) * (M->rln[jj + 1] - M->rln[jj - 1])) -
                                    .5 * (A2(tau33, J, I) + A2(tau33, J - 1, I)) * n_2j * (A2(h_rho, J, I) - A2(h_rho, J - 1, I)));
      }
    }
  }
}

/* uv_vertical_diffusion, :1940-2075: implicit vertical viscosity of U and V (layers 1 .. nk-1)
 * with the wall stress below, after the time step (plane it_uv) */
static int uv_vertical_diffusion(ep_model *M) {
  double *tau_wall = M->b2d[0], *zee = M->cz, *aaa = M->ca, *rho = M->crho, *ans = M->cans, *sf0 = M->sf0,
         *sf2 = M->sf2, *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3, gi;
  double *mu_b = M->cd + (KHI + 3);   /* crank_nicolson's band_improve residual reuses cd[0..n) */
  int K, J, I, kay;
  memset(tau_wall, 0, M->n2 * sizeof(double));
  tau_surface(M, WALL_U, tau_wall);
  for (J = 0; J <= NJ; J++)
    for (I = 1; I <= NI; I++) {
      gi = M->grav[2 * J + 1];
      stability_factor(M, J, I, sf2);
      stability_factor(M, J, I - 1, sf0);
      aaa[KHI] = 1.e+20;
      zee[KHI] = .5 * (A3(M->gz3, 0, J, I) + A3(M->gz3, 0, J, I - 1)) / gi;
      for (K = KHI - 1; K >= 1; K--) {
        kay = KHI - K;
        aaa[kay] = A3(U, K, J, I);
        zee[kay] = .5 * (A3(M->gz3, K, J, I) + A3(M->gz3, K, J, I - 1)) / gi;
        rho[kay] = .5 * (A3(M->rho3, K, J, I) + A3(M->rho3, K, J, I - 1));
      }
      for (K = KHI - 1; K >= 1; K--) {
        kay = KHI - K;
        mu_b[kay] = M->g.dynvisc + .5 * (sf2[2 * K] * A3(M->rho2, K, J, I) * .5 * (A3(M->dc_uv, K - 1, J, I) + A3(M->dc_uv, K, J, I)) +
                                         sf0[2 * K] * A3(M->rho2, K, J, I - 1) * .5 * (A3(M->dc_uv, K - 1, J, I - 1) + A3(M->dc_uv, K, J, I - 1)));
      }
      zee[0] = .5 * (A3(M->gz3, KHI, J, I) + A3(M->gz3, KHI, J, I - 1)) / gi;
      mu_b[0] = mu_b[1];
      aaa[0] = aaa[1] - A2(tau_wall, J, I) * (zee[1] - zee[0]) / mu_b[0];
      if (crank_nicolson(M, KHI - 1, DT, zee, aaa, mu_b, rho, ans)) return fail(M, "crank_nicolson: z not increasing (U, J=%d, I=%d)", J, I);
      for (K = KHI - 1; K >= 1; K--) A3(U, K, J, I) = ans[KHI - K];
    }
  bc3(M, U);
  tau_surface(M, WALL_V, tau_wall);
  for (J = 1; J <= NJ; J++)
    for (I = 1; I <= NI; I++) {
      gi = M->grav[2 * J];
      stability_factor(M, J, I, sf2);
      stability_factor(M, J - 1, I, sf0);
      aaa[KHI] = 1.e+20;
      zee[KHI] = .5 * (A3(M->gz3, 0, J, I) + A3(M->gz3, 0, J - 1, I)) / gi;
      for (K = KHI - 1; K >= 1; K--) {
        kay = KHI - K;
        aaa[kay] = A3(V, K, J, I);
        zee[kay] = .5 * (A3(M->gz3, K, J, I) + A3(M->gz3, K, J - 1, I)) / gi;
        rho[kay] = .5 * (A3(M->rho3, K, J, I) + A3(M->rho3, K, J - 1, I));
      }
      for (K = KHI - 1; K >= 1; K--) {
        kay = KHI - K;
        mu_b[kay] = M->g.dynvisc + .5 * (sf2[2 * K] * A3(M->rho2, K, J, I) * .5 * (A3(M->dc_uv, K - 1, J, I) + A3(M->dc_uv, K, J, I)) +
                                         sf0[2 * K] * A3(M->rho2, K, J - 1, I) * .5 * (A3(M->dc_uv, K - 1, J - 1, I) + A3(M->dc_uv, K, J - 1, I)));
      }
      zee[0] = .5 * (A3(M->gz3, KHI, J, I) + A3(M->gz3, KHI, J - 1, I)) / gi;
      mu_b[0] = mu_b[1];
      aaa[0] = aaa[1] - A2(tau_wall, J, I) * (zee[1] - zee[0]) / mu_b[0];
      if (crank_nicolson(M, KHI - 1, DT, zee, aaa, mu_b, rho, ans)) return fail(M, "crank_nicolson: z not increasing (V, J=%d, I=%d)", J, I);
      for (K = KHI - 1; K >= 1; K--) A3(V, K, J, I) = ans[KHI - K];
    }
  bc3(M, V);
  return 0;
}

static int turb_check(ep_model *M) {
  if (M->turb_err[0]) return fail(M, "%s", M->turb_err);
  return 0;
}

/* ---------------------------------------------------------------------------------------- */
/* Driver                                                                                   */
/* ---------------------------------------------------------------------------------------- */

int ep_stage(ep_model *M, int stage) {
  int rc = 0;
  switch (stage) {
    case EP_ST_ZERO_TEND:
      memset(M->dudt + (long)M->it_uv_tend * M->n3, 0, M->n3 * sizeof(double));
      memset(M->dvdt + (long)M->it_uv_tend * M->n3, 0, M->n3 * sizeof(double));
      break;
    case EP_ST_SOURCE_SINK: source_sink(M); break;
    case EP_ST_CALC_W: rc = calc_w(M); break;
    case EP_ST_UV_CORE: uv_core(M); break;
    case EP_ST_UV_DRAG: uv_drag(M); break;
    case EP_ST_SCALAR_HSUB:
      meridional_hyperviscosity(M, IDX_HDRY, M->hdry);
      zonal_hyperviscosity(M, IDX_HDRY, M->hdry);
      restore_mass(M);
      meridional_hyperviscosity(M, IDX_THETA, M->theta);
      zonal_hyperviscosity(M, IDX_THETA, M->theta);
      if (TURB_ON(M)) {
        meridional_hyperviscosity(M, IDX_OTHER, M->nu_turb);
        zonal_hyperviscosity(M, IDX_OTHER, M->nu_turb);
        restore_nu_turb(M);
      }
      break;
    case EP_ST_ADVECTION: advection(M); break;
    case EP_ST_PGRAD_VARS: rc = store_pgrad_vars(M); break;
    case EP_ST_GZ_FILTER: gz_filtered(M); break;
    case EP_ST_FILTER_TEND:
      rc = zonal_filter_3d(M, IDX_U, M->dudt + (long)M->it_uv_tend * M->n3);
      if (!rc) rc = zonal_filter_3d(M, IDX_V, M->dvdt + (long)M->it_uv_tend * M->n3);
      break;
    case EP_ST_FILTER_MASS:
      rc = zonal_filter_3d(M, IDX_HDRY, M->hdry);
      if (!rc) restore_mass(M);
      if (!rc) rc = zonal_filter_3d(M, IDX_THETA, M->theta);
      if (!rc && TURB_ON(M)) {
        rc = zonal_filter_3d(M, IDX_OTHER, M->nu_turb);
        if (!rc) restore_nu_turb(M);
      }
      break;
    case EP_ST_P2ETC_UPDATE: set_p2etc(M, 1); break;
    case EP_ST_UV_PGRAD: uv_pgrad_fv(M); break;
    case EP_ST_DIV_DAMP: divergence_damping(M); break;
    case EP_ST_UV_UPDATE: uv_update(M); break;
    case EP_ST_UV_HYPERVISC:
      meridional_hyperviscosity(M, IDX_U, M->u + (long)M->it_uv * M->n3);
      meridional_hyperviscosity(M, IDX_V, M->v + (long)M->it_uv * M->n3);
      zonal_hyperviscosity(M, IDX_U, M->u + (long)M->it_uv * M->n3);
      zonal_hyperviscosity(M, IDX_V, M->v + (long)M->it_uv * M->n3);
      break;
    case EP_ST_STORE_DIAG:
      store_diag(M);
      if (TURB_ON(M)) set_diffusion_coef(M);
      break;
    case EP_ST_CALC_HEATING: calc_heating(M); break;
    case EP_ST_P2ETC_NOUPDATE: set_p2etc(M, 0); break;
    case EP_ST_TURB_SOURCE: source_sink_sa(M); break;
    case EP_ST_SCALAR_HDIFF: scalar_horizontal_diffusion(M); break;
    case EP_ST_SCALAR_VDIFF: rc = scalar_vertical_diffusion(M); break;
    case EP_ST_UV_HDIFF: uv_horizontal_diffusion(M); break;
    case EP_ST_UV_VDIFF: rc = uv_vertical_diffusion(M); break;
    default: return fail(M, "unknown stage %d", stage);
  }
  if (!rc && TURB_ON(M)) rc = turb_check(M);
  return rc;
}

int ep_timestep(ep_model *M, int action) {
  int s, rc;
  static const int step[] = {EP_ST_ZERO_TEND, EP_ST_SOURCE_SINK, EP_ST_CALC_W, EP_ST_UV_CORE, EP_ST_UV_DRAG,
                             EP_ST_SCALAR_HSUB, EP_ST_ADVECTION, EP_ST_PGRAD_VARS, EP_ST_GZ_FILTER, EP_ST_FILTER_TEND,
                             EP_ST_FILTER_MASS, EP_ST_P2ETC_UPDATE, EP_ST_PGRAD_VARS, EP_ST_UV_PGRAD, EP_ST_DIV_DAMP,
                             EP_ST_UV_UPDATE, EP_ST_UV_HYPERVISC, -1, EP_ST_STORE_DIAG, EP_ST_CALC_HEATING};
  static const int sync[] = {EP_ST_P2ETC_UPDATE, EP_ST_PGRAD_VARS, EP_ST_STORE_DIAG, EP_ST_CALC_HEATING, EP_ST_CALC_W};
  /* with the turbulence closure (timestep, epic_timestep.c:130-290; the subgrid wrappers
   * scalar_horizontal_subgrid, scalar_vertical_subgrid, uv_horizontal_subgrid and
   * uv_vertical_subgrid, epic_subgrid.c:207,1241,1493,1894, choose by diffusion_direction) */
  int turb[40], nt = 0;
  if (!M->uploaded) return fail(M, "timestep before upload");
  if (action == EPIC_STEP_PROGS_AND_SYNC_DIAGS && TURB_ON(M)) {
    for (s = 0; s < (int)(sizeof(step) / sizeof(step[0])); s++) {
      if (step[s] == EP_ST_UV_CORE) turb[nt++] = EP_ST_TURB_SOURCE;
      if (step[s] == EP_ST_SCALAR_HSUB && DIFF_HORIZONTAL(M)) turb[nt++] = EP_ST_SCALAR_HDIFF;
      if (step[s] == EP_ST_DIV_DAMP && DIFF_HORIZONTAL(M)) turb[nt++] = EP_ST_UV_HDIFF;
      if (step[s] == EP_ST_UV_HYPERVISC && DIFF_VERTICAL(M)) turb[nt++] = EP_ST_UV_VDIFF;
      turb[nt++] = step[s];
      if (step[s] == EP_ST_SCALAR_HSUB && DIFF_VERTICAL(M)) turb[nt++] = EP_ST_SCALAR_VDIFF;
    }
    for (s = 0; s < nt; s++) {
      if (turb[s] < 0) { M->model_time += M->g.dt; continue; }
      rc = ep_stage(M, turb[s]);
      if (rc) return rc;
    }
  } else if (action == EPIC_STEP_PROGS_AND_SYNC_DIAGS) {
    for (s = 0; s < (int)(sizeof(step) / sizeof(step[0])); s++) {
      if (step[s] < 0) { M->model_time += M->g.dt; continue; }
      rc = ep_stage(M, step[s]);
      if (rc) return rc;
    }
  } else if (action == EPIC_SYNC_DIAGS_ONLY) {
    for (s = 0; s < 5; s++) {
      rc = ep_stage(M, sync[s]);
      if (rc) return rc;
    }
  } else return fail(M, "unrecognized action=%d", action);
  return 0;
}

int ep_run(ep_model *M, int nsteps) {
  int s, rc;
  for (s = 0; s < nsteps; s++) {
    rc = ep_timestep(M, EPIC_STEP_PROGS_AND_SYNC_DIAGS);
    if (rc) return rc;
    M->itime++;
  }
  return 0;
}

static double *dup1(const double *src, long n) {
  double *d = (double *)calloc((size_t)n, sizeof(double));
  if (d && src) memcpy(d, src, (size_t)n * sizeof(double));
  return d;
}

ep_model *ep_create(const epic_grid *g) {
  ep_model *M;
  int i, nj1, ni1, nk1;
  double eps;
  if (!g || g->ni < 4 || (g->ni & (g->ni - 1)) || g->nj < 3 || g->nk < 3 || g->globe_latbot != -90. || g->globe_lattop != 90.) {
    snprintf(create_err, sizeof(create_err), "unsupported grid");
    return NULL;
  }
  if (g->k_sigma < 2 || g->k_sigma > g->nk) {
    snprintf(create_err, sizeof(create_err), "k_sigma=%d out of range", g->k_sigma);
    return NULL;
  }
  M = (ep_model *)calloc(1, sizeof(ep_model));
  M->g = *g;
  M->ni = g->ni; M->nj = g->nj; M->nk = g->nk;
  M->iadim = g->ni + 2; M->jadim = g->nj + 3; M->kadim = g->nk + 2;
  M->n2 = (long)M->iadim * M->jadim;
  M->n3 = M->n2 * M->kadim;
  M->nvp = g->uv_scheme == EPIC_UV_AB3 ? 1 : 2;
  M->ntp = g->uv_scheme == EPIC_UV_AB3 ? 3 : 1;
  nj1 = 2 * (g->nj + 1) + 1; ni1 = 2 * (g->ni + 1) + 1; nk1 = 2 * (g->nk + 1) + 1;
  M->lon = dup1(g->lon, ni1); M->lat = dup1(g->lat, nj1); M->rln = dup1(g->rln, nj1); M->rlt = dup1(g->rlt, nj1);
  M->f = dup1(g->f, nj1); M->m = dup1(g->m, nj1); M->n = dup1(g->n, nj1); M->mn = dup1(g->mn, nj1);
  M->grav = dup1(g->g, nj1); M->sgth = dup1(g->sigmatheta, nk1); M->dsgth = dup1(g->dsgth, nk1);
  M->dsgth_inv = dup1(g->dsgth_inv, nk1); M->h_min = dup1(g->h_min, g->nk + 2);
  M->t_sponge_inv = dup1(g->t_sponge_inv, g->k_sponge + 1);
  M->u = dup1(NULL, M->nvp * M->n3); M->v = dup1(NULL, M->nvp * M->n3);
  M->dudt = dup1(NULL, M->ntp * M->n3); M->dvdt = dup1(NULL, M->ntp * M->n3);
#define NEW3(x) M->x = dup1(NULL, M->n3)
  NEW3(hdry); NEW3(theta); NEW3(p3); NEW3(h3); NEW3(p2); NEW3(theta2); NEW3(t2); NEW3(t3); NEW3(rho2); NEW3(rho3);
  NEW3(exner3); NEW3(gz3); NEW3(mont3); NEW3(heat3); NEW3(pv3); NEW3(ri2); NEW3(div_uv3); NEW3(w3); NEW3(dzdt3);
  NEW3(u_spinup); NEW3(gz); NEW3(sum_div); NEW3(unity); NEW3(old); NEW3(varz);
#undef NEW3
  M->gz_surface = dup1(NULL, M->n2);
  for (i = 0; i < 8; i++) M->b2d[i] = dup1(NULL, M->n2);
  M->data = dup1(NULL, g->ni + 1);
  M->table = (trip *)calloc(g->nk + 2, sizeof(trip));
  M->high_lat_h = dup1(NULL, M->n2);
  M->high_lat_pv = dup1(NULL, M->n2);
  M->h_coef = (trip *)calloc(g->nj + 2, sizeof(trip));
  M->v_coef = (trip *)calloc(g->nj + 2, sizeof(trip));
  M->mn_inv = dup1(NULL, nj1);
  for (i = 0; i < nj1; i++) M->mn_inv[i] = 1. / M->mn[i];
  M->wm = dup1(NULL, g->nk + 2); M->wp = dup1(NULL, g->nk + 2); M->w_a = dup1(NULL, g->nk + 2);
  M->w_a_pred = dup1(NULL, g->nk + 2); M->w_a_min = dup1(NULL, g->nk + 2); M->w_ff = dup1(NULL, g->nk + 2);
  M->w_a_diff1 = dup1(NULL, g->nk + 2); M->w_a_diff2 = dup1(NULL, g->nk + 2); M->w_aaa = dup1(NULL, g->nk + 2);
  /* machine_epsilon (epic_funcs_util.c:1247-1265), then its cube root as calc_w uses it */
  eps = 1.;
  while (1. + eps != 1.) eps *= .5;
  eps *= 2.;
  M->eps13 = pow(eps, 1. / 3.);
  M->mu_dry = 1. / (M->g.rgas / R_GAS);
  if (M->g.x_h2 > 0.) thermo_setup(M);
  if (g->turbulence != EPIC_TURB_OFF) {
    const int nc = g->nk + 3;
    if (g->turbulence != EPIC_TURB_SA_DES || g->diffusion_direction < 1 || g->diffusion_direction > 3) {
      snprintf(create_err, sizeof(create_err), "turbulence=%d, diffusion_direction=%d", g->turbulence, g->diffusion_direction);
      free(M);
      return NULL;
    }
    M->nu_turb = dup1(NULL, M->n3); M->dc_uv = dup1(NULL, M->n3); M->dc_theta = dup1(NULL, M->n3); M->dc_mass = dup1(NULL, M->n3);
    M->cz = dup1(NULL, nc); M->ca = dup1(NULL, nc); M->cd = dup1(NULL, 2 * nc); M->crho = dup1(NULL, nc);
    M->cans = dup1(NULL, nc); M->sf0 = dup1(NULL, 2 * nc); M->sf2 = dup1(NULL, 2 * nc); M->ri = dup1(NULL, 2 * nc);
    M->tb = dup1(NULL, 3 * nc); M->taorig = dup1(NULL, 3 * nc); M->tl = dup1(NULL, 3 * nc); M->tr = dup1(NULL, nc);
    M->tal = dup1(NULL, nc);
    M->tindex = (int *)calloc(nc, sizeof(int));
  }
  {
    /* set_max_nu, epic_subgrid.c:82-158 */
    double dt = (double)g->dt, dy2 = g->dy0 * g->dy0;
    for (i = 0; i < 9; i++) M->max_nu[i] = 0.;
    if (g->uv_scheme == EPIC_UV_AB3) {
      M->max_nu[0] = (1. / 3.) / dt; M->max_nu[2] = (dy2 / 30.) / dt; M->max_nu[4] = (dy2 / 240.) * (dy2 / dt);
      M->max_nu[6] = (dy2 / 800.) * (dy2 / dt) * dy2; M->max_nu[8] = (dy2 / 2400.) * (dy2 / dt) * dy2 * dy2;
    } else {
      M->max_nu[0] = .5 / dt; M->max_nu[2] = dy2 / (8. * dt); M->max_nu[4] = M->max_nu[2] * dy2 / 8.;
      M->max_nu[6] = M->max_nu[4] * dy2 / 8.; M->max_nu[8] = M->max_nu[6] * dy2 / 8.;
    }
  }
  filter_tables(M);
  visc_tables(M);
  M->it_zero = 0; M->it_minus1 = 1; M->it_minus2 = 2;
  return M;
}

void ep_destroy(ep_model *M) {
  int i;
  double **ps[] = {&M->lon, &M->lat, &M->rln, &M->rlt, &M->f, &M->m, &M->n, &M->mn, &M->grav, &M->sgth, &M->dsgth, &M->dsgth_inv,
                   &M->h_min, &M->t_sponge_inv, &M->u, &M->v, &M->dudt, &M->dvdt, &M->hdry, &M->theta, &M->p3, &M->h3, &M->p2,
                   &M->theta2, &M->t2, &M->t3, &M->rho2, &M->rho3, &M->exner3, &M->gz3, &M->mont3, &M->heat3, &M->pv3,
                   &M->ri2, &M->div_uv3, &M->w3, &M->dzdt3, &M->u_spinup, &M->gz_surface, &M->gz, &M->sum_div, &M->unity,
                   &M->old, &M->varz, &M->data, &M->high_lat_h, &M->high_lat_pv, &M->mn_inv, &M->wm, &M->wp, &M->w_a,
                   &M->w_a_pred, &M->w_a_min, &M->w_ff, &M->w_a_diff1, &M->w_a_diff2, &M->w_aaa};
  if (!M) return;
  for (i = 0; i < (int)(sizeof(ps) / sizeof(ps[0])); i++) free(*ps[i]);
  for (i = 0; i < 8; i++) free(M->b2d[i]);
  free(M->table); free(M->h_coef); free(M->v_coef);
  {
    double *turb[] = {M->nu_turb, M->dc_uv, M->dc_theta, M->dc_mass, M->cz, M->ca, M->cd, M->crho, M->cans, M->sf0,
                      M->sf2, M->ri, M->tb, M->taorig, M->tl, M->tr, M->tal};
    for (i = 0; i < (int)(sizeof(turb) / sizeof(turb[0])); i++) free(turb[i]);
    free(M->tindex);
  }
  free(M);
}

#define CP3(dst, src) do { if (dst) memcpy(dst, src, M->n3 * sizeof(double)); } while (0)

int ep_upload(ep_model *M, const epic_fields *f) {
  if (!f || !f->u || !f->v || !f->dudt || !f->dvdt || !f->hdry || !f->theta || !f->p3 || !f->gz_surface || !f->u_spinup)
    return fail(M, "ep_upload: missing field");
  memcpy(M->u, f->u, M->nvp * M->n3 * sizeof(double));
  memcpy(M->v, f->v, M->nvp * M->n3 * sizeof(double));
  memcpy(M->dudt, f->dudt, M->ntp * M->n3 * sizeof(double));
  memcpy(M->dvdt, f->dvdt, M->ntp * M->n3 * sizeof(double));
  memcpy(M->hdry, f->hdry, M->n3 * sizeof(double));
  memcpy(M->theta, f->theta, M->n3 * sizeof(double));
  memcpy(M->p3, f->p3, M->n3 * sizeof(double));
  memcpy(M->u_spinup, f->u_spinup, M->n3 * sizeof(double));
  memcpy(M->gz_surface, f->gz_surface, M->n2 * sizeof(double));
#define UP3(x) do { if (f->x) memcpy(M->x, f->x, M->n3 * sizeof(double)); } while (0)
  UP3(h3); UP3(p2); UP3(theta2); UP3(t2); UP3(t3); UP3(rho2); UP3(rho3); UP3(exner3); UP3(gz3); UP3(mont3); UP3(heat3);
  UP3(pv3); UP3(ri2); UP3(div_uv3); UP3(w3); UP3(dzdt3);
#undef UP3
  if (TURB_ON(M)) {
    if (!f->nu_turb) return fail(M, "ep_upload: the turbulence closure needs nu_turb");
    memcpy(M->nu_turb, f->nu_turb, M->n3 * sizeof(double));
#define UPT(x, y) do { if (f->y) memcpy(M->x, f->y, M->n3 * sizeof(double)); else memset(M->x, 0, M->n3 * sizeof(double)); } while (0)
    UPT(dc_uv, diffusion_coef_uv); UPT(dc_theta, diffusion_coef_theta); UPT(dc_mass, diffusion_coef_mass);
#undef UPT
    M->turb_err[0] = 0;
  }
  M->it_zero = f->it_zero; M->it_minus1 = f->it_minus1; M->it_minus2 = f->it_minus2;
  M->itime = (long)f->itime;
  M->model_time = (long)f->model_time;
  timeplane_bookkeeping(M);
  M->uploaded = 1;
  return 0;
}

int ep_download(ep_model *M, epic_fields *f) {
  if (f->u) memcpy(f->u, M->u, M->nvp * M->n3 * sizeof(double));
  if (f->v) memcpy(f->v, M->v, M->nvp * M->n3 * sizeof(double));
  if (f->dudt) memcpy(f->dudt, M->dudt, M->ntp * M->n3 * sizeof(double));
  if (f->dvdt) memcpy(f->dvdt, M->dvdt, M->ntp * M->n3 * sizeof(double));
  CP3(f->hdry, M->hdry); CP3(f->theta, M->theta); CP3(f->p3, M->p3); CP3(f->h3, M->h3); CP3(f->p2, M->p2);
  CP3(f->theta2, M->theta2); CP3(f->t2, M->t2); CP3(f->t3, M->t3); CP3(f->rho2, M->rho2); CP3(f->rho3, M->rho3);
  CP3(f->exner3, M->exner3); CP3(f->gz3, M->gz3); CP3(f->mont3, M->mont3); CP3(f->heat3, M->heat3); CP3(f->pv3, M->pv3);
  CP3(f->ri2, M->ri2); CP3(f->div_uv3, M->div_uv3); CP3(f->w3, M->w3); CP3(f->dzdt3, M->dzdt3); CP3(f->u_spinup, M->u_spinup);
  if (f->gz_surface) memcpy(f->gz_surface, M->gz_surface, M->n2 * sizeof(double));
  if (TURB_ON(M)) {
    CP3(f->nu_turb, M->nu_turb); CP3(f->diffusion_coef_uv, M->dc_uv); CP3(f->diffusion_coef_theta, M->dc_theta);
    CP3(f->diffusion_coef_mass, M->dc_mass);
  }
  f->it_zero = M->it_zero; f->it_minus1 = M->it_minus1; f->it_minus2 = M->it_minus2;
  f->itime = M->itime;
  f->model_time = M->model_time;
  return 0;
}

/* cfl_dt, epic_funcs_diag.c:4884-5022 (the limits before the truncation into cfl[0..2]: x, y, z) */
int ep_cfl_dt(ep_model *M, double *cfl) {
  const double *U = M->u + (long)M->it_uv * M->n3, *V = M->v + (long)M->it_uv * M->n3;
  double cflx = DBL_MAX, cfly = DBL_MAX, cflz = DBL_MAX, u, v, w, cs, dx, dy, dz, dt;
  int K, J, I;
  for (K = 1; K <= KHI; K++) {
    dz = M->dsgth[2 * K];
    for (J = 0; J <= NJ; J++)
      for (I = 1; I <= NI; I++) {
        w = A3(M->w3, K - 1, J, I);
        if (w > 0.) cflz = dmin(cflz, dz / w);
        w = A3(M->w3, K, J, I);
        if (w < 0.) cflz = dmin(cflz, -dz / w);
      }
  }
  for (J = 1; J <= NJ; J++) {
    dy = 1. / M->n[2 * J + 1];
    for (I = 1; I <= NI; I++)
      for (K = 1; K <= KHI; K++) {
        cs = sqrt(M->g.rgas * .5 * (A3(M->t3, K, J, I) + A3(M->t3, K, J - 1, I)) / (1. - M->g.kappa));
        v = A3(V, K, J + 1, I) + cs;
        if (v > 0.) cfly = dmin(cfly, dy / v);
        v = A3(V, K, J, I) - cs;
        if (v < 0.) cfly = dmin(cfly, -dy / v);
      }
  }
  for (J = 0; J <= NJ; J++) {
    if (fabs(M->lat[2 * J + 1]) <= LAT0) {
      dx = 1. / M->m[2 * J + 1];
      for (I = 1; I <= NI; I++)
        for (K = 1; K <= KHI; K++) {
          cs = sqrt(M->g.rgas * .5 * (A3(M->t3, K, J, I) + A3(M->t3, K, J, I - 1)) / (1. - M->g.kappa));
          u = A3(U, K, J, I + 1) + cs;
          if (u > 0.) cflx = dmin(cflx, dx / u);
          u = A3(U, K, J, I) - cs;
          if (u < 0.) cflx = dmin(cflx, -dx / u);
        }
    }
  }
  if (cfl) { cfl[0] = cflx; cfl[1] = cfly; cfl[2] = cflz; }
  dt = dmin(cflx, cfly);
  dt = dmin(dt, cflz);
  return (int)dt;
}

const char *ep_error(const ep_model *M) { return M->err; }
const char *ep_create_error(void) { return create_err; }
