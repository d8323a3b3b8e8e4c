// Host-side Held-Suarez grid and initial-state construction (no GPU).
//
// Restates, for planet "held_suarez" on the full globe, the grid set-up that the reference's
// `initial` program performs and that `epic` repeats at start-up:
//   geometry        set_lonlat / set_fmn / set_gravity   src/shared/epic_funcs_diag.c:1324-1633
//   dsgth           set_dsgth                            src/shared/epic_funcs_diag.c:1639-1686
//   vertical grid   p_ref, k_sigma, sigmatheta, h_min    src/shared/epic_initial.c:1758-2006
//   viscosity       set_max_nu / init_viscosity          src/shared/epic_subgrid.c:82-199
//   AB3/leapfrog start flags                             src/shared/epic_initial.c:1301-1330
//   HDRY from P3    get_h                                src/shared/epic_main.c:290-297
// The temperature sounding t_vs_p.held_suarez is replaced by the analytic Held-Suarez
// equilibrium profile at 45 degrees (temp_eq, src/shared/epic_sensible_heating.c:394-406), or
// by a constant-N^2 sounding for the zonal-jet state (epic_jet_initial_state).
// Compiled with -ffp-contract=off so the same bits come out on x86-64 and aarch64 hosts.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <string>
#include <vector>
#include "epic_gb300.h"
#include "epic_common.h"

namespace {

constexpr double kDeg = M_PI / 180.0;
constexpr double kHsKappa = 0.2857;
constexpr double kHsRgas = 286.86;
constexpr double kHsCp = 1004.0;
constexpr double kHsRe = 6371.e+3;
constexpr double kHsOmega = 7.2921e-5;
constexpr double kHsGM = 0.39860e+15;
constexpr double kHsJ2 = 1082.636e-6;
constexpr double kHsKinvisc = 14.60e-6;
constexpr double kAlphaBoundary = 0.5;   // ALPHA_BOUNDARY, epic_initial.c:110
constexpr double kPress0 = 1.e+5;        // grid.press0, epic_initial.c:242
constexpr double kSoundingGrav = 9.8;    // gravity of the constant-N^2 sounding's definition

struct Coord {  // the hybrid-coordinate constants get_sigma ... return_sigmatheta read
  double zeta0, zeta1, alpha, sigma_sigma;
};

// get_sigma, epic_funcs_diag.c:1751-1756
inline double get_sigma(double pbot, double p, double ptop) { return log(p / pbot) / log(ptop / pbot); }
// get_p_sigma, epic_funcs_diag.c:1765-1770
inline double get_p_sigma(double pbot, double sigma, double ptop) { return pbot * exp(sigma * log(ptop / pbot)); }
// g_sigma, epic_funcs_diag.c:1300-1314
inline double g_sigma(const Coord &c, double sigma) {
  const double coeff = 1. / (1 - exp(-c.alpha * (1. - c.sigma_sigma)));
  if (sigma <= c.sigma_sigma) return 0.;
  if (sigma >= 1.) return 1.;
  return coeff * (1. - exp(-c.alpha * (sigma - c.sigma_sigma)));
}
// f_sigma, epic_funcs_diag.c:1271-1289
inline double f_sigma(const Coord &c, double sigma) {
  if (sigma < 0.) return c.zeta0;
  if (sigma <= c.sigma_sigma) return c.zeta0 + sigma * (c.zeta1 - c.zeta0);
  if (sigma < 1.) return (1. - g_sigma(c, sigma)) * (c.zeta0 + sigma * (c.zeta1 - c.zeta0));
  return 0.;
}
// return_sigmatheta, epic_funcs_diag.c:1238-1260 (p > pbot is an error there; callers never pass it)
inline double return_sigmatheta(const Coord &c, double theta, double p, double pbot, double ptop) {
  if (p <= ptop) return theta;
  const double sigma = get_sigma(pbot, p, ptop);
  return f_sigma(c, sigma) + g_sigma(c, sigma) * theta;
}
// fcmp, epic_funcs_util.c:4275-4330 (binary64 epsilon)
inline int fcmp(double x1, double x2) {
  int exponent;
  frexp(fabs(x1) > fabs(x2) ? x1 : x2, &exponent);
  const double delta = ldexp(DBL_EPSILON, exponent);
  const double difference = x1 - x2;
  if (difference > delta) return 1;
  if (difference < -delta) return -1;
  return 0;
}
// onto_kk for P2_INDEX at a layer, epic_funcs_diag.c:2601-2618
inline double layer_pressure(double topval, double botval, double kappa) {
  if (fcmp(botval, topval) == 0) return .5 * (botval + topval);
  const double kappap1 = kappa + 1.;
  return pow((pow(botval, kappap1) - pow(topval, kappap1)) / (kappap1 * (botval - topval)), 1. / kappa);
}
// Held-Suarez equilibrium temperature, temp_eq, epic_sensible_heating.c:394-406
inline double hs_temp_eq(double lat_deg, double p, double kappa) {
  double cos2 = cos(lat_deg * kDeg);
  cos2 *= cos2;
  const double sin2 = 1. - cos2;
  const double p_p0 = p / (1000. * 100.);
  double ans = (315. - 60. * sin2 - 10. * log(p_p0) * cos2) * pow(p_p0, kappa);
  return ans > 200. ? ans : 200.;
}
inline double hs_theta_eq(double lat_deg, double p, double kappa) {
  return hs_temp_eq(lat_deg, p, kappa) * pow(kPress0 / p, kappa);
}

// A tabulated sounding, as get_sounding (epic_funcs_diag.c:3160-3290) prepares it from
// t_vs_p.<planet>: levels ordered by x = -ln p ascending (the reference stores them bottom first,
// epic_funcs_io.c:4074-4088), theta = T (p0/p)^kappa at each level (return_theta with x_h2 = 0,
// epic_funcs_diag.c:6408-6430), Fritsch-Carlson monotone slopes with three-point end conditions
// (spline_pchip, epic_funcs_util.c:715-846) taken before theta is ironed from the top down (a
// level warmer than the one above it takes that level's theta, the slopes stay), and the cubic
// Hermite piece of the interval holding x (splint_pchip, :926-946); below the table's lowest level
// its bottom value.
struct TableSounding {
  const double *src_p = nullptr, *src_t = nullptr;
  int n = 0;
  std::vector<double> x, y, z;
};

inline double sign_product(double a, double b) {   // pchst: the sign of a*b, 0 when either is 0
  return (a == 0. || b == 0.) ? 0. : ((a > 0.) == (b > 0.) ? 1. : -1.);
}

void pchip_slopes(const std::vector<double> &x, const std::vector<double> &y, std::vector<double> &z) {
  const int n = (int)x.size();
  z.assign(n, 0.);
  std::vector<double> h(n - 1), d(n - 1);
  for (int q = 0; q + 1 < n; q++) {
    h[q] = x[q + 1] - x[q];
    d[q] = (y[q + 1] - y[q]) / h[q];
  }
  if (n == 2) { z[0] = z[1] = d[0]; return; }
  // end points: three-point slopes, zeroed when against the end interval's slope, limited to three
  // times it when the first two intervals change direction
  {
    const double hs = h[0] + h[1];
    double t = ((h[0] + hs) / hs) * d[0] + (-h[0] / hs) * d[1];
    if (sign_product(t, d[0]) <= 0.) t = 0.;
    else if (sign_product(d[0], d[1]) < 0. && fabs(3. * d[0]) < fabs(t)) t = 3. * d[0];
    z[0] = t;
  }
  {
    const double h1 = h[n - 3], h2 = h[n - 2], d1 = d[n - 3], d2 = d[n - 2], hs = h1 + h2;
    double t = (-h2 / hs) * d1 + ((h2 + hs) / hs) * d2;
    if (sign_product(t, d2) <= 0.) t = 0.;
    else if (sign_product(d1, d2) < 0. && fabs(3. * d2) < fabs(t)) t = 3. * d2;
    z[n - 1] = t;
  }
  // interior: the weighted harmonic mean of the neighbouring slopes where they agree in sign, else 0
  for (int q = 1; q + 1 < n; q++) {
    const double h1 = h[q - 1], h2 = h[q], d1 = d[q - 1], d2 = d[q];
    if (sign_product(d1, d2) > 0.) {
      const double hs = h1 + h2, hs3 = 3. * hs;
      const double w1 = (hs + h1) / hs3, w2 = (hs + h2) / hs3;
      const double dmax = std::max(fabs(d1), fabs(d2)), dmin = std::min(fabs(d1), fabs(d2));
      z[q] = dmin / (w1 * (d1 / dmax) + w2 * (d2 / dmax));
    }
  }
}

const TableSounding &table_sounding(const epic_hs_params *p) {
  thread_local TableSounding s;
  if (s.src_p == p->table_p && s.src_t == p->table_t && s.n == p->table_n && !s.x.empty()) return s;
  const int n = p->table_n;
  std::vector<int> order(n);
  for (int q = 0; q < n; q++) order[q] = q;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return p->table_p[a] > p->table_p[b]; });
  s.x.resize(n);
  s.y.resize(n);
  for (int q = 0; q < n; q++) {
    const double pq = p->table_p[order[q]], tq = p->table_t[order[q]];
    s.x[q] = -log(pq);
    s.y[q] = tq * pow(kPress0 / pq, kHsKappa);
  }
  pchip_slopes(s.x, s.y, s.z);
  for (int q = n - 2; q >= 0; q--)
    if (s.y[q] > s.y[q + 1]) s.y[q] = s.y[q + 1];
  s.src_p = p->table_p;
  s.src_t = p->table_t;
  s.n = n;
  return s;
}

double table_theta(const epic_hs_params *p, double pres) {
  const TableSounding &s = table_sounding(p);
  const double x = -log(pres);
  const int n = (int)s.x.size();
  if (x < s.x[0]) return s.y[0];
  int q = 0;
  if (x >= s.x[n - 1]) q = n - 2;
  else {
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
      const int m = (lo + hi) / 2;
      if (x >= s.x[m]) lo = m; else hi = m;
    }
    q = lo;
  }
  const double h = s.x[q + 1] - s.x[q], delta = (s.y[q + 1] - s.y[q]) / h;
  const double del1 = (s.z[q] - delta) / h, del2 = (s.z[q + 1] - delta) / h;
  const double c3 = (del1 + del2) / h, c2 = -(del1 + del1 + del2), t = x - s.x[q];
  return s.y[q] + t * (s.z[q] + t * (c2 + t * c3));
}

// The sounding (theta at pressure pres) the vertical grid and the initial columns follow.
// EPIC_PROFILE_N2: theta(z) = theta_s exp(N^2 z / g) in hydrostatic balance from pbot up, i.e.
// 1/theta(p) = 1/theta_s + N^2 R / (g^2 kappa) ((p/p0)^kappa - (pbot/p0)^kappa), with the
// temperature held at t_iso above the level where it falls to t_iso.
inline double sounding_theta(const epic_hs_params *p, double pres) {
  if (p->profile == EPIC_PROFILE_TABLE) return table_theta(p, pres);
  if (p->profile != EPIC_PROFILE_N2) return hs_theta_eq(45., pres, kHsKappa);
  const double pbot = p->pbot > 0. ? p->pbot : 1.e+5;
  const double c = p->n2 * kHsRgas / (kSoundingGrav * kSoundingGrav * kHsKappa);
  const double pk = pow(pres / kPress0, kHsKappa);
  const double th = 1. / (1. / p->theta_surface + c * (pk - pow(pbot / kPress0, kHsKappa)));
  const double t = th * pk;
  return t > p->t_iso ? th : p->t_iso / pk;
}

// SplitMix64, one independent stream value per (seed, counter).
inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
inline double unit_open(uint64_t x) {  // (0, 1]
  return ((double)(x >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}
// Standard normal for cell `counter` of stream `seed` (Box-Muller on two SplitMix64 draws).
inline double gauss(uint64_t seed, uint64_t counter) {
  const uint64_t base = splitmix64(seed * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull);
  const double u1 = unit_open(splitmix64(base ^ (2 * counter)));
  const double u2 = unit_open(splitmix64(base ^ (2 * counter + 1)));
  return sqrt(-2. * log(u1)) * cos(2. * M_PI * u2);
}

}  // namespace

extern "C" int epic_hs_grid_build(const epic_hs_params *p, epic_grid *g, double *p_ref, double *theta_ref) {
  using epic::set_error;
  if (!p || !g || !p_ref || !theta_ref) return set_error(EPIC_ERR_ARG, "epic_hs_grid_build: NULL argument");
  const int ni = p->ni, nj = p->nj, nk = p->nk;
  if (ni < 4 || (ni & (ni - 1)) != 0) return set_error(EPIC_ERR_ARG, "ni=%d must be a power of 2 >= 4", ni);
  if (nj < 3 || nk < 3) return set_error(EPIC_ERR_ARG, "nj=%d, nk=%d too small", nj, nk);
  if (p->dt <= 0) return set_error(EPIC_ERR_ARG, "dt=%d", p->dt);
  if (p->uv_scheme != EPIC_UV_AB3 && p->uv_scheme != EPIC_UV_LEAPFROG) return set_error(EPIC_ERR_ARG, "uv_scheme=%d", p->uv_scheme);
  if (p->advection_scheme != EPIC_ADV_HSU && p->advection_scheme != EPIC_ADV_AKIMA)
    return set_error(EPIC_ERR_ARG, "advection_scheme=%d", p->advection_scheme);
  if (p->profile != EPIC_PROFILE_HS_EQ && p->profile != EPIC_PROFILE_N2 && p->profile != EPIC_PROFILE_TABLE)
    return set_error(EPIC_ERR_ARG, "profile=%d", p->profile);
  if (p->profile == EPIC_PROFILE_TABLE) {
    if (!p->table_p || !p->table_t || p->table_n < 3) return set_error(EPIC_ERR_ARG, "sounding table: need 3 or more levels");
    for (int q = 0; q < p->table_n; q++) {
      if (!(p->table_p[q] > 0.) || !(p->table_t[q] > 0.))
        return set_error(EPIC_ERR_ARG, "sounding table level %d: p=%g T=%g", q, p->table_p[q], p->table_t[q]);
      for (int r = 0; r < q; r++)
        if (p->table_p[r] == p->table_p[q]) return set_error(EPIC_ERR_ARG, "sounding table: pressure %g repeats", p->table_p[q]);
    }
  }
  if (p->profile == EPIC_PROFILE_N2) {
    const double pbot_chk = p->pbot > 0. ? p->pbot : 1.e+5;
    const double c = p->n2 * kHsRgas / (kSoundingGrav * kSoundingGrav * kHsKappa);
    if (!(p->n2 > 0.) || !(p->theta_surface > 0.) || !(p->t_iso > 0.) ||
        !(1. / p->theta_surface - c * pow(pbot_chk / kPress0, kHsKappa) > 0.))
      return set_error(EPIC_ERR_ARG, "N^2 sounding: n2=%g theta_surface=%g t_iso=%g", p->n2, p->theta_surface, p->t_iso);
  }
  double *lon = const_cast<double *>(g->lon), *lat = const_cast<double *>(g->lat);
  double *rln = const_cast<double *>(g->rln), *rlt = const_cast<double *>(g->rlt);
  double *fc = const_cast<double *>(g->f), *m = const_cast<double *>(g->m), *n = const_cast<double *>(g->n);
  double *mn = const_cast<double *>(g->mn), *grav = const_cast<double *>(g->g);
  double *sgth = const_cast<double *>(g->sigmatheta), *dsgth = const_cast<double *>(g->dsgth);
  double *dsgth_inv = const_cast<double *>(g->dsgth_inv), *h_min = const_cast<double *>(g->h_min);
  double *t_sponge_inv = const_cast<double *>(g->t_sponge_inv);
  if (!lon || !lat || !rln || !rlt || !fc || !m || !n || !mn || !grav || !sgth || !dsgth || !dsgth_inv || !h_min || !t_sponge_inv)
    return set_error(EPIC_ERR_ARG, "epic_hs_grid_build: grid array pointer is NULL");

  g->ni = ni; g->nj = nj; g->nk = nk; g->dt = p->dt; g->uv_scheme = p->uv_scheme;
  g->advection_scheme = p->advection_scheme;
  g->k_sponge = 0;               // held_suarez forces k_sponge = 0, epic_initial.c:1252-1254
  g->newt_cool_on = 1;           // epic_initial.c:473-475
  g->newt_cool_adjust = 0; g->prandtl = 0.;     // :488-490
  g->tau_drag = 1.e+20; g->drag_v = 0; g->drag_zonal_avg = 0;
  g->topo_scale = 1.;            // :1406-1408
  g->press0 = kPress0;
  g->zeta0 = 260.; g->zeta1 = 700.; g->hybrid_alpha = 50.;   // :1593-1601
  g->globe_latbot = -90.; g->globe_lattop = 90.;
  g->re = kHsRe; g->rp = kHsRe; g->cp = kHsCp; g->rgas = kHsRgas; g->kappa = kHsKappa; g->cpr = 3.5; g->kinvisc = kHsKinvisc;
  g->lat0 = p->lat0 > 0. ? p->lat0 : 45.;
  g->hs_kf = 1. / (24. * 60. * 60.);
  g->nudiv_nondim = p->nudiv_nondim;

  // Longitude/latitude spacing, epic_initial.c:1145-1150, 1198.
  const double lonbot = -180., lontop = 180.;
  g->dln = (lontop - lonbot) / ni;
  g->dlt = 180. / ((nj + 1) + sqrt(.5) + sqrt(.5));

  // set_lonlat, epic_funcs_diag.c:1324-1413 (globe with both poles).
  lon[0] = lonbot - g->dln;
  for (int ii = 1; ii <= 2 * (ni + 1); ii++) lon[ii] = lon[ii - 1] + g->dln * .5;
  lat[0] = -90. + g->dlt * sqrt(.5);
  for (int jj = 1; jj <= 2 * (nj + 1); jj++) lat[jj] = lat[jj - 1] + g->dlt * .5;
  lat[0] = -90.;
  lat[2 * (nj + 1)] = 90.;
  {
    int jjn = 2 * (nj + 1), jjs = 0;
    while (lat[jjs] < 0. && lat[jjn] > 0.) {
      for (; jjs < jjn; jjs++) {
        if (fabs(lat[jjs] + lat[jjn]) < 1.e-3) {
          lat[jjn--] = -lat[jjs++];
          break;
        }
      }
    }
  }

  // set_fmn, epic_funcs_diag.c:1424-1598 (globe).
  {
    const double omega = kHsOmega, re = g->re, rp = g->rp;
    const double dlnr = g->dln * kDeg, dltr = g->dlt * kDeg;
    for (int jj = 1; jj < 2 * (nj + 1); jj++) {
      const double la = kDeg * lat[jj];
      const double r_ln = re / sqrt(1. + pow(rp / re * tan(la), 2.));
      const double r_lt = r_ln / (cos(la) * (pow(sin(la), 2.) + pow(re / rp * cos(la), 2.)));
      rln[jj] = r_ln; rlt[jj] = r_lt;
      fc[jj] = 2. * omega * sin(la);
      m[jj] = 1. / (r_ln * dlnr);
      n[jj] = 1. / (r_lt * dltr);
      mn[jj] = m[jj] * n[jj];
    }
    double la = kDeg * lat[0];
    rln[0] = 0.; rlt[0] = re * re / rp; fc[0] = 2. * omega * sin(la);
    n[1] /= 1. + sqrt(.5);
    mn[1] = n[1] * n[1] / (.5 * dlnr);
    mn[0] = 2. * mn[1];
    const int jn = 2 * (nj + 1);
    la = kDeg * lat[jn];
    rln[jn] = 0.; rlt[jn] = re * re / rp; fc[jn] = 2. * omega * sin(la);
    n[jn - 1] /= 1. + sqrt(.5);
    mn[jn - 1] = n[jn - 1] * n[jn - 1] / (.5 * dlnr);
    mn[jn] = 2. * mn[jn - 1];
    // m[0], n[0], m[jn], n[jn] stay 0 as in the calloc'ed reference arrays.
    m[0] = n[0] = m[jn] = n[jn] = 0.;
    // dy0 at the filter latitude (LAT0 = 45 degrees in the reference).
    const double lat0 = g->lat0 * kDeg;
    const double r_ln = re / sqrt(1. + pow(rp / re * tan(lat0), 2.));
    const double r_lt = r_ln / (cos(lat0) * (pow(sin(lat0), 2.) + pow(re / rp * cos(lat0), 2.)));
    g->dy0 = r_lt * g->dlt * kDeg;
  }

  // set_gravity, epic_funcs_diag.c:1607-1633.
  {
    const double a = g->re, b = g->rp;
    const double spin_factor = (kHsOmega * a) * (kHsOmega * a) * (a / kHsGM);
    const double ge = (1. + 1.5 * kHsJ2 - spin_factor) * kHsGM / (a * a);
    const double gp = (1. - 3. * (a / b) * (a / b) * kHsJ2) * kHsGM / (b * b);
    for (int jj = 0; jj <= 2 * (nj + 1); jj++) {
      double s2 = sin(lat[jj] * kDeg); s2 *= s2;
      double c2 = cos(lat[jj] * kDeg); c2 *= c2;
      grav[jj] = (a * ge * c2 + b * gp * s2) / sqrt(a * a * c2 + b * b * s2);
    }
  }

  // grid.jtp: first h-row within dlt/2 of the equator, epic_initial.c:1434-1440.
  g->jtp = 0;
  for (int J = 0; J <= nj; J++) {
    if (fabs(lat[2 * J + 1] - 0.) <= .5 * g->dlt) { g->jtp = J; break; }
  }

  // Vertical grid, epic_initial.c:1758-2006 (terrestrial, SPACING_LOGP_W_BOUNDARIES).
  const int KHI = nk;
  const double ptop = p->ptop > 0. ? p->ptop : 10.;
  const double pbot = p->pbot > 0. ? p->pbot : 1.e+5;
  const double p_sigma = p->p_sigma > 0. ? p->p_sigma : 900. * 100.;
  for (int kk = 0; kk <= 2 * (nk + 1); kk++) { p_ref[kk] = 0.; theta_ref[kk] = 0.; sgth[kk] = 0.; }
  Coord c{g->zeta0, g->zeta1, g->hybrid_alpha, 0.};
  p_ref[1] = ptop;
  p_ref[2 * KHI + 1] = pbot;
  theta_ref[1] = sounding_theta(p, ptop);
  theta_ref[2 * KHI + 1] = sounding_theta(p, pbot);
  const double sgth_top = theta_ref[1];
  const double sgth_bot = return_sigmatheta(c, theta_ref[2 * KHI + 1], pbot, pbot, ptop);
  sgth[0] = sgth[1] = sgth_top;
  sgth[2 * KHI + 1] = sgth_bot;
  {
    const int nk_sponge = g->k_sponge;
    const int nk_pbl = nk / 5;
    const int nk_reg = nk - nk_pbl - nk_sponge;
    const double dlnp = log(pbot / ptop) /
                        ((1. - pow(1. + kAlphaBoundary, -nk_sponge)) / kAlphaBoundary + (double)nk_reg +
                         (1. - pow(1. + kAlphaBoundary, -nk_pbl)) / kAlphaBoundary);
    p_ref[2 * 1 + 1] = p_ref[1] * exp(dlnp * pow(1. + kAlphaBoundary, -nk_sponge));
    for (int K = 2; K <= g->k_sponge; K++)
      p_ref[2 * K + 1] = p_ref[2 * (K - 1) + 1] * pow(p_ref[2 * (K - 1) + 1] / p_ref[2 * (K - 2) + 1], 1. + kAlphaBoundary);
    for (int K = g->k_sponge + 1; K <= nk - nk_pbl; K++) p_ref[2 * K + 1] = p_ref[2 * (K - 1) + 1] * exp(dlnp);
    for (int K = nk - nk_pbl + 1; K < nk; K++)
      p_ref[2 * K + 1] = p_ref[2 * (K - 1) + 1] * pow(p_ref[2 * (K - 1) + 1] / p_ref[2 * (K - 2) + 1], 1. / (1. + kAlphaBoundary));
    for (int K = 1; K <= KHI; K++) p_ref[2 * K] = layer_pressure(p_ref[2 * K - 1], p_ref[2 * K + 1], kHsKappa);
  }
  // k_sigma: layer whose top is nearest p_sigma, epic_initial.c:1905-1923.
  {
    int k_sigma = -1;
    double best = DBL_MAX;
    for (int K = 1; K <= KHI; K++) {
      const double d = fabs(p_ref[2 * (K - 1) + 1] - p_sigma);
      if (d < best) { k_sigma = K; best = d; }
    }
    if (k_sigma < 2) return set_error(EPIC_ERR_ARG, "k_sigma=%d < 2 (nk too small for p_sigma)", k_sigma);
    g->k_sigma = k_sigma;
  }
  c.sigma_sigma = get_sigma(p_ref[2 * KHI + 1], p_ref[2 * (g->k_sigma - 1) + 1], p_ref[1]);
  for (int kk = 2; kk < 2 * KHI + 1; kk++) theta_ref[kk] = sounding_theta(p, p_ref[kk]);
  for (int kk = 2; kk < 2 * KHI + 1; kk++) sgth[kk] = return_sigmatheta(c, theta_ref[kk], p_ref[kk], pbot, ptop);
  g->sigma_sigma = (sgth[2 * g->k_sigma - 1] - g->zeta0) / (g->zeta1 - g->zeta0);

  // set_dsgth, epic_funcs_diag.c:1639-1686.
  for (int kk = 0; kk <= 2 * (nk + 1); kk++) { dsgth[kk] = 0.; dsgth_inv[kk] = 0.; }
  for (int K = 0; K <= KHI; K++) {
    const int kk = 2 * K;
    if (K == 0) dsgth[kk + 1] = sgth[kk + 1] - sgth[kk + 2];
    else if (K == KHI) dsgth[kk + 1] = sgth[kk] - sgth[kk + 1];
    else dsgth[kk + 1] = sgth[kk] - sgth[kk + 2];
    if (!(dsgth[kk + 1] > 0.)) return set_error(EPIC_ERR_MODEL, "dsgth[%d]=%g <= 0", kk + 1, dsgth[kk + 1]);
    dsgth_inv[kk + 1] = 1. / dsgth[kk + 1];
  }
  for (int K = 1; K <= KHI; K++) {
    const int kk = 2 * K;
    dsgth[kk] = sgth[kk - 1] - sgth[kk + 1];
    if (!(dsgth[kk] > 0.)) return set_error(EPIC_ERR_MODEL, "dsgth[%d]=%g <= 0", kk, dsgth[kk]);
    dsgth_inv[kk] = 1. / dsgth[kk];
  }

  // h_min, epic_initial.c:2001-2006.
  {
    const double tmp = 0.02 / grav[2 * g->jtp + 1];
    for (int K = 1; K <= KHI; K++)
      h_min[K] = tmp * (p_ref[2 * K + 1] - p_ref[2 * (K - 1) + 1]) * dsgth_inv[2 * K];
    h_min[0] = h_min[1];
    h_min[KHI + 1] = 0.;
  }
  t_sponge_inv[0] = 0.;  // k_sponge = 0: set_sponge() leaves the (harness-allocated) entry at 0

  // init_viscosity, epic_subgrid.c:169-199, with set_max_nu, :82-158.
  {
    double max_nu[9];
    epic::set_max_nu(g->dt, g->dy0, g->uv_scheme, max_nu);
    for (int i = 0; i < 9; i++) g->nu[i] = 0.;
    g->nu[2] = g->kinvisc < max_nu[2] ? g->kinvisc : max_nu[2];
    for (int ii = 4; ii <= 8; ii += 2) g->nu[ii] = p->nu_nondim[ii] * max_nu[ii];
  }
  return EPIC_OK;
}

namespace {

// P3 at the interfaces of a column with bottom pressure p_bot that follows the sounding, as
// init_with_u does from a sounding (src/shared/epic_funcs_init.c:1514-1662): get_p_sigma() in the
// pure-sigma region, bisection of return_sigmatheta(theta(p), p) = sigmatheta[2K+1] above it.
void sounding_column(const epic_grid *g, const epic_hs_params *p, double p_top, double p_bot, std::vector<double> &pcol) {
  const int KHI = g->nk, ksig = g->k_sigma;
  const Coord c{g->zeta0, g->zeta1, g->hybrid_alpha, g->sigma_sigma};
  const double *sgth = g->sigmatheta;
  pcol.assign(KHI + 1, 0.);
  pcol[0] = p_top;
  pcol[KHI] = p_bot;
  for (int K = ksig - 1; K < KHI; K++) {
    const double sigma = (sgth[2 * K + 1] - g->zeta0) / (g->zeta1 - g->zeta0);
    pcol[K] = get_p_sigma(p_bot, sigma, p_top);
  }
  for (int K = 1; K < ksig - 1; K++) {
    const double target = sgth[2 * K + 1];
    double lo = log(p_top), hi = log(pcol[ksig - 1]);
    for (int it = 0; it < 200; it++) {
      const double mid = .5 * (lo + hi);
      const double pm = exp(mid);
      const double v = return_sigmatheta(c, sounding_theta(p, pm), pm, p_bot, p_top) - target;
      if (v > 0.) lo = mid; else hi = mid;   // sigmatheta decreases downward
      if (hi - lo < 1.e-15) break;
    }
    pcol[K] = exp(.5 * (lo + hi));
  }
}

// HDRY = get_h(P3) in the layers, epic_main.c:290-297 with get_h, epic_funcs_diag.c:1780-1853.
void hdry_from_p3(const epic_grid *g, const epic::Layout &L, epic_fields *f) {
  for (int K = 1; K <= g->nk; K++)
    for (int J = 0; J <= g->nj; J++)
      for (int I = 1; I <= g->ni; I++)
        f->hdry[L.at(K, J, I)] = (f->p3[L.at(K, J, I)] - f->p3[L.at(K - 1, J, I)]) / (g->g[2 * J + 1] * g->dsgth[2 * K]);
}

// Time-plane indices and the first-step flags of the time scheme (epic_initial.c:1301-1330).
void start_flags(const epic_grid *g, const epic::Layout &L, epic_fields *f) {
  f->it_zero = 0; f->it_minus1 = 1; f->it_minus2 = 2;
  f->itime = 0; f->model_time = 0;
  const int64_t n3 = L.n3;
  if (g->uv_scheme == EPIC_UV_AB3) {
    for (int K = 1; K <= g->nk; K++)
      for (int J = 0; J <= g->nj; J++)
        for (int I = 1; I <= g->ni; I++) {
          f->dudt[2 * n3 + L.at(K, J, I)] = DBL_MAX;   // IT_MINUS2
          f->dudt[1 * n3 + L.at(K, J, I)] = DBL_MAX;   // IT_MINUS1
          f->dvdt[2 * n3 + L.at(K, J, I)] = DBL_MAX;
          f->dvdt[1 * n3 + L.at(K, J, I)] = DBL_MAX;
        }
  } else {
    // Leapfrog: the reference flags the whole IT_MINUS1 plane (epic_initial.c:1316-1325), which
    // leaves DBL_MAX in V's polar row after the first step.  Only the two cells that
    // leapfrog_step and timeplane_bookkeeping test are flagged here
    // (U at (KLO,JLO,ILO), V at (KLO,JFIRST,ILO)); the rest of IT_MINUS1 copies IT_ZERO.
    f->u[n3 + L.at(1, 0, 1)] = DBL_MAX;
    f->v[n3 + L.at(1, 1, 1)] = DBL_MAX;
  }
}

inline double uniform(uint64_t seed, uint64_t counter, double lo, double hi) {
  const uint64_t base = splitmix64(seed * 0x9E6C63D0676A9A99ull + 0x2545F4914F6CDD1Dull);
  return lo + (hi - lo) * (unit_open(splitmix64(base ^ counter)) - 0.5 / 9007199254740992.0);
}

}  // namespace

extern "C" int epic_hs_initial_state(const epic_grid *g, const epic_hs_params *p, uint64_t seed, double noise_k,
                                     epic_fields *f) {
  using epic::set_error;
  if (!g || !p || !f) return set_error(EPIC_ERR_ARG, "epic_hs_initial_state: NULL argument");
  if (!f->u || !f->v || !f->dudt || !f->dvdt || !f->hdry || !f->theta || !f->p3 || !f->gz_surface || !f->u_spinup)
    return set_error(EPIC_ERR_ARG, "epic_hs_initial_state: required field pointer is NULL");
  const epic::Layout L(g->ni, g->nj, g->nk);
  const int ni = g->ni, nj = g->nj, KHI = g->nk;
  const double p_top = p->ptop > 0. ? p->ptop : 10.;
  const double p_bot = p->pbot > 0. ? p->pbot : 1.e+5;
  start_flags(g, L, f);

  // Horizontally uniform column at rest, as the reference's own Held-Suarez runs start from a
  // single sounding (init_with_u with u_scale = 0, src/shared/epic_funcs_init.c:1514-1662):
  // P3 on the sigmatheta interfaces of the sounding, THETA = theta(P3).  Seeded N(0, noise_k^2)
  // noise is then added to THETA where it is prognostic (K >= k_sigma-1).
  const int ksig = g->k_sigma;
  std::vector<double> pcol, thcol(KHI + 1);
  sounding_column(g, p, p_top, p_bot, pcol);
  for (int K = 0; K <= KHI; K++) thcol[K] = sounding_theta(p, pcol[K]);
  for (int J = 0; J <= nj; J++) {
    for (int I = 1; I <= ni; I++) {
      for (int K = 0; K <= KHI; K++) {
        f->p3[L.at(K, J, I)] = pcol[K];
        double th = thcol[K];
        if (K >= ksig - 1 && noise_k > 0.) {
          const uint64_t counter = ((uint64_t)K * (uint64_t)(nj + 1) + (uint64_t)J) * (uint64_t)ni + (uint64_t)(I - 1);
          th += noise_k * gauss(seed, counter);
        }
        f->theta[L.at(K, J, I)] = th;
      }
    }
  }
  hdry_from_p3(g, L, f);
  // Zonal periodicity of everything that was filled (bc_lateral, src/single/s_epic_functions.c:39-87).
  double *fields3[] = {f->p3, f->theta, f->hdry};
  for (double *a : fields3) L.periodic3(a);
  return EPIC_OK;
}

extern "C" int epic_jet_initial_state(const epic_grid *g, const epic_hs_params *p, const epic_jet_params *jet, uint64_t seed,
                                      epic_fields *f) {
  using epic::set_error;
  if (!g || !p || !jet || !f) return set_error(EPIC_ERR_ARG, "epic_jet_initial_state: NULL argument");
  if (!f->u || !f->v || !f->dudt || !f->dvdt || !f->hdry || !f->theta || !f->p3 || !f->gz_surface || !f->u_spinup)
    return set_error(EPIC_ERR_ARG, "epic_jet_initial_state: required field pointer is NULL");
  if (jet->njets < 0 || jet->njets > 64 || !(jet->amp_min <= jet->amp_max) || !(jet->lat_min <= jet->lat_max) ||
      !(jet->width_min > 0.) || !(jet->width_min <= jet->width_max) || !(jet->vort_frac >= 0.))
    return set_error(EPIC_ERR_ARG, "epic_jet_initial_state: bad jet parameters");
  const epic::Layout L(g->ni, g->nj, g->nk);
  const int ni = g->ni, nj = g->nj, KHI = g->nk;
  const double p_top = p->ptop > 0. ? p->ptop : 10.;
  const double p_bot = p->pbot > 0. ? p->pbot : 1.e+5;
  const double a = g->re;
  start_flags(g, L, f);

  // the jets, u at the h rows
  std::vector<double> amp(jet->njets), cen(jet->njets), wid(jet->njets), uh(nj + 1, 0.);
  for (int q = 0; q < jet->njets; q++) {
    amp[q] = uniform(seed, 3 * (uint64_t)q, jet->amp_min, jet->amp_max);
    cen[q] = uniform(seed, 3 * (uint64_t)q + 1, jet->lat_min, jet->lat_max);
    wid[q] = uniform(seed, 3 * (uint64_t)q + 2, jet->width_min, jet->width_max);
  }
  for (int J = 0; J <= nj; J++) {
    const double la = g->lat[2 * J + 1];
    for (int q = 0; q < jet->njets; q++) {
      const double x = (la - cen[q]) / wid[q];
      uh[J] += amp[q] * exp(-x * x);
    }
  }
  // geopotential on pressure surfaces, relative to row 0, from gradient-wind balance at the v rows
  std::vector<double> phi(nj + 1, 0.);
  for (int J = 1; J <= nj; J++) {
    const double uv = .5 * (uh[J - 1] + uh[J]);
    const double dy = (g->lat[2 * J + 1] - g->lat[2 * J - 1]) * kDeg * a;
    phi[J] = phi[J - 1] - dy * (g->f[2 * J] + uv * tan(g->lat[2 * J] * kDeg) / a) * uv;
  }
  // the sounding's geopotential above p_bot, phiref(p) = int_p^p_bot R T dlnp, tabulated in ln p
  const int NT = 4096;
  const double l0 = log(p_top), l1 = log(1.5 * p_bot), dl = (l1 - l0) / (NT - 1);
  std::vector<double> tab(NT);
  auto temp = [&](double lp) { const double pr = exp(lp); return sounding_theta(p, pr) * pow(pr / kPress0, kHsKappa); };
  const int ib = (int)((log(p_bot) - l0) / dl);
  tab[0] = 0.;
  for (int q = 1; q < NT; q++) tab[q] = tab[q - 1] - .5 * kHsRgas * (temp(l0 + (q - 1) * dl) + temp(l0 + q * dl)) * dl;
  const double at_pbot = tab[ib] + (tab[ib + 1] - tab[ib]) * ((log(p_bot) - (l0 + ib * dl)) / dl);
  for (double &v : tab) v -= at_pbot;   // phiref(p_bot) = 0; phiref falls with p
  auto p_of_phi = [&](double target) {   // phiref^-1, linear in ln p between table points
    if (target >= tab[0]) return p_top;
    if (target <= tab[NT - 1]) return exp(l1);
    int lo = 0, hi = NT - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (tab[mid] >= target) lo = mid; else hi = mid;
    }
    return exp(l0 + dl * (lo + (target - tab[lo]) / (tab[hi] - tab[lo])));
  };
  // each row's bottom pressure: the surface (GZ_SURFACE = 0) is where phiref + phi - C = 0, with C
  // fixed by bisection so that the cos(lat)-weighted mean bottom pressure is p_bot
  std::vector<double> pb(nj + 1);
  auto mean_pb = [&](double C) {
    double sw = 0., s = 0.;
    for (int J = 0; J <= nj; J++) {
      pb[J] = p_of_phi(C - phi[J]);
      const double w = cos(g->lat[2 * J + 1] * kDeg);
      sw += w;
      s += w * pb[J];
    }
    return s / sw;
  };
  double clo = -1.e6, chi = 1.e6;   // mean_pb falls as C grows
  for (int it = 0; it < 200; it++) {
    const double mid = .5 * (clo + chi);
    if (mean_pb(mid) > p_bot) clo = mid; else chi = mid;
  }
  mean_pb(.5 * (clo + chi));
  for (int J = 0; J <= nj; J++)
    if (!(pb[J] > 2. * p_top && pb[J] < 1.4 * p_bot))
      return set_error(EPIC_ERR_ARG, "epic_jet_initial_state: row %d bottom pressure %g out of range", J, pb[J]);
  // P3 and THETA of each row's column
  std::vector<double> pcol;
  for (int J = 0; J <= nj; J++) {
    sounding_column(g, p, p_top, pb[J], pcol);
    for (int I = 1; I <= ni; I++)
      for (int K = 0; K <= KHI; K++) {
        f->p3[L.at(K, J, I)] = pcol[K];
        f->theta[L.at(K, J, I)] = sounding_theta(p, pcol[K]);
      }
  }
  hdry_from_p3(g, L, f);
  // the non-divergent perturbation: streamfunction psi at the vorticity points (v rows J,
  // u columns I), zero on the polar rows; u' = -dpsi/dy at the u points, v' = dpsi/dx at the v points
  std::vector<double> psi((size_t)(nj + 2) * (ni + 2), 0.), up((size_t)(nj + 1) * (ni + 2), 0.), vp((size_t)(nj + 2) * (ni + 2), 0.);
  auto PS = [&](int J, int I) -> double & { return psi[(size_t)J * (ni + 2) + I]; };
  for (int J = 1; J <= nj; J++) {
    for (int I = 1; I <= ni; I++) PS(J, I) = gauss(seed ^ 0x5DEECE66Dull, (uint64_t)J * ni + (I - 1));
    PS(J, ni + 1) = PS(J, 1);
    PS(J, 0) = PS(J, ni);
  }
  for (int J = 0; J <= nj; J++)
    for (int I = 1; I <= ni; I++) up[(size_t)J * (ni + 2) + I] = -(PS(J + 1, I) - PS(J, I)) * g->n[2 * J + 1];
  for (int J = 1; J <= nj; J++)
    for (int I = 1; I <= ni; I++) vp[(size_t)J * (ni + 2) + I] = (PS(J, I + 1) - PS(J, I)) * g->m[2 * J];
  // rms relative vorticity at the interior vorticity points, of the jets and of the perturbation
  double zj = 0., zp = 0.;
  for (int J = 1; J <= nj; J++)
    for (int I = 1; I <= ni; I++) {
      const double du = (up[(size_t)J * (ni + 2) + I] - up[(size_t)(J - 1) * (ni + 2) + I]) * g->n[2 * J];
      const int Im = I == 1 ? ni : I - 1;
      const double dv = (vp[(size_t)J * (ni + 2) + I] - vp[(size_t)J * (ni + 2) + Im]) * g->m[2 * J];
      zp += (dv - du) * (dv - du);
      const double zjet = -(uh[J] - uh[J - 1]) * g->n[2 * J];
      zj += zjet * zjet;
    }
  const double scale = zp > 0. ? jet->vort_frac * sqrt(zj / zp) : 0.;
  const int64_t n3 = L.n3;
  const int nplanes = g->uv_scheme == EPIC_UV_AB3 ? 1 : 2;
  for (int t = 0; t < nplanes; t++)
    for (int K = 1; K <= KHI; K++) {
      for (int J = 0; J <= nj; J++)
        for (int I = 1; I <= ni; I++) {
          double &u = f->u[t * n3 + L.at(K, J, I)];
          if (u != DBL_MAX) u = uh[J] + scale * up[(size_t)J * (ni + 2) + I];
        }
      for (int J = 1; J <= nj; J++)
        for (int I = 1; I <= ni; I++) {
          double &v = f->v[t * n3 + L.at(K, J, I)];
          if (v != DBL_MAX) v = scale * vp[(size_t)J * (ni + 2) + I];
        }
    }
  double *fields3[] = {f->p3, f->theta, f->hdry};
  for (double *x : fields3) L.periodic3(x);
  for (int t = 0; t < nplanes; t++) {
    L.periodic3(f->u + t * n3);
    L.periodic3(f->v + t * n3);
  }
  return EPIC_OK;
}
