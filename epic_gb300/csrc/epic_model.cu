// Host side of the GB300 timestep(): device state, the step sequence, CUDA-graph replay and
// the C ABI of include/epic_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include "device_common.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

using epic::Ctl;
using epic::DevModel;
using epic::set_error;

struct epic_model {
  epic_grid g;
  DevModel d;
  int precision;
  int device = -1;                   // the CUDA device that holds the pool and runs the stream
  cudaStream_t stream = nullptr;
  char *pool = nullptr;
  size_t pool_bytes = 0;
  void *fop = nullptr;               // the tensor-core filter's operator tiles, slot table and tensor map
                                     // (shared by the models of one grid on one device)
  uint64_t fop_hash = 0;             // equal for models with the same operator
  bool uploaded = false;
  cudaGraphExec_t run_graph = nullptr;
  bool graph_failed = false;
  int kernels_per_step = -1;
  // asynchronous snapshots (epic_model_snapshot_begin/_wait)
  char *snap = nullptr;              // device copy of the state region, gz_surface and Ctl
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t snap_taken = nullptr, snap_done = nullptr;
  Ctl *snap_ctl = nullptr;           // pinned host copy of the snapshot's Ctl
  epic_fields *snap_dst = nullptr;   // the pending snapshot's destination, or nullptr
};

namespace {

constexpr double kDeg = M_PI / 180.;

// Tables the reference builds in the initialisation blocks of its routines.
struct HostTables {
  std::vector<double> high_lat_h, high_lat_pv, h_coef, v_coef, mn_inv, tw;
  double m0 = 0., coef[9] = {0}, max_nu[9] = {0}, eps13 = 0.;
};

// zonal_filter's HIGH_LAT_H / HIGH_LAT_PV tables, src/shared/epic_adjust.c:132-241.
void filter_tables(const epic_grid &g, const epic::Layout &L, HostTables &T) {
  const double lat0 = g.lat0 * kDeg, re = g.re, rp = g.rp;
  const double rln0 = re / sqrt(1. + pow(rp / re * tan(lat0), 2.));
  const double rlt0 = rln0 / (cos(lat0) * (pow(sin(lat0), 2.) + pow(re / rp * cos(lat0), 2.)));
  const double m0 = 1. / (rln0 * g.dln * kDeg);
  const double n0 = 1. / (rlt0 * g.dlt * kDeg);
  T.m0 = m0;
  T.high_lat_h.assign(L.n2, 0.);
  T.high_lat_pv.assign(L.n2, 0.);
  auto fill = [&](std::vector<double> &hl, int J, int jj) {
    hl[L.at2(J, 1)] = 1.;
    const double r = g.mn[jj] / (g.m[jj] * g.n[jj]);
    double tmp0 = (g.n[jj] / n0) / (g.m[jj] / m0);
    tmp0 = pow(tmp0, 2.);
    for (int I = 2; I <= g.ni / 2 + 1; I++) {
      double tmp1 = sin((I - 1) * (g.dln) * kDeg / 2.);
      tmp1 = pow(tmp1, -2.);
      tmp1 *= r * tmp0;
      tmp1 = (tmp1 < 1.) ? tmp1 : 1.;
      hl[L.at2(J, I)] = tmp1;
    }
  };
  for (int J = 0; J <= g.nj; J++) fill(T.high_lat_h, J, 2 * J + 1);
  for (int J = 1; J <= g.nj; J++) fill(T.high_lat_pv, J, 2 * J);
}

// d2dy2's 3-point coefficients (a Legendre fit; one-sided at the ends), epic_subgrid.c:1049-1141.
void d2dy2_coef(double r2_inv, double l0, double l1, double l2, int where, double *c) {
  const double lat[3] = {l0 * kDeg, l1 * kDeg, l2 * kDeg};
  const double s0 = sin(lat[0]), s1 = sin(lat[1]), s2 = sin(lat[2]);
  if (where == 0) {
    c[0] = r2_inv * (1. + s0 * (-3. * s0 + s1 + s2)) / ((s1 - s0) * .5 * (s2 - s0));
    c[1] = -r2_inv * 2. * (cos(2. * lat[0]) + s0 * s2) / ((s1 - s0) * (s2 - s1));
    c[2] = r2_inv * (cos(2. * lat[0]) + s0 * s1) / (.5 * (s2 - s0) * (s2 - s1));
  } else if (where == 2) {
    c[0] = r2_inv * (cos(2. * lat[2]) + s1 * s2) / ((s1 - s0) * .5 * (s2 - s0));
    c[1] = -r2_inv * 2. * (cos(2. * lat[2]) + s0 * s2) / ((s1 - s0) * (s2 - s1));
    c[2] = r2_inv * (1. + s2 * (s0 + s1 - 3. * s2)) / (.5 * (s2 - s0) * (s2 - s1));
  } else {
    c[0] = r2_inv * (cos(2. * lat[1]) + s1 * s2) / ((s1 - s0) * .5 * (s2 - s0));
    c[1] = -r2_inv * 2. * (1. + s1 * (s0 - 3. * s1 + s2)) / ((s1 - s0) * (s2 - s1));
    c[2] = r2_inv * (cos(2. * lat[1]) + s0 * s1) / (.5 * (s2 - s0) * (s2 - s1));
  }
}

void visc_tables(const epic_grid &g, HostTables &T) {
  epic::set_max_nu(g.dt, g.dy0, g.uv_scheme, T.max_nu);
  double nu[9];
  for (int i = 0; i < 9; i++) nu[i] = g.nu[i];
  nu[2] = 0.;   // the hyperviscosity routines zero grid.nu[2] (epic_subgrid.c:651, :879)
  for (int itmp2 = 2; itmp2 <= 8; itmp2 += 2) {
    T.coef[itmp2] = nu[itmp2] > 0. ? nu[itmp2] : 0.01 * T.max_nu[itmp2];
    for (int itmp = 2; itmp < itmp2; itmp += 2) T.coef[itmp2] /= T.coef[itmp];
  }
  const int nj = g.nj;
  T.h_coef.assign(3 * (nj + 2), 0.);
  T.v_coef.assign(3 * (nj + 2), 0.);
  auto r2 = [&](int jj) { double r = g.rlt[jj]; return 1. / (r * r); };
  d2dy2_coef(r2(1), g.lat[1], g.lat[3], g.lat[5], 0, &T.h_coef[0]);
  for (int J = 1; J < nj; J++) d2dy2_coef(r2(2 * J + 1), g.lat[2 * J - 1], g.lat[2 * J + 1], g.lat[2 * J + 3], 1, &T.h_coef[3 * J]);
  d2dy2_coef(r2(2 * nj + 1), g.lat[2 * nj - 3], g.lat[2 * nj - 1], g.lat[2 * nj + 1], 2, &T.h_coef[3 * nj]);
  d2dy2_coef(r2(0), g.lat[0], g.lat[2], g.lat[4], 0, &T.v_coef[0]);
  for (int J = 1; J <= nj; J++) d2dy2_coef(r2(2 * J), g.lat[2 * J - 2], g.lat[2 * J], g.lat[2 * J + 2], 1, &T.v_coef[3 * J]);
  const int J = nj + 1;
  d2dy2_coef(r2(2 * J), g.lat[2 * J - 4], g.lat[2 * J - 2], g.lat[2 * J], 2, &T.v_coef[3 * J]);
}

double cube_root_machine_eps() {
  // machine_epsilon, epic_funcs_util.c:1247-1265, then pow(eps, 1/3) as calc_w uses it
  volatile double eps = 1.;
  while (1. + eps != 1.) eps *= .5;
  eps *= 2.;
  return pow((double)eps, 1. / 3.);
}

template <typename T>
T *carve(char *&p, size_t count) {
  T *r = reinterpret_cast<T *>(p);
  p += ((count * sizeof(T) + 255) / 256) * 256;
  return r;
}
// the state arrays are packed back to back (no padding), so that a caller whose host arrays are
// laid out the same way moves a whole state with one copy (enqueue_upload / enqueue_download)
template <typename T>
T *carve_packed(char *&p, size_t count) {
  T *r = reinterpret_cast<T *>(p);
  p += count * sizeof(T);
  return r;
}

int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(EPIC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return EPIC_OK;
}

// One reference-function stage of the step, in the reference's call order, for a model or
// (M.batch set) for every member of a batch.
int run_stage_on(const DevModel &M, cudaStream_t s, int stage) {
  using namespace epic;
  switch (stage) {
    case 0: launch_zero_tend(M, s); break;
    case 1: launch_source_sink(M, s); break;
    case 2: launch_calc_w(M, s); break;
    case 3: launch_uv_core(M, s); break;
    case 4: launch_uv_drag(M, s); break;
    case 5:
      launch_meridional_hyperviscosity(M, 2, M.hdry, PL_NONE, s);
      launch_zonal_hyperviscosity(M, 2, M.hdry, PL_NONE, s);   // then restore_mass, in the same kernel
      launch_meridional_hyperviscosity(M, 3, M.theta, PL_NONE, s);
      launch_zonal_hyperviscosity(M, 3, M.theta, PL_NONE, s);
      if (M.turb) {   // NU_TURB (layers 1..nk on the h-grid), then restore_mass(NU_TURB_INDEX)
        launch_meridional_hyperviscosity(M, 4, M.nu_turb, PL_NONE, s);
        launch_zonal_hyperviscosity(M, 4, M.nu_turb, PL_NONE, s);
        launch_restore_nu(M, s);
      }
      break;
    case 6: {
      // advection(), epic_flux.c:346-637: UNITY, THETA and HDRY with the grid's scheme
      auto vertical = M.akima ? launch_akima_vertical : launch_hsu_vertical;
      auto meridional = M.akima ? launch_akima_meridional : launch_hsu_meridional;
      auto zonal = M.akima ? launch_akima_zonal : launch_hsu_zonal;
      launch_advection_prep(M, 0, s);
      vertical(M, M.unity, 0, s);
      meridional(M, M.unity, 0, s);
      zonal(M, M.unity, 0, 1, s);
      launch_advection_prep(M, 1, s);
      vertical(M, M.theta, 1, s);
      meridional(M, M.theta, 1, s);
      zonal(M, M.theta, 0, M.k_sigma - 1, s);
      launch_advection_prep(M, 2, s);
      if (M.turb) {   // NU_TURB with the same scheme (UNITY stands), before HDRY, epic_flux.c:540-600
        launch_advection_prep(M, 3, s);
        vertical(M, M.nu_turb, 3, s);
        meridional(M, M.nu_turb, 3, s);
        zonal(M, M.nu_turb, 2, 1, s);
        launch_advection_prep(M, 4, s);
      }
      vertical(M, M.hdry, 2, s);
      meridional(M, M.hdry, 2, s);
      zonal(M, M.hdry, 1, 1, s);   // then restore_mass, in the same kernel
      // Its P2 is recomputed (stage 11) before the pressure gradient.  EPIC_PREC_MIXED runs the
      // double-float kernel here too: it writes the interfaces' logarithms that stage 7 reads.
      launch_set_p2etc(M, 0, s, true);
      break;
    }
    // GZ3 for the filtered copy (stage 8).  The copy places the 3-D filter's profiles (stages 9
    // and 10), which pass column-to-column rounding noise of GZ3 into the filtered fields, so
    // EPIC_PREC_MIXED computes it in double-float like stage 19 (the FP32 kernel made the wind
    // error after a day ~2x larger); EPIC_PREC_MIXED_FAST keeps the FP32 kernel.
    case 7: launch_store_pgrad_vars(M, s, true); break;
    case 8:
      launch_copy_gz(M, s);
      // The 3-D filter's profiles interpolate in the filtered GZ: filtering GZ itself in FP32
      // makes the mixed form's V error after a day grow from 4e-5 to 7e-5 (leapfrog: 1.7e-4 ->
      // 1.6e-3).  The mixed forms filter it on the tensor cores as GZ - GZ(i=1) per row (FP32
      // rounding of the zonal variations only) where the operator product applies, the FP64 form
      // in binary64.
      if (M.mixed && filter_gemm_usable(M)) launch_filter_planes(M, M.gz, PL_NONE, M.gz, 0, M.nk, 0, s, 1, 1);
      else launch_filter_planes(M, M.gz, PL_NONE, M.gz, 0, M.nk, 0, s);
      launch_gz_monotone(M, s);
      break;
    case 9:
      launch_varz_filter(M, M.dudt, PL_UV_TEND, 0, 1, M.nk, s);
      launch_varz_filter(M, M.dvdt, PL_UV_TEND, 1, 1, M.nk, s);
      break;
    case 10:
      launch_varz_filter(M, M.hdry, PL_NONE, 2, 1, M.nk, s);   // then restore_mass, in the same kernel
      launch_varz_filter(M, M.theta, PL_NONE, 3, M.k_sigma - 1, M.nk, s);
      if (M.turb) {   // NU_TURB (interfaces 0..nk), then restore_mass(NU_TURB_INDEX)
        launch_varz_filter(M, M.nu_turb, PL_NONE, 4, 0, M.nk, s);
        launch_restore_nu(M, s);
      }
      break;
    case 11: launch_set_p2etc(M, 1, s); break;
    case 12: launch_uv_pgrad(M, s); break;
    case 13: launch_divergence_damping(M, s); break;
    case 14: launch_uv_update(M, s); break;
    case 15:
      launch_meridional_hyperviscosity(M, 0, M.u, PL_UV, s);
      launch_meridional_hyperviscosity(M, 1, M.v, PL_UV, s);
      launch_zonal_hyperviscosity(M, 0, M.u, PL_UV, s);
      launch_zonal_hyperviscosity(M, 1, M.v, PL_UV, s);
      break;
    case 16:
      launch_store_diag(M, s);
      if (M.turb) launch_set_diffusion_coef(M, s);
      break;
    case 17: launch_calc_heating(M, s); break;
    case 18: launch_set_p2etc(M, 0, s); break;
    case 20: launch_calc_w(M, s, true); break;   // stages 1 and 2 in one pass over the columns
    case 19: launch_store_pgrad_vars(M, s); break;   // after stage 11: what the pressure gradient reads
    // the turbulence closure (epic_subgrid.c)
    case 21: if (M.turb) launch_source_sink_turb(M, s); break;
    case 22: if (M.turb) launch_scalar_hdiff(M, s); break;
    case 23: if (M.turb) launch_scalar_vdiff(M, s); break;
    case 24: if (M.turb) launch_uv_hdiff(M, s); break;
    case 25: if (M.turb) launch_uv_vdiff(M, s); break;
    default: return set_error(EPIC_ERR_ARG, "unknown stage %d", stage);
  }
  return check_launch("stage launch");
}

int run_stage(epic_model *m, int stage) { return run_stage_on(m->d, m->stream, stage); }

int enqueue_step_on(const DevModel &M, cudaStream_t s) {
  static const int step[] = {0, 20, 3, 4, 5, 6, 7, 8, 9, 10, 11, 19, 12, 13, 14, 15, 16, 17};
  // with the turbulence closure (timestep, epic_timestep.c:130-290): source_sink_turb after
  // calc_w; the scalar subgrid diffusion around the scalars' hyperviscosity; uv_horizontal_subgrid
  // before divergence damping, uv_vertical_subgrid after the time update (grid.diffusion_direction
  // chooses which diffusions run)
  static const int step_turb[] = {0, 20, 21, 3, 4, 22, 5, 23, 6, 7, 8, 9, 10, 11, 19, 12, 24, 13, 14, 25, 15, 16, 17};
  const int *seq = M.turb ? step_turb : step;
  const int n = M.turb ? (int)(sizeof(step_turb) / sizeof(int)) : (int)(sizeof(step) / sizeof(int));
  for (int q = 0; q < n; q++) {
    const int st = seq[q];
    if ((st == 22 || st == 24) && !M.turb_h) continue;
    if ((st == 23 || st == 25) && !M.turb_v) continue;
    int rc = run_stage_on(M, s, st);
    if (rc) return rc;
  }
  return EPIC_OK;
}

int enqueue_sync_on(const DevModel &M, cudaStream_t s) {
  static const int sync[] = {11, 19, 16, 17, 2};
  for (int st : sync) {
    int rc = run_stage_on(M, s, st);
    if (rc) return rc;
  }
  return EPIC_OK;
}

int enqueue_step(epic_model *m) { return enqueue_step_on(m->d, m->stream); }
int enqueue_sync(epic_model *m) { return enqueue_sync_on(m->d, m->stream); }

// Capture one step (and the step counter) on stream s into an executable graph; counts its
// kernel nodes.  Returns nullptr if capture is not possible.
cudaGraphExec_t capture_step(const DevModel &M, cudaStream_t s, int *kernels) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    int rc = enqueue_step_on(M, s);
    if (!rc) rc = epic::launch_itime_advance(M, s);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (rc == EPIC_OK && e == cudaSuccess && graph) {
      size_t nn = 0;
      if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess && nn > 0) {
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(graph, nodes.data(), &nn);
        int nk = 0;
        for (auto nd : nodes) {
          cudaGraphNodeType t;
          if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) nk++;
        }
        *kernels = nk;
      }
      if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
    }
    if (graph) cudaGraphDestroy(graph);
  }
  cudaGetLastError();
  return exec;
}

int read_ctl(epic_model *m, Ctl &c) {
  EPIC_CUDA_CHECK(cudaMemcpyAsync(&c, m->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, m->stream));
  EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  return EPIC_OK;
}

int model_error(const Ctl &c) {
  if (c.err_code == 0) return EPIC_OK;
  static const char *what[] = {"", "store_pgrad_vars: GZ3 not monotonic", "calc_w: p2 >= p4",
                               "zonal_filter: spline_pchip x not increasing", "non-finite value",
                               "tensor-core filter: product completion not signalled in time",
                               "turbulence closure (u_tau = 0, r_sa < 0, dwall <= 0, t_vis < 0 or z not increasing)"};
  return set_error(EPIC_ERR_MODEL, "%s at (k=%d, j=%d, i=%d), value %g", c.err_code < 7 ? what[c.err_code] : "model error",
                   c.err_k, c.err_j, c.err_i, c.err_val);
}

// thermo_setup's hydrogen tables (epic_funcs_diag.c:5864-6105) in DevModel::thermo's layout, with
// the correctly rounded log/exp/pow the FP64 form's kernels use (dd_math.cuh, host-compiled).
// Per temperature T_i = 500 (i+1)/128 K: the rotational partition sums of ortho and para H2
// (Dowling et al. 1998, appendix A), their enthalpies and potential temperatures; per para
// fraction n/15: the temperature on the mean potential temperature grid 20..600 K, inverted by
// linear interpolation (where the reference's search runs off the end of its arrays, the last
// interval extrapolates: mean potential temperatures the runs do not reach).
void thermo_tables(const epic_grid &g, const epic::MathTable &lt, std::vector<double> &out) {
  constexpr int NM = epic::TH_M, NN = epic::TH_N;
  auto xlog = [&](double x) { return epic::cr_log(x, lt); };
  auto xexp = [&](double x) { return epic::cr_exp(x, lt); };
  const double xh2 = g.x_h2, xhe = g.x_he, x3 = g.x_3;
  const double cpr = (2.5 * xh2 + 2.5 * xhe + 3.5 * x3) / (xh2 + xhe + x3);
  const double t0 = 1., p0 = 1.e+5, theta = 87.567, ndeg[2] = {3., 1.}, ln2 = 0.69314718055994530942;
  const double c1 = xlog(1.3806503e-23 * t0 / p0 *
                         epic::cr_pow(2. * M_PI * (1.67262158e-27 / 6.62606876e-34) * (1.3806503e-23 * t0 / 6.62606876e-34), 1.5, lt));
  const double c2 = xlog(9.), p = p0;
  std::vector<double> temp(NM), tho(NM), thp(NM), tvec(NM), thvec(NM), aa(NM);
  out.assign((size_t)NN * NM + 4 * NM + NN, 0.);
  double *T = out.data(), *HO = T + NN * NM, *HP = HO + NM, *TG = HP + NM, *THG = TG + NM, *FP = THG + NM;
  for (int i = 0; i < NM; i++) {
    const double temperature = 500. * (double)(i + 1) / (double)NM;
    double ho, hp, pottempo, pottempp;
    if (temperature < 10.) {   // placeholders of the reference below 10 K
      ho = 2.5 * temperature;
      hp = 2.5 * temperature;
      pottempo = temperature;
      pottempp = temperature;
    } else {
      double y = theta / temperature, z[3][2] = {{0., 0.}, {0., 0.}, {0., 0.}}, term = 0., a[7];
      y = y < 30. ? y : 30.;
      for (int j = 1; j <= 50; j++) {
        const int jn[2] = {2 * j - 1, 2 * j - 2};
        for (int n = 0; n < 2; n++) {
          term = ndeg[n] * (2 * jn[n] + 1) * xexp(-jn[n] * (jn[n] + 1) * y);
          for (int m = 0; m < 3; m++) {
            z[m][n] += term;
            if (m < 2) term *= jn[n] * (jn[n] + 1);
          }
        }
        if (j > 1 && term < 1.e-20) break;
      }
      for (int n = 0; n < 2; n++) {
        a[n + 1] = theta * z[1][n] / z[0][n];
        a[n + 5] = xlog(z[0][n]);
      }
      ho = a[1] + 2.5 * temperature - 2. * theta;
      hp = a[2] + 2.5 * temperature;
      const double so = -xlog(p / p0) + 2.5 * xlog(temperature) + 1.5 * ln2 + c1 + (ho + 2. * theta) / temperature + a[5];
      const double sp = -xlog(p / p0) + 2.5 * xlog(temperature) + 1.5 * ln2 + c1 + hp / temperature + a[6];
      pottempo = xexp(0.4 * (so - c2 - 1.5 * ln2 - c1 - 2.5));
      pottempp = xexp(0.4 * (sp - 1.5 * ln2 - c1 - 2.5));
    }
    temp[i] = temperature;
    tho[i] = pottempo;
    thp[i] = pottempp;
    HO[i] = ho;
    HP[i] = hp;
    TG[i] = temperature;
  }
  for (int m = 0; m < NM; m++) THG[m] = (20. * (double)(NM - (m + 1)) + 600. * (double)(m)) / (double)(NM - 1);
  for (int n = 0; n < NN; n++) {
    FP[n] = ((double)(n)) / (double)(NN - 1);
    for (int i = 0; i < NM; i++) {
      const double thetaln = (xh2 * 2.5 * ((1. - FP[n]) * xlog(tho[i]) + (FP[n]) * xlog(thp[i])) + (xhe * 2.5 + x3 * 3.5) * xlog(temp[i])) / cpr;
      thvec[i] = xexp(thetaln);
      tvec[i] = temp[i];
    }
    for (int j = 0; j < NM; j++) aa[j] = tvec[j];
    tvec[NM - 1] = aa[NM - 1];
    for (int i = 0; i < NM; i++) {
      int j = 1;
      for (; j < NM; j++)
        if (thvec[j] >= THG[i]) break;
      if (j == NM) j = NM - 1;
      tvec[i] = aa[j - 1] + (aa[j] - aa[j - 1]) * (THG[i] - thvec[j - 1]) / (thvec[j] - thvec[j - 1]);
    }
    for (int m = 0; m < NM; m++) T[n * NM + m] = tvec[m];
  }
}

// Device bytes of a model's pool: state, scratch and tables, carved in 256-byte units.
size_t model_pool_bytes(const epic_grid &g) {
  const epic::Layout L(g.ni, g.nj, g.nk);
  const size_t n3 = (size_t)L.n3, n2 = (size_t)L.n2;
  const size_t nvp = g.uv_scheme == EPIC_UV_AB3 ? 1 : 2, ntp = g.uv_scheme == EPIC_UV_AB3 ? 3 : 1;
  const size_t n_state3 = 2 * nvp + 2 * ntp + 20;   // u,v planes + tendencies + 20 single fields
  const size_t n_scratch3 = 8;                      // gz, unity, old, work0..3, lp3 (float2)
  const size_t nj1 = 2 * (g.nj + 1) + 1, ni1 = 2 * (g.ni + 1) + 1, nk1 = 2 * (g.nk + 1) + 1;
  const size_t ntw = epic::twiddle_doubles(g.ni);
  auto rnd = [](size_t b) { return ((b + 255) / 256) * 256; };
  return rnd(sizeof(Ctl)) + (n_state3 + n_scratch3) * rnd(n3 * 8) + 3 * rnd(n2 * 8) + rnd((size_t)(g.nj + 3) * (g.nk + 2) * 3 * 8) +
         rnd(ni1 * 8) + 10 * rnd(nj1 * 8) + 3 * rnd(nk1 * 8) + rnd((g.nk + 2) * 8) + rnd((g.k_sponge + 1) * 8) +
         2 * rnd(3 * (g.nj + 2) * 8) + rnd(ntw * 8) + rnd(ntw * 4) + 2 * rnd((g.nj + 1) * 8) + rnd(sizeof(epic::MathTable)) +
         rnd(32 * sizeof(float2)) + rnd(((size_t)epic::TH_N * epic::TH_M + 4 * epic::TH_M + epic::TH_N) * 8) +
         (g.turbulence ? 4 * rnd(n3 * 8) + rnd(2 * (size_t)(g.nk + 2) * 8) + rnd((size_t)(g.nj + 1) * 8) : 0) + 4096;
}

}  // namespace

extern "C" int64_t epic_model_bytes(const epic_grid *g, int32_t precision) {
  if (!g || g->ni < 4 || g->nj < 3 || g->nk < 3) return -1;
  // both forms store the state in binary64; the mixed ones add the tensor-core filter's operator
  return (int64_t)(model_pool_bytes(*g) + (epic::filter_operator_wanted(*g, precision) ? epic::filter_operator_bytes(*g) : 0));
}

extern "C" const char *epic_last_error(void) { return epic::error_buffer(); }

extern "C" int epic_model_create(const epic_grid *g, int32_t precision, epic_model **out) {
  if (!g || !out) return set_error(EPIC_ERR_ARG, "epic_model_create: NULL argument");
  *out = nullptr;
  if (precision != EPIC_PREC_FP64 && precision != EPIC_PREC_MIXED && precision != EPIC_PREC_MIXED_FAST)
    return set_error(EPIC_ERR_ARG, "precision form %d not available", precision);
  if (g->ni < 4 || (g->ni & (g->ni - 1)) || g->ni > EPIC_MAX_NI) return set_error(EPIC_ERR_ARG, "ni=%d: need a power of 2 in [4,%d]", g->ni, EPIC_MAX_NI);
  if (g->nj < 3 || g->nk < 3 || g->nk > EPIC_MAX_NK) return set_error(EPIC_ERR_ARG, "nj=%d nk=%d out of range", g->nj, g->nk);
  if (g->x_h2 < 0.) return set_error(EPIC_ERR_ARG, "x_h2=%g: negative", g->x_h2);
  if (g->turbulence != EPIC_TURB_OFF) {
    if (g->turbulence != EPIC_TURB_SA_DES) return set_error(EPIC_ERR_ARG, "turbulence=%d", g->turbulence);
    if (precision != EPIC_PREC_FP64) return set_error(EPIC_ERR_ARG, "the turbulence closure is in the FP64 form only");
    if (g->diffusion_direction < EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL || g->diffusion_direction > EPIC_DIFFUSION_JUST_VERTICAL)
      return set_error(EPIC_ERR_ARG, "diffusion_direction=%d", g->diffusion_direction);
    if (g->nk > EPIC_TURB_MAX_NK) return set_error(EPIC_ERR_ARG, "turbulence closure: nk=%d above %d", g->nk, EPIC_TURB_MAX_NK);
    if (!(g->kinvisc > 0.)) return set_error(EPIC_ERR_ARG, "turbulence closure: kinvisc=%g", g->kinvisc);
  }
  if (g->gas_giant && (g->jtp < 0 || g->jtp > g->nj))
    return set_error(EPIC_ERR_ARG, "gas giant: jtp=%d outside the rows 0..%d", g->jtp, g->nj);
  if (3. * (g->ni + 2) * (g->nj + 3) * (g->nk + 2) >= 2147483648.)
    return set_error(EPIC_ERR_ARG, "grid %dx%dx%d too large: a field's offsets must fit in 32 bits", g->ni, g->nj, g->nk);
  if (g->globe_latbot != -90. || g->globe_lattop != 90.) return set_error(EPIC_ERR_ARG, "only the full globe is supported");
  if (g->k_sigma < 2 || g->k_sigma > g->nk) return set_error(EPIC_ERR_ARG, "k_sigma=%d out of range", g->k_sigma);
  if (g->k_sponge != 0 || g->newt_cool_adjust) return set_error(EPIC_ERR_ARG, "k_sponge > 0 and newt_cool_adjust are not supported");
  if ((g->newt_cool_on && g->prandtl > 0.) || (g->tau_drag > 0. && g->tau_drag < 1.e+20))
    return set_error(EPIC_ERR_ARG, "zonal Rayleigh drag (prandtl/tau_drag) is not supported");
  if (g->uv_scheme != EPIC_UV_AB3 && g->uv_scheme != EPIC_UV_LEAPFROG) return set_error(EPIC_ERR_ARG, "uv_scheme=%d", g->uv_scheme);
  if (g->advection_scheme != EPIC_ADV_HSU && g->advection_scheme != EPIC_ADV_AKIMA)
    return set_error(EPIC_ERR_ARG, "advection_scheme=%d", g->advection_scheme);
  const char *ptrs[] = {(const char *)g->lon, (const char *)g->lat, (const char *)g->rln, (const char *)g->rlt, (const char *)g->f,
                        (const char *)g->m, (const char *)g->n, (const char *)g->mn, (const char *)g->g, (const char *)g->sigmatheta,
                        (const char *)g->dsgth, (const char *)g->dsgth_inv, (const char *)g->h_min, (const char *)g->t_sponge_inv};
  for (const char *p : ptrs)
    if (!p) return set_error(EPIC_ERR_ARG, "epic_model_create: grid array pointer is NULL");

  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess) return set_error(EPIC_ERR_CUDA, "epic_model_create: no CUDA device");
  epic_model *m = new epic_model();
  m->g = *g;
  m->precision = precision;
  m->device = device;
  const epic::Layout L(g->ni, g->nj, g->nk);
  DevModel &d = m->d;
  d.ni = g->ni; d.nj = g->nj; d.nk = g->nk;
  d.iadim = L.iadim; d.jadim = L.jadim; d.kadim = L.kadim;
  d.n2 = L.n2; d.n3 = L.n3;
  d.nvp = g->uv_scheme == EPIC_UV_AB3 ? 1 : 2;
  d.ntp = g->uv_scheme == EPIC_UV_AB3 ? 3 : 1;
  d.uv_scheme = g->uv_scheme; d.akima = g->advection_scheme == EPIC_ADV_AKIMA; d.k_sigma = g->k_sigma; d.k_sponge = g->k_sponge; d.newt_cool_on = g->newt_cool_on;
  d.drag_v = g->drag_v; d.drag_zonal_avg = g->drag_zonal_avg; d.rayleigh_on = 0;
  d.dt = (double)g->dt; d.press0 = g->press0; d.topo_scale = g->topo_scale; d.prandtl = g->prandtl; d.tau_drag = g->tau_drag;
  d.zeta0 = g->zeta0; d.zeta1 = g->zeta1; d.alpha = g->hybrid_alpha; d.sigma_sigma = g->sigma_sigma;
  d.g_coeff = 1. / (1 - exp(-g->hybrid_alpha * (1. - g->sigma_sigma)));
  d.kappa = g->kappa; d.cp = g->cp; d.cpr = g->cpr; d.rgas = g->rgas;
  d.mu_dry = 1. / (g->rgas / 8.314472e+3);
  d.hs_kf = g->hs_kf; d.lat0 = g->lat0;
  d.gas_giant = g->gas_giant != 0;
  d.jtp = g->jtp;
  d.turb = g->turbulence == EPIC_TURB_SA_DES;
  d.turb_h = d.turb && (g->diffusion_direction == EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL ||
                        g->diffusion_direction == EPIC_DIFFUSION_JUST_HORIZONTAL);
  d.turb_v = d.turb && (g->diffusion_direction == EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL ||
                        g->diffusion_direction == EPIC_DIFFUSION_JUST_VERTICAL);
  d.stab = g->stability_factor != 0;
  d.kinvisc = g->kinvisc;
  d.dynvisc = g->dynvisc;
  d.mixed = precision != EPIC_PREC_FP64;
  d.col64 = precision == EPIC_PREC_MIXED;
  d.cr = precision == EPIC_PREC_FP64;
  {
    auto split = [](double v) { return make_float2((float)v, (float)(v - (double)(float)v)); };
    d.dfc[epic::DFC_KAPPA] = split(d.kappa);
    d.dfc[epic::DFC_KAPPA_INV] = split(1. / d.kappa);
    d.dfc[epic::DFC_KAPPA1] = split(d.kappa + 1.);
    d.dfc[epic::DFC_SIGMA_SIGMA] = split(d.sigma_sigma);
    d.dfc[epic::DFC_ZETA0] = split(d.zeta0);
    d.dfc[epic::DFC_ZETA1] = split(d.zeta1);
    d.dfc[epic::DFC_G_COEFF] = split(d.g_coeff);
    d.dfc[epic::DFC_ALPHA] = split(d.alpha);
    d.dfc[epic::DFC_LOG_P0] = split(std::log(d.press0));
  }

  HostTables T;
  filter_tables(*g, L, T);
  visc_tables(*g, T);
  d.m0 = T.m0;
  d.eps13 = cube_root_machine_eps();
  for (int i = 0; i < 9; i++) { d.coef[i] = T.coef[i]; d.nu[i] = g->nu[i]; }
  d.nu[2] = 0.;
  d.nudiv = g->nudiv_nondim * T.max_nu[2];
  const int nj1 = 2 * (g->nj + 1) + 1, ni1 = 2 * (g->ni + 1) + 1, nk1 = 2 * (g->nk + 1) + 1;
  T.mn_inv.resize(nj1);
  for (int i = 0; i < nj1; i++) T.mn_inv[i] = 1. / g->mn[i];
  T.tw.assign(epic::twiddle_doubles(g->ni), 0.);
  epic::fill_twiddles(g->ni, T.tw.data());

  // One pool for everything: state, scratch, tables.
  const size_t n3 = (size_t)L.n3, n2 = (size_t)L.n2;
  const size_t bytes = model_pool_bytes(*g);
  cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete m; return set_error(EPIC_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
  e = cudaMalloc(&m->pool, bytes);
  if (e != cudaSuccess) {
    cudaStreamDestroy(m->stream);
    delete m;
    return set_error(EPIC_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  m->pool_bytes = bytes;
  cudaMemsetAsync(m->pool, 0, bytes, m->stream);
  char *p = m->pool;
  d.pool_base = m->pool;
  d.ctl = carve<Ctl>(p, 1);
  d.u = carve_packed<double>(p, d.nvp * n3); d.v = carve_packed<double>(p, d.nvp * n3);
  d.dudt = carve_packed<double>(p, d.ntp * n3); d.dvdt = carve_packed<double>(p, d.ntp * n3);
  double **f3[] = {&d.hdry, &d.theta, &d.p3, &d.h3, &d.p2, &d.theta2, &d.t2, &d.t3, &d.rho2, &d.rho3, &d.exner3, &d.gz3, &d.mont3,
                   &d.heat3, &d.pv3, &d.ri2, &d.div_uv3, &d.w3, &d.dzdt3, &d.u_spinup};
  for (double **q : f3) *q = carve_packed<double>(p, n3);
  p += (256 - ((size_t)(p - m->pool) & 255)) & 255;   // the scratch and tables start 256-aligned
  double **s3[] = {&d.gz, &d.unity, &d.old, &d.work0, &d.work1, &d.work2, &d.work3};
  for (double **q : s3) *q = carve<double>(p, n3);
  d.lp3 = carve<float2>(p, n3);
  d.gz_surface = carve<double>(p, n2);
  double *hlh = carve<double>(p, n2), *hlpv = carve<double>(p, n2);
  d.ptable = carve<double>(p, (size_t)(g->nj + 3) * (g->nk + 2) * 3);
  double *lon = carve<double>(p, ni1);
  double *j1[10];
  for (int i = 0; i < 10; i++) j1[i] = carve<double>(p, nj1);
  double *sg = carve<double>(p, nk1), *ds = carve<double>(p, nk1), *dsi = carve<double>(p, nk1);
  double *hmin = carve<double>(p, g->nk + 2), *tsp = carve<double>(p, g->k_sponge + 1);
  double *hc = carve<double>(p, 3 * (g->nj + 2)), *vc = carve<double>(p, 3 * (g->nj + 2));
  double *tw = carve<double>(p, T.tw.size());
  float *twf = carve<float>(p, T.tw.size());
  double *coslat = carve<double>(p, g->nj + 1);
  double *coslat4 = carve<double>(p, g->nj + 1);
  epic::MathTable *lt = carve<epic::MathTable>(p, 1);
  float2 *exp2tab = carve<float2>(p, 32);
  double *thermo_d = carve<double>(p, (size_t)epic::TH_N * epic::TH_M + 4 * epic::TH_M + epic::TH_N);
  if (d.turb) {   // the turbulence closure: NU_TURB, the three diffusivities (one stride apart, as
                  // relocate_field expects), scratch and a row table
    d.nu_turb = carve<double>(p, n3);
    d.dc_uv = carve<double>(p, n3);
    d.dc_theta = carve<double>(p, n3);
    d.dc_mass = carve<double>(p, n3);
    if ((const char *)d.dc_mass - (const char *)d.nu_turb != 3 * epic::scratch_stride(d.n3)) {
      epic_model_destroy(m);
      return set_error(EPIC_ERR_STATE, "internal pool layout of the turbulence arrays differs from the batch relocation's");
    }
    d.turb_pole = carve<double>(p, 2 * (size_t)(g->nk + 2));
    d.turb_maxnu2 = carve<double>(p, (size_t)g->nj + 1);
  }
  if ((size_t)(p - m->pool) > bytes) {
    epic_model_destroy(m);
    return set_error(EPIC_ERR_NOMEM, "internal pool layout overflow");
  }
  // the layout relocate_field (batches of mixed sizes) relies on: packed state planes, then the
  // seven scratch volumes at one stride
  if ((const char *)d.u_spinup - (const char *)d.u != (long long)(2 * d.nvp + 2 * d.ntp + 19) * d.n3 * 8 ||
      (const char *)d.work3 - (const char *)d.gz != 6 * epic::scratch_stride(d.n3)) {
    epic_model_destroy(m);
    return set_error(EPIC_ERR_STATE, "internal pool layout differs from the batch relocation's");
  }
  auto up = [&](double *dst, const double *src, size_t n) {
    return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, m->stream);
  };
  up(lon, g->lon, ni1);
  const double *src1[10] = {g->lat, g->rln, g->rlt, g->f, g->m, g->n, g->mn, g->g, T.mn_inv.data(), nullptr};
  for (int i = 0; i < 9; i++) up(j1[i], src1[i], nj1);
  up(sg, g->sigmatheta, nk1); up(ds, g->dsgth, nk1); up(dsi, g->dsgth_inv, nk1);
  up(hmin, g->h_min, g->nk + 2); up(tsp, g->t_sponge_inv, g->k_sponge + 1);
  up(hlh, T.high_lat_h.data(), n2); up(hlpv, T.high_lat_pv.data(), n2);
  up(hc, T.h_coef.data(), T.h_coef.size()); up(vc, T.v_coef.data(), T.v_coef.size());
  up(tw, T.tw.data(), T.tw.size());
  std::vector<float> twf_host(T.tw.begin(), T.tw.end());
  cudaMemcpyAsync(twf, twf_host.data(), twf_host.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  // cos of the h-row latitudes with the host libm (t_rad and temp_eq use them)
  std::vector<double> cl(g->nj + 1);
  for (int J = 0; J <= g->nj; J++) cl[J] = cos(g->lat[2 * J + 1] * kDeg);
  up(coslat, cl.data(), cl.size());
  std::vector<epic::MathTable> host_lt(1);   // ~34 KB, built per model in a few ms
  epic::fill_math_table(host_lt[0]);
  // t_rad's pow(cos(lat), 4.) once per row, with the device's correctly rounded pow (host-compiled)
  std::vector<double> cl4(g->nj + 1);
  for (int J = 0; J <= g->nj; J++) cl4[J] = epic::cr_pow(cl[J], 4., host_lt[0]);
  up(coslat4, cl4.data(), cl4.size());
  cudaMemcpyAsync(lt, host_lt.data(), sizeof(epic::MathTable), cudaMemcpyHostToDevice, m->stream);
  std::vector<double> thermo_host;   // hydrogen thermodynamics (x_h2 > 0)
  if (g->x_h2 > 0.) {
    thermo_tables(*g, host_lt[0], thermo_host);
    cudaMemcpyAsync(thermo_d, thermo_host.data(), thermo_host.size() * sizeof(double), cudaMemcpyHostToDevice, m->stream);
  }
  d.thermo = thermo_d;
  d.x_h2 = g->x_h2; d.x_he = g->x_he; d.x_3 = g->x_3;
  std::vector<double> maxnu2;
  if (d.turb) {
    // set_diffusion_coef's taper of max_nu[2] per row, MIN(1, pow(dy0 m, -2)) with the device's
    // correctly rounded pow (host-compiled)
    maxnu2.resize(g->nj + 1);
    for (int J = 0; J <= g->nj; J++) {
      const double p2 = epic::cr_pow(g->dy0 * g->m[2 * J + 1], -2., host_lt[0]);
      maxnu2[J] = T.max_nu[2] * (1. < p2 ? 1. : p2);
    }
    cudaMemcpyAsync((void *)d.turb_maxnu2, maxnu2.data(), maxnu2.size() * sizeof(double), cudaMemcpyHostToDevice, m->stream);
    d.max_nu2 = T.max_nu[2];
  }
  // 2^(j/32) as double-floats for the double-float exponential of the mixed form
  std::vector<float2> e2(32);
  for (int q = 0; q < 32; q++) {
    const double v = std::exp2(q / 32.);
    e2[q].x = (float)v;
    e2[q].y = (float)(v - (double)e2[q].x);
  }
  cudaMemcpyAsync(exp2tab, e2.data(), e2.size() * sizeof(float2), cudaMemcpyHostToDevice, m->stream);
  d.coslat = coslat;
  d.coslat4 = coslat4;
  d.lt = lt;
  d.exp2tab = exp2tab;
  d.lon = lon; d.lat = j1[0]; d.rln = j1[1]; d.rlt = j1[2]; d.f = j1[3]; d.m = j1[4]; d.n = j1[5]; d.mn = j1[6]; d.grav = j1[7];
  d.mn_inv = j1[8];
  d.sgth = sg; d.dsgth = ds; d.dsgth_inv = dsi; d.h_min = hmin; d.t_sponge_inv = tsp;
  d.high_lat_h = hlh; d.high_lat_pv = hlpv; d.h_coef = hc; d.v_coef = vc; d.tw = tw; d.twf = twf;
  d.fop_map = nullptr;
  d.fop_slot = nullptr;
  if (epic::filter_operator_wanted(*g, precision)) {   // the tensor-core filter's operator tiles
    const char *why = nullptr;
    if (epic::filter_operator_create(*g, T.high_lat_h.data(), T.high_lat_pv.data(), L.iadim, m->stream, d, &m->fop, &m->fop_hash, &why)) {
      epic_model_destroy(m);
      return set_error(EPIC_ERR_NOMEM, "epic_model_create: %s", why);
    }
  }
  epic::filter_kernels_init(g->ni);
  epic::column_kernels_init(g->nk);
  epic::column_acc_kernels_init();
  epic::filter_gemm_init(g->ni);
  e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) {
    epic_model_destroy(m);
    return set_error(EPIC_ERR_CUDA, "epic_model_create: %s", cudaGetErrorString(e));
  }
  *out = m;
  return EPIC_OK;
}

extern "C" void epic_model_destroy(epic_model *m) {
  if (!m) return;
  if (m->run_graph) cudaGraphExecDestroy(m->run_graph);
  if (m->copy_stream) {
    cudaStreamSynchronize(m->copy_stream);
    cudaStreamDestroy(m->copy_stream);
  }
  if (m->snap_taken) cudaEventDestroy(m->snap_taken);
  if (m->snap_done) cudaEventDestroy(m->snap_done);
  if (m->snap) cudaFree(m->snap);
  if (m->snap_ctl) cudaFreeHost(m->snap_ctl);
  if (m->stream) cudaStreamSynchronize(m->stream);
  if (m->pool) cudaFree(m->pool);
  if (m->fop) epic::filter_operator_release(m->fop);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

namespace {

// The copies of epic_model_upload, enqueued on stream s; *c receives the control block and must
// stay valid until s has run them.
// Whether the host's state arrays sit back to back in the device's order (u, v, dudt, dvdt, then
// the 20 single fields), as the device's do: then a state moves with one copy.
bool host_state_packed(const DevModel &d, const double *const *fld) {
  const size_t n3 = (size_t)d.n3;
  const double *base = fld[0];
  size_t off = 0;
  for (int i = 0; i < 24; i++) {
    if (fld[i] != base + off) return false;
    off += (i < 2 ? d.nvp : (i < 4 ? d.ntp : 1)) * n3;
  }
  return true;
}

// Planes of the state region that a copy moves: all of it, or (state_only) the prognostic
// prefix u, v, dudt, dvdt, hdry, theta -- the arrays a step advances and reads from the step
// before; the other 18 fields are diagnostics the step recomputes before it reads them (P3's top
// row and GZ_SURFACE are constants of the run).
int state_arrays(bool state_only) { return state_only ? 6 : 24; }
size_t state_planes(const DevModel &d, bool state_only) { return (size_t)(2 * d.nvp + 2 * d.ntp + (state_only ? 2 : 20)); }

int enqueue_upload(epic_model *m, const epic_fields *f, cudaStream_t s, Ctl *c, bool with_ctl = true, bool state_only = false) {
  if (!f->u || !f->v || !f->dudt || !f->dvdt || !f->hdry || !f->theta || !f->p3 || !f->gz_surface || !f->u_spinup)
    return set_error(EPIC_ERR_ARG, "epic_model_upload: a required field pointer is NULL");
  DevModel &d = m->d;
  const size_t b3 = (size_t)d.n3 * sizeof(double);
  const double *src[] = {f->u, f->v, f->dudt, f->dvdt, f->hdry, f->theta, f->p3, f->h3, f->p2, f->theta2, f->t2, f->t3, f->rho2,
                         f->rho3, f->exner3, f->gz3, f->mont3, f->heat3, f->pv3, f->ri2, f->div_uv3, f->w3, f->dzdt3, f->u_spinup};
  double *dst[] = {d.u, d.v, d.dudt, d.dvdt, d.hdry, d.theta, d.p3, d.h3, d.p2, d.theta2, d.t2, d.t3, d.rho2,
                   d.rho3, d.exner3, d.gz3, d.mont3, d.heat3, d.pv3, d.ri2, d.div_uv3, d.w3, d.dzdt3, d.u_spinup};
  if (host_state_packed(d, src)) {
    EPIC_CUDA_CHECK(cudaMemcpyAsync(d.u, f->u, state_planes(d, state_only) * b3, cudaMemcpyHostToDevice, s));
  } else {
    for (int i = 0; i < state_arrays(state_only); i++)
      if (src[i]) EPIC_CUDA_CHECK(cudaMemcpyAsync(dst[i], src[i], (i < 2 ? d.nvp : (i < 4 ? d.ntp : 1)) * b3, cudaMemcpyHostToDevice, s));
  }
  if (!state_only)
    EPIC_CUDA_CHECK(cudaMemcpyAsync(d.gz_surface, f->gz_surface, (size_t)d.n2 * sizeof(double), cudaMemcpyHostToDevice, s));
  if (d.turb) {   // NU_TURB is prognostic; the diffusivities are the previous step's store_diag's
    if (!f->nu_turb) return set_error(EPIC_ERR_ARG, "epic_model_upload: the turbulence closure needs nu_turb");
    EPIC_CUDA_CHECK(cudaMemcpyAsync(d.nu_turb, f->nu_turb, b3, cudaMemcpyHostToDevice, s));
    if (!state_only) {
      const double *tsrc[] = {f->diffusion_coef_uv, f->diffusion_coef_theta, f->diffusion_coef_mass};
      double *tdst[] = {d.dc_uv, d.dc_theta, d.dc_mass};
      for (int q = 0; q < 3; q++) {
        if (tsrc[q]) EPIC_CUDA_CHECK(cudaMemcpyAsync(tdst[q], tsrc[q], b3, cudaMemcpyHostToDevice, s));
        else EPIC_CUDA_CHECK(cudaMemsetAsync(tdst[q], 0, b3, s));
      }
    }
  }
  if (!with_ctl) return EPIC_OK;
  memset(c, 0, sizeof(*c));
  c->it_zero = f->it_zero; c->it_minus1 = f->it_minus1; c->it_minus2 = f->it_minus2;
  c->itime = f->itime; c->model_time = f->model_time;
  // timeplane_bookkeeping, epic_funcs_diag.c:7086-7124
  if (d.uv_scheme == EPIC_UV_AB3) {
    c->it_uv = 0; c->it_uv_dis = 0; c->it_uv_tend = c->it_zero;
  } else {
    c->it_uv = c->it_zero;
    const double flag = f->u[(size_t)c->it_minus1 * d.n3 + d.at(1, 0, 1)];
    c->it_uv_dis = flag == DBL_MAX ? c->it_zero : c->it_minus1;
    c->it_uv_tend = 0;
  }
  EPIC_CUDA_CHECK(cudaMemcpyAsync(d.ctl, c, sizeof(Ctl), cudaMemcpyHostToDevice, s));
  return EPIC_OK;
}

// The copies of epic_model_download, enqueued on stream s; *c receives the control block.
int enqueue_download(epic_model *m, epic_fields *f, cudaStream_t s, Ctl *c, bool state_only = false) {
  DevModel &d = m->d;
  const size_t b3 = (size_t)d.n3 * sizeof(double);
  double *dst[] = {f->u, f->v, f->dudt, f->dvdt, f->hdry, f->theta, f->p3, f->h3, f->p2, f->theta2, f->t2, f->t3, f->rho2,
                   f->rho3, f->exner3, f->gz3, f->mont3, f->heat3, f->pv3, f->ri2, f->div_uv3, f->w3, f->dzdt3, f->u_spinup};
  const double *src[] = {d.u, d.v, d.dudt, d.dvdt, d.hdry, d.theta, d.p3, d.h3, d.p2, d.theta2, d.t2, d.t3, d.rho2,
                         d.rho3, d.exner3, d.gz3, d.mont3, d.heat3, d.pv3, d.ri2, d.div_uv3, d.w3, d.dzdt3, d.u_spinup};
  if (host_state_packed(d, dst)) {
    EPIC_CUDA_CHECK(cudaMemcpyAsync(f->u, d.u, state_planes(d, state_only) * b3, cudaMemcpyDeviceToHost, s));
  } else {
    for (int i = 0; i < state_arrays(state_only); i++)
      if (dst[i]) EPIC_CUDA_CHECK(cudaMemcpyAsync(dst[i], src[i], (i < 2 ? d.nvp : (i < 4 ? d.ntp : 1)) * b3, cudaMemcpyDeviceToHost, s));
  }
  if (f->gz_surface && !state_only) EPIC_CUDA_CHECK(cudaMemcpyAsync(f->gz_surface, d.gz_surface, (size_t)d.n2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (d.turb) {
    if (f->nu_turb) EPIC_CUDA_CHECK(cudaMemcpyAsync(f->nu_turb, d.nu_turb, b3, cudaMemcpyDeviceToHost, s));
    if (!state_only) {
      double *tdst[] = {f->diffusion_coef_uv, f->diffusion_coef_theta, f->diffusion_coef_mass};
      const double *tsrc[] = {d.dc_uv, d.dc_theta, d.dc_mass};
      for (int q = 0; q < 3; q++)
        if (tdst[q]) EPIC_CUDA_CHECK(cudaMemcpyAsync(tdst[q], tsrc[q], b3, cudaMemcpyDeviceToHost, s));
    }
  }
  EPIC_CUDA_CHECK(cudaMemcpyAsync(c, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
  return EPIC_OK;
}

void fields_from_ctl(epic_fields *f, const Ctl &c) {
  f->it_zero = c.it_zero; f->it_minus1 = c.it_minus1; f->it_minus2 = c.it_minus2;
  f->itime = c.itime; f->model_time = c.model_time;
}

}  // namespace

extern "C" int epic_model_upload(epic_model *m, const epic_fields *f) {
  if (!m || !f) return set_error(EPIC_ERR_ARG, "epic_model_upload: NULL argument");
  Ctl c;
  int rc = enqueue_upload(m, f, m->stream, &c);
  EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  if (rc) return rc;
  m->uploaded = true;
  return EPIC_OK;
}

extern "C" int epic_model_timestep(epic_model *m, int32_t action) {
  if (!m) return set_error(EPIC_ERR_ARG, "epic_model_timestep: NULL model");
  if (!m->uploaded) return set_error(EPIC_ERR_STATE, "timestep before upload");
  if (action == EPIC_STEP_PROGS_AND_SYNC_DIAGS) return enqueue_step(m);
  if (action == EPIC_SYNC_DIAGS_ONLY) return enqueue_sync(m);
  return set_error(EPIC_ERR_ARG, "unrecognized action=%d", action);
}

extern "C" int epic_model_set_itime(epic_model *m, int64_t itime) {
  if (!m) return set_error(EPIC_ERR_ARG, "epic_model_set_itime: NULL model");
  if (!m->uploaded) return set_error(EPIC_ERR_STATE, "set_itime before upload");
  epic::launch_set_itime(m->d, (long long)itime, m->stream);
  return check_launch("epic_model_set_itime");
}

extern "C" int epic_model_run_stage(epic_model *m, int32_t stage) {
  if (!m) return set_error(EPIC_ERR_ARG, "epic_model_run_stage: NULL model");
  if (!m->uploaded) return set_error(EPIC_ERR_STATE, "stage before upload");
  return run_stage(m, stage);
}

extern "C" int epic_model_run(epic_model *m, int32_t nsteps) {
  if (!m) return set_error(EPIC_ERR_ARG, "epic_model_run: NULL model");
  if (!m->uploaded) return set_error(EPIC_ERR_STATE, "run before upload");
  if (nsteps <= 0) return EPIC_OK;
  if (!m->run_graph && !m->graph_failed) {
    m->run_graph = capture_step(m->d, m->stream, &m->kernels_per_step);
    if (!m->run_graph) m->graph_failed = true;
  }
  for (int s = 0; s < nsteps; s++) {
    if (m->run_graph) {
      EPIC_CUDA_CHECK(cudaGraphLaunch(m->run_graph, m->stream));
    } else {
      int rc = enqueue_step(m);
      if (rc) return rc;
      epic::launch_itime_advance(m->d, m->stream);
    }
  }
  return check_launch("epic_model_run");
}

extern "C" int epic_model_cfl_dt(epic_model *m, int32_t *dt_out, double *cfl) {
  if (!m || !dt_out) return set_error(EPIC_ERR_ARG, "epic_model_cfl_dt: NULL argument");
  if (!m->uploaded) return set_error(EPIC_ERR_STATE, "cfl_dt before upload");
  unsigned long long *lim = nullptr, host[3];
  EPIC_CUDA_CHECK(cudaMallocAsync((void **)&lim, 3 * sizeof(unsigned long long), m->stream));
  double big[3] = {DBL_MAX, DBL_MAX, DBL_MAX};
  EPIC_CUDA_CHECK(cudaMemcpyAsync(lim, big, sizeof(big), cudaMemcpyHostToDevice, m->stream));
  epic::launch_cfl_dt(m->d, lim, m->stream);
  int rc = check_launch("cfl_dt");
  EPIC_CUDA_CHECK(cudaMemcpyAsync(host, lim, sizeof(host), cudaMemcpyDeviceToHost, m->stream));
  EPIC_CUDA_CHECK(cudaFreeAsync(lim, m->stream));
  EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  if (rc) return rc;
  double c[3];
  memcpy(c, host, sizeof(c));
  double dt = c[0] < c[1] ? c[0] : c[1];   // MIN(cflx, cfly), then MIN(., cflz)
  dt = dt < c[2] ? dt : c[2];
  *dt_out = (int32_t)dt;
  if (cfl) memcpy(cfl, c, sizeof(c));
  return EPIC_OK;
}

extern "C" int epic_model_sync(epic_model *m) {
  if (!m) return set_error(EPIC_ERR_ARG, "epic_model_sync: NULL model");
  EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  Ctl c;
  int rc = read_ctl(m, c);
  if (rc) return rc;
  return model_error(c);
}

extern "C" int epic_model_download(epic_model *m, epic_fields *f) {
  if (!m || !f) return set_error(EPIC_ERR_ARG, "epic_model_download: NULL argument");
  Ctl c;
  int rc = enqueue_download(m, f, m->stream, &c);
  EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  if (rc) return rc;
  fields_from_ctl(f, c);
  return model_error(c);
}

extern "C" int epic_model_step_host(epic_model *m, epic_fields *f, int32_t prime, int32_t nsteps) {
  int rc = epic_model_upload(m, f);
  if (rc) return rc;
  if (prime) {
    rc = epic_model_timestep(m, EPIC_SYNC_DIAGS_ONLY);
    if (rc) return rc;
  }
  rc = epic_model_run(m, nsteps);
  if (rc) return rc;
  return epic_model_download(m, f);
}

extern "C" void *epic_model_stream(epic_model *m) { return m ? (void *)m->stream : nullptr; }

extern "C" int32_t epic_model_kernels_per_step(const epic_model *m) { return m ? m->kernels_per_step : -1; }

extern "C" int64_t epic_model_device_bytes(const epic_model *m) { return m ? (int64_t)m->pool_bytes : 0; }

extern "C" int32_t epic_model_device(const epic_model *m) { return m ? m->device : -1; }

// ---- the 3-D mass filter with a fixed scratch table (epic_model_filter_mass_noalloc) ----
//
// Some callers cannot allocate device memory at the point where they want the filter: a
// serving loop that has already handed every byte of its HBM budget to admitted runs, or code
// running beside other streams' work, where a cudaMalloc/cudaFree could stall on that work.
// For them the PCHIP profile tables, (nj+3)*(nk+2) entries of (x, y, slope), live in one array
// compiled into the library, sized for grids up to EPIC_NOALLOC_TABLE_ENTRIES entries
// (384 KiB).  Everything else the filter reads is the model's own, allocated once in
// epic_model_create.

static __device__ __align__(256) double g_noalloc_ptable[3 * EPIC_NOALLOC_TABLE_ENTRIES];

namespace {

// Address of g_noalloc_ptable in the current context, looked up on every call (no allocation):
// a context torn down and made again (cudaDeviceReset) reloads the module, possibly elsewhere.
int noalloc_table(int dev, double **out) {
  (void)dev;
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_ptable);
  if (e != cudaSuccess || !p) return set_error(EPIC_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  *out = static_cast<double *>(p);
  return EPIC_OK;
}

}  // namespace

extern "C" int epic_model_filter_mass_noalloc(epic_model *m) {
  if (!m) return set_error(EPIC_ERR_ARG, "epic_model_filter_mass_noalloc: NULL model");
  const long long entries = (long long)(m->d.nj + 3) * (m->d.nk + 2);
  if (entries > EPIC_NOALLOC_TABLE_ENTRIES)
    return set_error(EPIC_ERR_ARG, "epic_model_filter_mass_noalloc: (nj+3)*(nk+2) = %lld exceeds %d", entries,
                     EPIC_NOALLOC_TABLE_ENTRIES);
  if (!m->uploaded) return set_error(EPIC_ERR_STATE, "filter before upload");
  int dev = -1, cur = -1;
  EPIC_CUDA_CHECK(cudaStreamGetDevice(m->stream, &dev));
  EPIC_CUDA_CHECK(cudaGetDevice(&cur));
  if (dev != cur) EPIC_CUDA_CHECK(cudaSetDevice(dev));
  double *table = nullptr;
  int rc = noalloc_table(dev, &table);
  if (rc == EPIC_OK) {
    DevModel M = m->d;   // the model's description with only the table pointer replaced
    M.ptable = table;
    cudaStream_t s = m->stream;
    epic::launch_varz_filter(M, M.hdry, epic::PL_NONE, 2, 1, M.nk, s);   // with restore_mass
    epic::launch_varz_filter(M, M.theta, epic::PL_NONE, 3, M.k_sigma - 1, M.nk, s);
    rc = check_launch("epic_model_filter_mass_noalloc");
  }
  if (dev != cur) cudaSetDevice(cur);
  return rc;
}

// ---- batches: one launch per kernel for every member ----
//
// A batch is a view over models created by epic_model_create that share what shapes the step's
// sequence of launches: the layers (nk, k_sigma), the schemes, the precision form, which
// viscosity orders and whether divergence damping act, the filter latitude, and (in the mixed
// forms) whether the zonal filter runs on the tensor cores (ni a multiple of 128).  Members may
// differ in ni, nj, dt, their state and the Held-Suarez drag rate k_f.  The members' descriptions
// live in one device array; each kernel of the step is launched once with gridDim.z = members
// and a grid sized for the largest member, and takes member blockIdx.z's description on entry
// (epic_member): its own sizes bound its threads, its own coefficients and arrays are used.  So
// a 64-member ensemble, or runs of several grid sizes, cost the launches of one model.  Member
// state stays in each member's own device memory: upload and download go through the member
// models, after epic_batch_sync.

struct epic_batch {
  std::vector<epic_model *> members;
  DevModel d;                       // launch description: member 0's arrays, the largest sizes
  DevModel *dev_members = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t run_graph = nullptr;
  bool graph_failed = false;
  int kernels_per_step = -1;
  std::vector<epic_batch *> groups;  // sub-batches of epic_batch_step_host's pipeline
  Ctl *host_ctl = nullptr;           // pinned control blocks for the pipeline's copies
  size_t host_ctl_count = 0;
};

namespace {

bool tensor_filter(const DevModel &a) { return a.mixed && a.ni % 128 == 0 && a.ni <= 1024; }

// Whether two models can share every launch of a step (see above); *why names the difference.
bool batch_compatible(const DevModel &a, const DevModel &b, const char **why) {
  *why = nullptr;
  if (a.nk != b.nk || a.k_sigma != b.k_sigma) *why = "layers (nk, k_sigma)";
  else if (a.uv_scheme != b.uv_scheme || a.akima != b.akima) *why = "time or advection scheme";
  else if (a.mixed != b.mixed || a.col64 != b.col64) *why = "precision form";
  else if (a.k_sponge != b.k_sponge || a.newt_cool_on != b.newt_cool_on || a.drag_v != b.drag_v ||
           a.drag_zonal_avg != b.drag_zonal_avg || a.lat0 != b.lat0)
    *why = "physics options";
  else if ((a.nudiv == 0.) != (b.nudiv == 0.)) *why = "divergence damping on/off";
  else if (a.gas_giant != b.gas_giant) *why = "lower boundary (gas giant or terrain)";
  else if ((a.x_h2 > 0.) != (b.x_h2 > 0.)) *why = "thermodynamics (hydrogen tables or ideal cp)";
  else if (a.turb != b.turb || a.turb_h != b.turb_h || a.turb_v != b.turb_v)
    *why = "turbulence closure (on/off, diffusion directions)";
  else if (tensor_filter(a) != tensor_filter(b)) *why = "zonal filter path (ni a multiple of 128 or not)";
  else
    for (int i = 0; i < 9; i++)
      if ((a.nu[i] > 0.) != (b.nu[i] > 0.)) *why = "hyperviscosity orders";
  return *why == nullptr;
}

}  // namespace

extern "C" int epic_batch_create(epic_model *const *members, int32_t n, epic_batch **out) {
  if (!members || !out || n < 1) return set_error(EPIC_ERR_ARG, "epic_batch_create: bad arguments");
  *out = nullptr;
  for (int i = 0; i < n; i++) {
    if (!members[i]) return set_error(EPIC_ERR_ARG, "epic_batch_create: member %d is NULL", i);
    const char *why = nullptr;
    if (!batch_compatible(members[0]->d, members[i]->d, &why))
      return set_error(EPIC_ERR_ARG, "epic_batch_create: member %d differs from member 0 in %s", i, why);
    for (int q = 0; q < i; q++)
      if (members[q] == members[i]) return set_error(EPIC_ERR_ARG, "epic_batch_create: member %d repeats member %d", i, q);
    // every kernel of the batch reads and writes each member's pool: all on one device
    if (members[i]->device != members[0]->device)
      return set_error(EPIC_ERR_ARG, "epic_batch_create: member %d lives on device %d, member 0 on device %d", i,
                       members[i]->device, members[0]->device);
  }
  int cur = -1;
  EPIC_CUDA_CHECK(cudaGetDevice(&cur));
  if (cur != members[0]->device) EPIC_CUDA_CHECK(cudaSetDevice(members[0]->device));
  epic_batch *b = new epic_batch();
  b->members.assign(members, members + n);
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->dev_members, sizeof(DevModel) * (size_t)n);
  if (e != cudaSuccess) {
    epic_batch_destroy(b);
    if (cur != members[0]->device) cudaSetDevice(cur);
    return set_error(EPIC_ERR_NOMEM, "epic_batch_create: %s", cudaGetErrorString(e));
  }
  std::vector<DevModel> host(n);
  for (int i = 0; i < n; i++) host[i] = members[i]->d;
  e = cudaMemcpy(b->dev_members, host.data(), sizeof(DevModel) * (size_t)n, cudaMemcpyHostToDevice);
  if (cur != members[0]->device) cudaSetDevice(cur);
  if (e != cudaSuccess) {
    epic_batch_destroy(b);
    return set_error(EPIC_ERR_CUDA, "epic_batch_create: %s", cudaGetErrorString(e));
  }
  // the launch description: member 0's arrays (the kernels move pointer arguments to each
  // member's) with the largest sizes, which every grid, shared-memory size and loop bound of a
  // launch is computed from
  DevModel &d = b->d;
  d = members[0]->d;
  d.reloc_n3 = d.n3;
  for (int i = 1; i < n; i++) {
    const DevModel &m = members[i]->d;
    if (m.ni != members[0]->d.ni || m.nj != members[0]->d.nj) d.hetero = 1;
    d.ni = std::max(d.ni, m.ni);
    d.nj = std::max(d.nj, m.nj);
    d.iadim = std::max(d.iadim, m.iadim);
    d.jadim = std::max(d.jadim, m.jadim);
    d.n2 = std::max(d.n2, m.n2);
    d.n3 = std::max(d.n3, m.n3);
  }
  // one operator for all: a CTA of the filter serves several members with member 0's tiles
  d.fop_shared = !d.hetero && d.fop_map != nullptr;
  for (int i = 1; i < n && d.fop_shared; i++) d.fop_shared = members[i]->fop_hash == members[0]->fop_hash;
  d.batch = b->dev_members;
  d.nbatch = n;
  *out = b;
  return EPIC_OK;
}

extern "C" void epic_batch_destroy(epic_batch *b) {
  if (!b) return;
  for (auto *g : b->groups) epic_batch_destroy(g);
  if (b->host_ctl) cudaFreeHost(b->host_ctl);
  if (b->run_graph) cudaGraphExecDestroy(b->run_graph);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->dev_members) cudaFree(b->dev_members);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

static int batch_ready(epic_batch *b, const char *what) {
  if (!b) return set_error(EPIC_ERR_ARG, "%s: NULL batch", what);
  for (size_t i = 0; i < b->members.size(); i++)
    if (!b->members[i]->uploaded) return set_error(EPIC_ERR_STATE, "%s: member %zu has no state", what, i);
  // members' own streams may hold uploads; the batch runs after them
  for (auto *m : b->members) EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  return EPIC_OK;
}

extern "C" int epic_batch_timestep(epic_batch *b, int32_t action) {
  int rc = batch_ready(b, "epic_batch_timestep");
  if (rc) return rc;
  if (action == EPIC_STEP_PROGS_AND_SYNC_DIAGS) rc = enqueue_step_on(b->d, b->stream);
  else if (action == EPIC_SYNC_DIAGS_ONLY) rc = enqueue_sync_on(b->d, b->stream);
  else return set_error(EPIC_ERR_ARG, "unrecognized action=%d", action);
  if (rc) return rc;
  return check_launch("epic_batch_timestep");
}

extern "C" int epic_batch_run(epic_batch *b, int32_t nsteps) {
  int rc = batch_ready(b, "epic_batch_run");
  if (rc) return rc;
  if (nsteps <= 0) return EPIC_OK;
  if (!b->run_graph && !b->graph_failed) {
    b->run_graph = capture_step(b->d, b->stream, &b->kernels_per_step);
    if (!b->run_graph) b->graph_failed = true;
  }
  for (int s = 0; s < nsteps; s++) {
    if (b->run_graph) {
      EPIC_CUDA_CHECK(cudaGraphLaunch(b->run_graph, b->stream));
    } else {
      rc = enqueue_step_on(b->d, b->stream);
      if (rc) return rc;
      epic::launch_itime_advance(b->d, b->stream);
    }
  }
  return check_launch("epic_batch_run");
}

extern "C" int epic_batch_run_stage(epic_batch *b, int32_t stage) {
  int rc = batch_ready(b, "epic_batch_run_stage");
  if (rc) return rc;
  return run_stage_on(b->d, b->stream, stage);
}

// Every member's state to / from host arrays with all copies on the batch stream and one
// synchronisation (instead of one per member).
extern "C" int epic_batch_upload(epic_batch *b, const epic_fields *const *f) {
  if (!b || !f) return set_error(EPIC_ERR_ARG, "epic_batch_upload: NULL argument");
  for (auto *m : b->members) EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  EPIC_CUDA_CHECK(cudaStreamSynchronize(b->stream));
  std::vector<Ctl> ctl(b->members.size());
  int rc = EPIC_OK;
  for (size_t i = 0; i < b->members.size() && rc == EPIC_OK; i++) {
    if (!f[i]) rc = set_error(EPIC_ERR_ARG, "epic_batch_upload: member %zu has no fields", i);
    else rc = enqueue_upload(b->members[i], f[i], b->stream, &ctl[i]);
  }
  EPIC_CUDA_CHECK(cudaStreamSynchronize(b->stream));
  if (rc) return rc;
  for (auto *m : b->members) m->uploaded = true;
  return EPIC_OK;
}

extern "C" int epic_batch_download(epic_batch *b, epic_fields *const *f) {
  if (!b || !f) return set_error(EPIC_ERR_ARG, "epic_batch_download: NULL argument");
  std::vector<Ctl> ctl(b->members.size());
  int rc = EPIC_OK;
  for (size_t i = 0; i < b->members.size() && rc == EPIC_OK; i++) {
    if (!f[i]) rc = set_error(EPIC_ERR_ARG, "epic_batch_download: member %zu has no fields", i);
    else rc = enqueue_download(b->members[i], f[i], b->stream, &ctl[i]);
  }
  EPIC_CUDA_CHECK(cudaStreamSynchronize(b->stream));
  if (rc) return rc;
  for (size_t i = 0; i < b->members.size(); i++) {
    fields_from_ctl(f[i], ctl[i]);
    rc = model_error(ctl[i]);
    if (rc) {
      const std::string msg = epic::error_buffer();
      return set_error(EPIC_ERR_MODEL, "member %zu: %s", i, msg.c_str());
    }
  }
  return EPIC_OK;
}

extern "C" int epic_batch_sync(epic_batch *b) {
  if (!b) return set_error(EPIC_ERR_ARG, "epic_batch_sync: NULL batch");
  EPIC_CUDA_CHECK(cudaStreamSynchronize(b->stream));
  for (size_t i = 0; i < b->members.size(); i++) {
    Ctl c;
    int rc = read_ctl(b->members[i], c);
    if (rc) return rc;
    rc = model_error(c);
    if (rc) {
      const std::string msg = epic::error_buffer();
      return set_error(EPIC_ERR_MODEL, "member %zu: %s", i, msg.c_str());
    }
  }
  return EPIC_OK;
}

extern "C" int epic_batch_query(epic_batch *b) {
  if (!b) return set_error(EPIC_ERR_ARG, "epic_batch_query: NULL batch");
  const cudaError_t e = cudaStreamQuery(b->stream);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return set_error(EPIC_ERR_CUDA, "epic_batch_query: %s", cudaGetErrorString(e));
}

extern "C" void *epic_batch_stream(epic_batch *b) { return b ? (void *)b->stream : nullptr; }

extern "C" int32_t epic_batch_kernels_per_step(const epic_batch *b) { return b ? b->kernels_per_step : -1; }

// ---- autotuning of launch shapes ----
//
// For each kernel group (DevModel::tb) in turn, time whole steps of the batch with each candidate
// block size, the other groups at their best so far, and keep the fastest.  Every tuned kernel
// is pointwise or per row, so the choice changes no result.  The trial steps advance the
// members' state: tune before uploading the state a run starts from, or on scratch members.

extern "C" int epic_batch_autotune(epic_batch *b, int32_t trial_steps, int32_t *table_out) {
  int rc = batch_ready(b, "epic_batch_autotune");
  if (rc) return rc;
  if (trial_steps < 1) trial_steps = 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  EPIC_CUDA_CHECK(cudaEventCreate(&e0));
  EPIC_CUDA_CHECK(cudaEventCreate(&e1));
  auto time_steps = [&](float *ms) -> int {
    int r = enqueue_step_on(b->d, b->stream);   // warm-up step for this shape
    if (r) return r;
    cudaEventRecord(e0, b->stream);
    for (int q = 0; q < trial_steps && !r; q++) r = enqueue_step_on(b->d, b->stream);
    cudaEventRecord(e1, b->stream);
    if (r) return r;
    EPIC_CUDA_CHECK(cudaEventSynchronize(e1));
    EPIC_CUDA_CHECK(cudaEventElapsedTime(ms, e0, e1));
    return check_launch("epic_batch_autotune");
  };
  static const int cell_cand[] = {64, 128, 256, 512};
  static const int row_cand[] = {32, 64, 128, 256};
  static const int variant_cand[] = {1, 2};   // meridional Hsu pass: fused march, four passes
  for (int g = 0; g < TB_COUNT && rc == EPIC_OK; g++) {
    const int *cand = g == TB_ROW ? row_cand : (g == TB_HSU_MERID_VARIANT ? variant_cand : cell_cand);
    const int ncand = g == TB_HSU_MERID_VARIANT ? 2 : 4;
    int best = b->d.tb[g];
    float best_ms = 3.4e38f;
    for (int c = 0; c < ncand && rc == EPIC_OK; c++) {
      if (g == TB_ROW && c > 0 && cand[c] > b->d.ni / 2) continue;   // more threads than butterflies
      b->d.tb[g] = cand[c];
      float ms = 0.f;
      rc = time_steps(&ms);
      if (rc == EPIC_ERR_CUDA && c > 0 && cudaStreamSynchronize(b->stream) == cudaSuccess) {
        // a block size some kernel of the group cannot launch with (its registers per block):
        // the launch failed before running, nothing is in flight; skip the candidate
        rc = EPIC_OK;
        continue;
      }
      if (rc == EPIC_OK && ms < best_ms) { best_ms = ms; best = cand[c]; }
    }
    b->d.tb[g] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (b->run_graph) { cudaGraphExecDestroy(b->run_graph); b->run_graph = nullptr; }
  b->graph_failed = false;
  if (table_out)
    for (int g = 0; g < TB_COUNT; g++) table_out[g] = b->d.tb[g];
  return rc;
}

extern "C" int epic_batch_set_tuning(epic_batch *b, const int32_t *table) {
  if (!b || !table) return set_error(EPIC_ERR_ARG, "epic_batch_set_tuning: NULL argument");
  for (int g = 0; g < TB_COUNT; g++) b->d.tb[g] = table[g];
  if (b->run_graph) { cudaGraphExecDestroy(b->run_graph); b->run_graph = nullptr; }
  b->graph_failed = false;
  return EPIC_OK;
}

extern "C" int epic_model_set_tuning(epic_model *m, const int32_t *table) {
  if (!m || !table) return set_error(EPIC_ERR_ARG, "epic_model_set_tuning: NULL argument");
  for (int g = 0; g < TB_COUNT; g++) m->d.tb[g] = table[g];
  if (m->run_graph) { cudaGraphExecDestroy(m->run_graph); m->run_graph = nullptr; }
  m->graph_failed = false;
  return EPIC_OK;
}

// ---- asynchronous snapshots: the state copied out while the model keeps stepping ----
//
// The reference writes epic.nc/extract.nc from host `var` every itsave/itextract steps
// (src/shared/epic_main.c:338-411), which here would mean stopping the device for a full
// device-to-host copy.  A snapshot instead copies the state region device-to-device in stream
// order (between two steps; a few hundred microseconds even for a large grid) and then copies
// that copy to the host on a second stream while the following steps run.  The host-side
// writer (the reference's var_write) runs once epic_model_snapshot_wait returns.

namespace {

// [u, end of u_spinup): the state arrays, carved contiguously from the pool
size_t state_region_bytes(const DevModel &d) {
  return (size_t)((const char *)(d.u_spinup + d.n3) - (const char *)d.u);
}

int finish_snapshot(epic_model *m) {
  if (!m->snap_dst) return EPIC_OK;
  EPIC_CUDA_CHECK(cudaEventSynchronize(m->snap_done));
  epic_fields *f = m->snap_dst;
  m->snap_dst = nullptr;
  const Ctl &c = *m->snap_ctl;
  f->it_zero = c.it_zero; f->it_minus1 = c.it_minus1; f->it_minus2 = c.it_minus2;
  f->itime = c.itime; f->model_time = c.model_time;
  return model_error(c);
}

}  // namespace

extern "C" int epic_model_snapshot_begin(epic_model *m, epic_fields *f) {
  if (!m || !f) return set_error(EPIC_ERR_ARG, "epic_model_snapshot_begin: NULL argument");
  if (!m->uploaded) return set_error(EPIC_ERR_STATE, "snapshot before upload");
  int rc = finish_snapshot(m);   // one snapshot in flight per model
  if (rc) return rc;
  const DevModel &d = m->d;
  const size_t sb = state_region_bytes(d), gb = (size_t)d.n2 * sizeof(double);
  const size_t tb = d.turb ? 4 * (size_t)d.n3 * sizeof(double) : 0;   // NU_TURB and the diffusivities
  if (!m->snap) {
    EPIC_CUDA_CHECK(cudaStreamCreateWithFlags(&m->copy_stream, cudaStreamNonBlocking));
    EPIC_CUDA_CHECK(cudaEventCreateWithFlags(&m->snap_taken, cudaEventDisableTiming));
    EPIC_CUDA_CHECK(cudaEventCreateWithFlags(&m->snap_done, cudaEventDisableTiming));
    EPIC_CUDA_CHECK(cudaMallocHost(&m->snap_ctl, sizeof(Ctl)));
    cudaError_t e = cudaMalloc(&m->snap, sb + gb + sizeof(Ctl) + tb);
    if (e != cudaSuccess) {
      m->snap = nullptr;
      return set_error(EPIC_ERR_NOMEM, "snapshot buffer: %s", cudaGetErrorString(e));
    }
  }
  char *s_state = m->snap, *s_gzs = m->snap + sb, *s_ctl = s_gzs + gb, *s_turb = s_ctl + sizeof(Ctl);
  const size_t b3 = (size_t)d.n3 * sizeof(double);
  // in stream order, between the steps already enqueued and the ones that follow
  EPIC_CUDA_CHECK(cudaMemcpyAsync(s_state, d.u, sb, cudaMemcpyDeviceToDevice, m->stream));
  EPIC_CUDA_CHECK(cudaMemcpyAsync(s_gzs, d.gz_surface, gb, cudaMemcpyDeviceToDevice, m->stream));
  EPIC_CUDA_CHECK(cudaMemcpyAsync(s_ctl, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToDevice, m->stream));
  const double *turb_src[] = {d.nu_turb, d.dc_uv, d.dc_theta, d.dc_mass};
  double *turb_dst[] = {f->nu_turb, f->diffusion_coef_uv, f->diffusion_coef_theta, f->diffusion_coef_mass};
  if (d.turb)
    for (int q = 0; q < 4; q++) EPIC_CUDA_CHECK(cudaMemcpyAsync(s_turb + q * b3, turb_src[q], b3, cudaMemcpyDeviceToDevice, m->stream));
  EPIC_CUDA_CHECK(cudaEventRecord(m->snap_taken, m->stream));
  EPIC_CUDA_CHECK(cudaStreamWaitEvent(m->copy_stream, m->snap_taken, 0));
  auto at = [&](const double *dev) { return s_state + ((const char *)dev - (const char *)d.u); };
  cudaStream_t cs = m->copy_stream;
  if (d.turb)
    for (int q = 0; q < 4; q++)
      if (turb_dst[q]) EPIC_CUDA_CHECK(cudaMemcpyAsync(turb_dst[q], s_turb + q * b3, b3, cudaMemcpyDeviceToHost, cs));
  if (f->u) EPIC_CUDA_CHECK(cudaMemcpyAsync(f->u, at(d.u), d.nvp * b3, cudaMemcpyDeviceToHost, cs));
  if (f->v) EPIC_CUDA_CHECK(cudaMemcpyAsync(f->v, at(d.v), d.nvp * b3, cudaMemcpyDeviceToHost, cs));
  if (f->dudt) EPIC_CUDA_CHECK(cudaMemcpyAsync(f->dudt, at(d.dudt), d.ntp * b3, cudaMemcpyDeviceToHost, cs));
  if (f->dvdt) EPIC_CUDA_CHECK(cudaMemcpyAsync(f->dvdt, at(d.dvdt), d.ntp * b3, cudaMemcpyDeviceToHost, cs));
  double *dst[] = {f->hdry, f->theta, f->p3, f->h3, f->p2, f->theta2, f->t2, f->t3, f->rho2, f->rho3, f->exner3, f->gz3,
                   f->mont3, f->heat3, f->pv3, f->ri2, f->div_uv3, f->w3, f->dzdt3, f->u_spinup};
  const double *src[] = {d.hdry, d.theta, d.p3, d.h3, d.p2, d.theta2, d.t2, d.t3, d.rho2, d.rho3, d.exner3, d.gz3,
                         d.mont3, d.heat3, d.pv3, d.ri2, d.div_uv3, d.w3, d.dzdt3, d.u_spinup};
  for (int i = 0; i < 20; i++)
    if (dst[i]) EPIC_CUDA_CHECK(cudaMemcpyAsync(dst[i], at(src[i]), b3, cudaMemcpyDeviceToHost, cs));
  if (f->gz_surface) EPIC_CUDA_CHECK(cudaMemcpyAsync(f->gz_surface, s_gzs, gb, cudaMemcpyDeviceToHost, cs));
  EPIC_CUDA_CHECK(cudaMemcpyAsync(m->snap_ctl, s_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, cs));
  EPIC_CUDA_CHECK(cudaEventRecord(m->snap_done, cs));
  m->snap_dst = f;
  return EPIC_OK;
}

extern "C" int epic_model_snapshot_wait(epic_model *m) {
  if (!m) return set_error(EPIC_ERR_ARG, "epic_model_snapshot_wait: NULL model");
  return finish_snapshot(m);
}

// ---- the end-to-end step of a batch with host-resident state, pipelined ----
//
// Each step copies every member's state in from host arrays, steps it and copies it back (the
// drop-in's contract when `var` lives on the host).  The members are split into `groups`
// sub-batches, each with its own stream and captured graph, so one group's copies overlap the
// others' kernels and the two copy directions overlap each other.

extern "C" int epic_batch_step_host(epic_batch *b, epic_fields *const *f, int32_t groups, int32_t nsteps, int32_t io) {
  if (!b || !f) return set_error(EPIC_ERR_ARG, "epic_batch_step_host: NULL argument");
  if (io != EPIC_IO_ALL && io != EPIC_IO_STATE) return set_error(EPIC_ERR_ARG, "epic_batch_step_host: io=%d", io);
  const bool state_only = io == EPIC_IO_STATE;
  if (state_only)
    for (size_t i = 0; i < b->members.size(); i++)
      if (!b->members[i]->uploaded)
        return set_error(EPIC_ERR_STATE, "epic_batch_step_host: member %zu has no state on the device (EPIC_IO_STATE moves the prognostic arrays only)", i);
  const int n = (int)b->members.size();
  if (groups < 1) groups = 1;
  if (groups > n) groups = n;
  if ((int)b->groups.size() != groups) {
    for (auto *g : b->groups) epic_batch_destroy(g);
    b->groups.clear();
    for (int q = 0; q < groups; q++) {
      const int lo = (int)((long long)n * q / groups), hi = (int)((long long)n * (q + 1) / groups);
      epic_batch *g = nullptr;
      int rc = epic_batch_create(b->members.data() + lo, hi - lo, &g);
      if (rc) return rc;
      for (int t = 0; t < TB_COUNT; t++) g->d.tb[t] = b->d.tb[t];
      b->groups.push_back(g);
    }
  }
  // one upload and one download control block per member and step: the steps are not drained
  // one by one, each group's next upload follows its last download in stream order
  const size_t nctl = 2 * (size_t)n * (size_t)(nsteps > 0 ? nsteps : 1);
  if (b->host_ctl_count < nctl) {
    if (b->host_ctl) cudaFreeHost(b->host_ctl);
    b->host_ctl = nullptr;
    b->host_ctl_count = 0;
    EPIC_CUDA_CHECK(cudaMallocHost(&b->host_ctl, sizeof(Ctl) * nctl));
    b->host_ctl_count = nctl;
  }
  for (auto *m : b->members) EPIC_CUDA_CHECK(cudaStreamSynchronize(m->stream));
  for (int step = 0; step < nsteps; step++) {
    Ctl *ctl = b->host_ctl + 2 * (size_t)n * step;
    int idx = 0;
    for (auto *g : b->groups) {
      const int lo = idx;
      for (auto *m : g->members) {
        // after the first step the host arrays hold exactly what the device state was, and the
        // device's control block (time-plane indices, itime) is already the one they belong to
        int rc = enqueue_upload(m, f[idx], g->stream, &ctl[2 * idx], step == 0, state_only);
        if (rc) return rc;
        m->uploaded = true;
        idx++;
      }
      if (!g->run_graph && !g->graph_failed) {
        g->run_graph = capture_step(g->d, g->stream, &g->kernels_per_step);
        if (!g->run_graph) g->graph_failed = true;
      }
      if (g->run_graph) EPIC_CUDA_CHECK(cudaGraphLaunch(g->run_graph, g->stream));
      else {
        int rc = enqueue_step_on(g->d, g->stream);
        if (!rc) rc = epic::launch_itime_advance(g->d, g->stream);
        if (rc) return rc;
      }
      for (int q = lo; q < idx; q++) {
        int rc = enqueue_download(b->members[q], f[q], g->stream, &ctl[2 * q + 1], state_only);
        if (rc) return rc;
      }
    }
  }
  for (auto *g : b->groups) EPIC_CUDA_CHECK(cudaStreamSynchronize(g->stream));
  for (int step = 0; step < nsteps; step++)
    for (int q = 0; q < n; q++) {
      const Ctl &c = b->host_ctl[2 * ((size_t)n * step + q) + 1];
      if (step == nsteps - 1) fields_from_ctl(f[q], c);
      int rc = model_error(c);
      if (rc) {
        const std::string msg = epic::error_buffer();
        return set_error(EPIC_ERR_MODEL, "step %d, member %d: %s", step, q, msg.c_str());
      }
    }
  return check_launch("epic_batch_step_host");
}

