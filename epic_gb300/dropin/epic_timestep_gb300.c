/*
 * epic_timestep_gb300.c -- the GB300 step behind the reference's own entry point
 *
 *     void timestep(planetspec *planet, int action, EPIC_FLOAT **Buff2D);
 *         include/epic.h:654-656, src/shared/epic_timestep.c:62
 *
 * Compiled with the reference's headers (its include/ directory, EPIC_PRECISION=8) and linked
 * ahead of src/shared/epic_timestep.o together with libepic_gb300.so, it replaces the CPU step of
 * an unchanged `epic` driver: the globals `grid`, `planet` and `var` are read exactly as the
 * reference's timestep() reads them, and after every call `var` holds the stepped state (mirror
 * mode, the default) -- time-plane indices IT_ZERO/IT_MINUS1/IT_MINUS2 and var.model_time
 * included -- so var_write() and the save block of the driver loop (src/shared/epic_main.c:338-411)
 * need no change.  The driver keeps owning grid.itime and advances it after each call (:424).
 *
 * Environment (read on the first call):
 *   EPIC_GB300_MODE       "mirror" (default) or "resident": in resident mode the state stays on
 *                         the device and `var` is stale until epic_gpu_sync_to_host(), which a
 *                         driver calls before var_write() (no copies between saves)
 *   EPIC_GB300_PRECISION  "fp64" (default: the drop-in form, the reference's arithmetic), "mixed"
 *                         or "fast" (the mixed-precision forms)
 *
 * Errors follow the reference's convention: a failed call ends in epic_error("timestep", ...),
 * which prints the message and exits (src/shared/epic_funcs_io.c:4872-4889).
 * epic_gpu_status() reports the device's first error without exiting.
 */
#include <stdlib.h>
#include <string.h>

#include "epic.h"
#include "epic_gb300.h"

#if !defined(EPIC_PRECISION) || EPIC_PRECISION != 8
#error "the GB300 step works on binary64 state: build the reference with EPIC_PRECISION=8"
#endif

static epic_grid   g;
static epic_fields f;
static int         started = 0, mode = EPIC_DROPIN_MIRROR, precision = EPIC_PREC_FP64;

/* The gridspec/planetspec scalars and 1-D arrays the reference's step reads. */
static void grid_from_globals(planetspec *planet) {
  int i;
  memset(&g, 0, sizeof(g));
  g.ni = grid.ni;  g.nj = grid.nj;  g.nk = grid.nk;  g.dt = grid.dt;
  g.uv_scheme = strcmp(grid.uv_timestep_scheme, "3rd-order Adams-Bashforth") == 0 ? EPIC_UV_AB3 : EPIC_UV_LEAPFROG;
  /* advection() dispatches on var.theta.advection_scheme (epic_flux.c:390-397); HDRY uses the same scheme */
  g.advection_scheme = strcmp(var.theta.advection_scheme, "Monotonized, 4th-order centered (Akima)") == 0 ? EPIC_ADV_AKIMA
                                                                                                         : EPIC_ADV_HSU;
  g.k_sigma = grid.k_sigma;  g.k_sponge = grid.k_sponge;  g.newt_cool_on = grid.newt_cool_on;
  g.newt_cool_adjust = grid.newt_cool_adjust;  g.drag_v = grid.drag_v;  g.drag_zonal_avg = grid.drag_zonal_avg;
  g.jtp = grid.jtp;  g.dln = grid.dln;  g.dlt = grid.dlt;  g.dy0 = grid.dy0;
  g.globe_latbot = grid.globe_latbot;  g.globe_lattop = grid.globe_lattop;  g.press0 = grid.press0;
  g.topo_scale = grid.topo_scale;  g.prandtl = grid.prandtl;  g.tau_drag = grid.tau_drag;
  g.nudiv_nondim = grid.nudiv_nondim;  g.zeta0 = grid.zeta0;  g.zeta1 = grid.zeta1;
  g.hybrid_alpha = grid.hybrid_alpha;  g.sigma_sigma = grid.sigma_sigma;
  for (i = 0; i <= MAX_NU_ORDER && i < 9; i++) g.nu[i] = grid.nu[i];
  g.re = planet->re;  g.rp = planet->rp;  g.cp = planet->cp;  g.rgas = planet->rgas;
  g.kappa = planet->kappa;  g.cpr = planet->cpr;  g.kinvisc = planet->kinvisc;  g.dynvisc = planet->dynvisc;
  /* the gas-giant lower boundary (store_pgrad_vars' gz_from_u, epic_funcs_diag.c:3779-3811) and the
   * hydrogen thermodynamics (thermo_setup's tables when planet->x_h2 > 0; cpr is thermo_setup's) */
  g.gas_giant = strcmp(planet->type, "gas-giant") == 0;
  g.x_h2 = planet->x_h2;  g.x_he = planet->x_he;  g.x_3 = planet->x_3;
  /* the turbulence closure (epic_subgrid.c), as the reference's initial program chose it */
  g.turbulence = strcmp(grid.turbulence_scheme, "Spalart-Allmaras DES") == 0 ? EPIC_TURB_SA_DES : EPIC_TURB_OFF;
  g.diffusion_direction = grid.diffusion_direction;
  g.stability_factor = strcmp(grid.stability_factor, "Collins et al. (2004)") == 0;
  g.lat0 = LAT0;
  g.hs_kf = 1. / (24. * 60. * 60.);   /* HELD_SUAREZ_PBL_NU0, epic_timestep.c:1292 */
  g.lon = grid.lon;  g.lat = grid.lat;  g.rln = grid.rln;  g.rlt = grid.rlt;  g.f = grid.f;
  g.m = grid.m;  g.n = grid.n;  g.mn = grid.mn;  g.g = grid.g;  g.sigmatheta = grid.sigmatheta;
  g.dsgth = grid.dsgth;  g.dsgth_inv = grid.dsgth_inv;  g.h_min = grid.h_min;
  g.t_sponge_inv = grid.t_sponge_inv;
}

/* Host views of `var` (the arrays never move after make_arrays) and the time-plane indices. */
static void fields_from_var(void) {
  f.u = var.u.value;  f.v = var.v.value;  f.dudt = var.u.tendency;  f.dvdt = var.v.tendency;
  f.hdry = var.hdry.value;  f.theta = var.theta.value;  f.p3 = var.p3.value;  f.h3 = var.h3.value;
  f.p2 = var.p2.value;  f.theta2 = var.theta2.value;  f.t2 = var.t2.value;  f.t3 = var.t3.value;
  f.rho2 = var.rho2.value;  f.rho3 = var.rho3.value;  f.exner3 = var.exner3.value;
  f.gz3 = var.gz3.value;  f.mont3 = var.mont3.value;  f.heat3 = var.heat3.value;  f.pv3 = var.pv3.value;
  f.ri2 = var.ri2.value;  f.div_uv3 = var.div_uv3.value;  f.w3 = var.w3.value;  f.dzdt3 = var.dzdt3.value;
  f.u_spinup = var.u_spinup.value;  f.gz_surface = var.gz_surface.value;
  if (var.nu_turb.on) {   /* NU_TURB and the diffusivities store_diag leaves for the next step */
    f.nu_turb = var.nu_turb.value;  f.diffusion_coef_uv = var.diffusion_coef_uv.value;
    f.diffusion_coef_theta = var.diffusion_coef_theta.value;  f.diffusion_coef_mass = var.diffusion_coef_mass.value;
  }
  f.it_zero = IT_ZERO;  f.it_minus1 = IT_MINUS1;  f.it_minus2 = IT_MINUS2;
  f.itime = (int64_t)grid.itime;  f.model_time = (int64_t)var.model_time;
}

static void var_times_from_fields(void) {
  IT_ZERO = f.it_zero;  IT_MINUS1 = f.it_minus1;  IT_MINUS2 = f.it_minus2;
  var.model_time = (time_t)f.model_time;
}

static void fail(int rc) {
  char msg[1024];
  (void)rc;
  strncpy(msg, epic_dropin_message(), sizeof(msg) - 1);
  msg[sizeof(msg) - 1] = '\0';
  epic_error("timestep", msg);
}

void timestep(planetspec *planet, int action, EPIC_FLOAT **Buff2D) {
  int rc;
  (void)Buff2D;   /* the device keeps its own scratch planes */
  if (!started) {
    const char *m = getenv("EPIC_GB300_MODE"), *p = getenv("EPIC_GB300_PRECISION");
    mode = (m && strcmp(m, "resident") == 0) ? EPIC_DROPIN_RESIDENT : EPIC_DROPIN_MIRROR;
    precision = !p ? EPIC_PREC_FP64
                   : strcmp(p, "mixed") == 0 ? EPIC_PREC_MIXED : (strcmp(p, "fast") == 0 ? EPIC_PREC_MIXED_FAST : EPIC_PREC_FP64);
    grid_from_globals(planet);
    started = 1;
  }
  fields_from_var();
  rc = epic_dropin_timestep(&g, &f, precision, mode, action, (int64_t)grid.itime);
  if (rc) fail(rc);
  if (mode == EPIC_DROPIN_MIRROR) var_times_from_fields();
  else if (action == STEP_PROGS_AND_SYNC_DIAGS) var.model_time += (time_t)grid.dt;   /* epic_timestep.c:304 */
}

/* Resident mode: bring `var` (and IT_ZERO, IT_MINUS1, IT_MINUS2, var.model_time) up to date
 * before var_write() or any other host reader.  A no-op copy in mirror mode. */
void epic_gpu_sync_to_host(void) {
  int rc;
  fields_from_var();
  rc = epic_dropin_sync_to_host(&f);
  if (rc) fail(rc);
  var_times_from_fields();
}

/* 0 while the device step is healthy, else the EPIC_ERR_* code of its first error (the text is
 * epic_dropin_message()); waits for queued work, never exits. */
int epic_gpu_status(void) { return epic_dropin_status(); }
