/*
 * In-process harness around the reference EPIC step (test infrastructure only).
 *
 * Links the reference's own objects, compiled from their sources by oracle/Makefile, and
 * drives them the way src/shared/epic_main.c:236-303,336-427 does, with two changes that
 * work around crashes of the stock reference without touching its sources:
 *   - grid.t_sponge_inv is allocated for k_sponge = 0 (make_arrays only allocates it for
 *     k_sponge > 0, src/shared/epic_funcs_diag.c:859-861, but uv_drag reads entry 0,
 *     src/shared/epic_timestep.c:1363-1376);
 *   - nothing goes through netCDF: the grid and initial state arrive in the structs of
 *     include/epic_gb300.h instead of var_read() from epic.nc.
 * The grid arrays the reference computes itself (set_lonlat, set_fmn, set_gravity,
 * set_dsgth) are compared with the ones passed in (ref_geometry_maxdiff) and then replaced
 * by them, so both implementations step bit-identical inputs.
 *
 * The reference keeps static state inside its functions, so one process holds one model.
 */
#include <epic.h>
#include "epic_gb300.h"

static EPIC_FLOAT *ref_buff2d[NUM_WORKING_BUFFERS];
static int ref_ready = 0;
static double ref_geom_diff[8];

static double maxreldiff(const double *a, const double *b, int n) {
  double d = 0.;
  for (int i = 0; i < n; i++) {
    double s = fabs(a[i]) > fabs(b[i]) ? fabs(a[i]) : fabs(b[i]);
    double e = fabs(a[i] - b[i]);
    if (s > 0.) e /= s;
    if (e > d) d = e;
  }
  return d;
}

/* Index into a 3-D reference array. */
static long at3(int k, int j, int i) { return (long)i + (long)j * Iadim + (long)k * Nelem2d - Shift3d; }

int ref_init(const epic_grid *g, const epic_fields *f) {
  int K, J, I, n1j, n1k, n1i;
  if (ref_ready) return -1;
  memset(&grid, 0, sizeof(grid));
  memset(&var, 0, sizeof(var));

  planet = (planetspec *)malloc(sizeof(planetspec));
  *planet = held_suarez;
  /* the gas-giant lower boundary on the same planet: store_pgrad_vars then takes GZ_SURFACE
   * from gz_from_u (epic_funcs_diag.c:3779-3811) */
  if (g->gas_giant) strcpy(planet->type, "gas-giant");
  /* hydrogen thermodynamics on the same planet: the composition, then the reference's own
   * thermo_setup (its tables and cpr), as its initialisation calls it */
  if (g->x_h2 > 0.) {
    planet->x_h2 = g->x_h2;
    planet->x_he = g->x_he;
    planet->x_3 = g->x_3;
    thermo_setup(planet, &planet->cpr);
  }
  if (planet->re != g->re || planet->rp != g->rp || planet->cp != g->cp || planet->rgas != g->rgas ||
      planet->kappa != g->kappa || planet->cpr != g->cpr || planet->kinvisc != g->kinvisc ||
      (g->turbulence && planet->dynvisc != g->dynvisc))
    return -2;

  /* What var_read(SIZE_DATA) and (POST_SIZE_DATA) supply for a held_suarez epic.nc. */
  strcpy(grid.geometry, "globe");
  strcpy(grid.uv_timestep_scheme, g->uv_scheme == EPIC_UV_AB3 ? "3rd-order Adams-Bashforth" : "Leapfrog (Asselin filtered)");
  strcpy(grid.turbulence_scheme, g->turbulence == EPIC_TURB_SA_DES ? "Spalart-Allmaras DES" : "off");
  grid.diffusion_direction = g->diffusion_direction;
  strcpy(grid.stability_factor, g->stability_factor ? "Collins et al. (2004)" : "off");
  strcpy(grid.eos, "ideal");
  strcpy(grid.advection_scheme, g->advection_scheme == EPIC_ADV_AKIMA ? "Monotonized, 4th-order centered (Akima)"
                                                                      : "Predictor-corrector (Hsu, Konor, and Arakawa)");
  strcpy(var.theta.advection_scheme, grid.advection_scheme);
  strcpy(var.hdry.advection_scheme, grid.advection_scheme);
  strcpy(var.nu_turb.advection_scheme, grid.advection_scheme);
  grid.nk = g->nk; grid.nj = g->nj; grid.ni = g->ni; grid.dt = g->dt;
  grid.wrap[0] = 1; grid.wrap[1] = 0; grid.wrap[2] = 0;
  grid.pad[0] = grid.pad[1] = grid.pad[2] = 1;
  grid.jlo = 0; grid.jfirst = 1; grid.jlast = g->nj - 1;
  grid.globe_lonbot = -180.; grid.globe_lontop = 180.;
  grid.globe_latbot = g->globe_latbot; grid.globe_lattop = g->globe_lattop;
  grid.dln = g->dln; grid.dlt = g->dlt;
  grid.press0 = g->press0;
  grid.zeta0 = g->zeta0; grid.zeta1 = g->zeta1; grid.hybrid_alpha = g->hybrid_alpha; grid.sigma_sigma = g->sigma_sigma;
  grid.k_sponge = g->k_sponge; grid.k_sigma = g->k_sigma;
  grid.newt_cool_on = g->newt_cool_on; grid.newt_cool_adjust = g->newt_cool_adjust;
  grid.prandtl = g->prandtl; grid.tau_drag = g->tau_drag; grid.drag_v = g->drag_v; grid.drag_zonal_avg = g->drag_zonal_avg;
  grid.topo_scale = g->topo_scale; grid.nudiv_nondim = g->nudiv_nondim;
  grid.jtp = g->jtp;
  for (I = 0; I <= MAX_NU_ORDER; I++) grid.nu[I] = g->nu[I];
  grid.itime = 0;
  var.on_list[U_INDEX] = var.on_list[V_INDEX] = var.on_list[HDRY_INDEX] = var.on_list[THETA_INDEX] = 1;
  if (g->turbulence == EPIC_TURB_SA_DES) var.on_list[NU_TURB_INDEX] = 1;

  make_arrays(planet);   /* with the turbulence scheme on, this also allocates D_WALL (make_arrays_subgrid) */
  for (I = 0; I < NUM_WORKING_BUFFERS; I++) ref_buff2d[I] = fvector(0, Nelem2d - 1, "ref_harness");
  if (grid.t_sponge_inv == NULL) grid.t_sponge_inv = fvector(0, grid.k_sponge, "ref_harness");
  for (K = 0; K <= grid.k_sponge; K++) grid.t_sponge_inv[K] = g->t_sponge_inv[K];
  timeplane_bookkeeping();

  /* Reference geometry, then the caller's arrays in its place. */
  n1j = 2 * (grid.nj + 1) + 1; n1k = 2 * (grid.nk + 1) + 1; n1i = 2 * (grid.ni + 1) + 1;
  set_lonlat();
  set_fmn(planet);
  set_gravity(planet);
  ref_geom_diff[0] = maxreldiff(grid.lat, g->lat, n1j);
  ref_geom_diff[1] = maxreldiff(grid.lon, g->lon, n1i);
  ref_geom_diff[2] = fmax(maxreldiff(grid.m, g->m, n1j), maxreldiff(grid.n, g->n, n1j));
  ref_geom_diff[3] = fmax(maxreldiff(grid.mn, g->mn, n1j), maxreldiff(grid.f, g->f, n1j));
  ref_geom_diff[4] = fmax(maxreldiff(grid.rln, g->rln, n1j), maxreldiff(grid.rlt, g->rlt, n1j));
  ref_geom_diff[5] = maxreldiff(grid.g, g->g, n1j);
  ref_geom_diff[7] = fabs(grid.dy0 - g->dy0) / g->dy0;
  memcpy(grid.lat, g->lat, n1j * sizeof(double)); memcpy(grid.lon, g->lon, n1i * sizeof(double));
  memcpy(grid.m, g->m, n1j * sizeof(double)); memcpy(grid.n, g->n, n1j * sizeof(double));
  memcpy(grid.mn, g->mn, n1j * sizeof(double)); memcpy(grid.f, g->f, n1j * sizeof(double));
  memcpy(grid.rln, g->rln, n1j * sizeof(double)); memcpy(grid.rlt, g->rlt, n1j * sizeof(double));
  memcpy(grid.g, g->g, n1j * sizeof(double));
  grid.dy0 = g->dy0;
  memcpy(grid.sigmatheta, g->sigmatheta, n1k * sizeof(double));
  set_dsgth();
  ref_geom_diff[6] = fmax(maxreldiff(grid.dsgth, g->dsgth, n1k), maxreldiff(grid.dsgth_inv, g->dsgth_inv, n1k));
  memcpy(grid.dsgth, g->dsgth, n1k * sizeof(double)); memcpy(grid.dsgth_inv, g->dsgth_inv, n1k * sizeof(double));
  memcpy(grid.h_min, g->h_min, (grid.nk + 2) * sizeof(double));

  /* Prognostic state and the inputs the step reads before writing. */
  {
    int nvp = g->uv_scheme == EPIC_UV_AB3 ? 1 : 2, ntp = g->uv_scheme == EPIC_UV_AB3 ? 3 : 1;
    memcpy(var.u.value, f->u, (size_t)nvp * Nelem3d * sizeof(double));
    memcpy(var.v.value, f->v, (size_t)nvp * Nelem3d * sizeof(double));
    memcpy(var.u.tendency, f->dudt, (size_t)ntp * Nelem3d * sizeof(double));
    memcpy(var.v.tendency, f->dvdt, (size_t)ntp * Nelem3d * sizeof(double));
  }
  memcpy(var.hdry.value, f->hdry, Nelem3d * sizeof(double));
  memcpy(var.theta.value, f->theta, Nelem3d * sizeof(double));
  memcpy(var.p3.value, f->p3, Nelem3d * sizeof(double));
  memcpy(var.gz_surface.value, f->gz_surface, Nelem2d * sizeof(double));
  memcpy(var.u_spinup.value, f->u_spinup, Nelem3d * sizeof(double));
  if (g->turbulence == EPIC_TURB_SA_DES) {
    if (!f->nu_turb || !var.nu_turb.value) return -3;
    memcpy(var.nu_turb.value, f->nu_turb, Nelem3d * sizeof(double));
    if (f->diffusion_coef_uv) memcpy(var.diffusion_coef_uv.value, f->diffusion_coef_uv, Nelem3d * sizeof(double));
    if (f->diffusion_coef_theta) memcpy(var.diffusion_coef_theta.value, f->diffusion_coef_theta, Nelem3d * sizeof(double));
    if (f->diffusion_coef_mass) memcpy(var.diffusion_coef_mass.value, f->diffusion_coef_mass, Nelem3d * sizeof(double));
  }
  IT_ZERO = f->it_zero; IT_MINUS1 = f->it_minus1; IT_MINUS2 = f->it_minus2;
  grid.itime = f->itime;
  var.model_time = (time_t)f->model_time;
  timeplane_bookkeeping();
  ref_ready = 1;
  return 0;
}

/* HDRY as epic_main.c:290-297 rebuilds it (for checking the caller's HDRY). */
double ref_hdry_maxdiff(const double *hdry) {
  int K, J, I;
  double d = 0.;
  for (K = KLO; K <= KHI; K++)
    for (J = JLO; J <= JHI; J++)
      for (I = ILO; I <= IHI; I++) {
        double h = get_h(planet, 2 * K, J, I, DRY);
        double e = fabs(h - hdry[at3(K, J, I)]) / fabs(h);
        if (e > d) d = e;
      }
  return d;
}

void ref_geometry_maxdiff(double out[8]) { memcpy(out, ref_geom_diff, sizeof(ref_geom_diff)); }

int ref_timestep(int action) {
  if (!ref_ready) return -1;
  timestep(planet, action, ref_buff2d);
  return 0;
}

int ref_run(int nsteps) {
  int s;
  if (!ref_ready) return -1;
  for (s = 0; s < nsteps; s++) {
    timestep(planet, STEP_PROGS_AND_SYNC_DIAGS, ref_buff2d);
    grid.itime++;
  }
  return 0;
}

/* The reference's cfl_dt(planet) on its current state (var_write calls it before a save). */
int ref_cfl_dt(void) { return ref_ready ? cfl_dt(planet) : -1; }

static void cp3(double *dst, const double *src) { if (dst) memcpy(dst, src, Nelem3d * sizeof(double)); }

int ref_get(epic_fields *f) {
  int nvp, ntp;
  if (!ref_ready) return -1;
  nvp = strcmp(grid.uv_timestep_scheme, "3rd-order Adams-Bashforth") == 0 ? 1 : 2;
  ntp = nvp == 1 ? 3 : 1;
  if (f->u) memcpy(f->u, var.u.value, (size_t)nvp * Nelem3d * sizeof(double));
  if (f->v) memcpy(f->v, var.v.value, (size_t)nvp * Nelem3d * sizeof(double));
  if (f->dudt) memcpy(f->dudt, var.u.tendency, (size_t)ntp * Nelem3d * sizeof(double));
  if (f->dvdt) memcpy(f->dvdt, var.v.tendency, (size_t)ntp * Nelem3d * sizeof(double));
  cp3(f->hdry, var.hdry.value); cp3(f->theta, var.theta.value); cp3(f->p3, var.p3.value);
  cp3(f->h3, var.h3.value); cp3(f->p2, var.p2.value); cp3(f->theta2, var.theta2.value);
  cp3(f->t2, var.t2.value); cp3(f->t3, var.t3.value); cp3(f->rho2, var.rho2.value);
  cp3(f->rho3, var.rho3.value); cp3(f->exner3, var.exner3.value); cp3(f->gz3, var.gz3.value);
  cp3(f->mont3, var.mont3.value); cp3(f->heat3, var.heat3.value); cp3(f->pv3, var.pv3.value);
  cp3(f->ri2, var.ri2.value); cp3(f->div_uv3, var.div_uv3.value); cp3(f->w3, var.w3.value);
  cp3(f->dzdt3, var.dzdt3.value); cp3(f->u_spinup, var.u_spinup.value);
  if (f->gz_surface) memcpy(f->gz_surface, var.gz_surface.value, Nelem2d * sizeof(double));
  if (var.nu_turb.on) {
    cp3(f->nu_turb, var.nu_turb.value); cp3(f->diffusion_coef_uv, var.diffusion_coef_uv.value);
    cp3(f->diffusion_coef_theta, var.diffusion_coef_theta.value); cp3(f->diffusion_coef_mass, var.diffusion_coef_mass.value);
  }
  f->it_zero = IT_ZERO; f->it_minus1 = IT_MINUS1; f->it_minus2 = IT_MINUS2;
  f->itime = (int64_t)grid.itime;
  f->model_time = (int64_t)var.model_time;
  return 0;
}

/*
 * The reference's get_sounding(planet, p, "theta", &theta) (src/shared/epic_funcs_diag.c:3160-3290)
 * on a t_vs_p table -- ntp levels, pressures [Pa] and temperatures [K] bottom level first, as
 * read_t_vs_p stores them (src/shared/epic_funcs_io.c:4074-4088) -- at n pressures, for the
 * Held-Suarez planet with grid.press0 = press0.  get_sounding keeps its table in static storage,
 * so one table per process.
 */
int ref_sounding_theta(int ntp, const double *pdat, const double *tdat, double press0, int n, const double *pres, double *out) {
  int q;
  if (!planet) {
    planet = (planetspec *)malloc(sizeof(planetspec));
    *planet = held_suarez;
  }
  grid.press0 = press0;
  var.ntp = ntp;
  var.pdat = fvector(0, ntp - 1, "ref_harness");
  var.tdat = fvector(0, ntp - 1, "ref_harness");
  var.dtdat = fvector(0, ntp - 1, "ref_harness");
  for (q = 0; q < ntp; q++) { var.pdat[q] = pdat[q]; var.tdat[q] = tdat[q]; var.dtdat[q] = 0.; }
  for (q = 0; q < n; q++) get_sounding(planet, pres[q], "theta", out + q);
  return 0;
}

/* netCDF entry points referenced by src/shared/epic_funcs_io.c; the step never calls them. */
int nc_close(int a) { (void)a; return -1; }
int nc_create(const char *p, int m, int *id) { (void)p; (void)m; (void)id; return -1; }
int nc_def_dim(int a, const char *b, size_t c, int *d) { (void)a; (void)b; (void)c; (void)d; return -1; }
int nc_def_var(int a, const char *b, nc_type c, int d, const int *e, int *f) { (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; return -1; }
int nc_enddef(int a) { (void)a; return -1; }
int nc_get_att_double(int a, int b, const char *c, double *d) { (void)a; (void)b; (void)c; (void)d; return -1; }
int nc_get_att_int(int a, int b, const char *c, int *d) { (void)a; (void)b; (void)c; (void)d; return -1; }
int nc_get_att_text(int a, int b, const char *c, char *d) { (void)a; (void)b; (void)c; (void)d; return -1; }
int nc_get_vara_double(int a, int b, const size_t *c, const size_t *d, double *e) { (void)a; (void)b; (void)c; (void)d; (void)e; return -1; }
int nc_inq(int a, int *b, int *c, int *d, int *e) { (void)a; (void)b; (void)c; (void)d; (void)e; return -1; }
int nc_inq_attname(int a, int b, int c, char *d) { (void)a; (void)b; (void)c; (void)d; return -1; }
int nc_inq_atttype(int a, int b, const char *c, nc_type *d) { (void)a; (void)b; (void)c; (void)d; return -1; }
int nc_inq_varid(int a, const char *b, int *c) { (void)a; (void)b; (void)c; return -1; }
int nc_inq_varname(int a, int b, char *c) { (void)a; (void)b; (void)c; return -1; }
int nc_open(const char *a, int b, int *c) { (void)a; (void)b; (void)c; return -1; }
int nc_put_att_double(int a, int b, const char *c, nc_type d, size_t e, const double *f) { (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; return -1; }
int nc_put_att_int(int a, int b, const char *c, nc_type d, size_t e, const int *f) { (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; return -1; }
int nc_put_att_text(int a, int b, const char *c, size_t d, const char *e) { (void)a; (void)b; (void)c; (void)d; (void)e; return -1; }
int nc_put_var1_double(int a, int b, const size_t *c, const double *d) { (void)a; (void)b; (void)c; (void)d; return -1; }
int nc_put_vara_double(int a, int b, const size_t *c, const size_t *d, const double *e) { (void)a; (void)b; (void)c; (void)d; (void)e; return -1; }
int nc_redef(int a) { (void)a; return -1; }
const char *nc_strerror(int a) { (void)a; return "netCDF is not linked into the oracle harness"; }
