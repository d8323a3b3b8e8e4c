/*
 * epic_gb300.h -- C ABI of the GB300 dynamical core for EPIC's single-processor timestep().
 *
 * The reference entry point this library replaces is
 *
 *     void timestep(planetspec *planet, int action, EPIC_FLOAT **Buff2D);
 *         include/epic.h:654-656, defined at src/shared/epic_timestep.c:62
 *
 * which reads the globals `grid` (gridspec, include/epic_datatypes.h:279-394), `planet`
 * (planetspec, :238-274) and `var` (variablespec, :550-627).  This ABI carries the same
 * information through plain structs of scalars and host pointers:
 *
 *   epic_grid    the gridspec/planetspec scalars and 1-D grid arrays timestep() reads,
 *   epic_fields  host views of the variablespec 3-D arrays in the reference memory layout
 *                X(k,j,i) = base[i + (j+1)*(ni+2) + k*(ni+2)*(nj+3)], k = 0..nk+1,
 *                j = -1..nj+1, i = 0..ni+1 (include/epic.h:407-449; wind time planes
 *                are consecutive blocks of (ni+2)*(nj+3)*(nk+2) doubles, :407-411).
 *
 * All arithmetic types are IEEE binary64 unless a function says otherwise.  Every function
 * returns 0 on success or a negative EPIC_ERR_* code; epic_last_error() gives the text.
 * Nothing here calls exit(): the reference's epic_error() (src/shared/epic_funcs_io.c:4872)
 * becomes an error code plus message.
 */
#ifndef EPIC_GB300_H
#define EPIC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* timestep() actions, include/epic.h:294-295 */
#define EPIC_STEP_PROGS_AND_SYNC_DIAGS 0
#define EPIC_SYNC_DIAGS_ONLY           1

/* grid.uv_timestep_scheme, src/shared/epic_timestep.c:242,262 */
#define EPIC_UV_AB3      0   /* "3rd-order Adams-Bashforth"   */
#define EPIC_UV_LEAPFROG 1   /* "Leapfrog (Asselin filtered)" */

/* var.theta/hdry.advection_scheme (src/shared/epic_flux.c:346-637) */
#define EPIC_ADV_HSU   0   /* "Predictor-corrector (Hsu, Konor, and Arakawa)" */
#define EPIC_ADV_AKIMA 1   /* "Monotonized, 4th-order centered (Akima)"       */

/* grid.turbulence_scheme (src/shared/epic_initial.c:153-155) and grid.diffusion_direction
 * (include/epic.h:290-292) */
#define EPIC_TURB_OFF    0   /* "off"                  */
#define EPIC_TURB_SA_DES 1   /* "Spalart-Allmaras DES" */
#define EPIC_DIFFUSION_HORIZONTAL_AND_VERTICAL 1
#define EPIC_DIFFUSION_JUST_HORIZONTAL         2
#define EPIC_DIFFUSION_JUST_VERTICAL           3

/* Precision forms accepted by epic_model_create(). */
#define EPIC_PREC_FP64  0    /* every kernel in binary64 (the drop-in form)                    */
#define EPIC_PREC_MIXED 1    /* stencils/advection/hyperviscosity/filter/physics in binary32;
                                the vertical pressure and geopotential integration (set_p2etc,
                                store_pgrad_vars), the pressure gradient, the updates and the
                                global sums in binary64 (libdevice log/exp/pow)                */
#define EPIC_PREC_MIXED_FAST 2   /* as EPIC_PREC_MIXED, with the vertical integration and the
                                pressure gradient in binary32 too (binary64 running sums and
                                updates kept): faster, larger error in the meridional wind     */

/* Error codes. */
#define EPIC_OK               0
#define EPIC_ERR_ARG         -1   /* bad argument or unsupported configuration              */
#define EPIC_ERR_CUDA        -2   /* CUDA runtime error                                     */
#define EPIC_ERR_NOMEM       -3   /* device or host allocation failed                       */
#define EPIC_ERR_MODEL       -4   /* a model check failed (the reference would epic_error)  */
#define EPIC_ERR_STATE       -5   /* call order violated (e.g. step before upload)          */

/*
 * Scalars and 1-D arrays of `grid` and `planet` that the step reads.  Array lengths follow
 * make_arrays() (src/shared/epic_funcs_diag.c:577-1074): half-level index jj = 0..2*(nj+1),
 * ii = 0..2*(ni+1), kk = 0..2*(nk+1).  Only the full globe (latbot = -90, lattop = 90) with
 * Held-Suarez physics (planet "held_suarez", x_h2 = 0, ideal gas, nq = 0, turbulence "off",
 * Hsu or Akima advection), with the terrestrial or the gas-giant lower boundary (gas_giant), is
 * supported; anything else returns EPIC_ERR_ARG.
 */
typedef struct epic_grid {
  int32_t ni, nj, nk;          /* grid.ni, grid.nj, grid.nk                                     */
  int32_t dt;                  /* grid.dt [s]                                                   */
  int32_t uv_scheme;           /* EPIC_UV_AB3 or EPIC_UV_LEAPFROG                               */
  int32_t k_sigma;             /* grid.k_sigma                                                  */
  int32_t k_sponge;            /* grid.k_sponge                                                 */
  int32_t newt_cool_on;        /* grid.newt_cool_on                                             */
  int32_t newt_cool_adjust;    /* grid.newt_cool_adjust                                         */
  int32_t drag_v;              /* grid.drag_v                                                   */
  int32_t drag_zonal_avg;      /* grid.drag_zonal_avg                                           */
  int32_t jtp;                 /* grid.jtp                                                      */
  int32_t advection_scheme;    /* EPIC_ADV_HSU or EPIC_ADV_AKIMA, for THETA and HDRY alike      */
  int32_t gas_giant;           /* planet->type "gas-giant": store_pgrad_vars sets GZ_SURFACE in
                                  gradient balance with the bottom layer's zonal-mean U (gz_from_u,
                                  zero at J = jtp); 0 for "terrestrial" (GZ_SURFACE is the terrain) */
  double  dln, dlt, dy0;       /* grid.dln, grid.dlt [deg], grid.dy0 [m]                        */
  double  globe_latbot, globe_lattop;
  double  press0;              /* grid.press0 [Pa]                                              */
  double  topo_scale, prandtl, tau_drag, nudiv_nondim;
  double  zeta0, zeta1, hybrid_alpha, sigma_sigma;
  double  nu[9];               /* grid.nu[0..MAX_NU_ORDER]                                      */
  double  re, rp;              /* planet->re, planet->rp [m]                                    */
  double  cp, rgas, kappa;     /* planet->cp, planet->rgas, planet->kappa                       */
  double  cpr;                 /* planet->cpr, low-temperature cp/rgas (thermo_setup)           */
  double  kinvisc;             /* planet->kinvisc                                               */
  double  lat0;                /* filter/taper latitude [deg]; the reference's LAT0 is 45      */
  double  hs_kf;               /* Held-Suarez PBL drag rate k_f [1/s]; the reference hard-codes
                                  HELD_SUAREZ_PBL_NU0 = 1/86400 (epic_timestep.c:1292)         */
  double  x_h2, x_he, x_3;     /* planet->x_h2, x_he, x_3: mole fractions of molecular hydrogen,
                                  helium and the rest.  x_h2 > 0 takes the reference's hydrogen
                                  thermodynamics (thermo_setup's ortho/para tables, normal
                                  hydrogen, fpara = 0.25: return_temp and return_enthalpy by table
                                  interpolation); cpr must then be thermo_setup's
                                  (2.5 x_h2 + 2.5 x_he + 3.5 x_3) / (x_h2 + x_he + x_3).  Every
                                  precision form (the tables are read in binary64).             */
  double  dynvisc;             /* planet->dynvisc [kg/m/s] (the turbulence closure's molecular
                                  viscosity of the winds)                                       */
  int32_t turbulence;          /* grid.turbulence_scheme: EPIC_TURB_OFF or EPIC_TURB_SA_DES
                                  (Spalart-Allmaras DES: source_sink_turb, the subgrid diffusion
                                  of THETA, NU_TURB and the winds, epic_subgrid.c).  FP64 form only */
  int32_t diffusion_direction; /* grid.diffusion_direction: EPIC_DIFFUSION_* (1 horizontal and
                                  vertical, 2 horizontal only, 3 vertical only)                 */
  int32_t stability_factor;    /* grid.stability_factor: 0 "off", 1 "Collins et al. (2004)"    */
  int32_t pad1;
  const double *lon;           /* [2*(ni+1)+1]                                                  */
  const double *lat, *rln, *rlt, *f, *m, *n, *mn, *g;   /* [2*(nj+1)+1]                         */
  const double *sigmatheta, *dsgth, *dsgth_inv;         /* [2*(nk+1)+1]                         */
  const double *h_min;         /* [nk+2]                                                        */
  const double *t_sponge_inv;  /* [k_sponge+1]                                                  */
} epic_grid;

/*
 * Host views of `var`.  AB3: u, v hold 1 value plane and dudt, dvdt 3 tendency planes;
 * leapfrog: u, v hold 2 value planes and dudt, dvdt 1 plane (make_arrays, epic_funcs_diag.c:686-711).
 * With nq = 0 the reference aliases P3 = PDRY3, H2 = HDRY, H3 = HDRY3 (:891-927); here p3
 * and h3 are the only copies.  Any pointer may be NULL on download to skip that field.
 */
typedef struct epic_fields {
  double *u, *v, *dudt, *dvdt;
  double *hdry, *theta;
  double *p3, *h3, *p2, *theta2, *t2, *t3, *rho2, *rho3, *exner3;
  double *gz3, *mont3, *heat3, *pv3, *ri2, *div_uv3, *w3, *dzdt3, *u_spinup;
  double *gz_surface;          /* 2-D: [(nj+3)*(ni+2)]                                          */
  int32_t it_zero, it_minus1, it_minus2;  /* IT_ZERO, IT_MINUS1, IT_MINUS2 (include/epic.h:303) */
  int32_t pad0;
  int64_t itime;               /* grid.itime                                                    */
  int64_t model_time;          /* var.model_time [s]                                            */
  /* The turbulence closure's arrays (read only when epic_grid.turbulence is on): NU_TURB, the
   * Spalart-Allmaras working viscosity on the layer interfaces (prognostic), and the eddy
   * diffusivities that store_diag's set_diffusion_coef leaves for the next step
   * (DIFFUSION_COEF_UV, _THETA, _MASS).  On upload a NULL diffusivity uploads zeros. */
  double *nu_turb, *diffusion_coef_uv, *diffusion_coef_theta, *diffusion_coef_mass;
} epic_fields;

typedef struct epic_model epic_model;

/*
 * Allocate device state for one grid on the current CUDA device and upload the grid
 * arrays (the first-call work of timestep(), epic_timestep.c:88-101, plus the static
 * initialisation blocks of zonal_filter, d2dy2 and the hyperviscosity routines).
 */
int  epic_model_create(const epic_grid *grid, int32_t precision, epic_model **out);
void epic_model_destroy(epic_model *m);

/* Copy host `var` into the device state (no kernel runs). */
int  epic_model_upload(epic_model *m, const epic_fields *f);

/*
 * timestep(planet, action, Buff2D), src/shared/epic_timestep.c:62-390, on the device state.
 * Asynchronous on the model's stream; errors found by kernels surface on the next
 * epic_model_sync() or download.
 */
int  epic_model_timestep(epic_model *m, int32_t action);

/*
 * nsteps calls of timestep(STEP_PROGS_AND_SYNC_DIAGS) with grid.itime advancing by one
 * after each, as the driver loop does (src/shared/epic_main.c:336-427).  Replays a captured
 * CUDA graph of one step when possible.
 */
int  epic_model_run(epic_model *m, int32_t nsteps);

/*
 * Test hook: enqueue one stage of the step (the stage numbering of oracle/epic_port.h:
 * 0 zero tendencies, 1 source_sink, 2 calc_w, 3 uv_core, 4 uv_drag, 5 scalar hyperviscosity,
 * 6 advection, 7 store_pgrad_vars, 8 filtered GZ, 9 3-D filter of DUDT/DVDT, 10 3-D filter of
 * HDRY/THETA, 11 set_p2etc(UPDATE_THETA), 12 uv_pgrad, 13 divergence damping, 14 u/v time
 * update, 15 u/v hyperviscosity, 16 store_diag, 17 calc_heating, 18 set_p2etc(DONT_UPDATE),
 * 19 store_pgrad_vars after stage 11 -- the call whose output the pressure gradient reads: the
 * same kernels as 7 in the FP64 form; in the mixed forms the full ones, while 6 and 7 compute
 * only what is read before stages 11 and 19 recompute the rest), 20 stages 1 and 2 in one kernel
 * (the step's form of them).
 * It has no counterpart in the reference, which only exposes the whole step.
 */
int  epic_model_run_stage(epic_model *m, int32_t stage);

/*
 * Set grid.itime on the device, in stream order, to the value a driver that owns it holds (the
 * reference's loop advances grid.itime after each timestep() call, src/shared/epic_main.c:424;
 * store_pgrad_vars reads it, epic_funcs_diag.c:3666,3901).  epic_model_run advances it by one
 * per step; epic_model_timestep leaves it unchanged.
 */
int  epic_model_set_itime(epic_model *m, int64_t itime);

/* Wait for queued work and report any device-side model error. */
int  epic_model_sync(epic_model *m);

/* Copy the device state back into host `var` (called before var_write()). */
int  epic_model_download(epic_model *m, epic_fields *f);

/*
 * Asynchronous form of the download for the epic.nc/extract.nc saves of the driver loop
 * (src/shared/epic_main.c:338-411): the state as it stands after the work already enqueued is
 * copied on the device, in stream order, and then to f's host arrays on a second stream while
 * later epic_model_run/timestep calls proceed.  f must stay valid (and should be pinned host
 * memory for the copy to overlap) until epic_model_snapshot_wait returns; one snapshot is in
 * flight per model (a second begin first completes the first).  The first call allocates a
 * device buffer of the state's size.  No counterpart in the reference.
 */
int  epic_model_snapshot_begin(epic_model *m, epic_fields *f);
int  epic_model_snapshot_wait(epic_model *m);

/*
 * cfl_dt(planet), src/shared/epic_funcs_diag.c:4884-5022, on the device state as the work already
 * enqueued leaves it: the largest time step [s] the vertical, meridional and zonal advection
 * allow (sound speed for the horizontal gravity waves; the zonal limit only equatorward of the
 * filter latitude), truncated to int -- what var_write() stores as grid.cfl_dt before a save
 * (src/shared/epic_funcs_io.c:1772).  cfl (may be NULL) receives the three limits before the
 * truncation: cflx, cfly, cflz.  Waits for the model's queued work.
 */
int  epic_model_cfl_dt(epic_model *m, int32_t *dt_out, double *cfl);

/*
 * End-to-end form of the drop-in: upload f, run nsteps (after a SYNC_DIAGS_ONLY call when
 * prime != 0), download into f.  This is what a reference-side timestep() wrapper does.
 */
int  epic_model_step_host(epic_model *m, epic_fields *f, int32_t prime, int32_t nsteps);

/* Device stream the model runs on (a cudaStream_t), for callers that interleave work. */
void *epic_model_stream(epic_model *m);

/* Kernel launches in one step of epic_model_run (its captured graph), the step counter
 * included; -1 before the first epic_model_run.  No counterpart in the reference. */
int32_t epic_model_kernels_per_step(const epic_model *m);

/* Bytes of device memory the model holds. */
int64_t epic_model_device_bytes(const epic_model *m);

/* The CUDA device the model was created on (current at epic_model_create); -1 for NULL.  Its
 * state, stream and kernels stay there.  No counterpart in the reference. */
int32_t epic_model_device(const epic_model *m);

/* Bytes of device memory epic_model_create would take for this grid and precision form (-1 for
 * a bad grid): the pool, plus for the mixed forms at ni a multiple of 128 the tensor-core
 * filter's operator tiles (ni/32 x 32 KB per filtered row); for admission by memory budget.  No
 * counterpart in the reference. */
int64_t epic_model_bytes(const epic_grid *grid, int32_t precision);

/*
 * The 3-D zonal filter of the mass variables (stage 10 above: zonal_filter(HDRY_INDEX, ...,
 * THREEDIM), restore_mass, zonal_filter(THETA_INDEX, ..., THREEDIM); epic_timestep.c:207-222),
 * with its per-row PCHIP profile tables held in a fixed device array of the library instead of
 * the model's own scratch.  It allocates nothing: no cudaMalloc/cudaFree and no library call
 * that allocates.  No counterpart in the reference.
 *
 * Limit: (nj+3)*(nk+2) <= EPIC_NOALLOC_TABLE_ENTRIES; larger grids return EPIC_ERR_ARG.
 * The first call on a device resolves the array's address (cudaGetSymbolAddress with the
 * model's device current) and keeps it for the life of the process; make that first call before
 * any stream capture begins, and do not reset the device (cudaDeviceReset) while the library is
 * in use, which could move the array.  Nothing in
 * the array needs to start at zero: every table entry is written before it is read in the same
 * call.  The array is shared by every model on the device, so calls must not overlap: issue
 * them on one stream, or synchronise between them.  Results equal epic_model_run_stage(m, 10).
 */
#define EPIC_NOALLOC_TABLE_ENTRIES 16384
int  epic_model_filter_mass_noalloc(epic_model *m);

/*
 * Batches (no counterpart in the reference, which runs one model per process).  A batch is a
 * view over n models from epic_model_create that share sizes, scheme, precision form,
 * k_sigma, dt and viscosities (members may differ in state and in the drag rate hs_kf); every
 * kernel of a step is launched once for all members.  Member state stays in the member models:
 * upload and download through them (after epic_batch_sync).  The batch does not own them.
 * Members must live on one device (epic_model_device); the batch's stream is created there.
 */
typedef struct epic_batch epic_batch;
int  epic_batch_create(epic_model *const *members, int32_t n, epic_batch **out);
void epic_batch_destroy(epic_batch *b);
int  epic_batch_timestep(epic_batch *b, int32_t action);   /* every member, as epic_model_timestep */
int  epic_batch_run(epic_batch *b, int32_t nsteps);        /* every member, as epic_model_run */
int  epic_batch_run_stage(epic_batch *b, int32_t stage);   /* test/timing hook, as epic_model_run_stage */
/* every member's upload / download (f[i] for member i) with one synchronisation */
int  epic_batch_upload(epic_batch *b, const epic_fields *const *f);
int  epic_batch_download(epic_batch *b, epic_fields *const *f);
/*
 * nsteps end-to-end steps with host-resident state: each step uploads every member from f[i],
 * steps it and downloads it into f[i] (as epic_model_step_host does for one model).  The members
 * are split into `groups` sub-batches on their own streams so that copies overlap kernels, and a
 * group's next step starts as soon as its own download is done (no drain between steps; the
 * host's time-plane indices and itime in f[i] are updated once, after the last step).  f should
 * be pinned host memory; when a member's 3-D arrays sit back to back in the order u, v, dudt,
 * dvdt, hdry, theta, p3, h3, p2, theta2, t2, t3, rho2, rho3, exner3, gz3, mont3, heat3, pv3, ri2,
 * div_uv3, w3, dzdt3, u_spinup, its state moves with one copy each way (any layout works).
 * io = EPIC_IO_ALL moves every array (and GZ_SURFACE) each way; EPIC_IO_STATE moves the
 * prognostic arrays u, v, dudt, dvdt, hdry, theta only -- what a step advances and carries from
 * the step before -- and leaves the diagnostic fields on the device, which recomputes them from
 * those (every member must have been uploaded; epic_batch_download fetches the diagnostics when
 * they are wanted, e.g. before a save).
 */
#define EPIC_IO_ALL   0
#define EPIC_IO_STATE 1
int  epic_batch_step_host(epic_batch *b, epic_fields *const *f, int32_t groups, int32_t nsteps, int32_t io);
int  epic_batch_sync(epic_batch *b);                       /* wait; first member error, if any */
int  epic_batch_query(epic_batch *b);   /* 1: work queued on the batch finished, 0: still running */
void *epic_batch_stream(epic_batch *b);
int32_t epic_batch_kernels_per_step(const epic_batch *b);

/*
 * Launch-shape autotuning (no counterpart in the reference).  A tuning table holds one entry per
 * kernel group, 0 keeping the built-in choice: entries 0-8 are block sizes (uv_core, pgrad, Hsu
 * meridional, hyperviscosity, diagnostics, update, column, pointwise, row filter), entry 9 the
 * form of the meridional Hsu pass (1 one fused march per column of cells, 2 four passes over every
 * cell; by default the fused march once its threads fill the GPU).  Tuned kernels are pointwise,
 * per row or per column, and the two Hsu forms give the same bits, so a table changes no result.  epic_batch_autotune times whole steps
 * of the batch for each candidate (trial_steps timed steps each) and keeps the fastest; the
 * members must hold a primed state (after epic_batch_timestep(b, EPIC_SYNC_DIAGS_ONLY)), and the
 * trial steps advance it, so tune before uploading the state a run starts from.
 */
#define EPIC_TUNE_GROUPS 10
int  epic_batch_autotune(epic_batch *b, int32_t trial_steps, int32_t *table_out);
int  epic_batch_set_tuning(epic_batch *b, const int32_t *table);
int  epic_model_set_tuning(epic_model *m, const int32_t *table);

/* Text of the last error on this thread. */
const char *epic_last_error(void);

/*
 * The drop-in step, with the calling convention of the reference's
 *     void timestep(planetspec *planet, int action, EPIC_FLOAT **Buff2D)
 * (include/epic.h:654-656, src/shared/epic_timestep.c:62): one model per process, created by the
 * first call, as the reference's first call allocates and its callees keep static state.  A
 * timestep() wrapper compiled with the reference's headers (epic_gb300/dropin/epic_timestep_gb300.c)
 * fills *grid and *f from the globals `grid`, `planet` and `var` and calls these.
 *
 * epic_dropin_timestep: the first call creates the model from *grid on the current device
 * (precision form as for epic_model_create) and uploads *f.  Every call sets the device's itime
 * to `itime` (the driver's grid.itime, which the driver advances after the call) and runs
 * timestep(action): one step, or the synchronising call.  Mode EPIC_DROPIN_MIRROR (fixed by the
 * first call) then copies the state back into *f, time-plane indices, itime and model_time
 * included, so that the host arrays are current after every call and an unchanged driver works;
 * EPIC_DROPIN_RESIDENT leaves the host arrays stale until epic_dropin_sync_to_host (the driver
 * calls it before var_write).  The first error is kept: later calls return it without stepping
 * (the reference's epic_error() ends the run, src/shared/epic_funcs_io.c:4872).
 *
 * epic_dropin_status: EPIC_OK, or the code of the first error, after waiting for queued work
 * (the reference's epic_error text is epic_dropin_message()).  epic_dropin_release frees the
 * model; the next epic_dropin_timestep starts over.
 */
#define EPIC_DROPIN_MIRROR   0
#define EPIC_DROPIN_RESIDENT 1
int  epic_dropin_timestep(const epic_grid *grid, epic_fields *f, int32_t precision, int32_t mode, int32_t action, int64_t itime);
int  epic_dropin_sync_to_host(epic_fields *f);
int  epic_dropin_status(void);
const char *epic_dropin_message(void);
void epic_dropin_release(void);

/*
 * Host-side synthetic Held-Suarez set-up (no GPU needed).  These restate the grid
 * construction of the reference's `initial` program for planet "held_suarez"
 * (src/shared/epic_initial.c:1140-2006) and the geometry routines set_lonlat, set_fmn,
 * set_gravity, set_dsgth (src/shared/epic_funcs_diag.c:1324-1686), with the temperature
 * sounding replaced by the analytic Held-Suarez equilibrium profile at 45 degrees.
 *
 * epic_hs_grid_build fills *grid; every array pointer in *grid must already point at
 * caller-owned storage of the lengths documented in epic_grid (lon, lat, ... h_min,
 * t_sponge_inv).  p_ref and theta_ref (length 2*(nk+1)+1) receive grid.p_ref/theta_ref.
 */
typedef struct epic_hs_params {
  int32_t ni, nj, nk, dt;
  int32_t uv_scheme;
  int32_t advection_scheme;    /* EPIC_ADV_HSU (the Held-Suarez default) or EPIC_ADV_AKIMA */
  double  ptop, pbot, p_sigma; /* [Pa]; reference HS defaults 10, 1e5, 9e4 */
  double  nu_nondim[9];        /* grid.nu_nondim; HS runs use nu[4] = 0.5, the rest 0 */
  double  nudiv_nondim;
  double  lat0;                /* 45 reproduces the reference's LAT0 */
  /* the sounding the vertical grid (sigmatheta) and the initial column follow */
  int32_t profile;             /* EPIC_PROFILE_HS_EQ or EPIC_PROFILE_N2 */
  int32_t pad1;
  double  n2;                  /* EPIC_PROFILE_N2: buoyancy frequency squared [s^-2] below the ... */
  double  theta_surface;       /* ... isothermal layer: theta = theta_surface at pbot [K] ... */
  double  t_iso;               /* ... and T = max(t_iso, T_N2(p)) [K] */
  /* EPIC_PROFILE_TABLE: a temperature sounding as the reference reads it from t_vs_p.<planet>
   * (read_t_vs_p, src/shared/epic_funcs_io.c:4027-4088): table_n levels of pressure [Pa] and
   * temperature [K], in either order of pressure; the arrays are read during the call only */
  const double *table_p, *table_t;
  int32_t table_n, pad2;
} epic_hs_params;

/* Soundings: the Held-Suarez equilibrium column at 45 degrees (temp_eq); a column of constant
 * buoyancy frequency N^2 from theta_surface at pbot, isothermal at t_iso above the level where
 * it reaches that temperature (the stable jet sounding); or a table, interpolated as the
 * reference's get_sounding (src/shared/epic_funcs_diag.c:3160-3290) does: theta of the table's
 * levels, ironed from the top down so that it never decreases upward, by monotone cubic Hermite
 * interpolation (PCHIP) in -ln p, the table's bottom value below its lowest level. */
#define EPIC_PROFILE_HS_EQ 0
#define EPIC_PROFILE_N2    1
#define EPIC_PROFILE_TABLE 2

int epic_hs_grid_build(const epic_hs_params *p, epic_grid *grid, double *p_ref, double *theta_ref);

/*
 * Seeded initial state: rest (U = V = 0), P3 on the sigmatheta interfaces of the sounding
 * (p->profile), horizontally uniform, theta noise N(0, noise_k^2) in the pure-sigma region
 * (k >= k_sigma-1), HDRY = get_h(P3), GZ_SURFACE = 0, U_SPINUP = 0, and the first-step flags of
 * the chosen time scheme (src/shared/epic_initial.c:1301-1330).  Fields f must point at zeroed
 * storage.
 */
int epic_hs_initial_state(const epic_grid *grid, const epic_hs_params *p, uint64_t seed, double noise_k,
                          epic_fields *f);

/* Zonal jets: u(lat) = sum over njets of amp_i exp(-((lat - lat_i)/width_i)^2), the amplitudes,
 * centres and widths drawn uniformly from the ranges below (seeded), constant with height. */
typedef struct epic_jet_params {
  int32_t njets;
  int32_t pad0;
  double  amp_min, amp_max;       /* [m/s] */
  double  lat_min, lat_max;       /* jet centres [deg] */
  double  width_min, width_max;   /* [deg] */
  double  vort_frac;              /* rms relative vorticity of the seeded perturbation, as a
                                     fraction of the jets' */
} epic_jet_params;

/*
 * Seeded jet state, no counterpart in the reference (its jet runs start from `initial`'s
 * gradient-balance integration, src/shared/epic_funcs_init.c:1294-1342): the zonal jets of
 * *jet on every layer, theta horizontally uniform on pressure surfaces (the sounding of
 * p->profile), and each row's bottom pressure set so that the geopotential on pressure
 * surfaces balances the jets, d(phi)/dy = -(f + u tan(lat)/a) u, integrated from the south
 * row with the row-mean bottom pressure p->pbot; P3 on the sigmatheta interfaces of each row's
 * column, HDRY = get_h(P3); plus a seeded non-divergent wind perturbation (white streamfunction
 * noise at the vorticity points, the same on every layer) with vort_frac of the jets' rms
 * vorticity.  Grid built by epic_hs_grid_build with the same p.  Fields f must point at zeroed
 * storage.
 */
int epic_jet_initial_state(const epic_grid *grid, const epic_hs_params *p, const epic_jet_params *jet, uint64_t seed,
                           epic_fields *f);

#ifdef __cplusplus
}
#endif

#endif /* EPIC_GB300_H */
