/*
 * CPU restatement of the reference EPIC Held-Suarez timestep() -- test infrastructure only.
 *
 * This is the oracle the GPU kernels are checked against.  It restates, in plain C with
 * the same floating-point operation order, the reference functions on the path of
 * timestep() (src/shared/epic_timestep.c:62-390) for the configuration the GPU library
 * supports (include/epic_gb300.h).  Each function in epic_port.c cites the reference
 * lines it follows.  Unlike the reference it keeps all state in a context struct, so
 * several models can live in one process.
 */
#ifndef EPIC_PORT_H
#define EPIC_PORT_H

#include "epic_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ep_model ep_model;

/* Stages of one step, in call order (used to compare kernels one reference function at a time). */
enum ep_stage {
  EP_ST_ZERO_TEND = 0,       /* memset of DUDT, DVDT(it_uv_tend)           epic_timestep.c:107-108 */
  EP_ST_SOURCE_SINK = 1,     /* source_sink                                 epic_funcs_diag.c:4704 */
  EP_ST_CALC_W = 2,          /* calc_w                                      epic_flux.c:123        */
  EP_ST_UV_CORE = 3,         /* uv_core                                     epic_timestep.c:628    */
  EP_ST_UV_DRAG = 4,         /* uv_drag                                     epic_timestep.c:1303   */
  EP_ST_SCALAR_HSUB = 5,     /* scalar_horizontal_subgrid                   epic_subgrid.c:207     */
  EP_ST_ADVECTION = 6,       /* advection                                   epic_flux.c:346        */
  EP_ST_PGRAD_VARS = 7,      /* store_pgrad_vars                            epic_funcs_diag.c:3595 */
  EP_ST_GZ_FILTER = 8,       /* filtered, monotone GZ copy                  epic_timestep.c:176-196 */
  EP_ST_FILTER_TEND = 9,     /* 3-D filter of DUDT, DVDT                    epic_timestep.c:204-205 */
  EP_ST_FILTER_MASS = 10,    /* 3-D filter of HDRY (+restore_mass), THETA   epic_timestep.c:210-222 */
  EP_ST_P2ETC_UPDATE = 11,   /* set_p2etc(UPDATE_THETA)                     epic_funcs_diag.c:3352 */
  EP_ST_UV_PGRAD = 12,       /* uv_pgrad_finite_volume                      epic_timestep.c:909    */
  EP_ST_DIV_DAMP = 13,       /* divergence_damping                          epic_subgrid.c:1792    */
  EP_ST_UV_UPDATE = 14,      /* AB3 / leapfrog update, index rotation        epic_timestep.c:242-281 */
  EP_ST_UV_HYPERVISC = 15,   /* hyperviscosity of U, V                      epic_timestep.c:296-299 */
  EP_ST_STORE_DIAG = 16,     /* store_diag                                  epic_funcs_diag.c:3963 */
  EP_ST_CALC_HEATING = 17,   /* calc_heating                                epic_funcs_diag.c:4793 */
  EP_ST_P2ETC_NOUPDATE = 18, /* set_p2etc(DONT_UPDATE_THETA)                epic_funcs_diag.c:3352 */
  EP_ST_COUNT = 19,
  /* the turbulence closure (epic_grid.turbulence on); with it, stage 5 adds NU_TURB's
   * hyperviscosity, stage 10 NU_TURB's 3-D filter and stage 16 set_diffusion_coef */
  EP_ST_TURB_SOURCE = 21,    /* source_sink_turb (source_sink_SA)           epic_subgrid.c:2434    */
  EP_ST_SCALAR_HDIFF = 22,   /* scalar_horizontal_diffusion                 epic_subgrid.c:275     */
  EP_ST_SCALAR_VDIFF = 23,   /* scalar_vertical_diffusion                   epic_subgrid.c:1273    */
  EP_ST_UV_HDIFF = 24,       /* uv_horizontal_diffusion                     epic_subgrid.c:1571    */
  EP_ST_UV_VDIFF = 25        /* uv_vertical_diffusion                       epic_subgrid.c:1940    */
};

ep_model  *ep_create(const epic_grid *g);
void       ep_destroy(ep_model *m);
int        ep_upload(ep_model *m, const epic_fields *f);
int        ep_download(ep_model *m, epic_fields *f);
int        ep_timestep(ep_model *m, int action);
int        ep_cfl_dt(ep_model *m, double *cfl);   /* cfl_dt; cfl (may be NULL) = the x, y, z limits */
int        ep_run(ep_model *m, int nsteps);
int        ep_stage(ep_model *m, int stage);
const char *ep_error(const ep_model *m);
/* Last error text of ep_create (which has no model to hold it). */
const char *ep_create_error(void);

#ifdef __cplusplus
}
#endif

#endif
