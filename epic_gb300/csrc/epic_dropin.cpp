// The drop-in step with the reference's calling convention.
//
// The reference's timestep(planet, action, Buff2D) (src/shared/epic_timestep.c:62) works on the
// globals `grid` and `var`; its first call allocates (:88-101) and its callees keep static state,
// so a process runs one model.  The driver loop (src/shared/epic_main.c:336-427) owns grid.itime
// and advances it after every call, and reads the host `var` whenever it saves.  These entry
// points give a timestep() wrapper compiled with the reference's headers
// (epic_gb300/dropin/epic_timestep_gb300.c) exactly that behaviour over the device model:
//
//   * the first call creates the model on the current device and uploads the host state;
//   * every call first sets the device's itime to the driver's grid.itime (store_pgrad_vars
//     tests grid.itime > 1 for DZDT3, epic_funcs_diag.c:3666,3901), then runs the step (graph
//     replay) or the synchronising call;
//   * in mirror mode the state is copied back into the host arrays after every call, so an
//     unchanged driver sees a current `var`; in resident mode the host arrays are stale until
//     epic_dropin_sync_to_host;
//   * the first model error is kept: later calls return it without stepping, as the reference's
//     epic_error() would have ended the run.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include "epic_gb300.h"

namespace {

std::mutex g_mu;
epic_model *g_model = nullptr;
int g_mode = EPIC_DROPIN_MIRROR;
int g_status = EPIC_OK;
std::string g_message;

int fail(int rc) {
  if (g_status == EPIC_OK) {
    g_status = rc;
    g_message = epic_last_error();
  }
  return rc;
}

}  // namespace

extern "C" int epic_dropin_timestep(const epic_grid *grid, epic_fields *f, int32_t precision, int32_t mode, int32_t action,
                                    int64_t itime) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!grid || !f) return EPIC_ERR_ARG;
  if (g_status != EPIC_OK) return g_status;
  if (action != EPIC_STEP_PROGS_AND_SYNC_DIAGS && action != EPIC_SYNC_DIAGS_ONLY) {
    g_message = "timestep: unrecognized action";
    return g_status = EPIC_ERR_ARG;
  }
  int rc;
  if (!g_model) {
    if (mode != EPIC_DROPIN_MIRROR && mode != EPIC_DROPIN_RESIDENT) {
      g_message = "timestep: unknown drop-in mode";
      return g_status = EPIC_ERR_ARG;
    }
    g_mode = mode;
    if ((rc = epic_model_create(grid, precision, &g_model))) return fail(rc);
    if ((rc = epic_model_upload(g_model, f))) return fail(rc);
  }
  if ((rc = epic_model_set_itime(g_model, itime))) return fail(rc);
  rc = action == EPIC_STEP_PROGS_AND_SYNC_DIAGS ? epic_model_run(g_model, 1) : epic_model_timestep(g_model, EPIC_SYNC_DIAGS_ONLY);
  if (rc) return fail(rc);
  rc = g_mode == EPIC_DROPIN_MIRROR ? epic_model_download(g_model, f) : epic_model_sync(g_model);
  if (rc) return fail(rc);
  return EPIC_OK;
}

extern "C" int epic_dropin_sync_to_host(epic_fields *f) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!f) return EPIC_ERR_ARG;
  if (!g_model) {
    g_message = "epic_dropin_sync_to_host: no model yet (timestep() has not been called)";
    return EPIC_ERR_STATE;
  }
  const int rc = epic_model_download(g_model, f);
  return rc ? fail(rc) : EPIC_OK;
}

extern "C" int epic_dropin_status(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_status == EPIC_OK && g_model) {
    const int rc = epic_model_sync(g_model);
    if (rc) fail(rc);
  }
  return g_status;
}

extern "C" const char *epic_dropin_message(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  return g_message.c_str();
}

extern "C" void epic_dropin_release(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_model) epic_model_destroy(g_model);
  g_model = nullptr;
  g_status = EPIC_OK;
  g_message.clear();
  g_mode = EPIC_DROPIN_MIRROR;
}
