// Shared host-side helpers: error reporting, the reference array layout, viscosity limits.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>

namespace epic {

// Thread-local text of the last error (epic_last_error()).
inline char *error_buffer() {
  static thread_local char buf[512] = {0};
  return buf;
}

inline int set_error(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(error_buffer(), 512, fmt, ap);
  va_end(ap);
  return code;
}

// Reference layout X(k,j,i) = base[i + j*Iadim + k*Nelem2d - Shift3d] with Ishift = 0,
// Jshift = -1, Kshift = 0 (make_arrays, src/shared/epic_funcs_diag.c:660-670), i.e.
// base[i + (j+1)*Iadim + k*Nelem2d], Iadim = ni+2, Jadim = nj+3, Kadim = nk+2.
struct Layout {
  int ni, nj, nk;
  int iadim, jadim, kadim;
  int64_t n2, n3;
  Layout(int ni_, int nj_, int nk_)
      : ni(ni_), nj(nj_), nk(nk_), iadim(ni_ + 2), jadim(nj_ + 3), kadim(nk_ + 2),
        n2((int64_t)(ni_ + 2) * (nj_ + 3)), n3((int64_t)(ni_ + 2) * (nj_ + 3) * (nk_ + 2)) {}
  int64_t at(int k, int j, int i) const { return (int64_t)i + (int64_t)(j + 1) * iadim + (int64_t)k * n2; }
  int64_t at2(int j, int i) const { return (int64_t)i + (int64_t)(j + 1) * iadim; }
  // Zonal periodicity of a 3-D field for k = 0..nk+1, j = 0..nj+1 (bc_lateral THREEDIM,
  // src/single/s_epic_functions.c:69-82).
  void periodic3(double *a) const {
    for (int k = 0; k <= nk + 1; k++)
      for (int j = 0; j <= nj + 1; j++) {
        a[at(k, j, 0)] = a[at(k, j, ni)];
        a[at(k, j, ni + 1)] = a[at(k, j, 1)];
      }
  }
};

// set_max_nu, src/shared/epic_subgrid.c:82-158 (globe: dy0 from set_fmn).
inline void set_max_nu(int dt_s, double dy0, int uv_scheme, double max_nu[9]) {
  const double dt = (double)dt_s;
  const double dy2 = dy0 * dy0;
  for (int i = 0; i < 9; i++) max_nu[i] = 0.;
  if (uv_scheme == 0) {
    max_nu[0] = (1. / 3.) / dt;
    max_nu[2] = (dy2 / 30.) / dt;
    max_nu[4] = (dy2 / 240.) * (dy2 / dt);
    max_nu[6] = (dy2 / 800.) * (dy2 / dt) * dy2;
    max_nu[8] = (dy2 / 2400.) * (dy2 / dt) * dy2 * dy2;
  } else {
    max_nu[0] = .5 / dt;
    max_nu[2] = dy2 / (8. * dt);
    max_nu[4] = max_nu[2] * dy2 / 8.;
    max_nu[6] = max_nu[4] * dy2 / 8.;
    max_nu[8] = max_nu[6] * dy2 / 8.;
  }
}

}  // namespace epic
