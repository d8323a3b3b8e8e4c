// Launchers of the step kernels (each returns 0; launch errors surface through cudaGetLastError).
#pragma once
#include <cuda_runtime.h>
#include "device_common.cuh"
#include "epic_gb300.h"

namespace epic {

// Which time plane of a wind array a kernel works on; the index itself lives in Ctl so that
// one captured graph serves every step.
enum PlaneSel { PL_NONE = 0, PL_UV = 1, PL_UV_DIS = 2, PL_UV_TEND = 3 };

__device__ __forceinline__ int plane_offset(const DevModel &M, int sel) {
  const Ctl *c = M.ctl;
  switch (sel) {
    case PL_UV: return c->it_uv * (int)M.n3;
    case PL_UV_DIS: return c->it_uv_dis * (int)M.n3;
    case PL_UV_TEND: return c->it_uv_tend * (int)M.n3;
    default: return 0;
  }
}

// Grid of a launch over every member of a batch: blockIdx.z selects the member (one member
// when the model is not a batch).
inline dim3 zg(dim3 g, const DevModel &M) {
  g.z = M.nbatch > 1 ? (unsigned)M.nbatch : 1u;
  return g;
}

// Launch the FP32 (mixed form) or FP64 instantiation of a kernel template over every member
// (the launcher's `M` sets the batch).
#define EPIC_LAUNCH_R(mixed, kern, grid, block, smem, stream, ...)                              \
  do {                                                                                          \
    if (mixed) kern<float><<<zg((grid), M), (block), (smem), (stream)>>>(__VA_ARGS__);          \
    else kern<double><<<zg((grid), M), (block), (smem), (stream)>>>(__VA_ARGS__);              \
  } while (0)

// k_filter.cu -- zonal filter (epic_adjust.c) and the zonal pass of hsu_advection.
// fp32: filter in FP32 (the mixed forms; on the tensor cores for ni a multiple of 128).
// shift (tensor-core path only): filter x - x(i=1) of each row and add x(i=1) back in binary64,
// for fields whose zonal variations are small beside their value (the geopotential).
// pads_set: an in-place call whose rows 0..nj(+1) already carry their periodic pads (the
// tensor-core path then touches the filtered rows only).
int launch_filter_planes(const DevModel &M, const double *src, int src_sel, double *dst, int k0, int nplanes, int vgrid, cudaStream_t s,
                         int fp32 = 0, int shift = 0, int pads_set = 0);
int launch_varz_filter(const DevModel &M, double *buff, int sel, int index, int kstart, int kend, cudaStream_t s);
int launch_hsu_zonal(const DevModel &M, double *buff, int kind, int kstart, cudaStream_t s);
int filter_kernels_init(int ni);
// k_filter_gemm.cu -- the plane filter as a tcgen05 (3xTF32) operator product, mixed form
bool filter_gemm_usable(const DevModel &M);
int launch_filter_planes_gemm(const DevModel &M, const double *src, int src_sel, double *dst, int k0, int nplanes, int vgrid, cudaStream_t s,
                              int shift = 0);
int filter_gemm_init(int ni);

// k_column_acc.cu -- set_p2etc and store_pgrad_vars (column part) of the mixed form, with the
// quantities feeding the pressure gradient in double-float.
__global__ void k_set_p2etc_acc(DevModel M, int update_theta, int layers);
__global__ void k_pgrad_vars_column_acc(DevModel M);
__global__ void k_gz3_column_acc(DevModel M);   // GZ3 alone (the call before the filtered-GZ copy)
__global__ void k_pgrad_vars_column_acc_h2(DevModel M);   // the two above with hydrogen thermodynamics
__global__ void k_gz3_column_acc_h2(DevModel M);
int column_acc_kernels_init();
void fill_filter_kernels(int ni, int nj, const double *hl_h, const double *hl_pv, long long iadim, float *fh, float *fv);
bool filter_operator_wanted(const epic_grid &g, int precision);
size_t filter_operator_bytes(const epic_grid &g);
int filter_operator_create(const epic_grid &g, const double *hl_h, const double *hl_pv, long long iadim, cudaStream_t s, DevModel &d,
                           void **mem, uint64_t *hash, const char **why);
void filter_operator_release(void *mem);
size_t twiddle_doubles(int ni);
void fill_twiddles(int ni, double *tw);

// k_column.cu -- vertical (column) work
int launch_source_sink(const DevModel &M, cudaStream_t s);
// with_source_sink: source_sink first, in the same kernel (the step calls the two in a row)
int launch_calc_w(const DevModel &M, cudaStream_t s, bool with_source_sink = false);
int launch_uv_drag(const DevModel &M, cudaStream_t s);
int launch_hsu_vertical(const DevModel &M, double *buff, int kind, cudaStream_t s);
int launch_restore_mass(const DevModel &M, cudaStream_t s);
// early: the calls inside advection (set_p2etc) and before the filtered-GZ copy
// (store_pgrad_vars), whose outputs but P3, HDRY and GZ3 stage 11 and stage 19 rewrite before
// anything reads them.  The mixed forms compute only those there (EPIC_PREC_MIXED with its
// double-float kernels, which also leave the interfaces' logarithms for store_pgrad_vars:
// GZ3 places the 3-D filter's profiles, so it needs their accuracy; EPIC_PREC_MIXED_FAST with
// its FP32 ones).  The FP64 form writes everything in every call, as the reference does.
int launch_set_p2etc(const DevModel &M, int update_theta, cudaStream_t s, bool early = false);
int launch_store_pgrad_vars(const DevModel &M, cudaStream_t s, bool early = false);
int launch_gz_monotone(const DevModel &M, cudaStream_t s);
int launch_calc_heating(const DevModel &M, cudaStream_t s);
int launch_advection_prep(const DevModel &M, int phase, cudaStream_t s);
int column_kernels_init(int nk);

// k_stencil.cu -- horizontal stencils and the time update
int launch_copy_gz(const DevModel &M, cudaStream_t s);
int launch_zero_tend(const DevModel &M, cudaStream_t s);
int launch_uv_core(const DevModel &M, cudaStream_t s);
int launch_uv_pgrad(const DevModel &M, cudaStream_t s);
int launch_hsu_meridional(const DevModel &M, double *buff, int kind, cudaStream_t s);
// akima_advection (epic_flux.c:1502-1940), the other advection scheme: vertical (k_column.cu),
// meridional (k_stencil.cu) and zonal (k_filter.cu) passes, arguments as their Hsu counterparts
int launch_akima_vertical(const DevModel &M, double *buff, int kind, cudaStream_t s);
int launch_akima_meridional(const DevModel &M, double *buff, int kind, cudaStream_t s);
int launch_akima_zonal(const DevModel &M, double *buff, int kind, int kstart, cudaStream_t s);
int launch_meridional_hyperviscosity(const DevModel &M, int index, double *var, int sel, cudaStream_t s);
int launch_zonal_hyperviscosity(const DevModel &M, int index, double *var, int sel, cudaStream_t s);
int launch_divergence_damping(const DevModel &M, cudaStream_t s);
int launch_uv_update(const DevModel &M, cudaStream_t s);
int launch_store_diag(const DevModel &M, cudaStream_t s);
int launch_itime_advance(const DevModel &M, cudaStream_t s);
int launch_set_itime(const DevModel &M, long long itime, cudaStream_t s);

// k_turb.cu -- the Spalart-Allmaras DES turbulence closure (FP64 form): source_sink_turb,
// scalar_horizontal_diffusion (with its set_p2etc), scalar_vertical_diffusion (with its
// set_p2etc), uv_horizontal_diffusion, uv_vertical_diffusion, set_diffusion_coef, and
// restore_mass(NU_TURB_INDEX); scratch work0..3 and the model's turbulence arrays
int launch_source_sink_turb(const DevModel &M, cudaStream_t s);
int launch_scalar_hdiff(const DevModel &M, cudaStream_t s);
int launch_scalar_vdiff(const DevModel &M, cudaStream_t s);
int launch_uv_hdiff(const DevModel &M, cudaStream_t s);
int launch_uv_vdiff(const DevModel &M, cudaStream_t s);
int launch_set_diffusion_coef(const DevModel &M, cudaStream_t s);
int launch_restore_nu(const DevModel &M, cudaStream_t s);
// cfl_dt's three limits as the bits of positive binary64 values, minimised into lim[0..2]
// (x, y, z), which the caller sets to DBL_MAX's bits first
int launch_cfl_dt(const DevModel &M, unsigned long long *lim, cudaStream_t s);

}  // namespace epic
