// High-latitude zonal filter kernels (the reference's zonal_filter, src/shared/epic_adjust.c:102-480).
//
// The reference filters one latitude row at a time: realft() forward, multiply wavenumber m
// by HIGH_LAT(J,m+1), realft() inverse and scale by 2/ni (epic_adjust.c:412-456).  That is the
// real symmetric circulant operator F_J = IDFT diag(h_J) DFT.  Here one thread block owns one
// row: the ni reals are packed as ni/2 complex points, transformed by an in-shared-memory
// radix-2 FFT, split into the ni/2+1 real-input spectrum, scaled by h_J, and transformed back.
// Rows equatorward of lat0 are passed through unchanged.
#include "device_common.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

struct Cplx { double re, im; };
__device__ __forceinline__ Cplx cmul(Cplx a, Cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// Shared-memory workspace of one row filter: z[N], X[N+1], tw[N/2 + N+1].
struct FilterSmem {
  Cplx *z, *X, *w, *t;
};

__device__ __forceinline__ FilterSmem carve_filter(double *base, int ni) {
  const int N = ni / 2;
  FilterSmem s;
  s.z = reinterpret_cast<Cplx *>(base);
  s.X = s.z + N;
  s.w = s.X + (N + 1);
  s.t = s.w + N / 2;
  return s;
}
__host__ __device__ inline size_t filter_smem_doubles(int ni) {
  const int N = ni / 2;
  return 2 * ((size_t)N + (N + 1) + N / 2 + (N + 1));
}

__device__ __forceinline__ void load_twiddles(const DevModel &M, FilterSmem &s) {
  const int N = M.ni / 2;
  const Cplx *g = reinterpret_cast<const Cplx *>(M.tw);
  for (int k = threadIdx.x; k < N / 2 + N + 1; k += blockDim.x) s.w[k] = g[k];
}

// Radix-2 decimation-in-time FFT of z[0..N-1] (already in bit-reversed order).
// sign = -1 uses W = exp(-2 pi i/N) (forward), +1 its conjugate.
__device__ __forceinline__ void fft_stages(FilterSmem &s, int N, int lg, int sign) {
  for (int st = 1; st <= lg; st++) {
    const int half = 1 << (st - 1);
    for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
      const int pos = b & (half - 1);
      const int i0 = ((b >> (st - 1)) << st) + pos;
      const int i1 = i0 + half;
      Cplx w = s.w[pos << (lg - st)];
      if (sign > 0) w.im = -w.im;
      const Cplx tv = cmul(w, s.z[i1]);
      const Cplx a = s.z[i0];
      s.z[i1] = {a.re - tv.re, a.im - tv.im};
      s.z[i0] = {a.re + tv.re, a.im + tv.im};
    }
    __syncthreads();
  }
}

// Filter row x[1..ni] (1-based, shared memory) in place with weights h(m) = hl[rowbase + m + 1].
// Every thread of the block must call this; it synchronises internally.
__device__ void filter_row_smem(const DevModel &M, double *x, const double *hl, long long rowbase, FilterSmem &s) {
  const int ni = M.ni, N = ni / 2;
  const int lg = 31 - __clz(N);
  // pack and bit-reverse
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const int r = (int)(__brev((unsigned)k) >> (32 - lg));
    s.z[r] = {x[2 * k + 1], x[2 * k + 2]};
  }
  __syncthreads();
  fft_stages(s, N, lg, -1);
  // split into the real-input spectrum X_m, m = 0..N, and apply the filter weights
  for (int m = threadIdx.x; m <= N; m += blockDim.x) {
    const Cplx zm = s.z[m % N];
    const Cplx zc = s.z[(N - m) % N];
    const Cplx e = {0.5 * (zm.re + zc.re), 0.5 * (zm.im - zc.im)};
    const Cplx o = {0.5 * (zm.im + zc.im), -0.5 * (zm.re - zc.re)};
    const Cplx tm = s.t[m];
    const Cplx to = cmul(tm, o);
    const double h = hl[rowbase + m + 1];
    s.X[m] = {h * (e.re + to.re), h * (e.im + to.im)};
  }
  __syncthreads();
  // merge back into a half-length spectrum and bit-reverse
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    const Cplx ym = s.X[m];
    const Cplx yc = {s.X[N - m].re, -s.X[N - m].im};
    const Cplx e = {0.5 * (ym.re + yc.re), 0.5 * (ym.im + yc.im)};
    Cplx o = {0.5 * (ym.re - yc.re), 0.5 * (ym.im - yc.im)};
    const Cplx tc = {s.t[m].re, -s.t[m].im};
    o = cmul(o, tc);
    const int r = (int)(__brev((unsigned)m) >> (32 - lg));
    s.z[r] = {e.re - o.im, e.im + o.re};
  }
  __syncthreads();
  fft_stages(s, N, lg, +1);
  const double inv = 1.0 / (double)N;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    x[2 * k + 1] = s.z[k].re * inv;
    x[2 * k + 2] = s.z[k].im * inv;
  }
  __syncthreads();
}

__device__ __forceinline__ bool row_is_filtered(const DevModel &M, int j, int vgrid) {
  return fabs(M.lat[vgrid ? 2 * j : 2 * j + 1]) >= M.lat0;
}

// zonal_filter(index, plane, NULL, TWODIM) of planes k0..k0+gridDim.y-1, from src into dst
// (dst may equal src).  Block = one row j in -1..nj+1; rows outside the filtered set are
// copied; rows 0..nj+1 get periodic pads (bc_lateral).
__global__ void k_filter_planes(DevModel M, const double *src, int src_sel, double *dst, int k0, int vgrid) {
  extern __shared__ double sm[];
  src += plane_offset(M, src_sel);
  const int j = (int)blockIdx.x - 1;
  const int k = k0 + (int)blockIdx.y;
  const long long base = M.at(k, j, 0);
  double *x = sm;
  FilterSmem fs = carve_filter(sm + (M.ni + 2), M.ni);
  const bool valid = vgrid ? (j >= 1 && j <= M.nj) : (j >= 0 && j <= M.nj);
  const bool filt = valid && row_is_filtered(M, j, vgrid);
  if (!filt) {
    if (src != dst)
      for (int i = threadIdx.x; i <= M.ni + 1; i += blockDim.x) dst[base + i] = src[base + i];
    __syncthreads();
    if (j >= 0 && threadIdx.x == 0) {
      dst[base] = dst[base + M.ni];
      dst[base + M.ni + 1] = dst[base + 1];
    }
    return;
  }
  load_twiddles(M, fs);
  for (int i = threadIdx.x; i <= M.ni + 1; i += blockDim.x) x[i] = src[base + i];
  __syncthreads();
  filter_row_smem(M, x, vgrid ? M.high_lat_pv : M.high_lat_h, M.at2(j, 0), fs);
  for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) write_with_pads(dst, M, base, i, x[i]);
}

// Per-latitude var(gz) profile at the column of lowest bottom GZ, the first half of the
// THREEDIM branch of zonal_filter (epic_adjust.c:266-395).  One thread per row j.
// index: 0 = U, 1 = V, 2 = HDRY (log), 3 = THETA.
__global__ void k_varz_tables(DevModel M, const double *buff, int sel, int index, int kstart, int kend) {
  buff += plane_offset(M, sel);
  const int jstart = index == 1 ? 1 : 0;
  const int j = jstart + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (j > M.nj) return;
  const double *gz = M.gz;
  const int K = M.nk;
  int imin = 1;
  double gzmin = DBL_MAX;
  for (int i = 1; i <= M.ni; i++) {
    const double v = gz[M.at(K, j, i)];
    if (v < gzmin) { imin = i; gzmin = v; }
  }
  const int i = imin;
  Trip *t = reinterpret_cast<Trip *>(M.ptable) + (long long)(j + 1) * (M.nk + 2);
  for (int k = kend; k >= kstart; k--) {
    const int kay = kend - k;
    double x;
    switch (index) {
      case 0: x = .5 * (gz[M.at(k, j, i)] + gz[M.at(k, j, i - 1)]); break;
      case 1: x = .5 * (gz[M.at(k, j, i)] + gz[M.at(k, j - 1, i)]); break;
      case 2: x = .5 * (gz[M.at(k, j, i)] + gz[M.at(k - 1, j, i)]); break;
      default: x = gz[M.at(k, j, i)]; break;
    }
    t[kay].x = x;
    t[kay].y = index == 2 ? log(buff[M.at(k, j, i)]) : buff[M.at(k, j, i)];
  }
  if (!spline_pchip(kend - kstart + 1, t)) flag_error(M.ctl, ERR_PCHIP_X, kstart, j, i, t[0].x);
}

// The rest of the THREEDIM zonal_filter: subtract var(gz), filter, add it back.
// Block = one row (k = kstart + blockIdx.y, j = jstart + blockIdx.x).
__global__ void k_varz_filter_rows(DevModel M, double *buff, int sel, int index, int kstart, int kend) {
  extern __shared__ double sm[];
  buff += plane_offset(M, sel);
  const int jstart = index == 1 ? 1 : 0;
  const int j = jstart + (int)blockIdx.x;
  const int k = kstart + (int)blockIdx.y;
  const int vgrid = index == 1;
  double *x = sm, *vz = sm + (M.ni + 2);
  FilterSmem fs = carve_filter(sm + 2 * (M.ni + 2), M.ni);
  const Trip *t = reinterpret_cast<const Trip *>(M.ptable) + (long long)(j + 1) * (M.nk + 2);
  const int n = kend - kstart + 1;
  const double *gz = M.gz;
  const long long base = M.at(k, j, 0);
  const bool filt = row_is_filtered(M, j, vgrid);
  if (filt) load_twiddles(M, fs);
  for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) {
    double gzz;
    switch (index) {
      case 0: gzz = .5 * (gz[M.at(k, j, i)] + gz[M.at(k, j, i - 1)]); break;
      case 1: gzz = .5 * (gz[M.at(k, j, i)] + gz[M.at(k, j - 1, i)]); break;
      case 2: gzz = .5 * (gz[M.at(k, j, i)] + gz[M.at(k - 1, j, i)]); break;
      default: gzz = gz[M.at(k, j, i)]; break;
    }
    double dgz;
    const int kay = find_place_in_table(n, t, gzz, &dgz);
    double v = splint_pchip(gzz, t + kay, dgz);
    if (index == 2) v = exp(v);
    vz[i] = v;
    x[i] = buff[base + i] - v;
  }
  __syncthreads();
  if (filt) filter_row_smem(M, x, vgrid ? M.high_lat_pv : M.high_lat_h, M.at2(j, 0), fs);
  for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) write_with_pads(buff, M, base, i, x[i] + vz[i]);
}

// Zonal pass of hsu_advection (epic_flux.c:1316-1484) for one row: the fluxes come from a
// zonally filtered copy of the row, the update goes to the unfiltered field.
// kind: 0 = interface variable (unity, THETA), 1 = HDRY (layer; u averaged to the layer).
__global__ void k_hsu_zonal(DevModel M, double *buff, int kind, int kstart) {
  extern __shared__ double sm[];
  const int ni = M.ni, W = ni + 2;
  const int j = (int)blockIdx.x;
  const int k = kstart + (int)blockIdx.y;
  double *a = sm, *um = a + W, *up = um + W, *ff = up + W, *ap = ff + W, *d1 = ap + W, *d2 = d1 + W, *aa = d2 + W;
  FilterSmem fs = carve_filter(aa + W, ni);
  const double ep = 1.e-10, DT = M.dt;
  const double a_min = kind == 1 ? M.h_min[k] : 0.;
  const long long base = M.at(k, j, 0);
  const bool filt = row_is_filtered(M, j, 0);
  if (filt) load_twiddles(M, fs);
  const double *U = M.u + (long long)M.ctl->it_uv * M.n3;
  const double n_inv = 1. / M.n[2 * j + 1];
  const double mn1 = M.mn[2 * j + 1];
  for (int i = threadIdx.x; i <= ni + 1; i += blockDim.x) {
    a[i] = buff[base + i];
    // u2d, with periodic pads for the layer average (bc_lateral(u2d))
    const int ii = kind == 1 ? (i == 0 ? ni : (i == ni + 1 ? 1 : i)) : i;
    const double u2d = kind == 1 ? .5 * (U[M.at(k, j, ii)] + U[M.at(k - 1, j, ii)]) : U[M.at(k, j, i)];
    um[i] = dminr(0., u2d * n_inv);
    up[i] = dmaxr(0., u2d * n_inv);
  }
  __syncthreads();
  if (filt) filter_row_smem(M, a, M.high_lat_h, M.at2(j, 0), fs);
  if (threadIdx.x == 0) { a[0] = a[ni]; a[ni + 1] = a[1]; }
  __syncthreads();
  // predictor
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) ff[i] = up[i] * a[i - 1] + um[i] * a[i];
  __syncthreads();
  if (threadIdx.x == 0) { ff[0] = ff[ni]; ff[ni + 1] = ff[1]; }
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) ap[i] = a[i] + (ff[i] - ff[i + 1]) * mn1 * DT;
  __syncthreads();
  if (threadIdx.x == 0) { ap[0] = ap[ni]; ap[ni + 1] = ap[1]; }
  __syncthreads();
  // corrector
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) {
    ff[i] = .5 * (up[i] * (ap[i] + a[i - 1]) + um[i] * (ap[i - 1] + a[i]));
    d1[i] = ap[i] - a[i - 1];
    d2[i] = ap[i] - a[i + 1];
    const double tmp = fabs(a[i - 1] - 2. * a[i] + a[i + 1]) + ep;
    aa[i] = tmp * tmp;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    d1[0] = d1[ni]; d1[ni + 1] = d1[1];
    d2[0] = d2[ni]; d2[ni + 1] = d2[1];
    aa[0] = aa[ni]; aa[ni + 1] = aa[1];
  }
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) {
    const double uhatp = sqrt(up[i] * up[i - 1]);
    const double uhatm = -sqrt(um[i] * um[i + 1]);
    const double mu = (up[i] - um[i]) * mn1 * DT;
    const double al = (1. + mu) / 6.;
    double gap = aa[i - 1] / (aa[i - 1] + (a[i - 1] - a_min) * (a[i] - a_min));
    gap = gap * gap;
    double gam = aa[i] / (aa[i] + (a[i - 1] - a_min) * (a[i] - a_min));
    gam = gam * gam;
    const double bep = 1. + (1. / (2. * al) - 1.) * gap;
    const double bem = 1. + (1. / (2. * al) - 1.) * gam;
    const double g = -al * (up[i] * bep * d1[i] - uhatp * (1. - gap) * d1[i - 1] + um[i] * bem * d2[i - 1] - uhatm * (1. - gam) * d2[i]);
    ff[i] += g;
  }
  __syncthreads();
  if (threadIdx.x == 0) { ff[0] = ff[ni]; ff[ni + 1] = ff[1]; }
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) {
    const double val = buff[base + i] + (ff[i] - ff[i + 1]) * mn1 * DT;
    write_with_pads(buff, M, base, i, val);
  }
}

// ---- launchers ----

static int row_threads(int ni) { return ni >= 256 ? 128 : 64; }

int launch_filter_planes(const DevModel &M, const double *src, int src_sel, double *dst, int k0, int nplanes, int vgrid, cudaStream_t s) {
  if (nplanes <= 0) return 0;
  const size_t smem = ((size_t)(M.ni + 2) + filter_smem_doubles(M.ni)) * sizeof(double);
  dim3 grid(M.nj + 3, nplanes);
  k_filter_planes<<<grid, row_threads(M.ni), smem, s>>>(M, src, src_sel, dst, k0, vgrid);
  return 0;
}

int launch_varz_filter(const DevModel &M, double *buff, int sel, int index, int kstart, int kend, cudaStream_t s) {
  const int jstart = index == 1 ? 1 : 0;
  const int nrows = M.nj - jstart + 1;
  k_varz_tables<<<epic_blocks(nrows, 64), 64, 0, s>>>(M, buff, sel, index, kstart, kend);
  const size_t smem = (2 * (size_t)(M.ni + 2) + filter_smem_doubles(M.ni)) * sizeof(double);
  dim3 grid(nrows, kend - kstart + 1);
  k_varz_filter_rows<<<grid, row_threads(M.ni), smem, s>>>(M, buff, sel, index, kstart, kend);
  return 0;
}

int launch_hsu_zonal(const DevModel &M, double *buff, int kind, int kstart, cudaStream_t s) {
  const size_t smem = (8 * (size_t)(M.ni + 2) + filter_smem_doubles(M.ni)) * sizeof(double);
  dim3 grid(M.nj + 1, M.nk - kstart + 1);
  k_hsu_zonal<<<grid, row_threads(M.ni), smem, s>>>(M, buff, kind, kstart);
  return 0;
}

int filter_kernels_init(int ni) {
  const size_t big = (8 * (size_t)(ni + 2) + filter_smem_doubles(ni)) * sizeof(double);
  if (big > 48 * 1024) {
    cudaFuncSetAttribute(k_hsu_zonal, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)big);
    cudaFuncSetAttribute(k_varz_filter_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)big);
    cudaFuncSetAttribute(k_filter_planes, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)big);
  }
  return 0;
}

size_t twiddle_doubles(int ni) {
  const int N = ni / 2;
  return 2 * ((size_t)N / 2 + N + 1);
}

// Twiddles for the half-length FFT, W^k = exp(-2 pi i k/N) for k < N/2, followed by the
// real-split factors t^m = exp(-2 pi i m/ni) for m = 0..N.
void fill_twiddles(int ni, double *tw) {
  const int N = ni / 2;
  for (int k = 0; k < N / 2; k++) {
    const double a = -2. * M_PI * (double)k / (double)N;
    tw[2 * k] = cos(a);
    tw[2 * k + 1] = sin(a);
  }
  double *t = tw + 2 * (N / 2);
  for (int m = 0; m <= N; m++) {
    const double a = -2. * M_PI * (double)m / (double)ni;
    t[2 * m] = cos(a);
    t[2 * m + 1] = sin(a);
  }
}

}  // namespace epic
