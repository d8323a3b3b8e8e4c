// High-latitude zonal filter kernels (the reference's zonal_filter, src/shared/epic_adjust.c:102-480).
//
// The reference filters one latitude row at a time: realft() forward, multiply wavenumber m by
// HIGH_LAT(J,m+1), realft() inverse and scale by 2/ni (epic_adjust.c:412-456), where realft and
// four1 are the Numerical Recipes in C (2nd ed., pp. 507, 513) real and complex radix-2 FFTs
// (epic_funcs_util.c:4023-4132).  Here one thread block owns one row and carries out the same
// arithmetic in parallel: every butterfly of a four1 stage and every iteration of realft's
// post-processing loop touches its own data, so they run concurrently; the twiddle factors,
// which NR builds by a recurrence, are computed once on the host with exactly that recurrence.
// Compiled without FMA contraction, each filtered row is bit-identical to the reference's.
#include "device_common.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

struct Cplx { double re, im; };

// Twiddle table layout (pairs of doubles), N = ni/2 complex points:
//   [0, N-1)              four1 isign=+1, stage with half h at offset h-1, entries p = 0..h-1
//   [N-1, 2N-2)           four1 isign=-1, same layout
//   [2N-2, 2N-2 + N/2-1)  realft forward post-processing, q = 1..N/2-1
//   [.., + N/2-1)         realft inverse pre-processing, q = 1..N/2-1
__host__ __device__ inline size_t nr_twiddle_pairs(int ni) {
  const int N = ni / 2;
  return 2 * (size_t)(N - 1) + 2 * (size_t)(N / 2 - 1);
}

struct FilterSmem {
  Cplx *z, *w;   // row as N complex points; twiddles
};

__device__ __forceinline__ FilterSmem carve_filter(double *base, int ni) {
  const int N = ni / 2;
  FilterSmem s;
  s.z = reinterpret_cast<Cplx *>(base);
  s.w = s.z + N;
  return s;
}
__host__ __device__ inline size_t filter_smem_doubles(int ni) {
  return 2 * ((size_t)(ni / 2) + nr_twiddle_pairs(ni));
}

__device__ __forceinline__ void load_twiddles(const DevModel &M, FilterSmem &s) {
  const int n = (int)nr_twiddle_pairs(M.ni);
  const Cplx *g = reinterpret_cast<const Cplx *>(M.tw);
  for (int k = threadIdx.x; k < n; k += blockDim.x) s.w[k] = g[k];
}

// four1's Danielson-Lanczos stages on z (already bit-reversed); tw = this direction's table.
__device__ __forceinline__ void four1_stages(Cplx *z, const Cplx *tw, int N) {
  for (int h = 1; h < N; h <<= 1) {
    const Cplx *wt = tw + (h - 1);
    for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
      const int p = b & (h - 1);
      const int i0 = (b / h) * 2 * h + p;
      const int j0 = i0 + h;
      const double wr = wt[p].re, wi = wt[p].im;
      const double tempr = wr * z[j0].re - wi * z[j0].im;
      const double tempi = wr * z[j0].im + wi * z[j0].re;
      z[j0].re = z[i0].re - tempr;
      z[j0].im = z[i0].im - tempi;
      z[i0].re += tempr;
      z[i0].im += tempi;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void bitrev_permute(Cplx *z, int N, int lg) {
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const int r = (int)(__brev((unsigned)k) >> (32 - lg));
    if (r > k) {
      const Cplx t = z[k];
      z[k] = z[r];
      z[r] = t;
    }
  }
  __syncthreads();
}

// realft's split loop (i = 2..n/4, here q = i-1): c2 = -0.5 forward, +0.5 inverse.
__device__ __forceinline__ void realft_split(Cplx *z, const Cplx *tw, int N, double c2) {
  const double c1 = 0.5;
  for (int q = 1 + threadIdx.x; q < N / 2; q += blockDim.x) {
    const Cplx a = z[q], b = z[N - q];
    const double wr = tw[q - 1].re, wi = tw[q - 1].im;
    const double h1r = c1 * (a.re + b.re);
    const double h1i = c1 * (a.im - b.im);
    const double h2r = -c2 * (a.im + b.im);
    const double h2i = c2 * (a.re - b.re);
    z[q].re = h1r + wr * h2r - wi * h2i;
    z[q].im = h1i + wr * h2i + wi * h2r;
    z[N - q].re = h1r - wr * h2r + wi * h2i;
    z[N - q].im = -h1i + wr * h2i + wi * h2r;
  }
  __syncthreads();
}

// Filter row x[1..ni] (1-based, shared memory) in place with weights h(I) = hl[rowbase + I],
// I = 1..ni/2+1 (HIGH_LAT(J,I)).  Every thread of the block must call this.
__device__ void filter_row_smem(const DevModel &M, double *x, const double *hl, long long rowbase, FilterSmem &s) {
  const int ni = M.ni, N = ni / 2;
  const int lg = 31 - __clz(N);
  const Cplx *t4p = s.w, *t4m = s.w + (N - 1), *trp = s.w + 2 * (N - 1), *trm = trp + (N / 2 - 1);
  Cplx *z = s.z;
  // realft(data, n, 1): four1(data, n/2, 1) -- bit reversal, stages -- then the split loop
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const int r = (int)(__brev((unsigned)k) >> (32 - lg));
    z[r].re = x[2 * k + 1];
    z[r].im = x[2 * k + 2];
  }
  __syncthreads();
  four1_stages(z, t4p, N);
  realft_split(z, trp, N, -0.5);
  if (threadIdx.x == 0) {
    const double h1r = z[0].re;
    z[0].re = h1r + z[0].im;
    z[0].im = h1r - z[0].im;
  }
  __syncthreads();
  // spectral weights (epic_adjust.c:447-453)
  for (int q = threadIdx.x; q < N; q += blockDim.x) {
    if (q == 0) {
      z[0].re *= hl[rowbase + 1];
      z[0].im *= hl[rowbase + N + 1];
    } else {
      const double h = hl[rowbase + q + 1];
      z[q].re *= h;
      z[q].im *= h;
    }
  }
  __syncthreads();
  // realft(data, n, -1): split loop, then four1(data, n/2, -1)
  realft_split(z, trm, N, 0.5);
  if (threadIdx.x == 0) {
    const double h1r = z[0].re;
    z[0].re = 0.5 * (h1r + z[0].im);
    z[0].im = 0.5 * (h1r - z[0].im);
  }
  __syncthreads();
  bitrev_permute(z, N, lg);
  four1_stages(z, t4m, N);
  const double scale = 2. / (double)ni;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    x[2 * k + 1] = z[k].re * scale;
    x[2 * k + 2] = z[k].im * scale;
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
    t[kay].y = index == 2 ? xlog(M, buff[M.at(k, j, i)]) : buff[M.at(k, j, i)];
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
    if (index == 2) v = xexp(M, v);
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
    const double behatp = 1. - gap, behatm = 1. - gam;
    const double g = -al * (up[i] * bep * d1[i] - uhatp * behatp * d1[i - 1] + um[i] * bem * d2[i - 1] - uhatm * behatm * d2[i]);
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

size_t twiddle_doubles(int ni) { return 2 * nr_twiddle_pairs(ni); }

// Host: the twiddle factors four1 and realft generate by recurrence, in their order, with
// their arithmetic (epic_funcs_util.c:4047-4076, :4096-4120).  Compiled without contraction.
void fill_twiddles(int ni, double *tw) {
  const int N = ni / 2;
  const unsigned long n = (unsigned long)N << 1;
  double *out = tw;
  for (int isign = 1; isign >= -1; isign -= 2) {
    for (unsigned long mmax = 2; n > mmax; mmax <<= 1) {
      const double theta = isign * (2 * M_PI / mmax);
      double wtemp = sin(0.5 * theta);
      const double wpr = -2.0 * wtemp * wtemp;
      const double wpi = sin(theta);
      double wr = 1.0, wi = 0.0;
      for (unsigned long m = 1; m < mmax; m += 2) {
        *out++ = wr;
        *out++ = wi;
        wr = (wtemp = wr) * wpr - wi * wpi + wr;
        wi = wi * wpr + wtemp * wpi + wi;
      }
    }
  }
  for (int isign = 1; isign >= -1; isign -= 2) {
    double theta = M_PI / (double)((unsigned long)ni >> 1);
    if (isign != 1) theta = -theta;
    double wtemp = sin(0.5 * theta);
    const double wpr = -2.0 * wtemp * wtemp;
    const double wpi = sin(theta);
    double wr = 1.0 + wpr, wi = wpi;
    for (unsigned long i = 2; i <= ((unsigned long)ni >> 2); i++) {
      *out++ = wr;
      *out++ = wi;
      wr = (wtemp = wr) * wpr - wi * wpi + wr;
      wi = wi * wpr + wtemp * wpi + wi;
    }
  }
}

}  // namespace epic
