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

template <class R> struct Cplx { R re, im; };

// Twiddle table layout (pairs), N = ni/2 complex points:
//   [0, N-1)              four1 isign=+1, stage with half h at offset h-1, entries p = 0..h-1
//   [N-1, 2N-2)           four1 isign=-1, same layout
//   [2N-2, 2N-2 + N/2-1)  realft forward post-processing, q = 1..N/2-1
//   [.., + N/2-1)         realft inverse pre-processing, q = 1..N/2-1
// The FP64 table holds the recurrence values of the reference; the mixed form reads the same
// values rounded to float.
__host__ __device__ inline size_t nr_twiddle_pairs(int ni) {
  const int N = ni / 2;
  return 2 * (size_t)(N - 1) + 2 * (size_t)(N / 2 - 1);
}

template <class R>
struct FilterSmem {
  Cplx<R> *z, *w;   // row as N complex points; twiddles
};

template <class R>
__device__ __forceinline__ FilterSmem<R> carve_filter(R *base, int ni) {
  const int N = ni / 2;
  FilterSmem<R> s;
  s.z = reinterpret_cast<Cplx<R> *>(base);
  s.w = s.z + N;
  return s;
}
// shared-memory elements (of the compute type) one row filter needs
__host__ __device__ inline size_t filter_smem_elems(int ni) {
  return 2 * ((size_t)(ni / 2) + nr_twiddle_pairs(ni));
}

template <class R> __device__ __forceinline__ const R *twiddle_table(const DevModel &M);
template <> __device__ __forceinline__ const double *twiddle_table<double>(const DevModel &M) { return M.tw; }
template <> __device__ __forceinline__ const float *twiddle_table<float>(const DevModel &M) { return M.twf; }

template <class R>
__device__ __forceinline__ void load_twiddles(const DevModel &M, FilterSmem<R> &s) {
  const int n = (int)nr_twiddle_pairs(M.ni);
  const Cplx<R> *g = reinterpret_cast<const Cplx<R> *>(twiddle_table<R>(M));
  for (int k = threadIdx.x; k < n; k += blockDim.x) s.w[k] = g[k];
}

// four1's Danielson-Lanczos stages on z (already bit-reversed); tw = this direction's table.
template <class R>
__device__ __forceinline__ void four1_stages(Cplx<R> *z, const Cplx<R> *tw, int N) {
  for (int h = 1; h < N; h <<= 1) {
    const Cplx<R> *wt = tw + (h - 1);
    for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
      const int p = b & (h - 1);
      const int i0 = (b / h) * 2 * h + p;
      const int j0 = i0 + h;
      const R wr = wt[p].re, wi = wt[p].im;
      const R tempr = wr * z[j0].re - wi * z[j0].im;
      const R tempi = wr * z[j0].im + wi * z[j0].re;
      z[j0].re = z[i0].re - tempr;
      z[j0].im = z[i0].im - tempi;
      z[i0].re += tempr;
      z[i0].im += tempi;
    }
    __syncthreads();
  }
}

template <class R>
__device__ __forceinline__ void bitrev_permute(Cplx<R> *z, int N, int lg) {
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const int r = (int)(__brev((unsigned)k) >> (32 - lg));
    if (r > k) {
      const Cplx<R> t = z[k];
      z[k] = z[r];
      z[r] = t;
    }
  }
  __syncthreads();
}

// realft's split loop (i = 2..n/4, here q = i-1): c2 = -0.5 forward, +0.5 inverse.
template <class R>
__device__ __forceinline__ void realft_split(Cplx<R> *z, const Cplx<R> *tw, int N, R c2) {
  const R c1 = R(0.5);
  for (int q = 1 + threadIdx.x; q < N / 2; q += blockDim.x) {
    const Cplx<R> a = z[q], b = z[N - q];
    const R wr = tw[q - 1].re, wi = tw[q - 1].im;
    const R h1r = c1 * (a.re + b.re);
    const R h1i = c1 * (a.im - b.im);
    const R h2r = -c2 * (a.im + b.im);
    const R h2i = c2 * (a.re - b.re);
    z[q].re = h1r + wr * h2r - wi * h2i;
    z[q].im = h1i + wr * h2i + wi * h2r;
    z[N - q].re = h1r - wr * h2r + wi * h2i;
    z[N - q].im = -h1i + wr * h2i + wi * h2r;
  }
  __syncthreads();
}

// Filter row x[1..ni] (1-based, shared memory) in place with weights h(I) = hl[rowbase + I],
// I = 1..ni/2+1 (HIGH_LAT(J,I)).  Every thread of the block must call this.
template <class R>
__device__ void filter_row_smem(const DevModel &M, R *x, const double *hl, long long rowbase, FilterSmem<R> &s) {
  const int ni = M.ni, N = ni / 2;
  const int lg = 31 - __clz(N);
  const Cplx<R> *t4p = s.w, *t4m = s.w + (N - 1), *trp = s.w + 2 * (N - 1), *trm = trp + (N / 2 - 1);
  Cplx<R> *z = s.z;
  // realft(data, n, 1): four1(data, n/2, 1) -- bit reversal, stages -- then the split loop
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const int r = (int)(__brev((unsigned)k) >> (32 - lg));
    z[r].re = x[2 * k + 1];
    z[r].im = x[2 * k + 2];
  }
  __syncthreads();
  four1_stages(z, t4p, N);
  realft_split(z, trp, N, R(-0.5));
  if (threadIdx.x == 0) {
    const R h1r = z[0].re;
    z[0].re = h1r + z[0].im;
    z[0].im = h1r - z[0].im;
  }
  __syncthreads();
  // spectral weights (epic_adjust.c:447-453)
  for (int q = threadIdx.x; q < N; q += blockDim.x) {
    if (q == 0) {
      z[0].re *= cv<R>(hl[rowbase + 1]);
      z[0].im *= cv<R>(hl[rowbase + N + 1]);
    } else {
      const R h = cv<R>(hl[rowbase + q + 1]);
      z[q].re *= h;
      z[q].im *= h;
    }
  }
  __syncthreads();
  // realft(data, n, -1): split loop, then four1(data, n/2, -1)
  realft_split(z, trm, N, R(0.5));
  if (threadIdx.x == 0) {
    const R h1r = z[0].re;
    z[0].re = R(0.5) * (h1r + z[0].im);
    z[0].im = R(0.5) * (h1r - z[0].im);
  }
  __syncthreads();
  bitrev_permute(z, N, lg);
  four1_stages(z, t4m, N);
  const R scale = R(2.) / R(ni);
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
template <class R>
__global__ void k_filter_planes(DevModel M, const double *src, int src_sel, double *dst, int k0, int vgrid) {
  if (epic_member(M, src, dst)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sm = reinterpret_cast<R *>(smraw);
  src += plane_offset(M, src_sel);
  const int j = (int)blockIdx.x - 1;
  if (j > M.nj + 1) return;   // a member with fewer rows than the launch (batches of mixed sizes)
  const int k = k0 + (int)blockIdx.y;
  const long long base = M.at(k, j, 0);
  R *x = sm;
  FilterSmem<R> fs = carve_filter(sm + (M.ni + 2), M.ni);
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
  for (int i = threadIdx.x; i <= M.ni + 1; i += blockDim.x) x[i] = cv<R>(src[base + i]);
  __syncthreads();
  filter_row_smem(M, x, vgrid ? M.high_lat_pv : M.high_lat_h, M.at2(j, 0), fs);
  for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) write_with_pads(dst, M, base, i, x[i]);
}


// Per-latitude var(gz) profile at the column of lowest bottom GZ, the first half of the
// THREEDIM branch of zonal_filter (epic_adjust.c:266-395).  One warp per row j: the lanes find
// the first column of minimum bottom GZ (the reference's strict-less scan) and fill the table;
// lane 0 fits the spline.  index: 0 = U, 1 = V, 2 = HDRY (log), 3 = THETA.
__global__ void k_varz_tables(DevModel M, const double *buff, int sel, int index, int kstart, int kend) {
  if (epic_member(M, buff)) return;
  buff += plane_offset(M, sel);
  const int jstart = index == 1 ? 1 : 0;
  const int lane = (int)(threadIdx.x & 31);
  const int j = jstart + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (j > M.nj) return;
  // the mixed forms filter (and so tabulate) only the filtered rows
  if (M.mixed && !row_is_filtered(M, j, index == 1)) return;
  const double *gz = M.gz;
  const int K = M.nk;
  int imin = 1 << 30;
  double gzmin = DBL_MAX;
  for (int i = 1 + lane; i <= M.ni; i += 32) {
    const double v = gz[M.at(K, j, i)];
    if (v < gzmin) { imin = i; gzmin = v; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, gzmin, o);
    const int oi = __shfl_xor_sync(0xffffffffu, imin, o);
    if (ov < gzmin || (ov == gzmin && oi < imin)) { gzmin = ov; imin = oi; }
  }
  const int i = imin == (1 << 30) ? 1 : imin;
  Trip *t = reinterpret_cast<Trip *>(M.ptable) + (long long)(j + 1) * (M.nk + 2);
  for (int k = kend - lane; k >= kstart; k -= 32) {
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
  __syncwarp();
  // spline_pchip (epic_funcs_util.c:721-845): every slope uses only its two neighbouring
  // intervals, so the lanes compute them in parallel with the reference's expressions.
  const int n = kend - kstart + 1;
  bool bad = false;
  for (int q = 1 + lane; q < n; q += 32) bad |= t[q].x <= t[q - 1].x;
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) flag_error(M.ctl, ERR_PCHIP_X, kstart, j, i, t[0].x);
    return;
  }
  if (n == 2) {
    if (lane == 0) {
      const double del1 = (t[1].y - t[0].y) / (t[1].x - t[0].x);
      t[0].z = del1;
      t[1].z = del1;
    }
    return;
  }
  for (int q = lane; q < n; q += 32) {
    // the two intervals around point q (the first two for q = 0, the last two for q = n-1)
    const int m = q == 0 ? 1 : (q == n - 1 ? n - 2 : q);
    const double h1 = t[m].x - t[m - 1].x, h2 = t[m + 1].x - t[m].x;
    const double del1 = (t[m].y - t[m - 1].y) / h1, del2 = (t[m + 1].y - t[m].y) / h2;
    const double hsum = h1 + h2;
    double z;
    if (q == 0) {
      const double w1 = (h1 + hsum) / hsum, w2 = -h1 / hsum;
      z = w1 * del1 + w2 * del2;
      if (pchst(z, del1) <= 0.0) z = 0.0;
      else if (pchst(del1, del2) < 0.0) {
        const double dmx = 3.0 * del1;
        if (fabs(dmx) < fabs(z)) z = dmx;
      }
    } else if (q == n - 1) {
      const double w1 = -h2 / hsum, w2 = (h2 + hsum) / hsum;
      z = w1 * del1 + w2 * del2;
      if (pchst(z, del2) <= 0.0) z = 0.0;
      else if (pchst(del1, del2) < 0.0) {
        const double dmx = 3.0 * del2;
        if (fabs(dmx) < fabs(z)) z = dmx;
      }
    } else {
      z = 0.0;
      if (pchst(del1, del2) > 0.0) {
        const double hsumt3 = 3.0 * hsum;
        const double w1 = (hsum + h1) / hsumt3, w2 = (hsum + h2) / hsumt3;
        const double dmx = dmaxr(fabs(del1), fabs(del2)), dmn = dminr(fabs(del1), fabs(del2));
        z = dmn / (w1 * (del1 / dmx) + w2 * (del2 / dmx));
      }
    }
    t[q].z = z;
  }
}

// The mixed forms' profile: var(gz) to double-float accuracy (~48 bits) as the knot value plus the
// cubic's increment from the knot, evaluated in double-float on the distance gz - x_knot (gz and
// x_knot converted to double-floats on the integer pipe), with the cubic's coefficients computed
// in binary64 and split into double-floats; the deviation buff - var is formed in double-float
// and the filtered deviation added back to var in binary64 -- the field itself is never rounded
// to FP32, and the profile's own 48-bit rounding cancels between subtracting and adding it back.
// The profile has to be this accurate: out = var + F(buff - var) = buff - (I - F)(buff - var), so a
// rounding error of the profile that varies from column to column (an FP32 increment's does)
// passes the filter's high-wavenumber part (I - F) straight into THETA and HDRY on every filtered
// row, every step; with FP32 increments that was the largest single source of the mixed form's
// wind error after a simulated day (it halved the median member's U error to remove it).  HDRY is
// interpolated in log space: knot value exp(y) times exp(increment).  The knot values and the
// coefficients are tabulated once per row (varz_intervals_mixed); the interval is found in FP32
// (next to a knot either neighbouring cubic gives the same value, the pieces joining with their
// first derivative), the distance from its knot in double-float.
struct VarzInterval {
  float x, pad;
  float2 z0, c2, c3;   // double-float coefficients of the cubic in the distance from the knot
};
__device__ __forceinline__ float2 split_df(double v) {
  const dfl d = d2df(v);
  return make_float2(d.hi, d.lo);
}
__device__ __forceinline__ void varz_intervals_mixed(const Trip *t, int n, int index, double *knot, VarzInterval *iv) {
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    knot[q] = index == 2 ? ::exp(t[q].y) : t[q].y;
    VarzInterval v;
    v.x = d2f(t[q].x);
    v.pad = 0.f;
    v.z0 = split_df(t[q].z);
    v.c2 = v.c3 = make_float2(0.f, 0.f);
    if (q + 1 < n) {   // splint_pchip's cubic, epic_funcs_util.c:926-946
      const double h = t[q + 1].x - t[q].x;
      const double delta = (t[q + 1].y - t[q].y) / h;
      const double del1 = (t[q].z - delta) / h, del2 = (t[q + 1].z - delta) / h;
      v.c3 = split_df((del1 + del2) / h);
      v.c2 = split_df(-(del1 + del1 + del2));
    }
    iv[q] = v;
  }
}
__device__ __forceinline__ dfl varz_profile_mixed(const Trip *t, const double *knot, const VarzInterval *iv, int n, int index,
                                                  dfl gzd, const float2 *exp2tab) {
  const float g = gzd.hi;
  int kay;
  if (g <= iv[0].x) kay = 0;
  else if (g >= iv[n - 1].x) kay = n - 2;
  else {
    int il = -1, iu = n;
    while (iu - il > 1) {
      const int im = (iu + il) >> 1;
      if (g >= iv[im].x) il = im; else iu = im;
    }
    kay = il;
  }
  // a NaN argument fails every comparison: keep the interval index inside the table
  kay = kay < 0 ? 0 : (kay > n - 2 ? n - 2 : kay);
  const VarzInterval v = iv[kay];
  const dfl xx = gzd - d2df(t[kay].x);
  const dfl inc = xx * (dfl(v.z0.x, v.z0.y) + xx * (dfl(v.c2.x, v.c2.y) + xx * dfl(v.c3.x, v.c3.y)));
  return index == 2 ? d2df(knot[kay]) * exp_df(inc, exp2tab) : d2df(knot[kay]) + inc;
}

// The rest of the THREEDIM zonal_filter: subtract var(gz), filter, add it back.
// Block = one row (k = kstart + blockIdx.y, j = jstart + blockIdx.x).
template <class R>
__global__ void k_varz_filter_rows(DevModel M, double *buff, int sel, int index, int kstart, int kend) {
  if (epic_member(M, buff)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  buff += plane_offset(M, sel);
  const int jstart = index == 1 ? 1 : 0;
  const int j = jstart + (int)blockIdx.x;
  if (j > M.nj) return;   // a member with fewer rows than the launch (batches of mixed sizes)
  const int k = kstart + (int)blockIdx.y;
  const int vgrid = index == 1;
  const Trip *t = reinterpret_cast<const Trip *>(M.ptable) + (long long)(j + 1) * (M.nk + 2);
  const int n = kend - kstart + 1;
  const double *gz = M.gz;
  const long long base = M.at(k, j, 0);
  const bool filt = row_is_filtered(M, j, vgrid);
  // The mixed forms leave unfiltered rows untouched (their subtract-and-add-back is the identity
  // up to one rounding); the FP64 form repeats the reference's arithmetic on them.
  if (!filt && !std::is_same_v<R, double>) return;
  if constexpr (!std::is_same_v<R, double>) {
    double *vzd = reinterpret_cast<double *>(smraw), *knot = vzd + (M.ni + 2);
    VarzInterval *iv = reinterpret_cast<VarzInterval *>(knot + (M.nk + 2));
    R *x = reinterpret_cast<R *>(iv + (M.nk + 2));
    FilterSmem<R> fs = carve_filter(x + (M.ni + 2), M.ni);
    load_twiddles(M, fs);
    varz_intervals_mixed(t, n, index, knot, iv);
    __syncthreads();
    // the profile's argument, its value and the deviation in double-float (integer and FP32
    // pipes: this kernel had the FP64 unit half busy); the deviation is filtered in binary32 and
    // added back to the profile in binary64 below, the profile's own rounding cancelling
    for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) {
      dfl gzd;
      switch (index) {
        case 0: gzd = df_ldexp(d2df(gz[M.at(k, j, i)]) + d2df(gz[M.at(k, j, i - 1)]), -1); break;
        case 1: gzd = df_ldexp(d2df(gz[M.at(k, j, i)]) + d2df(gz[M.at(k, j - 1, i)]), -1); break;
        case 2: gzd = df_ldexp(d2df(gz[M.at(k, j, i)]) + d2df(gz[M.at(k - 1, j, i)]), -1); break;
        default: gzd = d2df(gz[M.at(k, j, i)]); break;
      }
      const dfl v = varz_profile_mixed(t, knot, iv, n, index, gzd, M.exp2tab);
      vzd[i] = df2d(v);
      x[i] = (d2df(buff[base + i]) - v).hi;
    }
    __syncthreads();
    filter_row_smem(M, x, vgrid ? M.high_lat_pv : M.high_lat_h, M.at2(j, 0), fs);
    // HDRY (index 2): restore_mass, which timestep() calls next (epic_timestep.c:212), on the
    // filtered value; unfiltered rows are untouched here and already restored
    for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) {
      const double v = f2d(x[i]) + vzd[i];
      write_with_pads(buff, M, base, i, index == 2 ? dmaxr(M.h_min[k], v) : v);
    }
    return;
  }
  R *sm = reinterpret_cast<R *>(smraw);
  R *x = sm, *vz = sm + (M.ni + 2);
  FilterSmem<R> fs = carve_filter(sm + 2 * (M.ni + 2), M.ni);
  if (filt) load_twiddles(M, fs);
  for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) {
    R gzz;
    switch (index) {
      case 0: gzz = R(.5) * (cv<R>(gz[M.at(k, j, i)]) + cv<R>(gz[M.at(k, j, i - 1)])); break;
      case 1: gzz = R(.5) * (cv<R>(gz[M.at(k, j, i)]) + cv<R>(gz[M.at(k, j - 1, i)])); break;
      case 2: gzz = R(.5) * (cv<R>(gz[M.at(k, j, i)]) + cv<R>(gz[M.at(k - 1, j, i)])); break;
      default: gzz = cv<R>(gz[M.at(k, j, i)]); break;
    }
    // find_place_in_table (epic_funcs_util.c:2908-2967) and splint_pchip (:926-946)
    int kay;
    if (RMath<R>::cmp(gzz, cv<R>(t[0].x)) <= 0) kay = 0;
    else if (RMath<R>::cmp(gzz, cv<R>(t[n - 1].x)) >= 0) kay = n - 2;
    else {
      int il = -1, iu = n;
      while (iu - il > 1) {
        const int im = (iu + il) >> 1;
        if (RMath<R>::cmp(gzz, cv<R>(t[im].x)) >= 0) il = im; else iu = im;
      }
      kay = il < 0 ? 0 : il;
    }
    const Trip *tk = t + kay;
    const R h = cv<R>(tk[1].x) - cv<R>(tk[0].x);
    const R delta = (cv<R>(tk[1].y) - cv<R>(tk[0].y)) / h;
    const R del1 = (cv<R>(tk[0].z) - delta) / h;
    const R del2 = (cv<R>(tk[1].z) - delta) / h;
    const R c3 = (del1 + del2) / h;
    const R c2 = -(del1 + del1 + del2);
    const R xx = gzz - cv<R>(tk[0].x);
    R v = cv<R>(tk[0].y) + xx * (cv<R>(tk[0].z) + xx * (c2 + xx * c3));
    if (index == 2) v = RMath<R>::exp(M, v);
    vz[i] = v;
    x[i] = cv<R>(buff[base + i] - to_d(v));
  }
  __syncthreads();
  if (filt) filter_row_smem(M, x, vgrid ? M.high_lat_pv : M.high_lat_h, M.at2(j, 0), fs);
  for (int i = threadIdx.x + 1; i <= M.ni; i += blockDim.x) {   // HDRY (index 2): restore_mass too
    const double v = to_d(x[i]) + to_d(vz[i]);
    write_with_pads(buff, M, base, i, index == 2 ? dmaxr(M.h_min[k], v) : v);
  }
}

// Zonal pass of hsu_advection (epic_flux.c:1316-1484) for one row: the fluxes come from a
// zonally filtered copy of the row, the update goes to the unfiltered field.
// kind: 0 = interface variable (unity, THETA), 1 = HDRY (layer; u averaged to the layer),
// 2 = NU_TURB (interface variable with the floor NU_TURB_MIN).
template <class R>
__global__ void k_hsu_zonal(DevModel M, double *buff, int kind, int kstart) {
  if (epic_member(M, buff)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sm = reinterpret_cast<R *>(smraw);
  const int ni = M.ni, W = ni + 2;
  const int j = (int)blockIdx.x;
  if (j > M.nj) return;   // a member with fewer rows than the launch (batches of mixed sizes)
  const int k = kstart + (int)blockIdx.y;
  R *a = sm, *um = a + W, *up = um + W, *ff = up + W, *ap = ff + W, *d1 = ap + W, *d2 = d1 + W, *aa = d2 + W;
  FilterSmem<R> fs = carve_filter(aa + W, ni);
  const R ep = R(1.e-10), DT = cv<R>(M.dt);
  const R a_min = kind == 1 ? cv<R>(M.h_min[k]) : (kind == 2 ? cv<R>(1.e-3 * M.kinvisc) : R(0.));
  const long long base = M.at(k, j, 0);
  const bool filt = row_is_filtered(M, j, 0);
  if (filt) load_twiddles(M, fs);
  const double *U = M.u + (long long)M.ctl->it_uv * M.n3;
  const R n_inv = R(1.) / cv<R>(M.n[2 * j + 1]);
  const R mn1 = cv<R>(M.mn[2 * j + 1]);
  for (int i = threadIdx.x; i <= ni + 1; i += blockDim.x) {
    a[i] = cv<R>(buff[base + i]);
    // u2d, with periodic pads for the layer average (bc_lateral(u2d))
    const int ii = kind == 1 ? (i == 0 ? ni : (i == ni + 1 ? 1 : i)) : i;
    const R u2d = kind == 1 ? R(.5) * (cv<R>(U[M.at(k, j, ii)]) + cv<R>(U[M.at(k - 1, j, ii)])) : cv<R>(U[M.at(k, j, i)]);
    um[i] = rmin(R(0.), u2d * n_inv);
    up[i] = rmax(R(0.), u2d * n_inv);
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
    ff[i] = R(.5) * (up[i] * (ap[i] + a[i - 1]) + um[i] * (ap[i - 1] + a[i]));
    d1[i] = ap[i] - a[i - 1];
    d2[i] = ap[i] - a[i + 1];
    const R tmp = fabs(a[i - 1] - R(2.) * a[i] + a[i + 1]) + ep;
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
    const R uhatp = sqrt(up[i] * up[i - 1]);
    const R uhatm = -sqrt(um[i] * um[i + 1]);
    const R mu = (up[i] - um[i]) * mn1 * DT;
    const R al = (R(1.) + mu) / R(6.);
    R gap = aa[i - 1] / (aa[i - 1] + (a[i - 1] - a_min) * (a[i] - a_min));
    gap = gap * gap;
    R gam = aa[i] / (aa[i] + (a[i - 1] - a_min) * (a[i] - a_min));
    gam = gam * gam;
    const R bep = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gap;
    const R bem = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gam;
    const R behatp = R(1.) - gap, behatm = R(1.) - gam;
    const R g = -al * (up[i] * bep * d1[i] - uhatp * behatp * d1[i - 1] + um[i] * bem * d2[i - 1] - uhatm * behatm * d2[i]);
    ff[i] += g;
  }
  __syncthreads();
  if (threadIdx.x == 0) { ff[0] = ff[ni]; ff[ni + 1] = ff[1]; }
  __syncthreads();
  // HDRY (kind 1): restore_mass (epic_adjust.c:45-96), which advection() calls next
  // (epic_flux.c:623), on the new value -- the same max per cell, one pass fewer
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) {
    const double v = buff[base + i] + to_d((ff[i] - ff[i + 1]) * mn1 * DT);
    write_with_pads(buff, M, base, i, kind == 1 ? dmaxr(M.h_min[k], v) : v);
  }
}

// Zonal pass of akima_advection (epic_flux.c:1826-1932) for one row: the fluxes come from a
// zonally filtered copy of the row, the update goes to the unfiltered field.
// kind: 0 = interface variable (unity, THETA), 1 = HDRY (layer; u averaged to the layer).
template <class R>
__global__ void k_akima_zonal(DevModel M, double *buff, int kind, int kstart) {
  if (epic_member(M, buff)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  R *sm = reinterpret_cast<R *>(smraw);
  const int ni = M.ni, W = ni + 2;
  const int j = (int)blockIdx.x;
  if (j > M.nj) return;   // a member with fewer rows than the launch (batches of mixed sizes)
  const int k = kstart + (int)blockIdx.y;
  R *a = sm, *u2d = a + W, *da = u2d + W, *dl = da + W, *ff = dl + W;
  FilterSmem<R> fs = carve_filter(ff + W, ni);
  const R DT = cv<R>(M.dt);
  const long long base = M.at(k, j, 0);
  const bool filt = row_is_filtered(M, j, 0);
  if (filt) load_twiddles(M, fs);
  const double *U = M.u + (long long)M.ctl->it_uv * M.n3;
  const R n_inv = R(1.) / cv<R>(M.n[2 * j + 1]);
  const R mn1 = cv<R>(M.mn[2 * j + 1]);
  for (int i = threadIdx.x; i <= ni + 1; i += blockDim.x) {
    a[i] = cv<R>(buff[base + i]);
    // u2d, with periodic pads for the layer average (bc_lateral(u2d))
    const int ii = kind == 1 ? (i == 0 ? ni : (i == ni + 1 ? 1 : i)) : i;
    u2d[i] = kind == 1 ? R(.5) * (cv<R>(U[M.at(k, j, ii)]) + cv<R>(U[M.at(k - 1, j, ii)])) : cv<R>(U[M.at(k, j, i)]);
  }
  __syncthreads();
  if (filt) filter_row_smem(M, a, M.high_lat_h, M.at2(j, 0), fs);
  if (threadIdx.x == 0) { a[0] = a[ni]; a[ni + 1] = a[1]; }
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) da[i] = a[i] - a[i - 1];
  __syncthreads();
  if (threadIdx.x == 0) { da[0] = da[ni]; da[ni + 1] = da[1]; }
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) {
    const R tmp = da[i] * da[i + 1];
    dl[i] = (tmp > R(0.)) ? R(2.) * tmp / (da[i] + da[i + 1]) : R(0.);
  }
  __syncthreads();
  if (threadIdx.x == 0) { dl[0] = dl[ni]; dl[ni + 1] = dl[1]; }
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) {
    const R aval = R(.5) * (a[i] + a[i - 1]) - (dl[i] - dl[i - 1]) / R(6.);
    ff[i] = u2d[i] * aval * n_inv;
  }
  __syncthreads();
  if (threadIdx.x == 0) { ff[0] = ff[ni]; ff[ni + 1] = ff[1]; }
  __syncthreads();
  for (int i = threadIdx.x + 1; i <= ni; i += blockDim.x) {   // HDRY (kind 1): restore_mass too
    const double v = buff[base + i] + to_d((ff[i] - ff[i + 1]) * mn1 * DT);
    write_with_pads(buff, M, base, i, kind == 1 ? dmaxr(M.h_min[k], v) : v);
  }
}

// The rows the tensor-core filter leaves alone (k_filter_planes_gemm filters the others): copied
// when dst is not src, periodic pads on rows 0..nj+1.  One warp per (row, plane).
__global__ void k_filter_rows_unfiltered(DevModel M, const double *src, int src_sel, double *dst, int k0, int nplanes, int vgrid) {
  if (epic_member(M, src, dst)) return;
  src += plane_offset(M, src_sel);
  const int lane = (int)(threadIdx.x & 31);
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int rows = M.nj + 3;
  if (w >= rows * nplanes) return;
  const int j = w % rows - 1, k = k0 + w / rows;
  const bool valid = vgrid ? (j >= 1 && j <= M.nj) : (j >= 0 && j <= M.nj);
  if (valid && row_is_filtered(M, j, vgrid)) return;
  const int base = M.at(k, j, 0);
  if (src != dst)
    for (int i = lane; i <= M.ni + 1; i += 32) dst[base + i] = src[base + i];
  __syncwarp();
  if (j >= 0 && lane == 0) {
    dst[base] = dst[base + M.ni];
    dst[base + M.ni + 1] = dst[base + 1];
  }
}

// ---- launchers ----

static int row_threads(const DevModel &M) { return M.tb[TB_ROW] > 0 ? M.tb[TB_ROW] : (M.ni >= 256 ? 128 : 64); }
static size_t relem(int fp32) { return fp32 ? sizeof(float) : sizeof(double); }

int launch_filter_planes(const DevModel &M, const double *src, int src_sel, double *dst, int k0, int nplanes, int vgrid, cudaStream_t s,
                         int fp32, int shift, int pads_set) {
  if (nplanes <= 0) return 0;
  const size_t smem = ((size_t)(M.ni + 2) + filter_smem_elems(M.ni)) * relem(fp32);
  dim3 grid(M.nj + 3, nplanes);
  if (fp32 && filter_gemm_usable(M)) {
    // The rows the operator leaves alone are copied (and padded) by a light kernel of their own:
    // done by the operator's blocks, each reserving the product's ~83 KB of shared memory, they
    // kept the filtered rows' blocks off the SMs (the step's filter time rose by a third).  In
    // place with the pads already set, those rows need nothing.
    const long long warps = (long long)(M.nj + 3) * nplanes;
    if (!(pads_set && src == dst && src_sel == PL_NONE))
      k_filter_rows_unfiltered<<<zg(epic_blocks(32 * warps, 128), M), 128, 0, s>>>(M, src, src_sel, dst, k0, nplanes, vgrid);
    return launch_filter_planes_gemm(M, src, src_sel, dst, k0, nplanes, vgrid, s, shift);
  }
  EPIC_LAUNCH_R(fp32, k_filter_planes, grid, row_threads(M), smem, s, M, src, src_sel, dst, k0, vgrid);
  return 0;
}

int launch_varz_filter(const DevModel &M, double *buff, int sel, int index, int kstart, int kend, cudaStream_t s) {
  const int jstart = index == 1 ? 1 : 0;
  const int nrows = M.nj - jstart + 1;
  k_varz_tables<<<zg(epic_blocks(32LL * nrows, 128), M), 128, 0, s>>>(M, buff, sel, index, kstart, kend);
  const size_t smem = M.mixed ? ((size_t)(M.ni + 2) + (M.nk + 2)) * sizeof(double) + (size_t)(M.nk + 2) * sizeof(VarzInterval) +
                                    ((size_t)(M.ni + 2) + filter_smem_elems(M.ni)) * sizeof(float)
                             : (2 * (size_t)(M.ni + 2) + filter_smem_elems(M.ni)) * sizeof(double);
  dim3 grid(nrows, kend - kstart + 1);
  EPIC_LAUNCH_R(M.mixed, k_varz_filter_rows, grid, row_threads(M), smem, s, M, buff, sel, index, kstart, kend);
  return 0;
}

int launch_akima_zonal(const DevModel &M, double *buff, int kind, int kstart, cudaStream_t s) {
  const size_t smem = (5 * (size_t)(M.ni + 2) + filter_smem_elems(M.ni)) * relem(M.mixed);
  dim3 grid(M.nj + 1, M.nk - kstart + 1);
  EPIC_LAUNCH_R(M.mixed, k_akima_zonal, grid, row_threads(M), smem, s, M, buff, kind, kstart);
  return 0;
}

int launch_hsu_zonal(const DevModel &M, double *buff, int kind, int kstart, cudaStream_t s) {
  const size_t smem = (8 * (size_t)(M.ni + 2) + filter_smem_elems(M.ni)) * relem(M.mixed);
  dim3 grid(M.nj + 1, M.nk - kstart + 1);
  EPIC_LAUNCH_R(M.mixed, k_hsu_zonal, grid, row_threads(M), smem, s, M, buff, kind, kstart);
  return 0;
}

template <class R>
static void filter_attrs(int bytes) {
  cudaFuncSetAttribute(k_hsu_zonal<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_akima_zonal<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_varz_filter_rows<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(k_filter_planes<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// Raised once to the largest row (ni = EPIC_MAX_NI), so models of different sizes in one process
// never lower the limit for one another.
int filter_kernels_init(int) {
  const size_t big = (8 * (size_t)(EPIC_MAX_NI + 2) + filter_smem_elems(EPIC_MAX_NI)) * sizeof(double);
  filter_attrs<double>((int)big);
  filter_attrs<float>((int)big);
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
