// Horizontal stencil kernels and the time update.  Each kernel restates the reference routine
// named in its comment; thread = one (k, j, i) cell unless stated otherwise.
#include "device_common.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

// Cell index helpers for 3-D launches over k in [k0, k0+nk), j in [j0, j0+nj), i in 1..ni.
struct Cell { int k, j, i; };
// The index arithmetic is 32-bit unsigned (two divisions, remainders by multiply-subtract): a
// launch covers fewer than 2^31 cells of a member (epic_model_create bounds a field below 2^31
// elements), and 64-bit divisions cost as many instructions as the stencil's own loads.
__device__ __forceinline__ bool cell3(const DevModel &M, int k0, int nkk, int j0, int njj, Cell &c) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)njj;
  if (t >= (unsigned)nkk * nr * ni) return false;
  const unsigned r = t / ni, q = r / nr;
  c.i = 1 + (int)(t - r * ni);
  c.j = j0 + (int)(r - q * nr);
  c.k = k0 + (int)q;
  return true;
}
// (k, j, i) of cell t of the interior layers k = 1..nk-1, rows j = 0..nj (the wind updates)
__device__ __forceinline__ void cell_kji(const DevModel &M, unsigned t, int &k, int &j, int &i) {
  const unsigned ni = (unsigned)M.ni, nr = (unsigned)(M.nj + 1);
  const unsigned r = t / ni, q = r / nr;
  i = 1 + (int)(t - r * ni);
  j = (int)(r - q * nr);
  k = 1 + (int)q;
}
static inline unsigned cells_blocks(const DevModel &M, int nkk, int njj, int th) {
  return epic_blocks((long long)nkk * njj * M.ni, th);
}
__device__ __forceinline__ int wrap_i(const DevModel &M, int i) { return i == 0 ? M.ni : (i == M.ni + 1 ? 1 : i); }

// The copy of GZ3 that the filtered geopotential starts from, epic_timestep.c:176-181.
__global__ void k_copy_gz(DevModel M) {
  if (epic_member(M)) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < M.n3) M.gz[t] = M.gz3[t];
}

// memset of DUDT, DVDT(it_uv_tend), epic_timestep.c:107-108
__global__ void k_zero_tend(DevModel M) {
  if (epic_member(M)) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.n3) return;
  const long long off = plane_offset(M, PL_UV_TEND);
  M.dudt[off + t] = 0.;
  M.dvdt[off + t] = 0.;
}

// ---------------------------------------------------------------------------------------------
// uv_core, epic_timestep.c:628-762, with get_kin (Suarez-Takacs blend for the Sadourney scheme,
// epic_funcs_diag.c:2694-2847) and the PV averages of include/epic_pv_schemes.h:48-61.
// ---------------------------------------------------------------------------------------------

// UH(j,i) for j = 0..nj (0 above), periodic in i
template <class R>
__device__ __forceinline__ R uh_at(const DevModel &M, const double *Uk, const double *Hk, int j, int i) {
  if (j < 0 || j > M.nj) return R(0.);
  i = wrap_i(M, i);
  const R havg = R(.5) * (cv<R>(Hk[M.at2(j, i)]) + cv<R>(Hk[M.at2(j, i - 1)]));
  return cv<R>(Uk[M.at2(j, i)]) * havg * (R(1.) / cv<R>(M.n[2 * j + 1]));
}
// VH(j,i) for j = 1..nj (0 at the poles), periodic in i
template <class R>
__device__ __forceinline__ R vh_at(const DevModel &M, const double *Vk, const double *Hk, int j, int i) {
  if (j < 1 || j > M.nj) return R(0.);
  i = wrap_i(M, i);
  const R havg = R(.5) * (cv<R>(Hk[M.at2(j, i)]) + cv<R>(Hk[M.at2(j - 1, i)]));
  return cv<R>(Vk[M.at2(j, i)]) * havg * (R(1.) / cv<R>(M.m[2 * j]));
}

// Kinetic energy per mass on the h grid, planes k = 1..nk-1, into work0 (with pads).
template <class R>
__global__ void k_uv_kin(DevModel M) {
  if (epic_member(M)) return;
  Cell c;
  if (!cell3(M, 1, M.nk - 1, 0, M.nj + 1, c)) return;
  const long long off = plane_offset(M, PL_UV);
  const double *Uk = M.u + off + c.k * M.n2, *Vk = M.v + off + c.k * M.n2;
  write_with_pads(M.work0, M, M.at(c.k, c.j, 0), c.i, kin_at<R>(M, Uk, Vk, c.j, c.i));
}

// DVDT += (PV*UH terms + KIN(j-1)-KIN(j))*n, then the vertical advection of V.
template <class R>
__global__ void k_uv_core_v(DevModel M) {
  if (epic_member(M)) return;
  Cell c;
  if (!cell3(M, 1, M.nk - 1, 1, M.nj, c)) return;
  const int k = c.k, j = c.j, i = c.i;
  const long long off = plane_offset(M, PL_UV);
  const double *U = M.u + off, *V = M.v + off;
  const double *Uk = U + k * M.n2, *Hk = M.h3 + k * M.n2;
  const double *PV = M.pv3 + k * M.n2, *KIN = M.work0 + k * M.n2;
  double *D = M.dvdt + plane_offset(M, PL_UV_TEND);
  auto pv = [&](int jj, int ii) { return cv<R>(PV[M.at2(jj, ii)]); };
  const R ga = (pv(j, i) + pv(j, i + 1) + pv(j + 1, i + 1));
  const R de = (pv(j, i) + pv(j + 1, i) + pv(j, i + 1));
  const R al = (pv(j - 1, i) + pv(j, i) + pv(j, i + 1));
  const R be = (pv(j, i) + pv(j, i + 1) + pv(j - 1, i + 1));
  const R core = ((-ga * uh_at<R>(M, Uk, Hk, j, i + 1) - de * uh_at<R>(M, Uk, Hk, j, i) - al * uh_at<R>(M, Uk, Hk, j - 1, i) -
                   be * uh_at<R>(M, Uk, Hk, j - 1, i + 1)) * (R(1.) / R(12.)) +
                  cv<R>(KIN[M.at2(j - 1, i)]) - cv<R>(KIN[M.at2(j, i)])) * cv<R>(M.n[2 * j]);
  const long long x = M.at(k, j, i);
  double d = D[x] + to_d(core);
  const int kk = 2 * k + 1;
  d -= to_d(R(.5) * (cv<R>(M.w3[x]) + cv<R>(M.w3[M.at(k, j - 1, i)])) * (cv<R>(V[M.at(k - 1, j, i)]) - cv<R>(V[M.at(k + 1, j, i)])) /
                (cv<R>(M.sgth[kk - 2]) - cv<R>(M.sgth[kk + 2])));
  D[x] = d;
}

// DUDT += (PV*VH terms + KIN(i-1)-KIN(i))*m with the filtered KIN, then the vertical advection of U.
template <class R>
__global__ void k_uv_core_u(DevModel M) {
  if (epic_member(M)) return;
  Cell c;
  if (!cell3(M, 1, M.nk - 1, 0, M.nj + 1, c)) return;
  const int k = c.k, j = c.j, i = c.i;
  const long long off = plane_offset(M, PL_UV);
  const double *U = M.u + off, *V = M.v + off;
  const double *Vk = V + k * M.n2, *Hk = M.h3 + k * M.n2;
  const double *PV = M.pv3 + k * M.n2, *KIN = M.work0 + k * M.n2;
  double *D = M.dudt + plane_offset(M, PL_UV_TEND);
  auto pv = [&](int jj, int ii) { return cv<R>(PV[M.at2(jj, ii)]); };
  const R al = (pv(j, i) + pv(j + 1, i) + pv(j + 1, i + 1));
  const R be = (pv(j + 1, i - 1) + pv(j + 1, i) + pv(j, i));
  const R ga = (pv(j, i - 1) + pv(j, i) + pv(j + 1, i));
  const R de = (pv(j, i) + pv(j + 1, i) + pv(j, i + 1));
  const R core = ((al * vh_at<R>(M, Vk, Hk, j + 1, i) + be * vh_at<R>(M, Vk, Hk, j + 1, i - 1) + ga * vh_at<R>(M, Vk, Hk, j, i - 1) +
                   de * vh_at<R>(M, Vk, Hk, j, i)) * (R(1.) / R(12.)) +
                  cv<R>(KIN[M.at2(j, i - 1)]) - cv<R>(KIN[M.at2(j, i)])) * cv<R>(M.m[2 * j + 1]);
  const long long x = M.at(k, j, i);
  double d = D[x] + to_d(core);
  const int kk = 2 * k + 1;
  d -= to_d(R(.5) * (cv<R>(M.w3[x]) + cv<R>(M.w3[M.at(k, j, i - 1)])) * (cv<R>(U[M.at(k - 1, j, i)]) - cv<R>(U[M.at(k + 1, j, i)])) /
                (cv<R>(M.sgth[kk - 2]) - cv<R>(M.sgth[kk + 2])));
  D[x] = d;
}

// ---------------------------------------------------------------------------------------------
// uv_pgrad_finite_volume, epic_timestep.c:909-1273
// ---------------------------------------------------------------------------------------------

// Pole boundary rows of GZ3 (zonal means of the adjacent row), epic_timestep.c:930-998.
// One block per k; thread 0 sums in the reference order.
__global__ void k_gz_pole_rows(DevModel M) {
  if (epic_member(M)) return;
  const int k = blockIdx.x;
  __shared__ double avg[2];
  if (threadIdx.x < 2) {
    const int j = threadIdx.x == 0 ? 0 : M.nj;
    double tmp = 0.;
    for (int i = 1; i <= M.ni; i++) tmp += M.gz3[M.at(k, j, i)];
    avg[threadIdx.x] = tmp / M.ni;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= M.ni + 1; i += blockDim.x) {
    M.gz3[M.at(k, -1, i)] = avg[0];
    M.gz3[M.at(k, M.nj + 1, i)] = avg[1];
    if (M.mixed) {
      put_split(M.work1, M.at(k, -1, i), avg[0]);
      put_split(M.work1, M.at(k, M.nj + 1, i), avg[1]);
    }
  }
}

// The finite-volume force is a sum of face integrals that is unchanged when every GZ3 (or every
// P2) of the stencil moves by one constant; the mixed form evaluates it in FP32 on
// GZ3 - GZ3(k,j,i) and P2 - P2(k,j,i), which keeps the FP32 products near the size of the
// differences the force is made of.  The differences are formed in FP32 from (hi, lo) splits of
// GZ3 and P2 (put_split: hi = float(x), lo = float(x - hi), in scratch work1 and work2, written by
// the kernels that computed the two fields) as (hi_x - hi_ref) + (lo_x - lo_ref): within a
// rounding or two of the FP64 difference, with no FP64 operation per stencil point.  The FP64
// form uses the values as they are.
// Double-float (dfl, the accurate mixed form) takes the same splits and forms the differences in
// double-float: the stencil's values then carry ~48 bits, and the face integrals' cancellation
// costs no accuracy that matters.
template <class R>
struct PgradRef {
  const DevModel &M;
  float2 zr, pr;
  __device__ __forceinline__ PgradRef(const DevModel &M_, int k, int j, int i) : M(M_) {
    if constexpr (!std::is_same_v<R, double>) {
      zr = reinterpret_cast<const float2 *>(M.work1)[M.at(k, j, i)];
      pr = reinterpret_cast<const float2 *>(M.work2)[M.at(k, j, i)];
    }
  }
  static __device__ __forceinline__ R diff(float2 v, float2 r) {
    if constexpr (std::is_same_v<R, float>) return (v.x - r.x) + (v.y - r.y);
    else return dfl(v.x, v.y) - dfl(r.x, r.y);
  }
  __device__ __forceinline__ R z(long long x) const {
    if constexpr (std::is_same_v<R, double>) return M.gz3[x];
    else return diff(reinterpret_cast<const float2 *>(M.work1)[x], zr);
  }
  __device__ __forceinline__ R p(long long x) const {
    if constexpr (std::is_same_v<R, double>) return M.p2[x];
    else return diff(reinterpret_cast<const float2 *>(M.work2)[x], pr);
  }
};
// Width of a u (v) control volume in longitude (latitude), radians, between the faces at
// half-levels ii-1 and ii+1: the FP64 form subtracts the two face coordinates in the compute
// type as the reference does; the mixed form subtracts in FP64 first (FP32 face coordinates
// of up to 2 pi would lose five digits to cancellation).
template <class R>
__device__ __forceinline__ R face_width(const double *deg, int iw, int ie) {
  if constexpr (std::is_same_v<R, double>) return deg[ie] * (M_PI / 180.) - deg[iw] * (M_PI / 180.);
  else return cv<R>((deg[ie] - deg[iw]) * (M_PI / 180.));
}

// Multiplication by a power of two, exact in every compute type: a double-float scales its two
// parts (two multiplications, where the general product takes seven operations).
struct Pow2 { float c; };
template <class R>
__device__ __forceinline__ R operator*(Pow2 s, R x) { return R(s.c) * x; }
__device__ __forceinline__ dfl operator*(Pow2 s, dfl x) { return dfl(s.c * x.hi, s.c * x.lo); }

// The four quarter sums and two half sums of a face (lon_face, lat_face): in the FP64 form in
// the reference's order; the mixed forms share the pair each two of them have in common.
template <class R, class G>
__device__ __forceinline__ void face_sums(G gz, R &zb0, R &zb2, R &zt0, R &zt2, R &zb, R &zt) {
  if constexpr (std::is_same_v<R, double>) {
    zb0 = R(.25) * (gz(1, 1) + gz(1, 0) + gz(2, 1) + gz(2, 0));
    zb2 = R(.25) * (gz(1, 1) + gz(1, 2) + gz(2, 1) + gz(2, 2));
    zt0 = R(.25) * (gz(1, 1) + gz(1, 0) + gz(0, 1) + gz(0, 0));
    zt2 = R(.25) * (gz(1, 1) + gz(1, 2) + gz(0, 1) + gz(0, 2));
    zb = R(.5) * (gz(1, 1) + gz(2, 1));
    zt = R(.5) * (gz(1, 1) + gz(0, 1));
  } else {
    const R sb = gz(1, 1) + gz(2, 1), st = gz(1, 1) + gz(0, 1);
    zb0 = Pow2{.25f} * (sb + gz(1, 0) + gz(2, 0));
    zb2 = Pow2{.25f} * (sb + gz(1, 2) + gz(2, 2));
    zt0 = Pow2{.25f} * (st + gz(1, 0) + gz(0, 0));
    zt2 = Pow2{.25f} * (st + gz(1, 2) + gz(0, 2));
    zb = Pow2{.5f} * sb;
    zt = Pow2{.5f} * st;
  }
}

template <class R>
struct LonFace { R zbse, zbne, ztse, ztne, zbe, zte, pbe, pte, east; };

// East face of the u control volume at column i+c-1 (the quantities the reference carries
// from one i to the next).  z[a][b][c]: GZ3 at level k+a-1, row j+b-1, column i+c-1;
// p[a][c]: P2 at level k+a, row j, column i+c-1 (shifted by the reference values, §PgradRef).
template <class R>
__device__ __forceinline__ LonFace<R> lon_face(const DevModel &M, const R (&z)[3][3][2], const R (&p)[2][2], int c, int i) {
  auto gz = [&](int a, int b) { return z[a][b][c]; };
  LonFace<R> f;
  face_sums<R>(gz, f.zbse, f.zbne, f.ztse, f.ztne, f.zbe, f.zte);
  f.pbe = p[1][c];
  f.pte = p[0][c];
  const R a1 = f.ztne + f.ztse, b1 = f.ztne * f.ztse, a2 = f.zbne + f.zbse, b2 = f.zbne * f.zbse;
  const R terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
  const R terms2 = R(3.) * (a1 - a2);
  f.east = (-terms1 * (f.pbe - f.pte) + terms2 * (f.zte * f.pbe - f.zbe * f.pte)) / (f.zte - f.zbe);
  return f;
}

// Rows shared by a block (ni divides the block: the launcher sizes the shared memory for it):
// each cell computes its east face once and takes its west face from the cell to its left --
// for i = 1 from the row's last cell, whose face at column ni equals the face at the periodic
// column 0 bit for bit (the fields' pad columns are copies).  The faces of one row then need one
// reference: the double-float form shifts by the row's value at i = 1 instead of each cell's own
// (its differences keep ~48 bits either way); the binary32 form keeps its per-cell reference and
// computes both faces.
template <class R>
__global__ void k_pgrad_lon(DevModel M) {
  if (epic_member(M)) return;
  Cell c;
  const bool share = !std::is_same_v<R, float> && (blockDim.x % (unsigned)M.ni) == 0u;
  const bool valid = cell3(M, 1, M.nk - 1, 0, M.nj + 1, c);
  if (!share && !valid) return;
  const int k = c.k, j = c.j, i = c.i;
  const R DLOGZ_TOL = R(1.e-2);
  LonFace<R> w, e;
  if (share) {
    extern __shared__ __align__(16) unsigned char pg_smem[];
    LonFace<R> *faces = reinterpret_cast<LonFace<R> *>(pg_smem);
    if (valid) {
      const PgradRef<R> ref(M, k, j, 1);
      R z[3][3][2], p[2][2];
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) z[a][b][1] = z[a][b][0] = ref.z(M.at(k + a - 1, j + b - 1, i));
#pragma unroll
      for (int a = 0; a < 2; a++) p[a][1] = p[a][0] = ref.p(M.at(k + a, j, i));
      e = lon_face<R>(M, z, p, 1, i);
      faces[threadIdx.x] = e;
    }
    __syncthreads();
    if (!valid) return;
    w = faces[i == 1 ? threadIdx.x + (unsigned)M.ni - 1u : threadIdx.x - 1u];
  } else {
    const PgradRef<R> ref(M, k, j, i);
    R z[3][3][2], p[2][2];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++)
#pragma unroll
        for (int q = 0; q < 2; q++) z[a][b][q] = ref.z(M.at(k + a - 1, j + b - 1, i + q - 1));
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
      for (int q = 0; q < 2; q++) p[a][q] = ref.p(M.at(k + a, j, i + q - 1));
    w = lon_face<R>(M, z, p, 0, i - 1);
    e = lon_face<R>(M, z, p, 1, i);
  }
  const R rho = Pow2{.5f} * (cv<R>(M.rho3[M.at(k, j, i)]) + cv<R>(M.rho3[M.at(k, j, i - 1)]));
  const R rlns = cv<R>(M.rln[2 * j]), rlnn = cv<R>(M.rln[2 * j + 2]);
  R a1 = e.ztne + e.ztse, a2 = w.ztne + w.ztse;
  R terms2 = R(3.) * (a1 - a2), top, bottom;
  if (fabs(R(2.) * (e.zte - w.zte) / (e.zte + w.zte - e.zbe - w.zbe)) > DLOGZ_TOL) {
    const R b1 = e.ztne * e.ztse, b2 = w.ztne * w.ztse;
    const R terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
    top = (-terms1 * (w.pte - e.pte) + terms2 * (e.zte * w.pte - w.zte * e.pte)) / (e.zte - w.zte);
  } else {
    top = Pow2{.5f} * (w.pte + e.pte) * terms2;
  }
  a1 = e.zbne + e.zbse;
  a2 = w.zbne + w.zbse;
  terms2 = R(3.) * (a1 - a2);
  if (fabs(R(2.) * (e.zbe - w.zbe) / (e.zte + w.zte - e.zbe - w.zbe)) > DLOGZ_TOL) {
    const R b1 = e.zbne * e.zbse, b2 = w.zbne * w.zbse;
    const R terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
    bottom = (-terms1 * (w.pbe - e.pbe) + terms2 * (e.zbe * w.pbe - w.zbe * e.pbe)) / (e.zbe - w.zbe);
  } else {
    bottom = Pow2{.5f} * (w.pbe + e.pbe) * terms2;
  }
  R pgflon = top - bottom + R(0.) - R(0.) + w.east - e.east;
  const R dzn = e.ztne - e.zbne + w.ztne - w.zbne;
  const R dzs = e.ztse - e.zbse + w.ztse - w.zbse;
  pgflon /= face_width<R>(M.lon, 2 * i - 1, 2 * i + 1) * rho * (rlns * (dzs + Pow2{.5f} * dzn) + rlnn * (dzn + Pow2{.5f} * dzs));
  const long long x = plane_offset(M, PL_UV_TEND) + M.at(k, j, i);
  M.dudt[x] = M.dudt[x] + to_d(pgflon);
}

template <class R>
struct LatFace { R zbnw, zbne, ztnw, ztne, zbn, ztn, pbn, ptn, north, rln; };

// North face of the v control volume at row j+b-1.  z[a][b][c]: GZ3 at level k+a-1, row j+b-1,
// column i+c-1; p[a][b][c]: P2 at level k+a, row j+b-1, column i+c-1 (shifted by the reference
// values).
template <class R>
__device__ __forceinline__ LatFace<R> lat_face(const DevModel &M, const R (&z)[3][2][3], const R (&p)[2][2][3], int b, int jrow) {
  auto gz = [&](int a, int c) { return z[a][b][c]; };
  LatFace<R> f;
  f.rln = cv<R>(M.rln[2 * jrow + 1]);
  face_sums<R>(gz, f.zbnw, f.zbne, f.ztnw, f.ztne, f.zbn, f.ztn);
  f.pbn = p[1][b][1];
  f.ptn = p[0][b][1];
  const R a1 = f.ztne + f.ztnw, b1 = f.ztne * f.ztnw, a2 = f.zbne + f.zbnw, b2 = f.zbne * f.zbnw;
  const R terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
  const R terms2 = R(3.) * (a1 - a2);
  f.north = f.rln * (-terms1 * (f.pbn - f.ptn) + terms2 * (f.ztn * f.pbn - f.zbn * f.ptn)) / (f.ztn - f.zbn);
  return f;
}

template <class R>
__global__ void k_pgrad_lat(DevModel M) {
  if (epic_member(M)) return;
  Cell c;
  if (!cell3(M, 1, M.nk - 1, 1, M.nj, c)) return;
  const int k = c.k, j = c.j, i = c.i;
  const R DLOGZ_TOL = R(1.e-2);
  const PgradRef<R> ref(M, k, j, i);
  R z[3][2][3], p[2][2][3];
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int q = 0; q < 3; q++) z[a][b][q] = ref.z(M.at(k + a - 1, j + b - 1, i + q - 1));
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int q = 0; q < 3; q++) p[a][b][q] = ref.p(M.at(k + a, j + b - 1, i + q - 1));
  // z(level k+a-1, row j+b-1, column i+q-1), pp(level k+a, row j+b-1, column i+q-1)
  auto gz = [&](int a, int b, int q) { return z[a][b][q]; };
  auto pp = [&](int a, int b, int q) { return p[a][b][q]; };
  const LatFace<R> s = lat_face<R>(M, z, p, 0, j - 1), n = lat_face<R>(M, z, p, 1, j);
  const R rho = Pow2{.5f} * (cv<R>(M.rho3[M.at(k, j, i)]) + cv<R>(M.rho3[M.at(k, j - 1, i)]));
  const R rlt = cv<R>(M.rlt[2 * j]);
  const R rlns = s.rln, rlnn = n.rln;
  const R south = s.north, north = n.north;
  // s-face values carried over from row j-1: zbsw = zbnw(j-1), zbse = zbne(j-1), ...
  const R zbsw = s.zbnw, zbse = s.zbne, ztsw = s.ztnw, ztse = s.ztne;
  const R zbs = s.zbn, zts = s.ztn, pbs = s.pbn, pts = s.ptn;
  R a1, a2, b1, b2, b3, terms1, terms2;
  // levels: a = 0 (k-1), 1 (k), 2 (k+1); rows: b = 0 (j-1), 1 (j); columns: q = 0 (i-1), 1 (i), 2 (i+1)
  // the 8-point means are the means of the faces' quarter sums and the 4-point P means share their
  // centre-column pair (mixed forms; the FP64 form sums in the reference's order)
  R zbe, zte, pbe, pte, zbw, ztw, pbw, ptw;
  if constexpr (std::is_same_v<R, double>) {
    zbe = R(.125) * (gz(1, 1, 1) + gz(1, 1, 2) + gz(1, 0, 1) + gz(1, 0, 2) + gz(2, 1, 1) + gz(2, 1, 2) + gz(2, 0, 1) + gz(2, 0, 2));
    zte = R(.125) * (gz(0, 1, 1) + gz(0, 1, 2) + gz(0, 0, 1) + gz(0, 0, 2) + gz(1, 1, 1) + gz(1, 1, 2) + gz(1, 0, 1) + gz(1, 0, 2));
    pbe = R(.25) * (pp(1, 1, 1) + pp(1, 1, 2) + pp(1, 0, 1) + pp(1, 0, 2));
    pte = R(.25) * (pp(0, 1, 1) + pp(0, 1, 2) + pp(0, 0, 1) + pp(0, 0, 2));
    zbw = R(.125) * (gz(1, 1, 1) + gz(1, 1, 0) + gz(1, 0, 1) + gz(1, 0, 0) + gz(2, 1, 1) + gz(2, 1, 0) + gz(2, 0, 1) + gz(2, 0, 0));
    ztw = R(.125) * (gz(0, 1, 1) + gz(0, 1, 0) + gz(0, 0, 1) + gz(0, 0, 0) + gz(1, 1, 1) + gz(1, 1, 0) + gz(1, 0, 1) + gz(1, 0, 0));
    pbw = R(.25) * (pp(1, 1, 1) + pp(1, 1, 0) + pp(1, 0, 1) + pp(1, 0, 0));
    ptw = R(.25) * (pp(0, 1, 1) + pp(0, 1, 0) + pp(0, 0, 1) + pp(0, 0, 0));
  } else {
    zbe = Pow2{.5f} * (n.zbne + s.zbne);
    zte = Pow2{.5f} * (n.ztne + s.ztne);
    zbw = Pow2{.5f} * (n.zbnw + s.zbnw);
    ztw = Pow2{.5f} * (n.ztnw + s.ztnw);
    const R cb = pp(1, 1, 1) + pp(1, 0, 1), ct = pp(0, 1, 1) + pp(0, 0, 1);
    pbe = Pow2{.25f} * (cb + pp(1, 1, 2) + pp(1, 0, 2));
    pte = Pow2{.25f} * (ct + pp(0, 1, 2) + pp(0, 0, 2));
    pbw = Pow2{.25f} * (cb + pp(1, 1, 0) + pp(1, 0, 0));
    ptw = Pow2{.25f} * (ct + pp(0, 1, 0) + pp(0, 0, 0));
  }
  a1 = n.ztne + ztse; b1 = n.ztne * ztse; a2 = n.zbne + zbse; b2 = n.zbne * zbse;
  terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
  terms2 = R(3.) * (a1 - a2);
  const R east = Pow2{.5f} * (rlns - rlnn) * (-terms1 * (pbe - pte) + terms2 * (zte * pbe - zbe * pte)) / (zte - zbe);
  a1 = n.ztnw + ztsw; b1 = n.ztnw * ztsw; a2 = n.zbnw + zbsw; b2 = n.zbnw * zbsw;
  terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
  terms2 = R(3.) * (a1 - a2);
  const R west = Pow2{.5f} * (rlns - rlnn) * (-terms1 * (pbw - ptw) + terms2 * (ztw * pbw - zbw * ptw)) / (ztw - zbw);
  R top, bottom;
  a1 = n.ztne + n.ztnw; a2 = ztse + ztsw;
  terms2 = R(3.) * (a1 - a2);
  if (fabs(R(2.) * (n.ztn - zts) / (n.ztn + zts - n.zbn - zbs)) > DLOGZ_TOL) {
    b1 = n.ztne * n.ztnw; b2 = ztse * ztsw; b3 = n.ztne * ztse + n.ztnw * ztsw;
    terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
    top = Pow2{.5f} * ((n.ptn - pts) * ((rlnn + rlns) * terms1 + (rlnn - rlns) * (b1 + b2 - b3)) + (rlnn + rlns) * terms2 * (n.ztn * pts - zts * n.ptn)) /
          (n.ztn - zts);
  } else {
    top = Pow2{.25f} * (rlnn + rlns) * (pts + n.ptn) * terms2;
  }
  a1 = n.zbne + n.zbnw; a2 = zbse + zbsw;
  terms2 = R(3.) * (a1 - a2);
  if (fabs(R(2.) * (n.zbn - zbs) / (n.ztn + zts - n.zbn - zbs)) > DLOGZ_TOL) {
    b1 = n.zbne * n.zbnw; b2 = zbse * zbsw; b3 = n.zbne * zbse + n.zbnw * zbsw;
    terms1 = a1 * a1 - b1 - (a2 * a2 - b2);
    bottom = Pow2{.5f} * ((n.pbn - pbs) * ((rlnn + rlns) * terms1 + (rlnn - rlns) * (b1 + b2 - b3)) + (rlnn + rlns) * terms2 * (n.zbn * pbs - zbs * n.pbn)) /
             (n.zbn - zbs);
  } else {
    bottom = Pow2{.25f} * (rlnn + rlns) * (pbs + n.pbn) * terms2;
  }
  R pgflat = top - bottom + south - (north + west + east);
  const R dzn = n.ztne - n.zbne + n.ztnw - n.zbnw;
  const R dzs = ztse - zbse + ztsw - zbsw;
  pgflat /= face_width<R>(M.lat, 2 * j - 1, 2 * j + 1) * rho * rlt * (rlns * (dzs + Pow2{.5f} * dzn) + rlnn * (dzn + Pow2{.5f} * dzs));
  const long long x = plane_offset(M, PL_UV_TEND) + M.at(k, j, i);
  M.dvdt[x] = M.dvdt[x] + to_d(pgflat);
}

// ---------------------------------------------------------------------------------------------
// Meridional pass of hsu_advection, epic_flux.c:1060-1310.  kind: 0/1 interface (unity,
// THETA), 2 = HDRY (v averaged to the layer), 3 = NU_TURB (interface, floor NU_TURB_MIN).  Four launches over all planes k0..nk.
// ---------------------------------------------------------------------------------------------

template <class R>
__device__ __forceinline__ void vmp(const DevModel &M, const double *V, int kind, int k, int j, int i, R &vm, R &vp) {
  R v2d;
  if (j < 0 || j > M.nj + 1) { vm = vp = R(0.); return; }
  if (kind == 2) v2d = (j >= 1 && j <= M.nj) ? R(.5) * (cv<R>(V[M.at(k, j, i)]) + cv<R>(V[M.at(k - 1, j, i)])) : R(0.);
  else v2d = cv<R>(V[M.at(k, j, i)]);
  const R mi = (fabs(M.lat[2 * j]) == 90.) ? R(0.) : R(1.) / cv<R>(M.m[2 * j]);
  vm = rmin(R(0.), v2d * mi);
  vp = rmax(R(0.), v2d * mi);
}

template <class R>
__global__ void k_hsu_merid_pred(DevModel M, const double *A, int kind, int k0) {
  if (epic_member(M, A)) return;
  Cell c;
  if (!cell3(M, k0, M.nk - k0 + 1, 0, M.nj + 2, c)) return;   // rows 0..nj+1
  const double *V = M.v + plane_offset(M, PL_UV);
  R ff = R(0.);
  if (c.j >= 1 && c.j <= M.nj) {
    R vm, vp;
    vmp<R>(M, V, kind, c.k, c.j, c.i, vm, vp);
    ff = vp * cv<R>(A[M.at(c.k, c.j - 1, c.i)]) + vm * cv<R>(A[M.at(c.k, c.j, c.i)]);
  }
  write_with_pads(M.work1, M, M.at(c.k, c.j, 0), c.i, ff);
}

template <class R>
__global__ void k_hsu_merid_apred(DevModel M, const double *A, int k0) {
  if (epic_member(M, A)) return;
  Cell c;
  if (!cell3(M, k0, M.nk - k0 + 1, 0, M.nj + 1, c)) return;
  const double *FF = M.work1;
  const long long x = M.at(c.k, c.j, c.i);
  const R da = (cv<R>(FF[x]) - cv<R>(FF[M.at(c.k, c.j + 1, c.i)])) * cv<R>(M.mn[2 * c.j + 1]) * cv<R>(M.dt);
  write_with_pads(M.work2, M, M.at(c.k, c.j, 0), c.i, A[x] + to_d(da));
}

template <class R>
__global__ void k_hsu_merid_corr(DevModel M, const double *A, int kind, int k0) {
  if (epic_member(M, A)) return;
  Cell c;
  if (!cell3(M, k0, M.nk - k0 + 1, 0, M.nj + 2, c)) return;
  const int k = c.k, j = c.j, i = c.i, nj = M.nj;
  R ffv = R(0.);
  if (j >= 1 && j <= nj) {
    const R ep = R(1.e-10), DT = cv<R>(M.dt);
    const R a_min = kind == 2 ? cv<R>(M.h_min[k]) : (kind == 3 ? cv<R>(1.e-3 * M.kinvisc) : R(0.));
    const double *V = M.v + plane_offset(M, PL_UV);
    const double *AP = M.work2;
    auto a = [&](int jj) { return cv<R>(A[M.at(k, jj, i)]); };
    auto ap = [&](int jj) { return cv<R>(AP[M.at(k, jj, i)]); };
    auto diff1 = [&](int jj) { return jj == 0 ? R(0.) : ap(jj) - a(jj - 1); };
    auto diff2 = [&](int jj) { return jj == nj ? R(0.) : ap(jj) - a(jj + 1); };
    auto aaa = [&](int jj) {
      R t;
      if (jj == 0) t = fabs(-a(0) + a(1)) + ep;
      else if (jj == nj) t = fabs(a(nj - 1) - a(nj)) + ep;
      else t = fabs(a(jj - 1) - R(2.) * a(jj) + a(jj + 1)) + ep;
      return t * t;
    };
    R vm, vp, vmm, vpm, vmp1, vpp1;
    vmp<R>(M, V, kind, k, j, i, vm, vp);
    vmp<R>(M, V, kind, k, j - 1, i, vmm, vpm);
    vmp<R>(M, V, kind, k, j + 1, i, vmp1, vpp1);
    ffv = R(.5) * (vp * (ap(j) + a(j - 1)) + vm * (ap(j - 1) + a(j)));
    const R vhatp = sqrt(vp * vpm);
    const R vhatm = -sqrt(vm * vmp1);
    const R mu = (vp - vm) * cv<R>(M.mn[2 * j]) * DT;
    const R al = (R(1.) + mu) / R(6.);
    const R am1 = aaa(j - 1), a0 = aaa(j);
    const R prod = (a(j - 1) - a_min) * (a(j) - a_min);
    R gap = am1 / (am1 + prod); gap = gap * gap;
    R gam = a0 / (a0 + prod); gam = gam * gam;
    const R bep = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gap;
    const R bem = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gam;
    ffv += -al * (vp * bep * diff1(j) - vhatp * (R(1.) - gap) * diff1(j - 1) + vm * bem * diff2(j - 1) - vhatm * (R(1.) - gam) * diff2(j));
  }
  write_with_pads(M.work3, M, M.at(k, j, 0), i, ffv);
}

template <class R>
__global__ void k_hsu_merid_update(DevModel M, double *A, int k0) {
  if (epic_member(M, A)) return;
  Cell c;
  if (!cell3(M, k0, M.nk - k0 + 1, 0, M.nj + 1, c)) return;
  const double *FF = M.work3;
  const long long x = M.at(c.k, c.j, c.i);
  const R da = (cv<R>(FF[x]) - cv<R>(FF[M.at(c.k, c.j + 1, c.i)])) * cv<R>(M.mn[2 * c.j + 1]) * cv<R>(M.dt);
  write_with_pads(A, M, M.at(c.k, c.j, 0), c.i, A[x] + to_d(da));
}

// The four meridional passes fused: one thread per (k, i) marches j = 0..nj and keeps, in a
// sliding register window, the original field A at rows j-2..j+2 (A is updated in place behind
// the march), the split velocity at rows j-1..j+2, the predictor fluxes FF at j+1, j+2, the
// predicted field AP at j-1..j+1 and the corrector flux FFV at j.  Every value is the same
// expression on the same operands as in the four passes (k_hsu_merid_pred/apred/corr/update),
// so the results are identical bit for bit, with no scratch traffic.  Row j+3's loads are issued
// at the top of iteration j, ahead of the arithmetic that does not need them.
template <class R>
__global__ void k_hsu_meridional(DevModel M, double *A, int kind, int k0) {
  if (epic_member(M, A)) return;
  const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  const int k = k0 + (int)blockIdx.y;
  if (i > M.ni) return;
  const int nj = M.nj;
  const double *V = M.v + plane_offset(M, PL_UV);
  const R ep = R(1.e-10), DT = cv<R>(M.dt);
  const R a_min = kind == 2 ? cv<R>(M.h_min[k]) : (kind == 3 ? cv<R>(1.e-3 * M.kinvisc) : R(0.));
  auto ld = [&](int jj) { return A[M.at(k, jj, i)]; };
  auto ff_of = [&](int jj, R vm, R vp, R am1, R a0) { return (jj >= 1 && jj <= nj) ? vp * am1 + vm * a0 : R(0.); };
  auto ap_of = [&](int jj, double ad, R ff0, R ff1) { return cv<R>(ad + to_d((ff0 - ff1) * cv<R>(M.mn[2 * jj + 1]) * DT)); };
  // window at the top of iteration j
  R a_m2 = R(0.), a_m1 = R(0.), a_0, a_1, a_2;   // A(j-2..j+2)
  double ad_0, ad_1, ad_2;                       // A(j..j+2) in binary64
  R vm_m1 = R(0.), vp_m1 = R(0.), vm_0, vp_0, vm_1, vp_1, vm_2, vp_2;   // split velocity at j-1..j+2
  R ff_1, ff_2;                                  // FF(j+1), FF(j+2)
  R ap_m1 = R(0.), ap_0, ap_1;                   // AP(j-1..j+1)
  R ffv_0 = R(0.);                               // FFV(j); FFV(0) = 0
  ad_0 = ld(0); ad_1 = ld(1); ad_2 = ld(2);
  a_0 = cv<R>(ad_0); a_1 = cv<R>(ad_1); a_2 = cv<R>(ad_2);
  vmp<R>(M, V, kind, k, 0, i, vm_0, vp_0);
  vmp<R>(M, V, kind, k, 1, i, vm_1, vp_1);
  vmp<R>(M, V, kind, k, 2, i, vm_2, vp_2);
  {
    const R ff_0 = R(0.);   // FF(0): row 0 is outside 1..nj
    ff_1 = ff_of(1, vm_1, vp_1, a_0, a_1);
    ff_2 = ff_of(2, vm_2, vp_2, a_1, a_2);
    ap_0 = ap_of(0, ad_0, ff_0, ff_1);
    ap_1 = ap_of(1, ad_1, ff_1, ff_2);
  }
  // aaa(jj) of the reference from a(jj-1), a(jj), a(jj+1)
  auto aaa = [&](int jj, R am, R a0v, R ap1) {
    R t;
    if (jj == 0) t = fabs(-a0v + ap1) + ep;
    else if (jj == nj) t = fabs(am - a0v) + ep;
    else t = fabs(am - R(2.) * a0v + ap1) + ep;
    return t * t;
  };
  for (int j = 0; j <= nj; j++) {
    // row j+3's inputs (rows beyond nj+1 do not exist and are not used)
    const int j3 = j + 3;
    double ad_3 = 0.;
    R vm_3 = R(0.), vp_3 = R(0.);
    if (j3 <= nj + 1) {
      ad_3 = ld(j3);
      vmp<R>(M, V, kind, k, j3, i, vm_3, vp_3);
    }
    // FFV(j+1): the corrector flux of row jj = j+1 (k_hsu_merid_corr)
    R ffv_1 = R(0.);
    const int jj = j + 1;
    if (jj >= 1 && jj <= nj) {
      const R diff1_jj = ap_1 - a_0;                              // diff1(jj), jj >= 1
      const R diff1_jm = (jj - 1 == 0) ? R(0.) : ap_0 - a_m1;     // diff1(jj-1)
      const R diff2_jm = (jj - 1 == nj) ? R(0.) : ap_0 - a_1;     // diff2(jj-1)
      const R diff2_jj = (jj == nj) ? R(0.) : ap_1 - a_2;         // diff2(jj)
      R f = R(.5) * (vp_1 * (ap_1 + a_0) + vm_1 * (ap_0 + a_1));
      const R vhatp = sqrt(vp_1 * vp_0);
      const R vhatm = -sqrt(vm_1 * vm_2);
      const R mu = (vp_1 - vm_1) * cv<R>(M.mn[2 * jj]) * DT;
      const R al = (R(1.) + mu) / R(6.);
      const R am1 = aaa(jj - 1, a_m1, a_0, a_1), a0 = aaa(jj, a_0, a_1, a_2);
      const R prod = (a_0 - a_min) * (a_1 - a_min);
      R gap = am1 / (am1 + prod); gap = gap * gap;
      R gam = a0 / (a0 + prod); gam = gam * gam;
      const R bep = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gap;
      const R bem = R(1.) + (R(1.) / (R(2.) * al) - R(1.)) * gam;
      f += -al * (vp_1 * bep * diff1_jj - vhatp * (R(1.) - gap) * diff1_jm + vm_1 * bem * diff2_jm - vhatm * (R(1.) - gam) * diff2_jj);
      ffv_1 = f;
    }
    // the update of row j (k_hsu_merid_update)
    const R da = (ffv_0 - ffv_1) * cv<R>(M.mn[2 * j + 1]) * cv<R>(M.dt);
    write_with_pads(A, M, M.at(k, j, 0), i, ad_0 + to_d(da));
    // advance the window to j+1: FF(j+3), AP(j+2)
    const R a_3 = cv<R>(ad_3);
    const R ff_3 = ff_of(j3, vm_3, vp_3, a_2, a_3);
    const R ap_2 = (j + 2 <= nj) ? ap_of(j + 2, ad_2, ff_2, ff_3) : R(0.);
    a_m2 = a_m1; a_m1 = a_0; a_0 = a_1; a_1 = a_2; a_2 = a_3;
    ad_0 = ad_1; ad_1 = ad_2; ad_2 = ad_3;
    vm_m1 = vm_0; vp_m1 = vp_0; vm_0 = vm_1; vp_0 = vp_1; vm_1 = vm_2; vp_1 = vp_2; vm_2 = vm_3; vp_2 = vp_3;
    ff_1 = ff_2; ff_2 = ff_3;
    ap_m1 = ap_0; ap_0 = ap_1; ap_1 = ap_2;
    ffv_0 = ffv_1;
  }
  (void)a_m2; (void)vm_m1; (void)vp_m1; (void)ap_m1;
}

// ---------------------------------------------------------------------------------------------
// Meridional pass of akima_advection, epic_flux.c:1752-1820.  kind: 0/1 interface (unity,
// THETA; V of the interface), 2 = HDRY (V averaged to the layer).  Two launches over planes
// k0..nk: the fluxes FF (v rows 1..nj, into work3), then the update of rows 0..nj.
// ---------------------------------------------------------------------------------------------

template <class R>
__device__ __forceinline__ R akima_mean(R d0, R d1) {   // the dela of akima_advection
  const R tmp = d0 * d1;
  return (tmp > R(0.)) ? R(2.) * tmp / (d0 + d1) : R(0.);
}

template <class R>
__global__ void k_akima_merid_flux(DevModel M, const double *A, int kind, int k0) {
  if (epic_member(M, A)) return;
  Cell c;
  if (!cell3(M, k0, M.nk - k0 + 1, 1, M.nj, c)) return;   // v rows 1..nj
  const int k = c.k, j = c.j, i = c.i, nj = M.nj;
  auto a = [&](int jj) { return cv<R>(A[M.at(k, jj, i)]); };
  // deltaa(jj) = A(jj) - A(jj-1) on rows 1..nj, 0 elsewhere
  auto deltaa = [&](int jj) { return (jj < 1 || jj > nj) ? R(0.) : a(jj) - a(jj - 1); };
  const R dl_j = akima_mean<R>(deltaa(j), deltaa(j + 1));
  const R dl_jm = akima_mean<R>(deltaa(j - 1), deltaa(j));
  const double *V = M.v + plane_offset(M, PL_UV);
  const R v2d = kind == 2 ? R(.5) * (cv<R>(V[M.at(k, j, i)]) + cv<R>(V[M.at(k - 1, j, i)])) : cv<R>(V[M.at(k, j, i)]);
  const R m_2j_inv = (fabs(M.lat[2 * j]) == 90.) ? R(0.) : R(1.) / cv<R>(M.m[2 * j]);
  const R aval = R(.5) * (a(j) + a(j - 1)) - (dl_j - dl_jm) / R(6.);
  write_with_pads(M.work3, M, M.at(k, j, 0), i, to_d(v2d * aval * m_2j_inv));
}

template <class R>
__global__ void k_akima_merid_update(DevModel M, double *A, int k0) {
  if (epic_member(M, A)) return;
  Cell c;
  if (!cell3(M, k0, M.nk - k0 + 1, 0, M.nj + 1, c)) return;   // rows 0..nj
  const int k = c.k, j = c.j, nj = M.nj;
  const double *FF = M.work3;
  auto ff = [&](int jj) { return (jj < 1 || jj > nj) ? R(0.) : cv<R>(FF[M.at(k, jj, c.i)]); };
  const long long x = M.at(k, j, c.i);
  const R da = (ff(j) - ff(j + 1)) * cv<R>(M.mn[2 * j + 1]) * cv<R>(M.dt);
  write_with_pads(A, M, M.at(k, j, 0), c.i, A[x] + to_d(da));
}

// ---------------------------------------------------------------------------------------------
// Hyperviscosity, epic_subgrid.c:590-1232
// ---------------------------------------------------------------------------------------------

// d2dy2 of planes k0..k1 of src into dst (coefficients per row from the init block, :1049-1141).
template <class R>
__global__ void k_d2dy2(DevModel M, const double *src, int src_sel, double *dst, int vgrid, int order, int k0, int nkk,
                        int of_state) {
  if (epic_member(M, src, dst)) return;
  // the member's own coefficient (it depends on dt and dy0): order 2, 4, 6 or 8, constant indices
  const double diff_coef = order == 2 ? M.coef[2] : (order == 4 ? M.coef[4] : (order == 6 ? M.coef[6] : M.coef[8]));
  Cell c;
  const int nrows = vgrid ? M.nj + 2 : M.nj + 1;   // v: j = 0..nj+1, h: j = 0..nj
  if (!cell3(M, k0, nkk, 0, nrows, c)) return;
  src += plane_offset(M, src_sel);
  const int k = c.k, j = c.j, i = c.i, nj = M.nj;
  const double *cf = (vgrid ? M.v_coef : M.h_coef) + 3 * j;
  const R a0 = cv<R>(diff_coef) * cv<R>(cf[0]), a1 = cv<R>(diff_coef) * cv<R>(cf[1]), a2 = cv<R>(diff_coef) * cv<R>(cf[2]);
  auto h = [&](int jj) { return cv<R>(src[M.at(k, jj, i)]); };
  R d;
  const int jlast = vgrid ? nj + 1 : nj;
  if (!std::is_same_v<R, double> && of_state) {
    // The mixed forms' second difference of a state field: the three coefficients sum to zero
    // (to ~1e-14 of the largest), so the stencil is a0 (h0 - h1) + a2 (h2 - h1) with the
    // differences taken in binary64 -- in binary32 the field's own rounding (1e-7 of its value,
    // 1e-4 of a neighbour difference) would enter the hyperviscous increment every step.
    const int m = j == 0 ? 1 : (j == jlast ? j - 1 : j);
    const double hm = src[M.at(k, m, i)];
    d = a0 * cv<R>(src[M.at(k, m - 1, i)] - hm) + a2 * cv<R>(src[M.at(k, m + 1, i)] - hm);
  } else if (j == 0) d = a0 * h(0) + a1 * h(1) + a2 * h(2);
  else if (j == jlast) d = a0 * h(j - 2) + a1 * h(j - 1) + a2 * h(j);
  else d = a0 * h(j - 1) + a1 * h(j) + a2 * h(j + 1);
  write_with_pads(dst, M, M.at(k, j, 0), i, d);
}

// The mixed forms' first two d2dy2 passes of meridional_hyperviscosity in one kernel: the first
// (of the state field, binary64 differences as in k_d2dy2) into shared memory, the second from
// there into dst.  Block = 32 columns of one layer k0 + blockIdx.y, every row; the values are
// those of two k_d2dy2<float> launches (the intermediate is a float either way), without the
// intermediate volume's write and read.
__global__ void k_d2dy2_pair_mixed(DevModel M, const double *src, int src_sel, double *dst, int vgrid, int k0) {
  if (epic_member(M, src, dst)) return;
  const double coef1 = M.coef[2], coef2 = M.coef[4];
  extern __shared__ __align__(16) unsigned char smraw[];
  float *d1 = reinterpret_cast<float *>(smraw);   // [row][lane]
  src += plane_offset(M, src_sel);
  const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5), nw = (int)(blockDim.x >> 5);
  const int i = (int)blockIdx.x * 32 + lane + 1;
  const int k = k0 + (int)blockIdx.y;
  const int nj = M.nj, jlast = vgrid ? nj + 1 : nj;
  const double *cfa = vgrid ? M.v_coef : M.h_coef;
  const bool live = i <= M.ni;
  for (int j = w; j <= jlast; j += nw) {
    float d = 0.f;
    if (live) {
      const double *cf = cfa + 3 * j;
      const float a0 = d2f(coef1) * d2f(cf[0]), a2 = d2f(coef1) * d2f(cf[2]);
      const int m = j == 0 ? 1 : (j == jlast ? j - 1 : j);
      const double hm = src[M.at(k, m, i)];
      d = a0 * d2f(src[M.at(k, m - 1, i)] - hm) + a2 * d2f(src[M.at(k, m + 1, i)] - hm);
    }
    d1[j * 32 + lane] = d;
  }
  __syncthreads();
  if (!live) return;
  for (int j = w; j <= jlast; j += nw) {
    const double *cf = cfa + 3 * j;
    const float a0 = d2f(coef2) * d2f(cf[0]), a1 = d2f(coef2) * d2f(cf[1]), a2 = d2f(coef2) * d2f(cf[2]);
    const int m = j == 0 ? 1 : (j == jlast ? j - 1 : j);
    const float d = a0 * d1[(m - 1) * 32 + lane] + a1 * d1[m * 32 + lane] + a2 * d1[(m + 1) * 32 + lane];
    write_with_pads(dst, M, M.at(k, j, 0), i, f2d(d));
  }
}

// A += dt*sign*D over the rows the reference updates (v: 1..nj, h: 0..nj).
template <class R>
__global__ void k_visc_apply(DevModel M, double *A, int sel, const double *D, int vgrid, double sign, int k0, int nkk) {
  if (epic_member(M, A, D)) return;
  Cell c;
  if (!cell3(M, k0, nkk, vgrid ? 1 : 0, vgrid ? M.nj : M.nj + 1, c)) return;
  A += plane_offset(M, sel);
  const long long x = M.at(c.k, c.j, c.i);
  write_with_pads(A, M, M.at(c.k, c.j, 0), c.i, A[x] + to_d(cv<R>(M.dt) * cv<R>(sign) * cv<R>(D[x])));
}

// zonal_hyperviscosity, epic_subgrid.c:715-808: one warp per row (j, k), rows_per_block rows
// per block.  The updated row stays in FP64 in both forms.  The FP64 form sums the row mean in
// the reference's order on lane 0; the mixed form sums it in FP64 with a warp reduction.
template <class R>
__global__ void k_zonal_visc(DevModel M, double *A, int sel, int jbot, int jhalf, int k0, int restore) {
  if (epic_member(M, A)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ni = M.ni, lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5), nw = (int)(blockDim.x >> 5);
  const int j = jbot + (int)blockIdx.x * nw + w;
  const int k = k0 + (int)blockIdx.y;
  if (j > M.nj) return;
  A += plane_offset(M, sel);
  const long long base = M.at(k, j, 0);
  const size_t row_bytes = (size_t)(ni + 2) * (sizeof(double) + 2 * sizeof(R));
  double *a = reinterpret_cast<double *>(smraw + w * row_bytes);
  R *hh = reinterpret_cast<R *>(a + (ni + 2)), *d = hh + (ni + 2);
  const unsigned full = 0xffffffffu;
  for (int i = lane; i <= ni + 1; i += 32) { a[i] = A[base + i]; hh[i] = cv<R>(a[i]); }
  __syncwarp();
  if (!std::is_same_v<R, double>) {
    // the mixed forms' first second difference is of the field itself: its neighbour
    // differences a(i+1) - a(i) in binary64, one per point (k_d2dy2)
    for (int i = lane; i <= ni; i += 32) hh[i] = cv<R>(a[i + 1] - a[i]);
    __syncwarp();
  }
  const bool taper = fabs(M.lat[2 * j + jhalf]) > M.lat0;
  const double mm = M.m[2 * j + jhalf];
  R sign = R(1.);
  bool any_applied = false;
  // fully unrolled so that M.coef[], M.nu[] are indexed by constants (M stays in registers)
#pragma unroll
  for (int itmp = 2; itmp <= 8; itmp += 2) {
    const R dc = cv<R>(taper ? M.coef[itmp] * M.m0 * M.m0 : M.coef[itmp] * mm * mm);
    if (!std::is_same_v<R, double> && itmp == 2)   // differences of the neighbour differences
      for (int i = lane + 1; i <= ni; i += 32) d[i] = dc * (hh[i] - hh[i - 1]);
    else
      for (int i = lane + 1; i <= ni; i += 32) d[i] = dc * (hh[i - 1] - R(2.) * hh[i] + hh[i + 1]);
    __syncwarp();
    R mean;
    if (sizeof(R) == sizeof(double)) {
      double mv = 0.;
      if (lane == 0) {
        d[ni + 1] = d[1];
        d[0] = d[ni];
        double fm = 0.;
        for (int i = 1; i <= ni; i++) fm += d[i];
        mv = fm / ni;
      }
      mean = cv<R>(__shfl_sync(full, mv, 0));
    } else {
      // the row sum of a periodic second difference vanishes but for rounding: FP32 suffices
      float fm = 0.f;
      for (int i = lane + 1; i <= ni; i += 32) fm += d[i];
      for (int o = 16; o > 0; o >>= 1) fm += __shfl_xor_sync(full, fm, o);
      mean = fm / (float)ni;
      if (lane == 0) {
        d[ni + 1] = d[1];
        d[0] = d[ni];
      }
    }
    __syncwarp();
    for (int i = lane; i <= ni + 1; i += 32) d[i] -= mean;
    __syncwarp();
    if (M.nu[itmp] > 0.) {
      for (int i = lane + 1; i <= ni; i += 32) a[i] += to_d(cv<R>(M.dt) * sign * d[i]);
      any_applied = true;
    }
    sign = -sign;
    double rest = 0.;
#pragma unroll
    for (int q = itmp + 2; q <= 8; q += 2) rest += M.nu[q];
    if (!(rest > 0.)) break;
    for (int i = lane; i <= ni + 1; i += 32) hh[i] = d[i];   // swap roles
    __syncwarp();
  }
  __syncwarp();
  // restore (HDRY): restore_mass, which the hyperviscosity step calls next (epic_subgrid.c:240),
  // on the new row -- the same max per cell, one pass fewer
  if (any_applied || restore)
    for (int i = lane + 1; i <= ni; i += 32) write_with_pads(A, M, base, i, restore ? dmaxr(M.h_min[k], a[i]) : a[i]);
}

// ---------------------------------------------------------------------------------------------
// divergence, vorticity, store_diag (epic_funcs_diag.c:3963-4445) and the Richardson number
// ---------------------------------------------------------------------------------------------

// DIV(j,i) of (UU, VV) on planes k0.., divergence() :4064-4117
template <class R>
__device__ __forceinline__ R div_at(const DevModel &M, const double *UU, const double *VV, int k, int j, int i) {
  const int jj = 2 * j + 1;
  const R n_inv = R(1.) / cv<R>(M.n[jj]);
  const R mn1 = cv<R>(M.mn[jj]);
  const R m2j_inv = (j == 0) ? R(0.) : R(1.) / cv<R>(M.m[jj - 1]);
  const R m2jp2_inv = (j == M.nj) ? R(0.) : R(1.) / cv<R>(M.m[jj + 1]);
  return mn1 * ((cv<R>(UU[M.at(k, j, i + 1)]) * n_inv - cv<R>(UU[M.at(k, j, i)]) * n_inv) +
                (cv<R>(VV[M.at(k, j + 1, i)]) * m2jp2_inv - cv<R>(VV[M.at(k, j, i)]) * m2j_inv));
}

template <class R>
__global__ void k_divergence(DevModel M, const double *UU, const double *VV, int vsel, double *DI, int k0, int nkk) {
  if (epic_member(M, UU, VV, DI)) return;
  Cell c;
  if (!cell3(M, k0, nkk, 0, M.nj + 1, c)) return;
  VV += plane_offset(M, vsel);
  write_with_pads(DI, M, M.at(c.k, c.j, 0), c.i, div_at<R>(M, UU, VV, c.k, c.j, c.i));
}

// Interior potential vorticity, vorticity(ON_SIGMATHETA, POTENTIAL) :4168-4186, planes 0..nk.
template <class R>
__global__ void k_pv_interior(DevModel M, const double *VV) {
  if (epic_member(M, VV)) return;
  Cell c;
  if (!cell3(M, 0, M.nk + 1, 1, M.nj, c)) return;
  const int k = c.k, j = c.j, i = c.i;
  const double *UU = M.u + plane_offset(M, PL_UV);
  const double *HH = M.h3;
  const R f2j = cv<R>(M.f[2 * j]), m2j = cv<R>(M.m[2 * j]), n2j = cv<R>(M.n[2 * j]);
  const R m_m1_inv = R(1.) / cv<R>(M.m[2 * j - 1]), m_p1_inv = R(1.) / cv<R>(M.m[2 * j + 1]);
  const R mn_m1_inv = R(1.) / cv<R>(M.mn[2 * j - 1]), mn_p1_inv = R(1.) / cv<R>(M.mn[2 * j + 1]);
  const R mn_pv = R(.5) / (mn_m1_inv + mn_p1_inv);
  const R ze = m2j * ((cv<R>(VV[M.at(k, j, i)]) - cv<R>(VV[M.at(k, j, i - 1)])) +
                      n2j * (cv<R>(UU[M.at(k, j - 1, i)]) * m_m1_inv - cv<R>(UU[M.at(k, j, i)]) * m_p1_inv));
  R pv = (ze + f2j);
  const R h_pv = ((cv<R>(HH[M.at(k, j, i)]) + cv<R>(HH[M.at(k, j, i - 1)])) * mn_p1_inv +
                  (cv<R>(HH[M.at(k, j - 1, i)]) + cv<R>(HH[M.at(k, j - 1, i - 1)])) * mn_m1_inv) * mn_pv;
  pv /= h_pv;
  write_with_pads(M.pv3, M, M.at(k, j, 0), i, pv);
}

// Polar potential vorticity from the circulation of the adjacent u row, :4279-4341.
// One block per plane; thread 0 forms the sums in the reference order.
__global__ void k_pv_poles(DevModel M) {
  if (epic_member(M)) return;
  const int k = blockIdx.x;
  const double *UU = M.u + plane_offset(M, PL_UV);
  const double *HH = M.h3;
  __shared__ double pole[2];
  // the four rows are staged by every thread, then summed by one thread in the reference's order
  extern __shared__ double rows[];   // [4][ni]: U(j=0), H(j=0), U(j=nj), H(j=nj)
  const int ni = M.ni, J = M.nj;
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    rows[i] = UU[M.at(k, 0, i + 1)];
    rows[ni + i] = HH[M.at(k, 0, i + 1)];
    rows[2 * ni + i] = UU[M.at(k, J, i + 1)];
    rows[3 * ni + i] = HH[M.at(k, J, i + 1)];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ze = 0., h = 0.;
    for (int i = 0; i < ni; i++) ze -= rows[i];
    ze *= M.mn[0] / ((M.m[1]) * (double)(M.ni));
    for (int i = 0; i < ni; i++) h += rows[ni + i];
    h /= (double)(M.ni);
    pole[0] = (ze + M.f[0]) / h;
    ze = 0.; h = 0.;
    for (int i = 0; i < ni; i++) ze += rows[2 * ni + i];
    ze *= M.mn[2 * (J + 1)] / (M.m[2 * J + 1] * (double)(M.ni));
    for (int i = 0; i < ni; i++) h += rows[3 * ni + i];
    h /= (double)(M.ni);
    pole[1] = (ze + M.f[2 * (J + 1)]) / h;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= M.ni + 1; i += blockDim.x) {
    M.pv3[M.at(k, 0, i)] = pole[0];
    M.pv3[M.at(k, M.nj + 1, i)] = pole[1];
  }
}

// Richardson number in the layers, get_richardson/get_brunt2 (:2885-3156).  The V term of
// dvdz2 keeps the reference's sign slip (:3127-3128); only dudz2 decides the 1e6 branch.
template <class R>
__global__ void k_ri2(DevModel M) {
  if (epic_member(M)) return;
  Cell c;
  if (!cell3(M, 1, M.nk, 0, M.nj + 1, c)) return;
  const int k = c.k, j = c.j, i = c.i;
  const long long off = plane_offset(M, PL_UV);
  const double *U = M.u + off, *V = M.v + off;
  auto u = [&](int kk, int jj, int ii) { return cv<R>(U[M.at(kk, jj, ii)]); };
  auto v = [&](int kk, int jj, int ii) { return cv<R>(V[M.at(kk, jj, ii)]); };
  R dudz2 = R(.5) * (u(k - 1, j, i) + u(k - 1, j, i + 1) - u(k, j, i) - u(k, j, i + 1));
  R dvdz2 = R(.5) * (v(k - 1, j, i) + v(k - 1, j + 1, i) - v(k, j, i) + v(k, j + 1, i));
  dudz2 *= dudz2;
  dvdz2 *= dvdz2;
  R ri;
  if (RMath<R>::cmp(dudz2, R(0.)) != 0) {
    const long long x = M.at(k, j, i);
    const R pressure = cv<R>(M.p2[x]), temperature = cv<R>(M.t2[x]), density = cv<R>(M.rho2[x]);
    const R cp = R(1004.), mu = cv<R>(M.mu_dry);
    const R deltap = R(0.001) * pressure, deltaT = R(0.001) * temperature;
    auto dens = [&](R p, R t) { return p * mu / (R(8.314472e+3) * t); };   // return_density
    const R drho_dp_T = (dens(pressure + deltap, temperature) - dens(pressure - deltap, temperature)) / (R(2.) * deltap);
    const R drho_dT_p = (dens(pressure, temperature + deltaT) - dens(pressure, temperature - deltaT)) / (R(2.) * deltaT);
    const R Drho_Dp = (cv<R>(M.rho3[x]) - cv<R>(M.rho3[M.at(k - 1, j, i)])) / (cv<R>(M.p3[x]) - cv<R>(M.p3[M.at(k - 1, j, i)]));
    const R g = cv<R>(M.grav[2 * j + 1]);
    const R brunt2 = g * g * (Drho_Dp - drho_dp_T + temperature / (cp * density * density) * drho_dT_p * drho_dT_p);
    ri = brunt2 / (dudz2 + dvdz2);
  } else {
    ri = R(1.e+6);
  }
  write_with_pads(M.ri2, M, M.at(k, j, 0), i, ri);
}

// divergence_damping apply step, epic_subgrid.c:1857-1881 (DIV from k_divergence in work2).
template <class R>
__global__ void k_divdamp_apply(DevModel M) {
  if (epic_member(M)) return;
  const double nudiv = M.nudiv;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned per = (unsigned)(M.nk - 1) * (unsigned)(M.nj + 1) * (unsigned)M.ni;
  if (t >= 2 * per) return;
  const int isv = t >= per;
  int i, j, k;
  cell_kji(M, isv ? t - per : t, k, j, i);
  const double *DIV = M.work2;
  const long long off = plane_offset(M, PL_UV_TEND);
  if (!isv) {
    const R coef = cv<R>((M.lat[2 * j + 1] > M.lat0) ? nudiv * M.m0 : nudiv * M.m[2 * j + 1]);
    const long long x = off + M.at(k, j, i);
    M.dudt[x] = M.dudt[x] + to_d(coef * (cv<R>(DIV[M.at(k, j, i)]) - cv<R>(DIV[M.at(k, j, i - 1)])));
  } else if (j >= 1) {
    const R coef = cv<R>(nudiv * M.n[2 * j]);
    const long long x = off + M.at(k, j, i);
    M.dvdt[x] = M.dvdt[x] + to_d(coef * (cv<R>(DIV[M.at(k, j, i)]) - cv<R>(DIV[M.at(k, j - 1, i)])));
  }
}

// ---------------------------------------------------------------------------------------------
// Time update: adams_bashforth_step / leapfrog_step (epic_timestep.c:406-615), the index
// rotation (:257-274) and timeplane_bookkeeping (epic_funcs_diag.c:7086-7124).
// ---------------------------------------------------------------------------------------------

__global__ void k_uv_decide(DevModel M) {
  if (epic_member(M)) return;
  Ctl *c = M.ctl;
  for (int w = 0; w < 2; w++) {
    const double *val = w == 0 ? M.u : M.v, *ten = w == 0 ? M.dudt : M.dvdt;
    const int jlo = w == 0 ? 0 : 1;
    const long long cell = M.at(1, jlo, 1);
    if (M.uv_scheme == EPIC_UV_AB3) {
      double *ab = c->ab[w];
      if (ten[(long long)c->it_minus2 * M.n3 + cell] == DBL_MAX) {
        if (ten[(long long)c->it_minus1 * M.n3 + cell] == DBL_MAX) { ab[0] = 1.; ab[1] = 0.; ab[2] = 0.; }
        else { ab[0] = 3. / 2.; ab[1] = -1. / 2.; ab[2] = 0.; }
      } else { ab[0] = 23. / 12.; ab[1] = -16. / 12.; ab[2] = 5. / 12.; }
      for (int q = 0; q < 3; q++) {
        const dfl d = d2df(ab[q]);
        c->abf[w][q] = make_float2(d.hi, d.lo);
      }
    } else {
      c->lf_first[w] = val[(long long)c->it_minus1 * M.n3 + cell] == DBL_MAX;
    }
  }
}

__global__ void k_uv_update(DevModel M) {
  if (epic_member(M)) return;
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned per = (unsigned)(M.nk - 1) * (unsigned)(M.nj + 1) * (unsigned)M.ni;
  if (t >= 2 * per) return;
  const int w = t >= per;
  int i, j, k;
  cell_kji(M, w ? t - per : t, k, j, i);
  if (w == 1 && j == 0) return;   // v is updated for j = 1..nj
  const Ctl *c = M.ctl;
  double *val = w == 0 ? M.u : M.v;
  const double *ten = w == 0 ? M.dudt : M.dvdt;
  const long long x = M.at(k, j, i), base = M.at(k, j, 0);
  const double DT = M.dt;
  if (M.uv_scheme == EPIC_UV_AB3 && M.mixed) {
    // the mixed forms: the Adams-Bashforth sum in double-float on the integer and FP32 pipes
    // (~1e-14 of the increment) added to the binary64 wind -- one FP64 addition a point instead
    // of seven, which had put this kernel at the FP64 unit's rate
    // (a zero coefficient -- the first steps -- drops its term: the planes not yet written hold
    // the DBL_MAX marker, which has no binary32 part)
    const float2 *ab = c->abf[w];
    double *X = val + (long long)c->it_uv * M.n3;
    dfl s = dfl(ab[0].x, ab[0].y) * d2df(ten[(long long)c->it_zero * M.n3 + x]);
    if (ab[1].x != 0.f) s += dfl(ab[1].x, ab[1].y) * d2df(ten[(long long)c->it_minus1 * M.n3 + x]);
    if (ab[2].x != 0.f) s += dfl(ab[2].x, ab[2].y) * d2df(ten[(long long)c->it_minus2 * M.n3 + x]);
    write_with_pads(X, M, base, i, X[x] + df2d(dfl(d2f(M.dt), 0.f) * s));
  } else if (M.uv_scheme == EPIC_UV_AB3) {
    const double *ab = c->ab[w];
    double *X = val + (long long)c->it_uv * M.n3;
    const double v = X[x] + DT * (ab[0] * ten[(long long)c->it_zero * M.n3 + x] + ab[1] * ten[(long long)c->it_minus1 * M.n3 + x] +
                                  ab[2] * ten[(long long)c->it_minus2 * M.n3 + x]);
    write_with_pads(X, M, base, i, v);
  } else {
    double *X0 = val + (long long)c->it_zero * M.n3, *Xm1 = val + (long long)c->it_minus1 * M.n3;
    const double d = ten[(long long)c->it_uv_tend * M.n3 + x];
    if (c->lf_first[w]) {
      write_with_pads(Xm1, M, base, i, X0[x] + DT * d);
    } else {
      const double old_filtered = Xm1[x], present = X0[x];
      const double new_leap = old_filtered + 2. * DT * d;
      write_with_pads(Xm1, M, base, i, new_leap);
      write_with_pads(X0, M, base, i, present * (1. - 2. * 0.06) + 0.06 * (old_filtered + new_leap));
    }
  }
}

__global__ void k_uv_rotate(DevModel M) {
  if (epic_member(M)) return;
  Ctl *c = M.ctl;
  if (M.uv_scheme == EPIC_UV_AB3) {
    const int itmp = c->it_minus2;
    c->it_minus2 = c->it_minus1;
    c->it_minus1 = c->it_zero;
    c->it_zero = itmp;
    c->it_uv = 0;
    c->it_uv_dis = 0;
    c->it_uv_tend = c->it_zero;
  } else {
    const int itmp = c->it_minus1;
    c->it_minus1 = c->it_zero;
    c->it_zero = itmp;
    c->it_uv = c->it_zero;
    c->it_uv_dis = (M.u[(long long)c->it_minus1 * M.n3 + M.at(1, 0, 1)] == DBL_MAX) ? c->it_zero : c->it_minus1;
    c->it_uv_tend = 0;
  }
  c->model_time += (long long)M.dt;
}

// End of a step: grid.itime += 1 (the driver loop, epic_main.c:424); a step that recorded a fatal
// error instead halts the model, as the reference's epic_error() ends the run in that step.
__global__ void k_itime_advance(DevModel M) {
  if (epic_member(M)) return;
  if (M.ctl->err_code != 0) M.ctl->halted = 1;
  else M.ctl->itime += 1;
}

// grid.itime as the caller's driver loop holds it (the drop-in: the driver advances it after each
// timestep() call, epic_main.c:424).  Runs on a halted model too.
__global__ void k_set_itime(DevModel M, long long itime) {
  epic_member(M);
  M.ctl->itime = itime;
}

// ---- launchers ----

int launch_copy_gz(const DevModel &M, cudaStream_t s) {
  k_copy_gz<<<zg(epic_blocks(M.n3, TB(M, TB_POINT)), M), TB(M, TB_POINT), 0, s>>>(M);
  return 0;
}

int launch_zero_tend(const DevModel &M, cudaStream_t s) {
  k_zero_tend<<<zg(epic_blocks(M.n3, TB(M, TB_POINT)), M), TB(M, TB_POINT), 0, s>>>(M);
  return 0;
}

int launch_uv_core(const DevModel &M, cudaStream_t s) {
  EPIC_LAUNCH_R(M.mixed, k_uv_kin, cells_blocks(M, M.nk - 1, M.nj + 1, TB(M, TB_UV_CORE)), TB(M, TB_UV_CORE), 0, s, M);
  EPIC_LAUNCH_R(M.mixed, k_uv_core_v, cells_blocks(M, M.nk - 1, M.nj, TB(M, TB_UV_CORE)), TB(M, TB_UV_CORE), 0, s, M);
  // k_uv_kin wrote KIN on rows 0..nj with their pads
  launch_filter_planes(M, M.work0, PL_NONE, M.work0, 1, M.nk - 1, 0, s, M.mixed, 0, 1);
  EPIC_LAUNCH_R(M.mixed, k_uv_core_u, cells_blocks(M, M.nk - 1, M.nj + 1, TB(M, TB_UV_CORE)), TB(M, TB_UV_CORE), 0, s, M);
  return 0;
}

// k_pgrad_lon's face exchange: one face per thread of the block
static size_t lon_smem(const DevModel &M, size_t face_bytes) { return (size_t)TB(M, TB_PGRAD) * face_bytes; }

int launch_uv_pgrad(const DevModel &M, cudaStream_t s) {
  k_gz_pole_rows<<<zg(M.nk + 1, M), 128, 0, s>>>(M);
  // FP64 form: binary64; mixed: double-float on the splits; fast mixed: binary32 on the splits
  const dim3 glon = zg(cells_blocks(M, M.nk - 1, M.nj + 1, TB(M, TB_PGRAD)), M), glat = zg(cells_blocks(M, M.nk - 1, M.nj, TB(M, TB_PGRAD)), M);
  if (!M.mixed) {
    k_pgrad_lon<double><<<glon, TB(M, TB_PGRAD), lon_smem(M, sizeof(LonFace<double>)), s>>>(M);
    k_pgrad_lat<double><<<glat, TB(M, TB_PGRAD), 0, s>>>(M);
    return 0;
  }
  if (M.col64) {
    k_pgrad_lon<dfl><<<glon, TB(M, TB_PGRAD), lon_smem(M, sizeof(LonFace<dfl>)), s>>>(M);
    k_pgrad_lat<dfl><<<glat, TB(M, TB_PGRAD), 0, s>>>(M);
  } else {
    k_pgrad_lon<float><<<glon, TB(M, TB_PGRAD), 0, s>>>(M);
    k_pgrad_lat<float><<<glat, TB(M, TB_PGRAD), 0, s>>>(M);
  }
  return 0;
}

// The fused march (k_hsu_meridional) has one thread per (k, i, member) walking nj+1 rows; it
// wins once those threads fill the GPU (large batches).  Smaller launches take the four passes,
// whose threads cover every cell.  Both give the same bits.  The tuning table's
// TB_HSU_MERID_VARIANT entry overrides the choice (1 fused, 2 four passes).
constexpr long long HSU_FUSED_MIN_THREADS = 65536;

int launch_akima_meridional(const DevModel &M, double *buff, int kind, cudaStream_t s) {
  const int k0 = kind == 1 ? M.k_sigma - 1 : 1;
  const int nkk = M.nk - k0 + 1;
  const int th = TB(M, TB_HSU);
  EPIC_LAUNCH_R(M.mixed, k_akima_merid_flux, cells_blocks(M, nkk, M.nj, th), th, 0, s, M, buff, kind, k0);
  EPIC_LAUNCH_R(M.mixed, k_akima_merid_update, cells_blocks(M, nkk, M.nj + 1, th), th, 0, s, M, buff, k0);
  return 0;
}

int launch_hsu_meridional(const DevModel &M, double *buff, int kind, cudaStream_t s) {
  const int k0 = kind == 1 ? M.k_sigma - 1 : 1;
  const int nkk = M.nk - k0 + 1;
  const int th = TB(M, TB_HSU);
  const int variant = M.tb[TB_HSU_MERID_VARIANT];
  const bool fused = variant == 1 ||
                     (variant == 0 && (long long)M.ni * nkk * (M.nbatch > 1 ? M.nbatch : 1) >= HSU_FUSED_MIN_THREADS);
  if (fused) {
    EPIC_LAUNCH_R(M.mixed, k_hsu_meridional, dim3(epic_blocks(M.ni, th), nkk), th, 0, s, M, buff, kind, k0);
    return 0;
  }
  EPIC_LAUNCH_R(M.mixed, k_hsu_merid_pred, cells_blocks(M, nkk, M.nj + 2, th), th, 0, s, M, buff, kind, k0);
  EPIC_LAUNCH_R(M.mixed, k_hsu_merid_apred, cells_blocks(M, nkk, M.nj + 1, th), th, 0, s, M, buff, k0);
  EPIC_LAUNCH_R(M.mixed, k_hsu_merid_corr, cells_blocks(M, nkk, M.nj + 2, th), th, 0, s, M, buff, kind, k0);
  EPIC_LAUNCH_R(M.mixed, k_hsu_merid_update, cells_blocks(M, nkk, M.nj + 1, th), th, 0, s, M, buff, k0);
  return 0;
}

// index: 0 = U, 1 = V, 2 = HDRY, 3 = THETA
static void visc_krange(const DevModel &M, int index, int &k0, int &k1) {
  k0 = 1;
  k1 = M.nk;
  if (index == 0 || index == 1) k1 = M.nk - 1;
  if (index == 3) k0 = M.k_sigma - 1;
}

int launch_meridional_hyperviscosity(const DevModel &M, int index, double *var, int sel, cudaStream_t s) {
  double rest4 = M.nu[4] + M.nu[6] + M.nu[8];
  if (!(rest4 > 0.)) return 0;
  int k0, k1;
  visc_krange(M, index, k0, k1);
  const int nkk = k1 - k0 + 1;
  const int vgrid = index == 1;
  const int nrows = vgrid ? M.nj + 2 : M.nj + 1;
  // The first second-derivative reads the (possibly time-plane selected) field itself; later
  // ones ping-pong between two scratch volumes, as hh and d2dy2var do in the reference.
  double *cur_src = var;
  int src_sel = sel;
  double *bufs[2] = {M.work1, M.work2};
  int which = 0;
  double sign = 1.;
  // the mixed forms fuse the first two passes when nothing is applied between them
  const size_t pair_smem = (size_t)nrows * 32 * sizeof(float);
  const bool pair = M.mixed && !(M.nu[2] > 0.) && M.nu[4] + M.nu[6] + M.nu[8] > 0. && pair_smem <= 48 * 1024;
  for (int itmp = 2; itmp <= 8; itmp += 2) {
    double *dst = bufs[which];
    if (pair && itmp == 2) {
      // the second pass's output goes where the unfused loop leaves it
      dst = bufs[1];
      k_d2dy2_pair_mixed<<<zg(dim3((unsigned)((M.ni + 31) / 32), (unsigned)nkk), M), 256, pair_smem, s>>>(M, var, sel, dst, vgrid, k0);
      itmp = 4;
      which = 1;
      sign = -sign;
    } else {
      EPIC_LAUNCH_R(M.mixed, k_d2dy2, cells_blocks(M, nkk, nrows, TB(M, TB_VISC)), TB(M, TB_VISC), 0, s, M, cur_src, src_sel, dst, vgrid, itmp, k0,
                    nkk, cur_src == var);
    }
    src_sel = PL_NONE;
    if (M.nu[itmp] > 0.) {
      // k_d2dy2 / k_d2dy2_pair_mixed wrote every row of dst with its pads
      launch_filter_planes(M, dst, PL_NONE, dst, k0, nkk, vgrid, s, M.mixed, 0, 1);
      EPIC_LAUNCH_R(M.mixed, k_visc_apply, cells_blocks(M, nkk, vgrid ? M.nj : M.nj + 1, TB(M, TB_VISC)), TB(M, TB_VISC), 0, s, M, var, sel, dst, vgrid, sign, k0, nkk);
    }
    sign = -sign;
    double rest = 0.;
    for (int q = itmp + 2; q <= 8; q += 2) rest += M.nu[q];
    if (!(rest > 0.)) break;
    cur_src = dst;
    which ^= 1;
  }
  return 0;
}

// index 2 (HDRY) applies restore_mass as well (in the kernel, or alone without hyperviscosity)
int launch_zonal_hyperviscosity(const DevModel &M, int index, double *var, int sel, cudaStream_t s) {
  if (M.ni < 2 || !(M.nu[4] + M.nu[6] + M.nu[8] > 0.)) return index == 2 ? launch_restore_mass(M, s) : 0;
  int k0, k1;
  visc_krange(M, index, k0, k1);
  const int jbot = index == 1 ? 1 : 0, jhalf = index == 1 ? 0 : 1;
  const size_t row_bytes = (size_t)(M.ni + 2) * (sizeof(double) + 2 * (M.mixed ? sizeof(float) : sizeof(double)));
  int rows = (int)((40 * 1024) / row_bytes);
  rows = rows < 1 ? 1 : (rows > 4 ? 4 : rows);
  const int nrows = M.nj - jbot + 1;
  dim3 grid((nrows + rows - 1) / rows, k1 - k0 + 1);
  EPIC_LAUNCH_R(M.mixed, k_zonal_visc, grid, 32 * rows, rows * row_bytes, s, M, var, sel, jbot, jhalf, k0, index == 2);
  return 0;
}

int launch_divergence_damping(const DevModel &M, cudaStream_t s) {
  if (M.nudiv == 0.) return 0;
  launch_filter_planes(M, M.u, PL_UV_DIS, M.work1, 1, M.nk - 1, 0, s, M.mixed);
  EPIC_LAUNCH_R(M.mixed, k_divergence, cells_blocks(M, M.nk - 1, M.nj + 1, TB(M, TB_DIAG)), TB(M, TB_DIAG), 0, s, M, M.work1, M.v, PL_UV_DIS, M.work2, 1, M.nk - 1);
  EPIC_LAUNCH_R(M.mixed, k_divdamp_apply, epic_blocks(2LL * (M.nk - 1) * (M.nj + 1) * M.ni, TB(M, TB_UPDATE)), TB(M, TB_UPDATE), 0, s, M);
  return 0;
}

int launch_uv_update(const DevModel &M, cudaStream_t s) {
  k_uv_decide<<<zg(1, M), 1, 0, s>>>(M);
  k_uv_update<<<zg(epic_blocks(2LL * (M.nk - 1) * (M.nj + 1) * M.ni, TB(M, TB_UPDATE)), M), TB(M, TB_UPDATE), 0, s>>>(M);
  k_uv_rotate<<<zg(1, M), 1, 0, s>>>(M);
  return 0;
}

int launch_store_diag(const DevModel &M, cudaStream_t s) {
  // PV3: filtered copy of V (v rows), then the interior and polar values.
  launch_filter_planes(M, M.v, PL_UV, M.work1, 0, M.nk + 1, 1, s, M.mixed);
  EPIC_LAUNCH_R(M.mixed, k_pv_interior, cells_blocks(M, M.nk + 1, M.nj, TB(M, TB_DIAG)), TB(M, TB_DIAG), 0, s, M, M.work1);
  k_pv_poles<<<zg(M.nk + 1, M), 128, 4 * M.ni * sizeof(double), s>>>(M);
  // DIV_UV3 from a filtered copy of U.
  launch_filter_planes(M, M.u, PL_UV, M.work2, 0, M.nk + 1, 0, s, M.mixed);
  EPIC_LAUNCH_R(M.mixed, k_divergence, cells_blocks(M, M.nk + 1, M.nj + 1, TB(M, TB_DIAG)), TB(M, TB_DIAG), 0, s, M, M.work2, M.v, PL_UV, M.div_uv3, 0, M.nk + 1);
  EPIC_LAUNCH_R(M.mixed, k_ri2, cells_blocks(M, M.nk, M.nj + 1, TB(M, TB_DIAG)), TB(M, TB_DIAG), 0, s, M);
  return 0;
}

int launch_itime_advance(const DevModel &M, cudaStream_t s) {
  k_itime_advance<<<zg(1, M), 1, 0, s>>>(M);
  return 0;
}

int launch_set_itime(const DevModel &M, long long itime, cudaStream_t s) {
  k_set_itime<<<zg(1, M), 1, 0, s>>>(M, itime);
  return 0;
}

}  // namespace epic
