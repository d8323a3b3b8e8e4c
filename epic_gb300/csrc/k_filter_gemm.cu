// The zonal filter of whole planes (zonal_filter TWODIM, src/shared/epic_adjust.c:412-456) as a
// dense filter-operator product on the fifth-generation tensor cores, for the mixed form
// (ni a multiple of 128).
//
// The reference filters one latitude row at a time: realft forward, wavenumber q scaled by
// HIGH_LAT(J,q+1), realft inverse, times 2/ni.  That is a circulant, symmetric operator:
// y(i) = sum_i' f_J((i - i') mod ni) x(i'), with
//     f_J(d) = (w_0 + (-1)^d w_{ni/2} + 2 sum_{q=1}^{ni/2-1} w_q cos(2 pi q d / ni)) / ni,
// w_q = HIGH_LAT(J, q+1).  For row J of every plane at once this is the product
//     D[m][n] = sum_k A[m][k] B[n][k],   A[m][k] = f_J((m0 + m - k) mod ni),  B[n][k] = x_n(k+1),
// in tiles of M = 128 output points, N = 32 planes and K = ni.  A CTA owns one row and 32 planes
// and accumulates every 128-point tile of the row in its own tensor-memory columns, so it reads
// the whole input row before it writes any output (the filter may run in place).  Operands are staged
// in shared memory in the 128-byte-swizzled K-major layout (8-row atoms of 1024 bytes; the
// 16-byte chunk c of row r sits at chunk c ^ (r % 8)), multiplied by tcgen05.mma kind::tf32 issued
// by one thread into a 128 x 32 FP32 accumulator in tensor memory, and read back with tcgen05.ld.
// Three products per K step give FP32 accuracy from TF32 inputs ("3xTF32"): with a = a_hi + a_lo,
// a_hi = tf32(a), the sum a_hi b_hi + a_hi b_lo + a_lo b_hi misses only the a_lo b_lo term.
//
// With shift set, each row of each plane is filtered as x - x(1), and x(1) is added back to the
// output in binary64: the operator passes a constant unchanged (its wavenumber-0 weight is 1), so
// the result is the same while the FP32 rounding acts on the zonal variations only -- for the
// geopotential, ~1e-5 of its value.
//
// Every wait is bounded: a CTA whose MMA completion does not arrive within the limit records
// ERR_TIMEOUT, waits (bounded) for its last commit, frees its tensor memory and returns.
#include <cmath>
#include <vector>
#include "device_common.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

namespace {

constexpr int FG_M = 128;        // output points per CTA (tensor-memory lanes)
constexpr int FG_N = 32;         // planes per CTA (accumulator columns)
constexpr int FG_KC = 32;        // K elements per staged chunk: one 128-byte swizzle row of FP32
constexpr int FG_THREADS = 128;  // four warps: one per 32-lane quarter of tensor memory
constexpr unsigned FG_WAIT_LIMIT = 1u << 22;

// Byte offset of element (r, e), 0 <= e < 32, in a 128B-swizzled K-major tile of FP32 rows.
__device__ __forceinline__ unsigned sw128(int r, int e) {
  return (unsigned)((r >> 3) * 1024 + (r & 7) * 128 + ((((e >> 2) ^ (r & 7)) & 7) << 4) + (e & 3) * 4);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension byte offset
// (unused for swizzled K-major operands; 16 bytes), stride-dimension byte offset 1024 (between
// 8-row atoms), descriptor version 1, layout SWIZZLE_128B.
__device__ __forceinline__ uint64_t smem_desc(unsigned saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor for kind::tf32: D FP32, A and B TF32, both K-major, N = 32, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(FG_N >> 3) << 17) | ((uint32_t)(FG_M >> 4) << 24);

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(unsigned mbar, unsigned phase) {
  for (unsigned it = 0; it < FG_WAIT_LIMIT; it++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace

// Block = one row j in -1..nj+1 (x), a chunk of 32 planes (y), the member (z).  Rows outside
// the filtered set return at once (k_filter_rows_unfiltered copies them).
//
// The product runs as a two-stage pipeline over steps t = (K chunk kc, output tile mt): the A
// (operator) and B (input) tiles are double-buffered in shared memory; while the tensor cores
// multiply step t, the threads stage step t+1 and the next K chunk's inputs are already on their
// way from global memory into registers.  Each step's products are committed to the mbarrier of
// its buffer; a buffer is restaged only after the commit of the step that last read it (commits
// complete in issue order).
__global__ void __launch_bounds__(FG_THREADS) k_filter_planes_gemm(DevModel M, const double *src, int src_sel, double *dst, int k0,
                                                                     int nplanes, int vgrid, int shift) {
  if (epic_member(M, src, dst)) return;
  extern __shared__ __align__(16) unsigned char fg_raw[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  __shared__ double x1[FG_N];   // the subtracted value of each plane's row (shift), else 0
  const int ni = M.ni, mtiles = ni / FG_M, nchunks = ni / FG_KC, nsteps = nchunks * mtiles;
  const int j = (int)blockIdx.x - 1;
  if (j > M.nj + 1) return;   // a member with fewer rows than the launch (batches of mixed sizes)
  const bool valid = vgrid ? (j >= 1 && j <= M.nj) : (j >= 0 && j <= M.nj);
  src += plane_offset(M, src_sel);
  const int n0 = (int)blockIdx.y * FG_N;
  if (!valid || fabs(M.lat[vgrid ? 2 * j : 2 * j + 1]) < M.lat0) return;
  const int tid = (int)threadIdx.x, warp = tid >> 5;
  const uint32_t tcols = (uint32_t)(mtiles * FG_N);   // 32, 64, 128 or 256: a power of 2

  // two buffers of A_hi, A_lo (128 x 32 FP32 each) and B_hi, B_lo (32 x 32 each), then the
  // row's kernel f; the swizzle atoms need a 1024-byte aligned base
  constexpr unsigned A_BYTES = FG_M * FG_KC * 4, B_BYTES = FG_N * FG_KC * 4, BUF_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  unsigned char *fg_smem = fg_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(fg_raw) & 1023u)) & 1023u);
  float *fk = reinterpret_cast<float *>(fg_smem + 2 * BUF_BYTES);
  const float *fsrc = (vgrid ? M.fkern_v : M.fkern_h) + (long long)(j + 1) * ni;
  for (int d = tid; d < ni; d += FG_THREADS) fk[d] = fsrc[d];
  if (tid < FG_N) x1[tid] = shift && n0 + tid < nplanes ? src[M.at(k0 + n0 + tid, j, 1)] : 0.;
  const unsigned mbar_s = (unsigned)__cvta_generic_to_shared(&mbar[0]);
  if (tid == 0) {
    fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_s));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_s + 8));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    const unsigned dst_s = (unsigned)__cvta_generic_to_shared(&tmem_base);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_s), "r"(tcols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t dtmem = tmem_base;
  const unsigned smem_s = (unsigned)__cvta_generic_to_shared(fg_smem);

  // B[n][e] = x_{n0+n}(kc + e + 1), zero beyond the last plane: two 16-byte chunks (4 values
  // each) per thread and K chunk, loaded into registers one chunk ahead
  constexpr int BQ = FG_N * FG_KC / 4 / FG_THREADS;   // 2
  double bnext[BQ][4];
  auto load_b = [&](int kc) {
#pragma unroll
    for (int u = 0; u < BQ; u++) {
      const int q = tid + u * FG_THREADS, n = q / (FG_KC / 4), e0 = 4 * (q % (FG_KC / 4));
      if (n0 + n < nplanes) {
        const double *row = src + M.at(k0 + n0 + n, j, kc + e0 + 1);
        if (shift) {
          const double c = x1[n];
#pragma unroll
          for (int v = 0; v < 4; v++) bnext[u][v] = row[v] - c;
        } else {
#pragma unroll
          for (int v = 0; v < 4; v++) bnext[u][v] = row[v];
        }
      } else {
#pragma unroll
        for (int v = 0; v < 4; v++) bnext[u][v] = 0.;
      }
    }
  };
  load_b(0);
  int t = 0;
  for (; t < nsteps; t++) {
    const int c = t / mtiles, mt = t - c * mtiles, kc = c * FG_KC, buf = t & 1;
    // the buffer was last read by the products of step t-2
    if (t >= 2 && !mbar_wait(mbar_s + 8 * buf, (unsigned)(((t - 2) >> 1) & 1))) atomicExch(&fail, 1);
    __syncthreads();
    if (fail) break;
    unsigned char *a_hi = fg_smem + buf * BUF_BYTES, *a_lo = a_hi + A_BYTES, *b_hi = a_lo + A_BYTES, *b_lo = b_hi + B_BYTES;
    // B of this K chunk (every output tile of the chunk restages it into its own buffer)
#pragma unroll
    for (int u = 0; u < BQ; u++) {
      const int q = tid + u * FG_THREADS, n = q / (FG_KC / 4), e0 = 4 * (q % (FG_KC / 4));
      const float b0 = d2f(bnext[u][0]), b1 = d2f(bnext[u][1]), b2 = d2f(bnext[u][2]), b3 = d2f(bnext[u][3]);
      const float4 hv = make_float4(tf32_hi(b0), tf32_hi(b1), tf32_hi(b2), tf32_hi(b3));
      const float4 lv = make_float4(b0 - hv.x, b1 - hv.y, b2 - hv.z, b3 - hv.w);
      const unsigned off = sw128(n, e0);
      *reinterpret_cast<float4 *>(b_hi + off) = hv;
      *reinterpret_cast<float4 *>(b_lo + off) = lv;
    }
    // A[m][e] = f((128 mt + m - (kc + e)) mod ni), ni a power of 2
    for (int q = tid; q < FG_M * FG_KC / 4; q += FG_THREADS) {
      const int m = q / (FG_KC / 4), e0 = 4 * (q % (FG_KC / 4));
      const int d0 = mt * FG_M + m - (kc + e0) + ni;
      float a[4];
#pragma unroll
      for (int u = 0; u < 4; u++) a[u] = fk[(d0 - u) & (ni - 1)];
      const float4 hv = make_float4(tf32_hi(a[0]), tf32_hi(a[1]), tf32_hi(a[2]), tf32_hi(a[3]));
      const float4 lv = make_float4(a[0] - hv.x, a[1] - hv.y, a[2] - hv.z, a[3] - hv.w);
      const unsigned off = sw128(m, e0);
      *reinterpret_cast<float4 *>(a_hi + off) = hv;
      *reinterpret_cast<float4 *>(a_lo + off) = lv;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const unsigned a_hi_s = smem_s + buf * BUF_BYTES, a_lo_s = a_hi_s + A_BYTES, b_hi_s = a_lo_s + A_BYTES, b_lo_s = b_hi_s + B_BYTES;
      const uint32_t d_mt = dtmem + (uint32_t)(mt * FG_N);
      for (int ks = 0; ks < FG_KC / 8; ks++) {   // K = 8 TF32 (32 bytes) per instruction
        const unsigned koff = (unsigned)ks * 32;
        const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
        mma_tf32(d_mt, smem_desc(a_hi_s + koff), smem_desc(b_hi_s + koff), acc);
        mma_tf32(d_mt, smem_desc(a_hi_s + koff), smem_desc(b_lo_s + koff), 1u);
        mma_tf32(d_mt, smem_desc(a_lo_s + koff), smem_desc(b_hi_s + koff), 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_s + 8 * buf) : "memory");
    }
    // the next K chunk's inputs travel while the products run
    if (mt == mtiles - 1 && c + 1 < nchunks) load_b(kc + FG_KC);
  }
  // all products done: the last commit covers every earlier one (bounded also after a failure,
  // so that no product is in flight when the tensor memory is freed)
  if (t > 0 && !mbar_wait(mbar_s + 8 * ((t - 1) & 1), (unsigned)(((t - 1) >> 1) & 1))) atomicExch(&fail, 1);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (!fail) {
    const int lane = tid & 31;
    for (int mt = 0; mt < mtiles; mt++) {
      // warp w reads tensor-memory lanes 32w..32w+31: output point 128 mt + 32w + lane, 32 planes
      uint32_t r[FG_N];
      const uint32_t taddr = dtmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(mt * FG_N);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
          "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
            "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
            "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
            "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int i = mt * FG_M + warp * 32 + lane + 1;
#pragma unroll
      for (int n = 0; n < FG_N; n++)
        if (n0 + n < nplanes) {
          const double y = f2d(__uint_as_float(r[n]));
          write_with_pads(dst, M, M.at(k0 + n0 + n, j, 0), i, shift ? y + x1[n] : y);
        }
    }
  } else if (tid == 0) {
    flag_error(M.ctl, ERR_TIMEOUT, k0 + n0, j, 0, 0.);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(dtmem), "r"(tcols));
}

size_t filter_gemm_smem_bytes(int ni) {
  return 1024 + (size_t)2 * (2 * FG_M * FG_KC * 4 + 2 * FG_N * FG_KC * 4) + (size_t)ni * 4;
}

bool filter_gemm_usable(const DevModel &M) { return M.fkern_h && M.ni % FG_M == 0 && M.ni <= 8 * FG_M; }

int launch_filter_planes_gemm(const DevModel &M, const double *src, int src_sel, double *dst, int k0, int nplanes, int vgrid, cudaStream_t s,
                              int shift) {
  dim3 grid(M.nj + 3, (nplanes + FG_N - 1) / FG_N);
  k_filter_planes_gemm<<<zg(grid, M), FG_THREADS, filter_gemm_smem_bytes(M.ni), s>>>(M, src, src_sel, dst, k0, nplanes, vgrid, shift);
  return 0;
}

// 86 KB at ni = 1024: the shared-memory limit is raised once to that maximum.
int filter_gemm_init(int) {
  return cudaFuncSetAttribute(k_filter_planes_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)filter_gemm_smem_bytes(8 * FG_M)) == cudaSuccess ? 0 : -1;
}

// Host: the circulant kernel f_J(d) of every row (h rows from HIGH_LAT_H, v rows from
// HIGH_LAT_PV), rows indexed J+1 = 0..nj+2, rounded to FP32.
void fill_filter_kernels(int ni, int nj, const double *hl_h, const double *hl_pv, long long iadim, float *fh, float *fv) {
  const int N = ni / 2;
  std::vector<double> cs(ni);
  for (int mq = 0; mq < ni; mq++) cs[mq] = cos(2. * M_PI * mq / ni);
  for (int g = 0; g < 2; g++) {
    const double *hl = g ? hl_pv : hl_h;
    float *out = g ? fv : fh;
    for (int row = 0; row < nj + 3; row++) {
      const double *w = hl + (long long)row * iadim;   // w[I], I = 1..N+1
      for (int d = 0; d < ni; d++) {
        double f = w[1] + ((d & 1) ? -w[N + 1] : w[N + 1]);
        for (int q = 1; q < N; q++) f += 2. * w[q + 1] * cs[(long long)q * d % ni];
        out[(long long)row * ni + d] = (float)(f / ni);
      }
    }
  }
}

}  // namespace epic
