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
// in tiles of M = 128 output points, N columns and K = ni.  The columns are (member, plane) pairs:
// one CTA filters row J of up to 64 planes of several members of a batch at once (members that
// share the grid, so the operator), which is what amortises the operator's staging.  A CTA
// accumulates every 128-point tile of the row in its own tensor-memory columns, so it reads the
// whole input row before it writes any output (the filter may run in place).  Operands are staged
// in shared memory in the 128-byte-swizzled K-major layout (8-row atoms of 1024 bytes; the
// 16-byte chunk c of row r sits at chunk c ^ (r % 8)), multiplied by tcgen05.mma kind::tf32 issued
// by one thread into a 128 x N FP32 accumulator in tensor memory, and read back with tcgen05.ld.
// Three products per K step give FP32 accuracy from TF32 inputs ("3xTF32"): with a = a_hi + a_lo,
// a_hi = tf32(a), the sum a_hi b_hi + a_hi b_lo + a_lo b_hi misses only the a_lo b_lo term.
//
// The operator is circulant, so the 128 x 32 tile of output tile mt and K chunk kc depends on
// (128 mt - kc) mod ni alone: ni/32 distinct tiles per row.  They are built once per model on
// the host, already split into TF32 hi and lo parts, and kept in HBM for the filtered rows only
// (ni/32 x 32 KB per row); the TMA engine copies each step's pair into shared memory
// (cp.async.bulk.tensor with the 128-byte swizzle, completion counted on an mbarrier) while the
// threads convert and stage the planes' values.
//
// With shift set, each row of each plane is filtered as x - x(1), and x(1) is added back to the
// output in binary64: the operator passes a constant unchanged (its wavenumber-0 weight is 1), so
// the result is the same while the FP32 rounding acts on the zonal variations only -- for the
// geopotential, ~1e-5 of its value.
//
// Every wait is bounded: a CTA whose operator copy or MMA completion does not arrive within the
// limit records ERR_TIMEOUT, waits (bounded) for what it has in flight, frees its tensor memory
// and returns.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>
#include <cuda.h>
#include <cudaTypedefs.h>
#include "device_common.cuh"
#include "kernels.h"
#include "epic_common.h"
#include "epic_gb300.h"

namespace epic {

namespace {

constexpr int FG_M = 128;        // output points per tile (tensor-memory lanes)
constexpr int FG_KC = 32;        // K elements per staged chunk: one 128-byte swizzle row of FP32
constexpr int FG_NMAX = 64;      // columns per CTA ((member, plane) pairs), a multiple of 32
constexpr int FG_THREADS = 128;  // four warps: one per 32-lane quarter of tensor memory
constexpr unsigned FG_WAIT_LIMIT = 1u << 22;
constexpr unsigned FG_A_BYTES = FG_M * FG_KC * 4;   // one operator tile (hi or lo): 16 KB

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

// Instruction descriptor for kind::tf32: D FP32, A and B TF32, both K-major, M = 128, N columns
// (a multiple of 16 up to 256).
__device__ __forceinline__ uint32_t idesc_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(FG_M >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

// One operator tile (128 rows of 32 FP32) from the tensor map's row y into shared memory at
// dst (1024-byte aligned), counted on mbarrier mbar.  x is 0: the rows are exactly one 128-byte
// box wide, so the copy starts on the 16-byte boundary TMA requires.
__device__ __forceinline__ void tma_tile(unsigned dst, const void *map, int y, unsigned mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(map), "r"(0), "r"(y), "r"(mbar)
      : "memory");
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

// Block = one row j in -1..nj+1 (x) and, in y, one group of G members times one chunk of pc
// planes: column n = g pc + p is plane k0 + chunk pc + p of member q0 + g, N = G pc rounded up to
// 32 (idle columns stay zero).  Rows outside the filtered set return at once
// (k_filter_rows_unfiltered copies them).  A member the batch has halted keeps its planes
// untouched.  G > 1 only when the members share the launch's geometry and operator (fop_shared).
//
// The product runs as a two-stage pipeline over steps t = (K chunk c, output tile mt): the
// operator tiles are double-buffered by step, the planes' tile by K chunk (staged once per chunk,
// read by its mtiles output tiles); while the tensor cores multiply step t, TMA brings step t+1's
// operator tiles and the threads stage the next chunk, whose inputs are already on their way from
// global memory into registers.  Each step's products are committed to the mbarrier of its buffer;
// a buffer is refilled only after the commit of the step that last read it (commits complete in
// issue order).
__global__ void __launch_bounds__(FG_THREADS) k_filter_planes_gemm(DevModel M, const double *src, int src_sel, double *dst, int k0,
                                                                     int nplanes, int vgrid, int shift, int pc, int G, int N, int msplit) {
  extern __shared__ __align__(16) unsigned char fg_raw[];
  __shared__ __align__(8) uint64_t bars[4];   // products of buffer 0 / 1 done; operator tiles of buffer 0 / 1 landed
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  __shared__ const double *s_src[FG_NMAX];
  __shared__ double *s_dst[FG_NMAX];
  __shared__ int s_col[FG_NMAX];             // offset of the column's row (i = 0) in its member's field, -1 when idle
  __shared__ unsigned char s_colg[FG_NMAX];  // the column's member slot g
  __shared__ double s_x1[FG_NMAX];           // the subtracted value of each column's row (shift), else 0
  const int tid = (int)threadIdx.x, warp = tid >> 5;
  const int j = (int)blockIdx.x - 1;
  const int nch = (nplanes + pc - 1) / pc;
  const int yq = (int)blockIdx.y / msplit, msi = (int)blockIdx.y - yq * msplit;
  const int chunk = yq % nch, q0 = (yq / nch) * G;
  const int members = M.batch ? M.nbatch : 1;
  // geometry: a one-member CTA takes its member's own (batches of mixed sizes); the members of
  // a larger group share the launch's
  const DevModel &Mg = M.batch ? M.batch[q0] : M;
  const DevModel &opm = M.fop_shared ? M : Mg;
  const int ni = Mg.ni, mtiles = ni / FG_M, nchunks = ni / FG_KC, ntiles = ni / FG_KC;
  // this CTA's output tiles: msplit CTAs share a row's mtiles (a member narrower than the launch
  // may leave some of them without a tile)
  const int mts = mtiles >= msplit ? mtiles / msplit : 1, mt0 = msi * mts;
  if (mt0 >= mtiles) return;
  if (j > Mg.nj + 1) return;   // a member with fewer rows than the launch
  const int slot = opm.fop_slot[vgrid * (Mg.nj + 3) + j + 1];
  if (slot < 0) return;
  if (tid < G) {
    const int q = q0 + tid;
    const double *sp = nullptr;
    double *dp = nullptr;
    if (q < members) {
      const DevModel &mq = M.batch ? M.batch[q] : M;
      if (!mq.ctl->halted) {
        sp = member_ptr(M, mq, src) + plane_offset(mq, src_sel);
        dp = member_ptr(M, mq, dst);
      }
    }
    s_src[tid] = sp;
    s_dst[tid] = dp;
  }
  __syncthreads();
  int live = 0;
  if (tid < N) {
    const int g = tid / pc, p = tid - g * pc, plane = chunk * pc + p;
    int base = -1;
    if (g < G && plane < nplanes && s_src[g]) base = Mg.at(k0 + plane, j, 0);
    s_col[tid] = base;
    s_colg[tid] = (unsigned char)(g < G ? g : 0);
    s_x1[tid] = shift && base >= 0 ? s_src[g][base + 1] : 0.;
    live = base >= 0;
  }
  if (!__syncthreads_or(live)) return;   // every member of the group halted

  // two operator buffers of A_hi, A_lo (128 x 32 FP32 each), then two plane buffers of B_hi,
  // B_lo (N x 32 each); the swizzle atoms need a 1024-byte aligned base
  const unsigned b_bytes = (unsigned)N * FG_KC * 4;
  unsigned char *fg_smem = fg_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(fg_raw) & 1023u)) & 1023u);
  const unsigned smem_s = (unsigned)__cvta_generic_to_shared(fg_smem);
  const unsigned a_s = smem_s, b_s = smem_s + 4 * FG_A_BYTES;
  const unsigned bars_s = (unsigned)__cvta_generic_to_shared(&bars[0]);
  const uint32_t tcols = (uint32_t)(mts * N) <= 32 ? 32u : 1u << (32 - __clz(mts * N - 1));   // a power of 2 >= 32
  if (tid == 0) {
    fail = 0;
    for (int b = 0; b < 4; b++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars_s + 8 * b));
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
  const uint32_t idesc = idesc_tf32(N);

  // B[n][e] = x_n(kc + e + 1) - x1_n, zero in idle columns: N/16 16-byte chunks (4 values each)
  // per thread and K chunk, loaded into registers two chunks ahead (two register sets, the chunks
  // taken in pairs), so that a chunk's loads have two chunks' products to arrive in
  constexpr int BQMAX = FG_NMAX * FG_KC / 4 / FG_THREADS;   // 4
  const int nq = N * (FG_KC / 4) / FG_THREADS;
  double breg0[BQMAX][4], breg1[BQMAX][4];
  auto load_b = [&](int kc, double (&bn)[BQMAX][4]) {
#pragma unroll
    for (int u = 0; u < BQMAX; u++) {
      if (u >= nq) break;
      const int q = tid + u * FG_THREADS, n = q / (FG_KC / 4), e0 = 4 * (q % (FG_KC / 4));
      const int base = s_col[n];
      if (base >= 0) {
        const double *row = s_src[s_colg[n]] + base + kc + e0 + 1;
        const double c = s_x1[n];
#pragma unroll
        for (int v = 0; v < 4; v++) bn[u][v] = row[v] - c;
      } else {
#pragma unroll
        for (int v = 0; v < 4; v++) bn[u][v] = 0.;
      }
    }
  };
  load_b(0, breg0);
  if (nchunks > 1) load_b(FG_KC, breg1);
  int last_tma = -1, last_commit = -1;
  // step t = (K chunk c, output tile mt); false once the CTA must stop
  auto step = [&](int c, int mt, double (&bn)[BQMAX][4]) -> bool {
    const int t = c * mts + (mt - mt0), kc = c * FG_KC, abuf = t & 1, bbuf = c & 1;
    // both buffers were last read by the products of step t-2 or earlier
    if (t >= 2 && !mbar_wait(bars_s + 8 * abuf, (unsigned)(((t - 2) >> 1) & 1))) atomicExch(&fail, 1);
    __syncthreads();
    if (fail) return false;
    const unsigned a_hi_s = a_s + abuf * 2 * FG_A_BYTES, a_lo_s = a_hi_s + FG_A_BYTES;
    const unsigned b_hi_s = b_s + bbuf * 2 * b_bytes, b_lo_s = b_hi_s + b_bytes;
    if (tid == 0) {
      // the operator tile for offset (128 mt - kc) mod ni, hi then lo
      const int tt = ((mt * FG_M - kc) & (ni - 1)) / FG_KC;
      const int y = ((slot * ntiles + tt) * 2) * FG_M;
      const unsigned tb = bars_s + 8 * (2 + abuf);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tb), "r"(2 * FG_A_BYTES) : "memory");
      tma_tile(a_hi_s, opm.fop_map, y, tb);
      tma_tile(a_lo_s, opm.fop_map, y + FG_M, tb);
      last_tma = t;
    }
    if (mt == mt0) {   // the planes' tile of this K chunk, then the loads of chunk c+2 into its registers
      unsigned char *bh = fg_smem + (b_hi_s - smem_s), *bl = bh + b_bytes;
#pragma unroll
      for (int u = 0; u < BQMAX; u++) {
        if (u >= nq) break;
        const int q = tid + u * FG_THREADS, n = q / (FG_KC / 4), e0 = 4 * (q % (FG_KC / 4));
        const float b0 = d2f(bn[u][0]), b1 = d2f(bn[u][1]), b2 = d2f(bn[u][2]), b3 = d2f(bn[u][3]);
        const float4 hv = make_float4(tf32_hi(b0), tf32_hi(b1), tf32_hi(b2), tf32_hi(b3));
        const float4 lv = make_float4(b0 - hv.x, b1 - hv.y, b2 - hv.z, b3 - hv.w);
        const unsigned off = sw128(n, e0);
        *reinterpret_cast<float4 *>(bh + off) = hv;
        *reinterpret_cast<float4 *>(bl + off) = lv;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (c + 2 < nchunks) load_b(kc + 2 * FG_KC, bn);
    }
    __syncthreads();
    if (tid == 0) {
      if (!mbar_wait(bars_s + 8 * (2 + abuf), (unsigned)((t >> 1) & 1))) {
        fail = 1;
      } else {
        last_tma = -1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t d_mt = dtmem + (uint32_t)((mt - mt0) * N);
        for (int ks = 0; ks < FG_KC / 8; ks++) {   // K = 8 TF32 (32 bytes) per instruction
          const unsigned koff = (unsigned)ks * 32;
          const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
          mma_tf32(d_mt, smem_desc(a_hi_s + koff), smem_desc(b_hi_s + koff), idesc, acc);
          mma_tf32(d_mt, smem_desc(a_hi_s + koff), smem_desc(b_lo_s + koff), idesc, 1u);
          mma_tf32(d_mt, smem_desc(a_lo_s + koff), smem_desc(b_hi_s + koff), idesc, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bars_s + 8 * abuf) : "memory");
        last_commit = t;
      }
    }
    return true;
  };
  bool going = true;
  for (int c = 0; c < nchunks && going; c += 2) {   // nchunks = ni/32 is even
    for (int mt = mt0; mt < mt0 + mts && going; mt++) going = step(c, mt, breg0);
    for (int mt = mt0; mt < mt0 + mts && going; mt++) going = step(c + 1, mt, breg1);
  }
  // drain: the last commit covers every earlier one; an operator copy whose wait gave up is
  // waited for again (both bounded), so that nothing writes this CTA's shared or tensor memory
  // after it is released
  __shared__ int s_last_commit;
  if (tid == 0) {
    s_last_commit = last_commit;
    if (last_tma >= 0 && !mbar_wait(bars_s + 8 * (2 + (last_tma & 1)), (unsigned)((last_tma >> 1) & 1))) fail = 1;
  }
  __syncthreads();
  const int lc = s_last_commit;
  if (lc >= 0 && !mbar_wait(bars_s + 8 * (lc & 1), (unsigned)((lc >> 1) & 1))) atomicExch(&fail, 1);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (!fail) {
    const int lane = tid & 31;
    for (int mt = mt0; mt < mt0 + mts; mt++)
      for (int cg = 0; cg < N; cg += 32) {
        // warp w reads tensor-memory lanes 32w..32w+31: output point 128 mt + 32w + lane, columns cg..cg+31
        uint32_t r[32];
        const uint32_t taddr = dtmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((mt - mt0) * N + cg);
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
        for (int n = 0; n < 32; n++) {
          const int col = cg + n, base = s_col[col];
          if (base >= 0) {
            const double y = f2d(__uint_as_float(r[n]));
            write_with_pads(s_dst[s_colg[col]], Mg, base, i, shift ? y + s_x1[col] : y);
          }
        }
      }
  } else if (tid == 0) {
    flag_error(Mg.ctl, ERR_TIMEOUT, k0 + chunk * pc, j, 0, 0.);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(dtmem), "r"(tcols));
}

// dynamic shared memory of a CTA with N columns: two operator buffers, two plane buffers, the
// alignment slack of the swizzle atoms
size_t filter_gemm_smem_bytes(int n) { return 1024 + 4 * (size_t)FG_A_BYTES + 4 * (size_t)n * FG_KC * 4; }

static int g_sms = 0;   // SMs of the device (filter_gemm_init, at model creation: not during a graph capture)

bool filter_gemm_usable(const DevModel &M) { return M.fop_map && M.ni % FG_M == 0 && M.ni <= 8 * FG_M; }

// Columns per CTA: up to 64 (32 at ni = 1024), so that two CTAs fit an SM in shared memory
// (~98 KB each) and in tensor memory (mtiles x N <= 256 columns each).  Planes beyond that split
// into chunks; members of one operator fill the rest of the columns.
int launch_filter_planes_gemm(const DevModel &M, const double *src, int src_sel, double *dst, int k0, int nplanes, int vgrid, cudaStream_t s,
                              int shift) {
  const int members = M.batch ? M.nbatch : 1;
  const int nmax = M.ni / FG_M <= 4 ? FG_NMAX : 32;
  const int pc = nplanes < nmax ? nplanes : nmax;
  const int nch = (nplanes + pc - 1) / pc;
  int G = M.fop_shared ? nmax / pc : 1;
  if (G > members) G = members;
  const int N = ((G * pc + 31) / 32) * 32;
  const int groups = (members + G - 1) / G;
  // Few members (a single model): about half of the nj+3 rows are filtered, and one CTA per
  // (row, group, plane chunk) leaves SMs idle while each CTA walks all its output tiles; split a
  // row's 128-point output tiles over up to mtiles CTAs (each tile's sums are unchanged) until
  // there are two CTAs with work per SM.  Not in place: a CTA writes its tiles while the others
  // of its row still read the whole row.
  const int sms = g_sms > 0 ? g_sms : 152;
  const int mtiles = M.ni / FG_M;
  const long long working = (long long)(M.nj + 3) / 2 * nch * groups;
  int msplit = 1;
  if (src != dst)
    while (2 * msplit <= mtiles && working * msplit < 2LL * sms) msplit *= 2;
  dim3 grid((unsigned)(M.nj + 3), (unsigned)(nch * groups * msplit), 1u);
  k_filter_planes_gemm<<<grid, FG_THREADS, filter_gemm_smem_bytes(N), s>>>(M, src, src_sel, dst, k0, nplanes, vgrid, shift, pc, G, N,
                                                                          msplit);
  return 0;
}

int filter_gemm_init(int) {
  int dev = 0;
  if (g_sms == 0 && cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
  return cudaFuncSetAttribute(k_filter_planes_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)filter_gemm_smem_bytes(FG_NMAX)) ==
                 cudaSuccess
             ? 0
             : -1;
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

namespace {

// cvt.rna.tf32.f32 on the host: round to nearest (ties away from zero) to 10 fraction bits, the
// 13 bits below cleared
float tf32_rna(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

// which rows the filter changes: |lat| >= lat0 among the h rows j = 0..nj and the v rows 1..nj
// (row_is_filtered); slot[g (nj+3) + j+1], g = 0 for h rows and 1 for v rows
int filter_slots(const epic_grid &g, std::vector<int> &slot) {
  slot.assign(2 * (size_t)(g.nj + 3), -1);
  int n = 0;
  for (int gr = 0; gr < 2; gr++)
    for (int j = gr ? 1 : 0; j <= g.nj; j++)
      if (std::fabs(g.lat[gr ? 2 * j : 2 * j + 1]) >= g.lat0) slot[(size_t)gr * (g.nj + 3) + j + 1] = n++;
  return n;
}

}  // namespace

bool filter_operator_wanted(const epic_grid &g, int precision) {
  return precision != EPIC_PREC_FP64 && g.ni % FG_M == 0 && g.ni <= 8 * FG_M;
}

// Device bytes of a model's operator allocation: the tiles (ni/32 x 2 x 16 KB per filtered row),
// the slot table and the tensor map, with the alignments TMA wants.
size_t filter_operator_bytes(const epic_grid &g) {
  std::vector<int> slot;
  const int n = filter_slots(g, slot);
  return (size_t)n * (g.ni / FG_KC) * 2 * FG_A_BYTES + 1024 + ((slot.size() * sizeof(int) + 255) / 256) * 256 + 256;
}

// Host: the operator tiles of the filtered rows.  For slot s (row J of the h or v grid), tile t
// (offset 32 t) and part h (0: the TF32 part hi = tf32(f), 1: the rest f - hi), row m and column e
// hold the two parts of f_J((32 t + m - e) mod ni), f_J the row's circulant kernel rounded to FP32
// (fill_filter_kernels); the rows of 32 FP32 are stored one after another, tile (s, t, h) at row
// ((s ni/32 + t) 2 + h) 128.  They are copied into one device allocation with the slot table and
// the TMA tensor map that describes them (2-D: 32 FP32 per row, boxes of 32 x 128 with the
// 128-byte swizzle of the kernel's operand layout).  hash identifies the operator (equal hashes:
// the same tiles): models of one grid on one device share one allocation (released by
// filter_operator_release when its last model goes), and a batch of them filters with member 0's.
namespace {
// Operators are shared between the models of one grid on one device: a process-wide table of the
// allocations, keyed by device and hash, counted by the models that use them.
struct OperatorCopy {
  int device;
  uint64_t hash;
  void *base;
  const void *map;
  const int *slot;
  int users;
};
std::mutex g_op_mu;
std::vector<OperatorCopy> g_ops;
}  // namespace

void filter_operator_release(void *mem) {
  if (!mem) return;
  std::lock_guard<std::mutex> lock(g_op_mu);
  for (size_t q = 0; q < g_ops.size(); q++)
    if (g_ops[q].base == mem) {
      if (--g_ops[q].users == 0) {
        cudaFree(g_ops[q].base);
        g_ops.erase(g_ops.begin() + (long)q);
      }
      return;
    }
}

int filter_operator_create(const epic_grid &g, const double *hl_h, const double *hl_pv, long long iadim, cudaStream_t s, DevModel &d,
                           void **mem, uint64_t *hash, const char **why) {
  *mem = nullptr;
  const int ni = g.ni, ntiles = ni / FG_KC;
  std::vector<int> slot;
  const int nslots = filter_slots(g, slot);
  std::vector<float> fh((size_t)(g.nj + 3) * ni), fv((size_t)(g.nj + 3) * ni);
  fill_filter_kernels(ni, g.nj, hl_h, hl_pv, iadim, fh.data(), fv.data());
  uint64_t hs = 1469598103934665603ull;   // FNV-1a over everything the tiles are made of
  auto mix = [&](const void *p, size_t n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    for (size_t q = 0; q < n; q++) hs = (hs ^ c[q]) * 1099511628211ull;
  };
  mix(&ni, sizeof ni);
  mix(slot.data(), slot.size() * sizeof(int));
  mix(fh.data(), fh.size() * sizeof(float));
  mix(fv.data(), fv.size() * sizeof(float));
  *hash = hs;
  int device = -1;
  cudaGetDevice(&device);
  std::lock_guard<std::mutex> lock(g_op_mu);
  for (auto &c : g_ops)
    if (c.device == device && c.hash == hs) {   // a model of the same grid made it already
      c.users++;
      d.fop_map = c.map;
      d.fop_slot = c.slot;
      *mem = c.base;
      return 0;
    }
  const size_t tile_floats = (size_t)FG_M * FG_KC;
  std::vector<float> tiles((size_t)(nslots > 0 ? nslots : 1) * ntiles * 2 * tile_floats, 0.f);
  for (int gr = 0; gr < 2; gr++)
    for (int r = 0; r < g.nj + 3; r++) {
      const int sl = slot[(size_t)gr * (g.nj + 3) + r];
      if (sl < 0) continue;
      const float *f = (gr ? fv.data() : fh.data()) + (size_t)r * ni;
      for (int t = 0; t < ntiles; t++) {
        float *hi = tiles.data() + (((size_t)sl * ntiles + t) * 2) * tile_floats, *lo = hi + tile_floats;
        for (int m = 0; m < FG_M; m++)
          for (int e = 0; e < FG_KC; e++) {
            const float a = f[(FG_KC * t + m - e + 2 * ni) & (ni - 1)], h = tf32_rna(a);
            hi[m * FG_KC + e] = h;
            lo[m * FG_KC + e] = a - h;
          }
      }
    }
  const size_t tile_bytes = tiles.size() * sizeof(float), slot_bytes = ((slot.size() * sizeof(int) + 255) / 256) * 256;
  char *base = nullptr;
  if (cudaMalloc(&base, tile_bytes + 1024 + slot_bytes + 256) != cudaSuccess) {
    *why = "cudaMalloc of the filter operator tiles failed";
    return -1;
  }
  char *tiles_d = base + ((1024 - ((uintptr_t)base & 1023)) & 1023);   // cudaMalloc gives 256-byte alignment
  int *slot_d = reinterpret_cast<int *>(tiles_d + tile_bytes);
  CUtensorMap *map_d = reinterpret_cast<CUtensorMap *>(reinterpret_cast<char *>(slot_d) + slot_bytes);

  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaFree(base);
      *why = "cuTensorMapEncodeTiled not available from the driver";
      return -1;
    }
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  CUtensorMap map;
  std::memset(&map, 0, sizeof map);
  const cuuint64_t gdim[2] = {(cuuint64_t)FG_KC, (cuuint64_t)(tiles.size() / FG_KC)};
  const cuuint64_t gstride[1] = {(cuuint64_t)FG_KC * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)FG_KC, (cuuint32_t)FG_M}, estride[2] = {1, 1};
  if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, tiles_d, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    cudaFree(base);
    *why = "cuTensorMapEncodeTiled rejected the filter operator's layout";
    return -1;
  }
  cudaError_t e = cudaMemcpyAsync(tiles_d, tiles.data(), tile_bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(slot_d, slot.data(), slot.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(map_d, &map, sizeof map, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // the host vectors go out of scope
  if (e != cudaSuccess) {
    cudaFree(base);
    *why = "copy of the filter operator failed";
    return -1;
  }
  d.fop_map = map_d;
  d.fop_slot = slot_d;
  *mem = base;
  g_ops.push_back({device, hs, base, map_d, slot_d, 1});
  return 0;
}

}  // namespace epic
