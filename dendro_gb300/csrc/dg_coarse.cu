// Dense FP32 inverse of the coarsest multigrid operator.  The reference
// factors its coarsest operator with PETSc's LU (bin/options:206,
// -mg_coarse_pc_type lu).  Here the coarsest level is small (at most a few
// thousand nodes) and is solved many times per solve, so it is inverted
// once and applied as a dense matrix-vector product; the FP64 refinement
// rounds of the coarse solve (dg_mg.cu, k_cs_apply) take the result to FP64
// accuracy.
//
// In-place block Gauss-Jordan without pivoting (the operator is SPD).  For
// the pivot block K = [k0, k0 + 64), R the other indices and P = inv(X_KK):
//   X_RR -= X_RK (P X_KR),  X_KR = P X_KR,  X_RK = -(X_RK P),  X_KK = P;
// after the last block X holds the inverse.  Three launches per block:
//   k_gj_diag    P, one CTA (64 serial pivots held in registers);
//   k_gj_strips  Cs = X_RK and Rs = P X_KR into scratch strips, and the new
//                row and column blocks of X (2 * 64^2 * n multiply-adds on
//                the CUDA cores);
//   k_gj_update  X_RR -= Cs Rs: a rank-64 update, n^2 * 64 multiply-adds,
//                on the tensor cores (tcgen05.mma kind::tf32, accumulators in
//                tensor memory), 128 x 128 tiles of X, one persistent CTA
//                per SM.
// The update splits each operand entry a = a_hi + a_lo, a_hi the nearest
// TF32 value and a_lo = a - a_hi (exact in FP32), and accumulates
// lo * hi + hi * lo + hi * hi in FP32 ("3xTF32"): the dropped lo * lo term
// and the TF32 truncation of lo are below 2^-21 of each product, so the
// inverse keeps close to FP32 accuracy.
#include "dg_mg.cuh"
#include "dg_elem.cuh"

#include <algorithm>

namespace dg {

namespace {

constexpr int GJB = 64;      // pivots per block
constexpr int GJT = 64 + 4;  // shared tile row stride (floats)

// ---- k_gj_diag: P = inv(X_KK) for one diagonal block (one CTA of 256
// threads): thread t holds 16 entries of row t / 4 in registers.  Per pivot
// the pivot row's threads scale their row by the reciprocal of the pivot
// (the pivot column entry becomes that reciprocal) and store it in shared
// memory (double-buffered, one barrier per pivot); every other row zeroes
// its pivot-column entry and subtracts its former value times the scaled
// row.  A row's pivot-column entry comes by a shuffle within the row's four
// threads.  A partial last block is padded with the identity; P is written
// as a full GJB x GJB block.  The 64 pivots form a chain of dependent
// steps (about 20 us); the host overlaps it with the previous block's
// trailing update.
__global__ void __launch_bounds__(256) k_gj_diag(const float *__restrict__ X, size_t n, size_t k0, int b,
                                                 float *__restrict__ P) {
  static_assert(GJB == 64, "one CTA of 256 threads covers a 64 x 64 block");
  __shared__ __align__(16) float prow[2][GJB];
  const int t = threadIdx.x, r = t >> 2, q = t & 3, c0 = q * 16;
  const int lane = t & 31, base = lane & ~3;
  float v[16];
#pragma unroll
  for (int i = 0; i < 16; i++) {
    const int c = c0 + i;
    v[i] = (r < b && c < b) ? X[(k0 + r) * n + k0 + c] : (r == c ? 1.f : 0.f);
  }
#pragma unroll
  for (int p = 0; p < GJB; p++) {
    float *pr = prow[p & 1];
    const float f = __shfl_sync(0xffffffffu, v[p & 15], base | (p >> 4));  // this row's column-p entry
    if (r == p) {
      const float inv = 1.0f / f;
#pragma unroll
      for (int i = 0; i < 16; i++) v[i] *= inv;
      if (q == (p >> 4)) v[p & 15] = inv;
      float4 *dst = reinterpret_cast<float4 *>(pr + c0);
#pragma unroll
      for (int i = 0; i < 4; i++) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    }
    __syncthreads();
    if (r != p) {
      if (q == (p >> 4)) v[p & 15] = 0.f;
      const float4 *src = reinterpret_cast<const float4 *>(pr + c0);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const float4 s4 = src[i];
        v[4 * i] -= f * s4.x;
        v[4 * i + 1] -= f * s4.y;
        v[4 * i + 2] -= f * s4.z;
        v[4 * i + 3] -= f * s4.w;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 16; i++) P[r * GJB + c0 + i] = v[i];
}

// acc[4][4] += L R over a 64-deep product, L given transposed (Lt[m][r]), R
// as is (Rm[m][c]); thread (ty, tx) of 256 owns rows 4ty.., columns 4tx..
__device__ __forceinline__ void gj_mma(const float *Lt, const float *Rm, float2 (&acc)[4][2]) {
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
#pragma unroll 8
  for (int m = 0; m < 64; m++) {
    const float4 a = *reinterpret_cast<const float4 *>(&Lt[m * GJT + ty * 4]);
    const float4 c4 = *reinterpret_cast<const float4 *>(&Rm[m * GJT + tx * 4]);
    const float av[4] = {a.x, a.y, a.z, a.w};
    const float2 b01 = make_float2(c4.x, c4.y), b23 = make_float2(c4.z, c4.w);
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const float2 ar = make_float2(av[r], av[r]);
      acc[r][0] = ffma2(ar, b01, acc[r][0]);
      acc[r][1] = ffma2(ar, b23, acc[r][1]);
    }
  }
}

__device__ __forceinline__ float acc_at(const float2 (&acc)[4][2], int r, int c) {
  return c < 2 ? (c == 0 ? acc[r][0].x : acc[r][0].y) : (c == 2 ? acc[r][1].x : acc[r][1].y);
}

// ---- k_gj_strips: CTA t takes index tile I = [64 t, 64 t + 64).  For
// I != K: (a) rows I: Cs[I, :] = X_IK, X_IK = -(X_IK P); (b) columns I:
// Rs[:, I] = P X_KI, X_KI = Rs[:, I].  For I = K: X_KK = P and Rs[:, K] = 0.
// The tiles of different CTAs are disjoint, so no CTA reads what another
// writes.  Columns k >= b of a partial last block are zero in Cs and Rs,
// and so are the rows of K in Cs and the columns of K in Rs.
__global__ void __launch_bounds__(256) k_gj_strips(float *__restrict__ X, size_t n, size_t k0, int b,
                                                   const float *__restrict__ P, float *__restrict__ Cs,
                                                   float *__restrict__ Rs) {
  __shared__ __align__(16) float Lt[64 * GJT];
  __shared__ __align__(16) float Rm[64 * GJT];
  const size_t t = blockIdx.x, base = t * GJB;
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
  if (base == k0) {
    for (int q = threadIdx.x; q < GJB * GJB; q += 256) {
      const int r = q / GJB, c = q % GJB;
      if (r < b && c < b) X[(k0 + r) * n + k0 + c] = P[q];
      if (c < b) Rs[(size_t)r * n + k0 + c] = 0.f;
      if (r < b) Cs[(k0 + r) * GJB + c] = 0.f;
    }
    return;
  }
  const int rows = (int)(n - base < (size_t)GJB ? n - base : (size_t)GJB);
  float2 acc[4][2];
  // (a) the rows of I in column block K (loads first, so that they overlap)
  {
    float xv[16], pv[16];
#pragma unroll
    for (int e = 0; e < 16; e++) {
      const int q = threadIdx.x + e * 256, r = q / GJB, m = q % GJB;
      xv[e] = (r < rows && m < b) ? X[(base + r) * n + k0 + m] : 0.f;
      pv[e] = P[q];
    }
#pragma unroll
    for (int e = 0; e < 16; e++) {
      const int q = threadIdx.x + e * 256, r = q / GJB, m = q % GJB;
      Lt[m * GJT + r] = xv[e];
      if (r < rows) Cs[(base + r) * GJB + m] = xv[e];
      Rm[r * GJT + m] = pv[e];
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 4; r++) acc[r][0] = acc[r][1] = make_float2(0.f, 0.f);
  gj_mma(Lt, Rm, acc);
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int rr = ty * 4 + r, cc = tx * 4 + c;
      if (rr < rows && cc < b) X[(base + rr) * n + k0 + cc] = -acc_at(acc, r, c);
    }
  __syncthreads();  // Lt and Rm are read again below
  // (b) row block K in the columns of I
  {
    float xv[16], pv[16];
#pragma unroll
    for (int e = 0; e < 16; e++) {
      const int q = threadIdx.x + e * 256, m = q / GJB, c = q % GJB;
      xv[e] = (m < b && c < rows) ? X[(k0 + m) * n + base + c] : 0.f;
      pv[e] = P[q];
    }
#pragma unroll
    for (int e = 0; e < 16; e++) {
      const int q = threadIdx.x + e * 256, m = q / GJB, c = q % GJB;
      Lt[c * GJT + m] = pv[e];  // Lt[m'][r'] = P[r'][m']
      Rm[m * GJT + c] = xv[e];
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 4; r++) acc[r][0] = acc[r][1] = make_float2(0.f, 0.f);
  gj_mma(Lt, Rm, acc);
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int rr = ty * 4 + r, cc = tx * 4 + c;
      if (cc < rows) {
        const float v = acc_at(acc, r, c);
        Rs[(size_t)rr * n + base + cc] = v;  // rows rr >= b are zero (P is the identity there)
        if (rr < b) X[(k0 + rr) * n + base + cc] = v;
      }
    }
}

// ---- tensor-core helpers (tcgen05, tensor memory, mbarrier)
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of a K-major operand without swizzling:
// the operand is stored as core matrices of 8 rows x 16 bytes (128
// contiguous bytes, row after row); lbo is the byte step between core
// matrices adjacent along K, sbo the byte step between 8-row groups.
// Fields: start address >> 4 (bits 0-13), lbo >> 4 (16-29), sbo >> 4
// (32-45), descriptor version 1 (46-47), base offset 0, swizzle mode 0.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32: D in F32 (bits 4-5 = 1), A and B in
// TF32 (bits 7-9 and 10-12 = 2), both K-major (bits 15 and 16 clear), no
// negation or sparsity, N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t tc_idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :
      : "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// arrive on the mbarrier once every tcgen05 operation this thread issued
// has completed
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// a bounded wait: false when the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, unsigned limit) {
  for (unsigned i = 0; i < limit; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    __nanosleep(64);
  }
  return false;
}

// 32 consecutive FP32 columns of this warp's 32 tensor-memory lanes (lane =
// thread), starting at taddr
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- k_gj_update: X_ij -= sum_k Cs[i][k] Rs[k][j] for i, j outside K
constexpr int TC_M = 128, TC_N = 128, TC_K = GJB;
constexpr int TC_PROD_WARPS = 4, TC_CONS_WARPS = 8;
constexpr int TC_THREADS = 32 * (TC_PROD_WARPS + TC_CONS_WARPS);
constexpr int TC_PROD = 32 * TC_PROD_WARPS;
constexpr uint32_t TC_LBO = 128;               // core matrices along K: adjacent
constexpr uint32_t TC_SBO = (TC_K / 4) * 128;  // an 8-row group holds TC_K / 4 core matrices
constexpr int TC_OPER = TC_M * TC_K * 4;       // bytes of one operand tile (A or B, hi or lo)
constexpr int TC_TSTRIDE = 33;                 // transpose scratch row stride (floats)
constexpr int TC_TBYTES = TC_CONS_WARPS * 32 * TC_TSTRIDE * 4;
// A hi/lo, two stages of B hi/lo, the consumers' transpose scratch, 4 mbarriers, the tensor-memory address
constexpr int TC_SMEM = 6 * TC_OPER + TC_TBYTES + 48;
constexpr uint32_t TC_TMEM_COLS = 2 * TC_N;    // two accumulator buffers
constexpr unsigned TC_WAIT_LIMIT = 1u << 22;   // polls of one mbarrier wait
static_assert(TC_M == TC_N, "A and B tiles share one layout");
static_assert(TC_SMEM <= 227 * 1024, "shared memory per CTA");

// byte offset of entry (row, k) of a K-major operand tile
__device__ __forceinline__ uint32_t kmaj_off(int row, int k) {
  return (uint32_t)((row >> 3) * TC_SBO + (k >> 2) * TC_LBO + (row & 7) * 16 + (k & 3) * 4);
}

// a = hi + lo, hi the TF32 value nearest to a (ties away from zero), lo
// exact in FP32
__device__ __forceinline__ void tf32_split(float a, float &hi, float &lo) {
  hi = __uint_as_float((__float_as_uint(a) + 0x1000u) & 0xFFFFE000u);
  lo = a - hi;
}

__device__ __forceinline__ void store_split(unsigned char *hi_tile, unsigned char *lo_tile, uint32_t off,
                                            float4 v) {
  float4 h, l;
  tf32_split(v.x, h.x, l.x);
  tf32_split(v.y, h.y, l.y);
  tf32_split(v.z, h.z, l.z);
  tf32_split(v.w, h.w, l.w);
  *reinterpret_cast<float4 *>(hi_tile + off) = h;
  *reinterpret_cast<float4 *>(lo_tile + off) = l;
}

// AND of v over the producer warps (named barrier 1), so that they leave
// their loop together
__device__ __forceinline__ bool producers_all(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.and.pred p, 1, %2, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(TC_PROD)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}

// The tiles one launch covers: every tile (GJ_ALL), the panel of the next
// pivot block (GJ_PANEL: tile row tp and tile column tp, 2 nt - 1 tiles) or
// the rest (GJ_REST: (nt - 1)^2 tiles); gj_tile maps a launch's tile number
// to its tile row and column.
enum GjTiles { GJ_ALL = 0, GJ_PANEL = 1, GJ_REST = 2 };

__host__ __device__ inline size_t gj_tile_count(int mode, size_t nt) {
  return mode == GJ_ALL ? nt * nt : mode == GJ_PANEL ? 2 * nt - 1 : (nt - 1) * (nt - 1);
}

__device__ __forceinline__ void gj_tile(int mode, size_t nt, size_t tp, size_t u, size_t &tr, size_t &tc) {
  if (mode == GJ_ALL) {
    tr = u / nt;
    tc = u % nt;
  } else if (mode == GJ_PANEL) {
    if (u < nt) {
      tr = tp;
      tc = u;
    } else {
      const size_t w = u - nt;
      tr = w < tp ? w : w + 1;
      tc = tp;
    }
  } else {
    const size_t a = u / (nt - 1), b = u % (nt - 1);
    tr = a < tp ? a : a + 1;
    tc = b < tp ? b : b + 1;
  }
}

// Persistent and warp-specialised: CTA c of G takes the tiles
// [c T / G, (c + 1) T / G) of the T tiles of its tile set (128 x 128 each,
// row-major within the set, so that a CTA mostly stays in one tile row and
// stages the A operand, rows of Cs, once per row).  The CTA's tile number
// lt picks the B stage and the accumulator buffer (lt & 1).
//   producers (warps 0-3): stage B[c][k] = Rs[k][j0 + c] (and A[r][k] =
//     Cs[i0 + r][k] when the row changes) split into hi and lo, K-major;
//     thread 0 then issues the 8 K-steps x 3 MMAs of 128 x 128 x 8 into the
//     accumulator buffer and commits them to mma_done[lt & 1];
//   consumers (warps 4-11; lane quadrant warp % 4, column half): wait for
//     mma_done, read their 32 rows x 64 columns 32 columns at a time, free
//     the buffer (tmem_free[lt & 1]), transpose through shared memory and
//     update X row by row (coalesced).
// Staging of tile lt + 1 and the MMAs of tile lt overlap the write-back of
// tile lt - 1.  Every wait is bounded; when one runs out, DGF_TIMEOUT is
// raised, both roles stop, and the tensor memory is freed after a last
// bounded wait.
__global__ void __launch_bounds__(TC_THREADS, 1) k_gj_update(float *__restrict__ X, size_t n, size_t k0,
                                                             const float *__restrict__ Cs,
                                                             const float *__restrict__ Rs, size_t nt, int mode,
                                                             size_t tp, uint32_t *__restrict__ flags) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char *Ahi = tsm, *Alo = tsm + TC_OPER;
  unsigned char *Bst = tsm + 2 * TC_OPER;  // stage s: hi at Bst + 2 s TC_OPER, lo after it
  uint64_t *bar = reinterpret_cast<uint64_t *>(tsm + 6 * TC_OPER + TC_TBYTES);
  uint64_t *mma_done = bar, *tmem_free = bar + 2;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 4);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(bar + 5);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t ntile = gj_tile_count(mode, nt), G = gridDim.x;
  const size_t t_begin = blockIdx.x * ntile / G, t_end = (blockIdx.x + 1) * ntile / G;
  const size_t L = t_end - t_begin;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&mma_done[0], 1);
    mbar_init(&mma_done[1], 1);
    mbar_init(&tmem_free[0], TC_CONS_WARPS);
    mbar_init(&tmem_free[1], TC_CONS_WARPS);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  auto fail = [&]() {
    *abort_flag = 1;
    atomicOr(flags, DGF_TIMEOUT);
  };

  if (warp < TC_PROD_WARPS) {
    // ---- producers
    size_t a_row = ~(size_t)0;
    for (size_t lt = 0; lt < L; lt++) {
      size_t tr, tc;
      gj_tile(mode, nt, tp, t_begin + lt, tr, tc);
      const size_t i0 = tr * TC_M, j0 = tc * TC_N;
      const int st = (int)(lt & 1);
      unsigned char *Bhi = Bst + 2 * st * TC_OPER, *Blo = Bhi + TC_OPER;
      bool ok = true;
      // B stage st was last read by the MMAs of tile lt - 2; A by those of lt - 1
      if (lt >= 2) ok = mbar_wait_bounded(&mma_done[st], (uint32_t)(((lt - 2) >> 1) & 1), TC_WAIT_LIMIT);
      if (ok && tr != a_row && lt >= 1)
        ok = mbar_wait_bounded(&mma_done[st ^ 1], (uint32_t)(((lt - 1) >> 1) & 1), TC_WAIT_LIMIT);
      // every producer takes the same branch (a bar.sync below waits for all of them)
      const bool go = producers_all(ok && !*abort_flag);
      if (!go) {
        if (!ok) fail();
        break;
      }
      if (tr != a_row) {
        a_row = tr;
#pragma unroll 1
        for (int h = 0; h < 2; h++) {
          float4 va[8];
#pragma unroll
          for (int e = 0; e < 8; e++) {
            const int g = tid + (h * 8 + e) * TC_PROD, row = g >> 4, k4 = (g & 15) * 4;
            va[e] = i0 + row < n ? *reinterpret_cast<const float4 *>(Cs + (i0 + row) * TC_K + k4)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
          }
#pragma unroll
          for (int e = 0; e < 8; e++) {
            const int g = tid + (h * 8 + e) * TC_PROD, row = g >> 4, k4 = (g & 15) * 4;
            store_split(Ahi, Alo, kmaj_off(row, k4), va[e]);
          }
        }
      }
#pragma unroll 1
      for (int h = 0; h < 2; h++) {
        float4 vb[8];
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int g = tid + (h * 8 + e) * TC_PROD, c = g & (TC_N - 1), k4 = (g / TC_N) * 4;
          vb[e] = make_float4(0.f, 0.f, 0.f, 0.f);
          if (j0 + c < n) {
            const float *src = Rs + (size_t)k4 * n + j0 + c;
            vb[e] = make_float4(src[0], src[n], src[2 * n], src[3 * n]);
          }
        }
#pragma unroll
        for (int e = 0; e < 8; e++) {
          const int g = tid + (h * 8 + e) * TC_PROD, c = g & (TC_N - 1), k4 = (g / TC_N) * 4;
          store_split(Bhi, Blo, kmaj_off(c, k4), vb[e]);
        }
      }
      // the generic-proxy writes become visible to the tensor cores
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("bar.sync 1, %0;" ::"n"(TC_PROD) : "memory");
      if (tid == 0) {
        // accumulator buffer st was last read by the write-back of tile lt - 2
        if (lt >= 2 && !mbar_wait_bounded(&tmem_free[st], (uint32_t)(((lt - 2) >> 1) & 1), TC_WAIT_LIMIT)) {
          fail();
        } else {
          tc_fence_after();
          constexpr uint32_t idesc = tc_idesc_tf32(TC_M, TC_N);
          const uint32_t d = tmem + (uint32_t)st * TC_N;
          const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo), bh = smem_u32(Bhi), bl = smem_u32(Blo);
#pragma unroll
          for (int s = 0; s < TC_K / 8; s++) {
            const uint32_t off = (uint32_t)s * 2 * TC_LBO;  // 8 TF32 entries of K = two core matrices
            tc_mma_tf32(d, tc_desc(al + off, TC_LBO, TC_SBO), tc_desc(bh + off, TC_LBO, TC_SBO), idesc, s > 0);
            tc_mma_tf32(d, tc_desc(ah + off, TC_LBO, TC_SBO), tc_desc(bl + off, TC_LBO, TC_SBO), idesc, 1);
            tc_mma_tf32(d, tc_desc(ah + off, TC_LBO, TC_SBO), tc_desc(bh + off, TC_LBO, TC_SBO), idesc, 1);
          }
          tc_commit(&mma_done[st]);
        }
      }
    }
  } else {
    // ---- consumers
    const int cw = warp - TC_PROD_WARPS, q = warp & 3, half = cw >> 2;
    float *T = reinterpret_cast<float *>(tsm + 6 * TC_OPER) + cw * 32 * TC_TSTRIDE;
    for (size_t lt = 0; lt < L; lt++) {
      const int st = (int)(lt & 1);
      bool ok = false;
      for (int tries = 0; tries < 64 && !ok && !*abort_flag; tries++)  // bounded in total by the poll limit
        ok = mbar_wait_bounded(&mma_done[st], (uint32_t)((lt >> 1) & 1), TC_WAIT_LIMIT / 64);
      if (!ok) {
        if (!*abort_flag) fail();
        break;
      }
      tc_fence_after();
      size_t tr, tc;
      gj_tile(mode, nt, tp, t_begin + lt, tr, tc);
      const size_t i0 = tr * TC_M, j0 = tc * TC_N;
      const uint32_t tbase = tmem + (uint32_t)st * TC_N + ((uint32_t)(q * 32) << 16) + (uint32_t)(half * 64);
      // chunk 0 into the transpose scratch, chunk 1 held in registers; then
      // the accumulator buffer is free for the MMAs of tile lt + 2
      uint32_t v[32];
      tc_ld32(tbase, v);
#pragma unroll
      for (int c = 0; c < 32; c++) T[lane * TC_TSTRIDE + c] = __uint_as_float(v[c]);
      tc_ld32(tbase + 32u, v);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tmem_free[st]);
#pragma unroll 1
      for (int ch = 0; ch < 2; ch++) {
        if (ch == 1) {
#pragma unroll
          for (int c = 0; c < 32; c++) T[lane * TC_TSTRIDE + c] = __uint_as_float(v[c]);
          __syncwarp();
        }
        const size_t j = j0 + (size_t)(half * 64 + ch * 32 + lane);
        const bool jok = j < n && (j < k0 || j >= k0 + GJB);
        float xv[32];
#pragma unroll
        for (int rr = 0; rr < 32; rr++) {
          const size_t i = i0 + (size_t)(q * 32 + rr);
          xv[rr] = (jok && i < n && (i < k0 || i >= k0 + GJB)) ? X[i * n + j] : 0.f;
        }
#pragma unroll
        for (int rr = 0; rr < 32; rr++) {
          const size_t i = i0 + (size_t)(q * 32 + rr);
          if (jok && i < n && (i < k0 || i >= k0 + GJB)) X[i * n + j] = xv[rr] - T[rr * TC_TSTRIDE + lane];
        }
        __syncwarp();
      }
    }
  }
  __syncthreads();
  if (*abort_flag && tid == 0) {  // MMAs may still be running: a last bounded wait on both buffers
    mbar_wait_bounded(&mma_done[0], 0, TC_WAIT_LIMIT);
    mbar_wait_bounded(&mma_done[1], 0, TC_WAIT_LIMIT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS)
                 : "memory");
}

}  // namespace

// The host loop overlaps each block's serial part with the previous
// block's update: the update of block k first covers the panel of block
// k + 1 (its tile row and column); a side stream then runs k_gj_diag and
// k_gj_strips for block k + 1 (they read and write only rows and columns
// of block k + 1, final after the panel) while the main stream updates the
// remaining tiles of block k.  The strips and P alternate between two
// buffers; the main stream waits for block k + 1's strips before its
// update.
void coarse_inverse(Context &ctx, float *X, size_t n) {
  if (n == 0) return;
  cudaStream_t s = ctx.stream;
  ProfScope _prof(ctx, "mg_coarse_inverse", (double)n * n * 4 * 2 * ((n + GJB - 1) / GJB));
  const size_t nb = (n + GJB - 1) / GJB, nt = (n + TC_M - 1) / TC_M;
  DBuf<float> P(2 * GJB * GJB, s), Cs(2 * n * GJB, s), Rs(2 * GJB * n, s);
  ensure_smem_attr(ctx, k_gj_update, TC_SMEM);
  if (!ctx.side) {
    DG_CUDA(cudaStreamCreateWithFlags(&ctx.side, cudaStreamNonBlocking));
    DG_CUDA(cudaEventCreateWithFlags(&ctx.side_ev[0], cudaEventDisableTiming));
    DG_CUDA(cudaEventCreateWithFlags(&ctx.side_ev[1], cudaEventDisableTiming));
  }
  cudaStream_t side = ctx.side;
  cudaEvent_t ev_panel = ctx.side_ev[0], ev_strips = ctx.side_ev[1];
  auto blk = [&](size_t k, cudaStream_t st) {  // diag + strips of block k into buffer k & 1
    const size_t k0 = k * GJB, o = k & 1;
    const int b = (int)std::min<size_t>(GJB, n - k0);
    k_gj_diag<<<1, 256, 0, st>>>(X, n, k0, b, P.get() + o * GJB * GJB);
    k_gj_strips<<<(unsigned)nb, 256, 0, st>>>(X, n, k0, b, P.get() + o * GJB * GJB, Cs.get() + o * n * GJB,
                                             Rs.get() + o * GJB * n);
  };
  // an update CTA fills its SM (shared memory), so the update of the
  // remaining tiles leaves some SMs to the side stream's diag and strips
  const size_t side_sms = std::min<size_t>(16, (size_t)ctx.num_sms / 8);
  auto update = [&](size_t k, int mode, size_t tp) {
    const size_t o = k & 1, cnt = gj_tile_count(mode, nt);
    if (cnt == 0) return;
    const size_t sms = mode == GJ_REST ? (size_t)ctx.num_sms - side_sms : (size_t)ctx.num_sms;
    const unsigned grid = (unsigned)std::min<size_t>(cnt, sms);
    k_gj_update<<<grid, TC_THREADS, TC_SMEM, s>>>(X, n, k * GJB, Cs.get() + o * n * GJB, Rs.get() + o * GJB * n,
                                                  nt, mode, tp, ctx.d_flags);
  };
  try {
    blk(0, s);
    for (size_t k = 0; k < nb; k++) {
      if (k + 1 < nb) {
        const size_t tp = (k + 1) * GJB / TC_M;
        update(k, GJ_PANEL, tp);
        DG_CUDA(cudaEventRecord(ev_panel, s));
        DG_CUDA(cudaStreamWaitEvent(side, ev_panel, 0));
        blk(k + 1, side);
        DG_CUDA(cudaEventRecord(ev_strips, side));
        update(k, GJ_REST, tp);
        DG_CUDA(cudaStreamWaitEvent(s, ev_strips, 0));
      } else {
        update(k, GJ_ALL, 0);
      }
    }
    DG_LAUNCH_CHECK();
  } catch (...) {
    cudaStreamSynchronize(side);  // the scratch buffers are freed on the main stream
    throw;
  }
}

}  // namespace dg
