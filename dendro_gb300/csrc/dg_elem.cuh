// Element-loop building blocks shared by the matVec kernels.
//
// Canonical stencils: every (child, type) stencil is a relabelling of the
// child-0 stencil of the same type by one of the 48 symmetries of the cube,
// S(c,t)[k][j] = S(0,t)[p[k]][p[j]] (equal to rounding), so 18 full 8x8
// Laplacian + mass stencils (18 KB in FP64, 9 KB in FP32) and one 8-entry
// relabelling per (child, type) stand for all 144.  Full rows load as
// 16-byte vectors; the elements of a patch are ordered by (type, level), so
// the threads of a warp mostly read the same stencil (a broadcast).
//
// Patches: PATCH consecutive elements form a patch.  Its incidence table
// lists the 8 x PATCH (element, vertex) pairs grouped by node (one run per
// node, runs in the order of a per-patch hash table, the pairs of a run by
// slot), 16 bits each:
//   bits 0..11  slot = vertex * PATCH + element within the patch
//   bit 12      first pair of a node's run
//   bit 13      the run holds every pair of its node in the whole mesh, so
//               the node's sum is complete in this patch (stored, not added)
// pnode[poff[p] + u] is the node of run u of patch p, pexc[p][t] the number
// of runs that start before pair 8t, and pmeta[p][t] the meta word of the
// patch's element t in (type, level) order (the order slots use).  An element loop over a patch
// gathers x once per node into the slots, applies the element stencils
// slot-to-slot in shared memory, and sums each run with a segmented scan:
// no shared-memory atomics, and global atomics only for nodes that other
// patches also touch.
#pragma once

#include "dg_prims.cuh"

namespace dg {

// per type: 8x8 Laplacian rows, then 8x8 mass rows, then 16 bytes of padding
// so that the same row of two neighbouring types sits in different banks
template <typename T>
constexpr int fsten_stride() {
  return 128 + 16 / (int)sizeof(T);
}
template <typename T>
constexpr int fsten_entries() {
  return 18 * fsten_stride<T>();
}
constexpr int PATCH = 512;
constexpr int PATCH_ENT = 8 * PATCH;
// per-patch combined stencils: one 8x8 S = f1(l) L_t + f2(l) M_t per
// (type, level) present in the patch, up to PKEY_MAX of them; rows padded by
// 16 bytes so neighbouring keys sit in different banks
constexpr int PKEY_MAX = 64;
template <typename T>
constexpr int sstride() {
  return 64 + 16 / (int)sizeof(T);
}
constexpr uint32_t ENT_SLOT = 0xfffu, ENT_START = 1u << 12, ENT_COMPLETE = 1u << 13;
constexpr uint32_t RUN_BDY = 1u << 31;  // run node flag in shared memory (Dirichlet)

// 2^-l exactly, from the exponent bits (0 <= l <= 30)
__device__ __forceinline__ float exp2_neg(float, unsigned l) { return __int_as_float((int)(127u - l) << 23); }
__device__ __forceinline__ double exp2_neg(double, unsigned l) {
  return __longlong_as_double((long long)(1023u - l) << 52);
}

// combined stencils of every (type, level), 32 levels per type:
// comb[(t * 32 + l) * 64 + q] = lapf 2^-l / 2 L_t[q] + massf 2^-3l / 8 M_t[q]
// (the element loop copies the ones a patch uses into shared memory)
constexpr int COMB_LEVELS = 32;
constexpr int COMB_ENTRIES = 18 * COMB_LEVELS * 64;
template <typename T>
__global__ void k_comb_table(const T *__restrict__ cs, T lapf, T massf, T *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= COMB_ENTRIES) return;
  const int t = i / (COMB_LEVELS * 64), l = (i / 64) % COMB_LEVELS, q = i % 64;
  const T h = exp2_neg((T)0, (unsigned)l);
  const T *st = cs + t * fsten_stride<T>();
  out[i] = lapf * h * (T)0.5 * st[q] + massf * h * h * h * (T)0.125 * st[64 + q];
}

// two FP32 fused multiply-adds in one instruction (Blackwell f32x2)
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

// paired FP32 add, subtract and multiply (Blackwell f32x2), round to nearest
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

// y_k = f1 sum_j L[k][j] x_j + f2 sum_j M[k][j] x_j (full-row stencil S),
// handing each y_k to emit(k, y_k)
template <typename Emit>
__device__ __forceinline__ void apply_full(const float *__restrict__ S, float f1, float f2, const float (&xv)[8],
                                           Emit &&emit) {
  const float2 x0 = make_float2(xv[0], xv[1]), x1 = make_float2(xv[2], xv[3]);
  const float2 x2 = make_float2(xv[4], xv[5]), x3 = make_float2(xv[6], xv[7]);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float4 l0 = reinterpret_cast<const float4 *>(S + 8 * k)[0];
    const float4 l1 = reinterpret_cast<const float4 *>(S + 8 * k)[1];
    const float4 m0 = reinterpret_cast<const float4 *>(S + 64 + 8 * k)[0];
    const float4 m1 = reinterpret_cast<const float4 *>(S + 64 + 8 * k)[1];
    float2 aL = ffma2(make_float2(l0.x, l0.y), x0, make_float2(0.f, 0.f));
    aL = ffma2(make_float2(l0.z, l0.w), x1, aL);
    aL = ffma2(make_float2(l1.x, l1.y), x2, aL);
    aL = ffma2(make_float2(l1.z, l1.w), x3, aL);
    float2 aM = ffma2(make_float2(m0.x, m0.y), x0, make_float2(0.f, 0.f));
    aM = ffma2(make_float2(m0.z, m0.w), x1, aM);
    aM = ffma2(make_float2(m1.x, m1.y), x2, aM);
    aM = ffma2(make_float2(m1.z, m1.w), x3, aM);
    emit(k, f1 * (aL.x + aL.y) + f2 * (aM.x + aM.y));
  }
}

template <typename Emit>
__device__ __forceinline__ void apply_full(const double *__restrict__ S, double f1, double f2, const double (&xv)[8],
                                           Emit &&emit) {
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double aL = 0, aM = 0;
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      const double2 l = reinterpret_cast<const double2 *>(S + 8 * k + j)[0];
      const double2 m = reinterpret_cast<const double2 *>(S + 64 + 8 * k + j)[0];
      aL = fma(l.x, xv[j], aL);
      aL = fma(l.y, xv[j + 1], aL);
      aM = fma(m.x, xv[j], aM);
      aM = fma(m.y, xv[j + 1], aM);
    }
    emit(k, f1 * aL + f2 * aM);
  }
}

// y'_k = sum_j S[k][j] x_j with a combined, already scaled stencil S
template <typename Emit>
__device__ __forceinline__ void apply_comb(const float *__restrict__ S, const float (&xv)[8], Emit &&emit) {
  const float2 x0 = make_float2(xv[0], xv[1]), x1 = make_float2(xv[2], xv[3]);
  const float2 x2 = make_float2(xv[4], xv[5]), x3 = make_float2(xv[6], xv[7]);
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float4 s0 = reinterpret_cast<const float4 *>(S + 8 * k)[0];
    const float4 s1 = reinterpret_cast<const float4 *>(S + 8 * k)[1];
    float2 a = ffma2(make_float2(s0.x, s0.y), x0, make_float2(0.f, 0.f));
    a = ffma2(make_float2(s0.z, s0.w), x1, a);
    a = ffma2(make_float2(s1.x, s1.y), x2, a);
    a = ffma2(make_float2(s1.z, s1.w), x3, a);
    emit(k, a.x + a.y);
  }
}

template <typename Emit>
__device__ __forceinline__ void apply_comb(const double *__restrict__ S, const double (&xv)[8], Emit &&emit) {
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double a = 0;
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      const double2 sv = reinterpret_cast<const double2 *>(S + 8 * k + j)[0];
      a = fma(sv.x, xv[j], a);
      a = fma(sv.y, xv[j + 1], a);
    }
    emit(k, a);
  }
}

// y = (lapf K + massf M) x over the elements of every patch; with DIR the
// Dirichlet form: boundary rows are the identity (y = x), boundary columns
// are dropped.  One block of PATCH threads per patch, grid-strided; thread t
// holds pairs 8t..8t+7 of the patch's table and is element t of the patch.
// The slot buffer and the run-node array are single (a patch costs four
// barriers) so that more blocks fit an SM: three in FP32 (40 registers per
// thread), two in FP64; one block's gathers and sums overlap another's
// stencil phase.  (Double-buffering them by patch parity saves a barrier
// but halves the blocks; measured slower.)  The next patch's table words are
// loaded one patch ahead.
template <typename T>
constexpr int patch_nbuf() {
  return 1;
}

// With COEF, element e's factors are coef[2e] (Laplacian) and coef[2e + 1]
// (mass) instead of lapf and massf (pperm gives e from the patch order).
template <typename T, bool DIR, bool COEF = false>
__global__ void __launch_bounds__(PATCH, sizeof(T) == 4 ? 3 : 2)
    k_patch_matvec(const uint32_t *__restrict__ pmeta, const uint16_t *__restrict__ pinc,
                   const uint16_t *__restrict__ pexc, const uint32_t *__restrict__ pnode,
                   const uint64_t *__restrict__ poff, const uint16_t *__restrict__ pkeys,
                   const uint16_t *__restrict__ pkcount, size_t E, size_t n_patch, const T *__restrict__ fsten,
                   const T *__restrict__ ctab, const uint32_t *__restrict__ cperm, const uint8_t *__restrict__ bdy,
                   const T *__restrict__ x, T *__restrict__ y, T lapf, T massf,
                   const double *__restrict__ coef = nullptr, const uint16_t *__restrict__ pperm = nullptr) {
  constexpr int NW = PATCH / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *cs = reinterpret_cast<T *>(smem_raw);
  constexpr int NBUF = patch_nbuf<T>();
  T *bufs = cs + fsten_entries<T>();
  uint32_t *gns = reinterpret_cast<uint32_t *>(bufs + NBUF * PATCH_ENT);
  uint32_t *cp = gns + NBUF * PATCH_ENT;
  T *sc = reinterpret_cast<T *>(cp + 8 * 18 + 4);  // PKEY_MAX combined stencils (16-byte aligned)
  __shared__ T ws_v[2][NW];
  __shared__ int ws_f[2][NW];
  __shared__ int ws_first[2][NW + 1];
  for (int i = threadIdx.x; i < fsten_entries<T>(); i += PATCH) cs[i] = fsten[i];
  for (int i = threadIdx.x; i < 8 * 18; i += PATCH) cp[i] = cperm[i];
  __syncthreads();  // step 1 of the first patch already reads cs
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  auto patch_ne = [&](size_t q) { return (int)((E - q * PATCH) < (size_t)PATCH ? (E - q * PATCH) : (size_t)PATCH); };
  size_t p = blockIdx.x;
  uint4 w = make_uint4(0, 0, 0, 0);
  uint32_t ex = 0, me = 0, kc = 0;
  uint64_t ub = 0;
  if (p < n_patch) {
    ub = poff[p];
    kc = pkcount[p];
    if (tid < patch_ne(p)) {
      w = reinterpret_cast<const uint4 *>(pinc + p * PATCH_ENT)[tid];
      ex = pexc[p * PATCH + tid];
      me = pmeta[p * PATCH + tid];
    }
  }
  int par = 0;
  for (; p < n_patch; p += gridDim.x, par ^= (NBUF - 1)) {
    const int ne = patch_ne(p);
    const bool have = tid < ne;
    const uint4 cw = w;
    const uint32_t cex = ex, cme = me, ckc = kc;
    const uint64_t cub = ub;
    // the next patch's table words, one patch ahead
    const size_t pn = p + gridDim.x;
    if (pn < n_patch) {
      ub = poff[pn];
      kc = pkcount[pn];
      if (tid < patch_ne(pn)) {
        w = reinterpret_cast<const uint4 *>(pinc + pn * PATCH_ENT)[tid];
        ex = pexc[pn * PATCH + tid];
        me = pmeta[pn * PATCH + tid];
      }
    }
    auto ent = [&](int j) -> uint32_t {
      const uint32_t word = j < 2 ? cw.x : j < 4 ? cw.y : j < 6 ? cw.z : cw.w;
      return (j & 1) ? word >> 16 : word & 0xffffu;
    };
    T *buf = bufs + par * PATCH_ENT;
    uint32_t *gn = gns + par * PATCH_ENT;
    // 1. x of each run's node into its slots; the run's node into gn
    if (have) {
      int u = (int)cex - 1;
      T xv = (T)0;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const uint32_t e = ent(j);
        if (e & ENT_START) {
          u++;
          const uint32_t g = pnode[cub + u];
          xv = x[g];
          uint32_t tag = g;
          if (DIR && bdy[g]) {
            xv = (T)0;
            tag |= RUN_BDY;
          }
          gn[u] = tag;
        } else if (j == 0) {
          xv = x[pnode[cub + u]];  // the run began in an earlier thread
          if (DIR && bdy[pnode[cub + u]]) xv = (T)0;
        }
        buf[e & ENT_SLOT] = xv;
      }
    }
    // the patch's combined stencils (read only in step 2 of this patch, and
    // rewritten only after every thread has passed that step's barrier)
    const bool comb = !COEF && ckc <= (uint32_t)PKEY_MAX;
    if (comb) {
      for (int i = tid; i < (int)ckc * 64; i += PATCH) {
        const uint32_t key = pkeys[p * PKEY_MAX + (i >> 6)];
        const unsigned t = key >> 5, l = key & 31u;
        if constexpr (sizeof(T) == 8) {
          // FP64 issue is scarce: copy the precomputed entry
          sc[(i >> 6) * sstride<T>() + (i & 63)] = ctab[(t * COMB_LEVELS + l) * 64 + (i & 63)];
        } else {
          const T h = exp2_neg((T)0, l);
          const T *st = cs + t * fsten_stride<T>();
          sc[(i >> 6) * sstride<T>() + (i & 63)] =
              lapf * h * (T)0.5 * st[i & 63] + massf * h * h * h * (T)0.125 * st[64 + (i & 63)];
        }
      }
    }
    if (lane == 0) ws_first[par][wid] = (ent(0) & ENT_START) ? 1 : 0;
    if (tid == 0) ws_first[par][NW] = 1;
    __syncthreads();
    // 2. element stencils, slot to slot (canonical stencil, relabelled slots)
    if (have) {
      const unsigned l = cme & 255u, c = (cme >> 8) & 7u, t = cme >> 24;
      const uint32_t sig = cp[c * 18 + t];
      T xv[8];
#pragma unroll
      for (int m = 0; m < 8; m++) xv[m] = buf[((sig >> (3 * m)) & 7u) * PATCH + tid];
      auto put = [&](int m, T ym) { buf[((sig >> (3 * m)) & 7u) * PATCH + tid] = ym; };
      if (comb) {
        apply_comb(sc + ((cme >> 16) & 255u) * sstride<T>(), xv, put);
      } else {
        const T h = exp2_neg((T)0, l);
        T lf = lapf, mf = massf;
        if constexpr (COEF) {
          const size_t e = p * PATCH + pperm[p * PATCH + tid];
          lf = (T)coef[2 * e];
          mf = (T)coef[2 * e + 1];
        }
        apply_full(cs + t * fsten_stride<T>(), lf * h * (T)0.5, mf * h * h * h * (T)0.125, xv, put);
      }
    }
    __syncthreads();
    // 3. run sums: segmented scan of the threads' trailing partial sums
    T v[8];
    T tail = (T)0;
    int head = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const uint32_t e = ent(j);
      v[j] = have ? buf[e & ENT_SLOT] : (T)0;
      if (e & ENT_START) {
        head = 1;
        tail = (T)0;
      }
      tail += v[j];
    }
    T s = tail;
    int f = head;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T s2 = __shfl_up_sync(0xffffffffu, s, o);
      const int f2 = __shfl_up_sync(0xffffffffu, f, o);
      if (lane >= o) {
        if (!f) s += s2;
        f |= f2;
      }
    }
    if (lane == 31) {
      ws_v[par][wid] = s;
      ws_f[par][wid] = f;
    }
    __syncthreads();
    T wv = lane < NW ? ws_v[par][lane] : (T)0;
    int wf = lane < NW ? ws_f[par][lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T s2 = __shfl_up_sync(0xffffffffu, wv, o);
      const int f2 = __shfl_up_sync(0xffffffffu, wf, o);
      if (lane >= o) {
        if (!wf) wv += s2;
        wf |= f2;
      }
    }
    const T wpre = __shfl_sync(0xffffffffu, wv, wid > 0 ? wid - 1 : 0);
    const T wprefix = wid > 0 ? wpre : (T)0;
    const T ex_s = __shfl_up_sync(0xffffffffu, s, 1);
    const int ex_f = __shfl_up_sync(0xffffffffu, f, 1);
    const T carry = (lane == 0) ? wprefix : (ex_f ? ex_s : wprefix + ex_s);
    const int nxt = __shfl_down_sync(0xffffffffu, (ent(0) & ENT_START) ? 1 : 0, 1);
    if (have) {
      const bool last_run_ends = tid + 1 >= ne || (lane < 31 ? nxt : ws_first[par][wid + 1]);
      auto emit = [&](int u, T acc, uint32_t e) {
        const uint32_t tag = gn[u];
        const uint32_t g = tag & ~RUN_BDY;
        if (DIR && (tag & RUN_BDY)) y[g] = x[g];
        else if (e & ENT_COMPLETE) y[g] = acc;
        else atomicAdd(&y[g], acc);
      };
      int u = (int)cex - 1;
      T acc = carry;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const uint32_t e = ent(j);
        if (e & ENT_START) {
          if (j > 0) emit(u, acc, ent(j - 1));
          u++;
          acc = (T)0;
        }
        acc += v[j];
      }
      if (last_run_ends) emit(u, acc, ent(7));
    }
    if (NBUF == 1) __syncthreads();  // the next patch rewrites buf and gn
  }
}

// The same operator from run-indexed tables (run form).  Per
// patch: plid[p][t] holds, for the element at (type, level) position t, the
// patch-local run (node) index of each of its 8 vertices in the canonical
// (relabelled) order of its stencil, and prun[poff[p] + u] the node of run u
// with bit 31 set when the run holds every pair of its node in the mesh.
// One block of PATCH threads per patch, grid-strided, three barriers per
// patch:
//   1. x of every run's node into xs[u] (runs spread over the threads, so
//      the node ids are read coalesced), ys[u] = 0;
//   2. thread t = element t: x from xs through its 8 run indices, the
//      element stencil, the 8 results added into ys with shared-memory
//      atomics;
//   3. each run's sum stored (complete runs) or added atomically to y.
// No per-pair slots and no segmented scan: the shared traffic per element
// is 8 loads and 8 atomic adds, against 8 stores, 16 loads and 8 stores in
// the pair form above.
constexpr uint32_t PRUN_COMPLETE = 1u << 31;
constexpr uint32_t PRUN_BDY = 1u << 30;  // the run's node lies on the domain boundary
constexpr uint32_t PRUN_NODE = PRUN_BDY - 1;

template <typename T, bool DIR>
__global__ void __launch_bounds__(PATCH, sizeof(T) == 4 ? 3 : 2)
    k_patch_matvec_runs(const uint32_t *__restrict__ pmeta, const uint4 *__restrict__ plid,
                        const uint32_t *__restrict__ prun, const uint64_t *__restrict__ poff,
                        const uint16_t *__restrict__ pkeys, const uint16_t *__restrict__ pkcount, size_t E,
                        size_t n_patch, const T *__restrict__ fsten, const T *__restrict__ ctab,
                        const T *__restrict__ x, T *__restrict__ y, T lapf, T massf) {
  // FP32 keeps the canonical stencils in shared memory and forms the
  // patch's combined stencils from them; FP64 (whose arithmetic is the
  // scarce resource) copies the combined stencils from the (type, level)
  // table and reads the canonical ones from global memory on the rare
  // patches with more than PKEY_MAX keys
  constexpr bool F32 = sizeof(T) == 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *cs = reinterpret_cast<T *>(smem_raw);
  T *xs = cs + (F32 ? fsten_entries<T>() : 0);
  T *ys = xs + PATCH_ENT;
  T *sc = ys + PATCH_ENT;  // PKEY_MAX combined stencils (16-byte aligned)
  if (F32)
    for (int i = threadIdx.x; i < fsten_entries<T>(); i += PATCH) cs[i] = fsten[i];
  const T *gst = F32 ? cs : fsten;
  const int tid = threadIdx.x;
  for (size_t p = blockIdx.x; p < n_patch; p += gridDim.x) {
    const int ne = (int)((E - p * PATCH) < (size_t)PATCH ? (E - p * PATCH) : (size_t)PATCH);
    const uint64_t ub = poff[p];
    const int nr = (int)(poff[p + 1] - ub);
    const uint32_t kc = pkcount[p];
    const bool comb = kc <= (uint32_t)PKEY_MAX;
    // this element's tables, loaded before the gather so that their latency
    // overlaps it
    uint32_t me = 0;
    uint4 lw = make_uint4(0, 0, 0, 0);
    if (tid < ne) {
      me = pmeta[p * PATCH + tid];
      lw = plid[p * PATCH + tid];
    }
    __syncthreads();  // the previous patch is done with xs, ys and sc (and cs is loaded)
    // 1. gather
    for (int u = tid; u < nr; u += PATCH) {
      const uint32_t r = prun[ub + u];
      xs[u] = (DIR && (r & PRUN_BDY)) ? (T)0 : x[r & PRUN_NODE];
      ys[u] = (T)0;
    }
    if (comb) {
      for (int i = tid; i < (int)kc * 64; i += PATCH) {
        const uint32_t key = pkeys[p * PKEY_MAX + (i >> 6)];
        const unsigned t = key >> 5, l = key & 31u;
        if constexpr (F32) {
          const T h = exp2_neg((T)0, l);
          const T *st = cs + t * fsten_stride<T>();
          sc[(i >> 6) * sstride<T>() + (i & 63)] =
              lapf * h * (T)0.5 * st[i & 63] + massf * h * h * h * (T)0.125 * st[64 + (i & 63)];
        } else {
          sc[(i >> 6) * sstride<T>() + (i & 63)] = ctab[(t * COMB_LEVELS + l) * 64 + (i & 63)];
        }
      }
    }
    __syncthreads();
    // 2. element stencils
    if (tid < ne) {
      const uint32_t lv[4] = {lw.x, lw.y, lw.z, lw.w};
      int lid[8];
#pragma unroll
      for (int m = 0; m < 8; m++) lid[m] = (int)((lv[m >> 1] >> ((m & 1) * 16)) & 0xffffu);
      T xv[8];
#pragma unroll
      for (int m = 0; m < 8; m++) xv[m] = xs[lid[m]];
      auto put = [&](int m, T ym) { atomicAdd(&ys[lid[m]], ym); };
      if (comb) {
        apply_comb(sc + ((me >> 16) & 255u) * sstride<T>(), xv, put);
      } else {
        const unsigned l = me & 255u, t = me >> 24;
        const T h = exp2_neg((T)0, l);
        apply_full(gst + t * fsten_stride<T>(), lapf * h * (T)0.5, massf * h * h * h * (T)0.125, xv, put);
      }
    }
    __syncthreads();
    // 3. run sums out (the run words are read again: cached since step 1)
    for (int u = tid; u < nr; u += PATCH) {
      const uint32_t r = prun[ub + u], g = r & PRUN_NODE;
      if (DIR && (r & PRUN_BDY)) y[g] = x[g];
      else if (r & PRUN_COMPLETE) y[g] = ys[u];
      else atomicAdd(&y[g], ys[u]);
    }
  }
}

// ---- double-single (FP32 pair) form of the run-form loop: the CG operator
// of the FP32-V-cycle solve.  GB300 issues FP64 at 2 multiply-adds per
// clock per SM, and the FP64 loop is bound by that.  Here each stencil
// entry a and each gathered x are pairs (hi, lo) of FP32 values with
// hi + lo equal to the FP64 value to about 2^-48; each product is formed
// exactly (hi * hi and its rounding error by an FMA, plus the two cross
// terms) and the 8 products of a row are summed with an error-free sum
// (TwoSum) into a (hi, lo) pair, so a row is exact to about 2^-46 of the
// sum of its terms' magnitudes.  The row results are summed per run in
// 64-bit fixed point (below), so an element costs no FP64 operation at all;
// only the split of each gathered x and each run's final sum use the FP64
// pipe.  The paired instructions (f32x2) keep the compiler from fusing the
// sums with the products, as the explicit FMAs do for the exact products.
//
// ds_term2: two rows k, k + 1 at once; a = (hi_k, hi_k+1, lo_k, lo_k+1) of
// column j, x = (hi, lo) of x_j; (sh, sl) hold the two rows' running
// (hi, lo) sums
__device__ __forceinline__ void ds_term2(float2 &sh, float2 &sl, float4 a, float2 x) {
  const float2 ah = make_float2(a.x, a.y), al = make_float2(a.z, a.w);
  const float2 xh = make_float2(x.x, x.x), xl = make_float2(x.y, x.y);
  const float2 ph = fmul2(ah, xh);
  float2 pl = make_float2(fmaf(a.x, x.x, -ph.x), fmaf(a.y, x.x, -ph.y));  // exact: hi * hi - ph
  pl = ffma2(ah, xl, pl);
  pl = ffma2(al, xh, pl);
  const float2 s = fadd2(sh, ph);
  const float2 v = fsub2(s, sh);
  const float2 e = fadd2(fsub2(sh, fsub2(s, v)), fsub2(ph, v));
  sl = fadd2(sl, fadd2(e, pl));
  sh = s;
}

// round(f * 2^s) as a 64-bit integer, by integer operations (the ALU
// pipe): FP32 normal and subnormal values; the caller keeps |f| * 2^s below
// 2^62
__device__ __forceinline__ long long f2fix(float f, int s) {
  const uint32_t u = __float_as_uint(f);
  if (!(u & 0x7fffffffu)) return 0;
  const int e = (int)((u >> 23) & 0xffu);
  const long long m = e ? (long long)((u & 0x7fffffu) | 0x800000u) : (long long)(u & 0x7fffffu);
  const int sh = (e ? e : 1) - 150 + s;  // f * 2^s = m * 2^sh
  long long r;
  if (sh >= 0) r = m << (sh < 39 ? sh : 39);
  else if (sh > -63) r = (m + (1ll << (-sh - 1))) >> (-sh);
  else r = 0;
  return (u >> 31) ? -r : r;
}

constexpr int DS_STRIDE = 32;  // float4 entries per combined stencil: (row pair, column)

// ctab: the combined stencils of every (type, level) as (hi, lo) pairs,
// laid out per (row pair p, column j) as (hi[2p][j], hi[2p+1][j],
// lo[2p][j], lo[2p+1][j]);
// rowabs: per (type, level) the largest row sum of |entries| (rounded up).
// x is scaled by xscale = 2^k on the way in and the results by 2^yshift =
// 2^-k on the way out (both exact), so that the FP32 parts stay far from
// FP32's underflow whatever the vectors' magnitude.  The row results are
// summed per run in 64-bit fixed point (shared-memory integer atomic adds;
// FP64 shared-memory atomic adds cost about three FP64 operations each on
// GB300's narrow FP64 pipe): the patch's scale 2^s makes (largest |x| of
// the patch) x (largest row sum of its stencils) x 4096 (the most pairs a
// run can have) smaller than 2^62, so no sum overflows, and a row result is
// kept to 2^-50 of that bound.
template <bool DIR>
__global__ void __launch_bounds__(PATCH, 2)
    k_patch_matvec_runs_ds(const uint32_t *__restrict__ pmeta, const uint4 *__restrict__ plid,
                           const uint32_t *__restrict__ prun, const uint64_t *__restrict__ poff,
                           const uint16_t *__restrict__ pkeys, const uint16_t *__restrict__ pkcount, size_t E,
                           size_t n_patch, const float4 *__restrict__ ctab, const float *__restrict__ rowabs,
                           const double *__restrict__ x, double *__restrict__ y, double xscale, int yshift) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *xs = reinterpret_cast<float2 *>(smem_raw);
  unsigned long long *ys = reinterpret_cast<unsigned long long *>(xs + PATCH_ENT);
  float4 *sc = reinterpret_cast<float4 *>(ys + PATCH_ENT);  // PKEY_MAX combined stencils
  __shared__ uint32_t xmax_bits[2], smax_bits[2];  // per patch parity: largest |x|, largest row sum
  const int tid = threadIdx.x;
  if (tid < 2) xmax_bits[tid] = smax_bits[tid] = 0;
  int par = 0;
  for (size_t p = blockIdx.x; p < n_patch; p += gridDim.x, par ^= 1) {
    const int ne = (int)((E - p * PATCH) < (size_t)PATCH ? (E - p * PATCH) : (size_t)PATCH);
    const uint64_t ub = poff[p];
    const int nr = (int)(poff[p + 1] - ub);
    const uint32_t kc = pkcount[p];
    const bool comb = kc <= (uint32_t)PKEY_MAX;
    uint32_t me = 0;
    uint4 lw = make_uint4(0, 0, 0, 0);
    float rmax = 0.f;
    if (tid < ne) {
      me = pmeta[p * PATCH + tid];
      lw = plid[p * PATCH + tid];
      rmax = rowabs[(me >> 24) * COMB_LEVELS + (me & 31u)];
    }
    __syncthreads();  // the previous patch is done with xs, ys, sc and its bounds
    // 1. gather, each x split into (hi, lo); the patch's bounds
    float xmax = 0.f;
    for (int u = tid; u < nr; u += PATCH) {
      const uint32_t r = prun[ub + u];
      const double xv = (DIR && (r & PRUN_BDY)) ? 0.0 : x[r & PRUN_NODE] * xscale;
      const float hi = __double2float_rn(xv);
      xs[u] = make_float2(hi, __double2float_rn(xv - (double)hi));
      ys[u] = 0ull;
      xmax = fmaxf(xmax, fabsf(hi));
    }
    const uint32_t wx = __reduce_max_sync(0xffffffffu, __float_as_uint(xmax));  // non-negative: bits order as values
    const uint32_t ws = __reduce_max_sync(0xffffffffu, __float_as_uint(rmax));
    if ((tid & 31) == 0) {
      atomicMax(&xmax_bits[par], wx);
      atomicMax(&smax_bits[par], ws);
    }
    if (comb) {
      for (int i = tid; i < (int)kc * DS_STRIDE; i += PATCH) {
        const uint32_t key = pkeys[p * PKEY_MAX + i / DS_STRIDE];
        sc[i] = ctab[((key >> 5) * COMB_LEVELS + (key & 31u)) * DS_STRIDE + i % DS_STRIDE];
      }
    }
    __syncthreads();
    const double bound = (double)__uint_as_float(xmax_bits[par]) * (double)__uint_as_float(smax_bits[par]);
    const int fs = bound > 0.0 ? 49 - ilogb(bound) : 0;  // the fixed-point scale 2^fs
    const double out_scale = ldexp(1.0, yshift - fs);
    if (tid == 0) xmax_bits[par ^ 1] = smax_bits[par ^ 1] = 0;  // for the next patch
    // 2. element stencils
    if (tid < ne) {
      const uint32_t lv[4] = {lw.x, lw.y, lw.z, lw.w};
      int lid[8];
#pragma unroll
      for (int m = 0; m < 8; m++) lid[m] = (int)((lv[m >> 1] >> ((m & 1) * 16)) & 0xffffu);
      float2 xv[8];
#pragma unroll
      for (int m = 0; m < 8; m++) xv[m] = xs[lid[m]];
      const float4 *S = comb ? sc + ((me >> 16) & 255u) * DS_STRIDE
                             : ctab + ((me >> 24) * COMB_LEVELS + (me & 31u)) * DS_STRIDE;
#pragma unroll
      for (int pr = 0; pr < 4; pr++) {
        float2 sh = make_float2(0.f, 0.f), sl = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 8; j++) ds_term2(sh, sl, S[pr * 8 + j], xv[j]);
        atomicAdd(&ys[lid[2 * pr]], (unsigned long long)(f2fix(sh.x, fs) + f2fix(sl.x, fs)));
        atomicAdd(&ys[lid[2 * pr + 1]], (unsigned long long)(f2fix(sh.y, fs) + f2fix(sl.y, fs)));
      }
    }
    __syncthreads();
    // 3. run sums out
    for (int u = tid; u < nr; u += PATCH) {
      const uint32_t r = prun[ub + u], g = r & PRUN_NODE;
      const double v = (double)(long long)ys[u] * out_scale;
      if (DIR && (r & PRUN_BDY)) y[g] = x[g];
      else if (r & PRUN_COMPLETE) y[g] = v;
      else atomicAdd(&y[g], v);
    }
  }
}

constexpr size_t patch_runs_ds_smem() {
  return PATCH_ENT * sizeof(float2) + PATCH_ENT * sizeof(unsigned long long) + PKEY_MAX * DS_STRIDE * sizeof(float4);
}

template <typename T>
constexpr size_t patch_runs_smem() {
  return (sizeof(T) == 4 ? fsten_entries<T>() * sizeof(T) : 0) + 2 * PATCH_ENT * sizeof(T) +
         PKEY_MAX * sstride<T>() * sizeof(T);
}

template <typename T>
constexpr size_t patch_smem() {
  return fsten_entries<T>() * sizeof(T) + patch_nbuf<T>() * PATCH_ENT * (sizeof(T) + sizeof(uint32_t)) +
         (8 * 18 + 4) * sizeof(uint32_t) + PKEY_MAX * sstride<T>() * sizeof(T);
}

}  // namespace dg
