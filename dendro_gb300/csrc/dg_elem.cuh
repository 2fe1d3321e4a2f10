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
// Patches: PATCH consecutive elements form a patch.  Its tables:
//   pinc   the 8 x PATCH (element, vertex) pairs as slots (vertex * PATCH +
//          element within the patch, 12 bits), grouped into runs, one run per
//          node (runs in any order, the pairs of a run by slot);
//   pnode  the node of each run (pnode[poff[p] + u]);
//   prend  the end of each run's pairs, with RUN_COMPLETE when the run holds
//          every pair of its node in the whole mesh (its sum is then stored,
//          not added);
//   pmeta  the meta words of the patch's elements in (type, level) order (the
//          order slots use), bits 16..23 the element's stencil key;
//   pkeys  the patch's distinct (type, level) pairs.
// The element loop gathers x once per node into the slots, applies the
// element stencils slot to slot in shared memory and sums each run: no
// shared-memory atomics, and global atomics only for nodes that other
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
constexpr uint32_t ENT_SLOT = 0xfffu;
constexpr uint32_t RUN_END = 0x7fffu, RUN_COMPLETE = 0x8000u;  // run-end words
constexpr uint32_t RUN_BDY = 1u << 31;  // run node flag in shared memory (Dirichlet)

// 2^-l exactly, from the exponent bits (0 <= l <= 30)
__device__ __forceinline__ float exp2_neg(float, unsigned l) { return __int_as_float((int)(127u - l) << 23); }
__device__ __forceinline__ double exp2_neg(double, unsigned l) {
  return __longlong_as_double((long long)(1023u - l) << 52);
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
    double a = 0, b = 0;
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      const double2 sv = reinterpret_cast<const double2 *>(S + 8 * k + j)[0];
      a = fma(sv.x, xv[j], a);
      b = fma(sv.y, xv[j + 1], b);
    }
    emit(k, a + b);
  }
}

// y = (lapf K + massf M) x over the elements of every patch; with DIR the
// Dirichlet form: boundary rows are the identity (y = x), boundary columns
// are dropped.  One block of PATCH threads per patch, grid-strided:
//   stage  the patch's pair slots (in run order), each run's node and end,
//          its meta words and its combined stencils into shared memory;
//   1.     thread per run: x of the run's node into every slot of the run;
//   2.     thread per element: the element stencil, slot to slot;
//   3.     thread per run: the sum over the run's slots, stored (the run holds
//          every pair of its node) or added atomically (other patches share
//          the node).
template <typename T, bool DIR>
__global__ void __launch_bounds__(PATCH, sizeof(T) == 4 ? 2 : 1)
    k_patch_matvec(const uint32_t *__restrict__ pmeta, const uint16_t *__restrict__ pinc,
                   const uint16_t *__restrict__ prend, const uint32_t *__restrict__ pnode,
                   const uint64_t *__restrict__ poff, const uint16_t *__restrict__ pkeys,
                   const uint16_t *__restrict__ pkcount, size_t E, size_t n_patch, const T *__restrict__ fsten,
                   const uint32_t *__restrict__ cperm, const uint8_t *__restrict__ bdy, const T *__restrict__ x,
                   T *__restrict__ y, T lapf, T massf) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *cs = reinterpret_cast<T *>(smem_raw);
  T *buf = cs + fsten_entries<T>();
  T *sc = buf + PATCH_ENT;  // PKEY_MAX combined stencils
  uint32_t *rn = reinterpret_cast<uint32_t *>(sc + PKEY_MAX * sstride<T>());
  uint16_t *ents = reinterpret_cast<uint16_t *>(rn + PATCH_ENT);
  uint16_t *re = ents + PATCH_ENT;
  uint32_t *cp = reinterpret_cast<uint32_t *>(re + PATCH_ENT);
  for (int i = threadIdx.x; i < fsten_entries<T>(); i += PATCH) cs[i] = fsten[i];
  for (int i = threadIdx.x; i < 8 * 18; i += PATCH) cp[i] = cperm[i];
  __syncthreads();
  const int tid = threadIdx.x;
  for (size_t p = blockIdx.x; p < n_patch; p += gridDim.x) {
    const size_t e0 = p * PATCH;
    const int ne = (int)((E - e0) < (size_t)PATCH ? (E - e0) : (size_t)PATCH);
    const bool have = tid < ne;
    const uint64_t ub = poff[p];
    const int nr = (int)(poff[p + 1] - ub);
    const uint32_t kc = pkcount[p];
    // stage
    if (have) reinterpret_cast<uint4 *>(ents)[tid] = reinterpret_cast<const uint4 *>(pinc + p * PATCH_ENT)[tid];
    const uint32_t me = have ? pmeta[e0 + tid] : 0u;
    for (int u = tid; u < nr; u += PATCH) {
      const uint32_t g = pnode[ub + u];
      rn[u] = (DIR && bdy[g]) ? (g | RUN_BDY) : g;
      re[u] = prend[ub + u];
    }
    const bool comb = kc <= (uint32_t)PKEY_MAX;
    if (comb) {
      for (int i = tid; i < (int)kc * 64; i += PATCH) {
        const uint32_t key = pkeys[p * PKEY_MAX + (i >> 6)];
        const unsigned t = key >> 5, l = key & 31u;
        const T h = exp2_neg((T)0, l);
        const T *st = cs + t * fsten_stride<T>();
        sc[(i >> 6) * sstride<T>() + (i & 63)] =
            lapf * h * (T)0.5 * st[i & 63] + massf * h * h * h * (T)0.125 * st[64 + (i & 63)];
      }
    }
    __syncthreads();
    // 1. x of each run's node into the run's slots
    for (int u = tid; u < nr; u += PATCH) {
      const int b = u ? (int)(re[u - 1] & RUN_END) : 0, e = (int)(re[u] & RUN_END);
      const uint32_t tag = rn[u];
      const T xv = (DIR && (tag & RUN_BDY)) ? (T)0 : x[tag & ~RUN_BDY];
      for (int i = b; i < e; i++) buf[ents[i] & ENT_SLOT] = xv;
    }
    __syncthreads();
    // 2. element stencils, slot to slot (canonical stencil, relabelled slots)
    if (have) {
      const unsigned l = me & 255u, c = (me >> 8) & 7u, t = me >> 24;
      const uint32_t sig = cp[c * 18 + t];
      T xv[8];
#pragma unroll
      for (int m = 0; m < 8; m++) xv[m] = buf[((sig >> (3 * m)) & 7u) * PATCH + tid];
      auto put = [&](int m, T ym) { buf[((sig >> (3 * m)) & 7u) * PATCH + tid] = ym; };
      if (comb) {
        apply_comb(sc + ((me >> 16) & 255u) * sstride<T>(), xv, put);
      } else {
        const T h = exp2_neg((T)0, l);
        apply_full(cs + t * fsten_stride<T>(), lapf * h * (T)0.5, massf * h * h * h * (T)0.125, xv, put);
      }
    }
    __syncthreads();
    // 3. each run's sum to its node
    for (int u = tid; u < nr; u += PATCH) {
      const int b = u ? (int)(re[u - 1] & RUN_END) : 0, e = (int)(re[u] & RUN_END);
      T acc = (T)0;
      for (int i = b; i < e; i++) acc += buf[ents[i] & ENT_SLOT];
      const uint32_t tag = rn[u];
      const uint32_t g = tag & ~RUN_BDY;
      if (DIR && (tag & RUN_BDY)) y[g] = x[g];
      else if (re[u] & RUN_COMPLETE) y[g] = acc;
      else atomicAdd(&y[g], acc);
    }
    __syncthreads();
  }
}

template <typename T>
constexpr size_t patch_smem() {
  return fsten_entries<T>() * sizeof(T) + PATCH_ENT * sizeof(T) + PKEY_MAX * sstride<T>() * sizeof(T) +
         PATCH_ENT * sizeof(uint32_t) + 2 * PATCH_ENT * sizeof(uint16_t) + 8 * 18 * sizeof(uint32_t);
}

}  // namespace dg
