// Element-loop building blocks shared by the matVec kernels.
//
// Packed stencils: every type-2 stencil is symmetric, so a (child, type)
// pair keeps 36 Laplacian + 36 mass entries (lower triangle, row-major:
// entry (k, j), k >= j, at k(k+1)/2 + j).  All 144 pairs fit in shared
// memory in FP64 (83 KB) and FP32 (41 KB).
//
// Block accumulation: the elements of a block are consecutive in Morton
// order, and node ids follow the element order of their owners, so the
// nodes a block touches sit mostly in a short id window starting at the
// smallest id the block touches.  Contributions inside the window are summed
// with shared-memory atomics, the window is flushed with one global atomic
// per touched node, and the few contributions outside it go to global
// memory directly.
#pragma once

#include "dg_common.cuh"

namespace dg {

constexpr int PSTEN_PER_TYPE = 72;                   // 36 + 36
constexpr int PSTEN_ENTRIES = 8 * 18 * PSTEN_PER_TYPE;

__host__ __device__ constexpr int tri_index(int k, int j) { return k >= j ? k * (k + 1) / 2 + j : j * (j + 1) / 2 + k; }

// node ids summed in shared memory per chunk: 16 KB of accumulators
template <typename T>
constexpr int acc_window() {
  return 16384 / (int)sizeof(T);
}

// window accumulator: W consecutive node ids from lo
template <typename T, int W>
struct WindowAccum {
  T *val;          // W entries, zero between chunks
  uint32_t *lo_s;  // shared word
  __device__ __forceinline__ void init() {
    for (int i = threadIdx.x; i < W; i += blockDim.x) val[i] = (T)0;
  }
  // block-wide: lo = smallest id of the chunk (call with UINT_MAX for idle threads)
  __device__ __forceinline__ void set_lo(uint32_t my_min) {
    if (threadIdx.x == 0) *lo_s = 0xffffffffu;
    __syncthreads();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_min = min(my_min, __shfl_xor_sync(0xffffffffu, my_min, o));
    if ((threadIdx.x & 31) == 0) atomicMin(lo_s, my_min);
    __syncthreads();
  }
  __device__ __forceinline__ void add(uint32_t id, T v, T *__restrict__ gy) {
    const uint32_t off = id - *lo_s;
    if (off < (uint32_t)W) atomicAdd(&val[off], v);
    else atomicAdd(&gy[id], v);
  }
  // flush touched entries and zero them for the next chunk (after a barrier)
  __device__ __forceinline__ void flush(T *__restrict__ gy, size_t n) {
    const uint32_t lo = *lo_s;
    for (int i = threadIdx.x; i < W; i += blockDim.x) {
      T v = val[i];
      if (v != (T)0) {
        if ((size_t)lo + i < n) atomicAdd(&gy[lo + i], v);
        val[i] = (T)0;
      }
    }
  }
};

// y_k = sum_j (f1 L[k][j] + f2 M[k][j]) x_j for k = 0..7 from a packed stencil
template <typename T>
__device__ __forceinline__ void apply_packed(const T *__restrict__ P, T f1, T f2, const T (&xv)[8], T (&yv)[8]) {
#pragma unroll
  for (int k = 0; k < 8; k++) {
    T aL = 0, aM = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      aL += P[tri_index(k, j)] * xv[j];
      aM += P[36 + tri_index(k, j)] * xv[j];
    }
    yv[k] = f1 * aL + f2 * aM;
  }
}

// same, handing each y_k to emit(k, y_k) as soon as it is formed (keeps
// fewer values live than a y array)
template <typename T, typename Emit>
__device__ __forceinline__ void apply_packed_emit(const T *__restrict__ P, T f1, T f2, const T (&xv)[8], Emit &&emit) {
#pragma unroll
  for (int k = 0; k < 8; k++) {
    T aL = 0, aM = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      aL += P[tri_index(k, j)] * xv[j];
      aM += P[36 + tri_index(k, j)] * xv[j];
    }
    emit(k, f1 * aL + f2 * aM);
  }
}

}  // namespace dg
