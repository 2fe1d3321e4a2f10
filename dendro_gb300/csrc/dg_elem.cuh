// Element-loop building blocks shared by the matVec kernels.
//
// Packed stencils: every type-2 stencil is symmetric, so a (child, type)
// pair keeps 36 Laplacian + 36 mass entries (lower triangle, row-major:
// entry (k, j), k >= j, at k(k+1)/2 + j).  All 144 pairs fit in shared
// memory in FP64 (83 KB) and FP32 (41 KB).
//
// Block accumulation: the elements of a block are consecutive in Morton
// order and share most of their nodes, so their 8 contributions each are
// first summed in a shared-memory hash table keyed by node id, then flushed
// with one global atomic per distinct node.  This cuts the global atomics
// several-fold and removes same-address contention between neighbouring
// elements.
#pragma once

#include "dg_common.cuh"

namespace dg {

constexpr int PSTEN_PER_TYPE = 72;                   // 36 + 36
constexpr int PSTEN_ENTRIES = 8 * 18 * PSTEN_PER_TYPE;

__host__ __device__ constexpr int tri_index(int k, int j) { return k >= j ? k * (k + 1) / 2 + j : j * (j + 1) / 2 + k; }

constexpr int ACC_SLOTS = 4096;
constexpr uint32_t ACC_EMPTY = 0xffffffffu;

template <typename T>
struct BlockAccum {
  uint32_t *key;
  T *val;

  __device__ __forceinline__ void clear() {
    for (int i = threadIdx.x; i < ACC_SLOTS; i += blockDim.x) {
      key[i] = ACC_EMPTY;
      val[i] = (T)0;
    }
  }
  // add v to node id; falls back to a global atomic when the probe bound is hit
  __device__ __forceinline__ void add(uint32_t id, T v, T *__restrict__ gy) {
    uint32_t h = (id * 2654435761u) >> 20;  // 12 bits
#pragma unroll 1
    for (int probe = 0; probe < 64; probe++) {
      uint32_t k = *(volatile uint32_t *)&key[h];
      if (k == id) {
        atomicAdd(&val[h], v);
        return;
      }
      if (k == ACC_EMPTY) {
        uint32_t old = atomicCAS(&key[h], ACC_EMPTY, id);
        if (old == ACC_EMPTY || old == id) {
          atomicAdd(&val[h], v);
          return;
        }
      }
      h = (h + 1) & (ACC_SLOTS - 1);
    }
    atomicAdd(&gy[id], v);
  }
  __device__ __forceinline__ void flush(T *__restrict__ gy) {
    for (int i = threadIdx.x; i < ACC_SLOTS; i += blockDim.x) {
      uint32_t k = key[i];
      if (k != ACC_EMPTY) atomicAdd(&gy[k], val[i]);
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

}  // namespace dg
