// Shared device/host helpers for the GB300 octree hot path.
//
// Octant keys: the Morton (bit-interleaved, z above y above x) index of the
// anchor at the finest level D, right-aligned in a 128-bit value; an octant
// at level l has its low 3*(D-l) key bits zero.  Linear octrees are stored as
// a key array plus a level array (one byte per octant); since a linear
// octree never holds two octants with the same anchor, the key alone orders
// it exactly like the reference's TreeNode::operator< (TreeNode.tcc:211-236).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>

#include "dendro_gb300.h"

namespace dg {

typedef unsigned __int128 u128;

struct __align__(16) Key128 {
  uint64_t lo, hi;
};

__host__ __device__ __forceinline__ u128 to_u128(Key128 k) { return ((u128)k.hi << 64) | (u128)k.lo; }
__host__ __device__ __forceinline__ Key128 from_u128(u128 v) {
  Key128 k;
  k.lo = (uint64_t)v;
  k.hi = (uint64_t)(v >> 64);
  return k;
}
__host__ __device__ __forceinline__ bool key_eq(Key128 a, Key128 b) { return a.lo == b.lo && a.hi == b.hi; }
__host__ __device__ __forceinline__ bool key_lt(Key128 a, Key128 b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__host__ __device__ __forceinline__ bool key_le(Key128 a, Key128 b) { return !key_lt(b, a); }

// spread the low 21 bits of v to every third bit (bit i -> bit 3i)
__host__ __device__ __forceinline__ uint64_t spread21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}
// inverse of spread21
__host__ __device__ __forceinline__ uint32_t compact21(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v | (v >> 2)) & 0x10c30c30c30c30c3ull;
  v = (v | (v >> 4)) & 0x100f00f00f00f00full;
  v = (v | (v >> 8)) & 0x1f0000ff0000ffull;
  v = (v | (v >> 16)) & 0x1f00000000ffffull;
  v = (v | (v >> 32)) & 0x1fffffull;
  return (uint32_t)v;
}

// Morton key of 32-bit coordinates (96 bits used)
__host__ __device__ __forceinline__ Key128 morton3(uint32_t x, uint32_t y, uint32_t z) {
  uint64_t lo63 = spread21(x) | (spread21(y) << 1) | (spread21(z) << 2);
  uint64_t hi33 = spread21(x >> 21) | (spread21(y >> 21) << 1) | (spread21(z >> 21) << 2);
  Key128 k;
  k.lo = lo63 | (hi33 << 63);
  k.hi = hi33 >> 1;
  return k;
}

__host__ __device__ __forceinline__ void demorton3(Key128 k, uint32_t &x, uint32_t &y, uint32_t &z) {
  uint64_t lo63 = k.lo & 0x7fffffffffffffffull;
  uint64_t hi33 = (k.hi << 1) | (k.lo >> 63);
  x = compact21(lo63) | (compact21(hi33) << 21);
  y = compact21(lo63 >> 1) | (compact21(hi33 >> 1) << 21);
  z = compact21(lo63 >> 2) | (compact21(hi33 >> 2) << 21);
}

__host__ __device__ __forceinline__ Key128 key_shr(Key128 k, unsigned s) {
  if (s == 0) return k;
  if (s >= 128) return Key128{0, 0};
  if (s >= 64) return Key128{k.hi >> (s - 64), 0};
  return Key128{(k.lo >> s) | (k.hi << (64 - s)), k.hi >> s};
}
__host__ __device__ __forceinline__ Key128 key_shl(Key128 k, unsigned s) {
  if (s == 0) return k;
  if (s >= 128) return Key128{0, 0};
  if (s >= 64) return Key128{0, k.lo << (s - 64)};
  return Key128{k.lo << s, (k.hi << s) | (k.lo >> (64 - s))};
}
__host__ __device__ __forceinline__ Key128 key_or(Key128 a, Key128 b) { return Key128{a.lo | b.lo, a.hi | b.hi}; }
__host__ __device__ __forceinline__ Key128 key_xor(Key128 a, Key128 b) { return Key128{a.lo ^ b.lo, a.hi ^ b.hi}; }

// number of leading zero bits of k within a `bits`-wide field (bits <= 128)
__device__ __forceinline__ int key_clz(Key128 k, int bits) {
  int lz;
  if (k.hi) lz = __clzll((long long)k.hi);
  else if (k.lo) lz = 64 + __clzll((long long)k.lo);
  else lz = 128;
  return lz - (128 - bits);
}

// status codes: DG_OK / DG_ERR_* of the C ABI (include/dendro_gb300.h)

// device-side error flags (bitmask written by kernels, read by the host)
enum {
  DGF_DOMAIN = 1u,         // a point outside [0, gLen)^3 or not finite
  DGF_NOT_BALANCED = 2u,   // DA input not 2:1 balanced / not complete
  DGF_TIMEOUT = 4u,        // a bounded spin gave up
  DGF_INTERNAL = 8u,       // internal consistency check failed
  DGF_ORDER = 16u,         // input not sorted / unique as the caller declared
};

}  // namespace dg
