// Device-wide primitives: exclusive scan, stream compaction, key OR/AND
// reduction and a stable LSD radix sort of 64- or 128-bit keys that skips
// the digits on which all keys agree.
//
// Radix sort, per 8-bit digit: (1) per-tile 256-bin histograms (shared
// atomics), (2) one exclusive scan of the digit-major histogram matrix,
// (3) a stable scatter in which each warp ranks its keys in order with
// __match_any_sync and per-warp running digit counters in shared memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dg_common.cuh"
#include "dg_runtime.cuh"

namespace dg {

// ------------------------------------------------------------------------
// key traits
// ------------------------------------------------------------------------
template <typename K>
struct KeyOps;

template <>
struct KeyOps<uint64_t> {
  static constexpr int BITS = 64;
  __device__ __forceinline__ static unsigned digit(uint64_t k, int shift) { return (unsigned)(k >> shift) & 0xffu; }
  __device__ __forceinline__ static bool eq(uint64_t a, uint64_t b) { return a == b; }
  __device__ __forceinline__ static uint64_t bor(uint64_t a, uint64_t b) { return a | b; }
  __device__ __forceinline__ static uint64_t band(uint64_t a, uint64_t b) { return a & b; }
};

template <>
struct KeyOps<Key128> {
  static constexpr int BITS = 128;
  __device__ __forceinline__ static unsigned digit(Key128 k, int shift) {
    if (shift >= 64) return (unsigned)(k.hi >> (shift - 64)) & 0xffu;
    if (shift <= 56) return (unsigned)(k.lo >> shift) & 0xffu;
    return (unsigned)((k.lo >> shift) | (k.hi << (64 - shift))) & 0xffu;
  }
  __device__ __forceinline__ static bool eq(Key128 a, Key128 b) { return a.lo == b.lo && a.hi == b.hi; }
  __device__ __forceinline__ static Key128 bor(Key128 a, Key128 b) { return Key128{a.lo | b.lo, a.hi | b.hi}; }
  __device__ __forceinline__ static Key128 band(Key128 a, Key128 b) { return Key128{a.lo & b.lo, a.hi & b.hi}; }
};

// ------------------------------------------------------------------------
// scans
// ------------------------------------------------------------------------
constexpr int SCAN_BLOCK = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= (unsigned)o) v += t;
  }
  return v;
}

// block-wide exclusive scan of one value per thread; returns the block total
template <typename T, int BLOCK>
__device__ __forceinline__ T block_excl_scan(T v, T &total) {
  __shared__ T warp_sums[BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T incl = warp_incl_scan(v);
  if (lane == 31) warp_sums[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    T s = (lane < BLOCK / 32) ? warp_sums[lane] : T(0);
    s = warp_incl_scan(s);
    if (lane < BLOCK / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  T prefix = (wid > 0) ? warp_sums[wid - 1] : T(0);
  total = warp_sums[BLOCK / 32 - 1];
  __syncthreads();
  return prefix + incl - v;
}

template <typename Tin, typename Tout>
__global__ void k_scan_tile_sums(const Tin *__restrict__ in, size_t n, Tout *__restrict__ sums) {
  size_t base = (size_t)blockIdx.x * SCAN_TILE;
  Tout s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    size_t idx = base + (size_t)i * SCAN_BLOCK + threadIdx.x;
    if (idx < n) s += (Tout)in[idx];
  }
  Tout total;
  block_excl_scan<Tout, SCAN_BLOCK>(s, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <typename Tin, typename Tout>
__global__ void k_scan_tiles(const Tin *__restrict__ in, size_t n, Tout *__restrict__ out,
                             const Tout *__restrict__ tile_offsets, Tout *__restrict__ total_out) {
  __shared__ Tout sm[SCAN_TILE];
  size_t base = (size_t)blockIdx.x * SCAN_TILE;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    size_t idx = base + (size_t)i * SCAN_BLOCK + threadIdx.x;
    sm[i * SCAN_BLOCK + threadIdx.x] = (idx < n) ? (Tout)in[idx] : Tout(0);
  }
  __syncthreads();
  Tout v[SCAN_ITEMS];
  Tout s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    v[i] = sm[threadIdx.x * SCAN_ITEMS + i];
    s += v[i];
  }
  Tout total;
  Tout pre = block_excl_scan<Tout, SCAN_BLOCK>(s, total);
  pre += tile_offsets ? tile_offsets[blockIdx.x] : Tout(0);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    Tout t = v[i];
    sm[threadIdx.x * SCAN_ITEMS + i] = pre;
    pre += t;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; i++) {
    size_t idx = base + (size_t)i * SCAN_BLOCK + threadIdx.x;
    if (idx < n) out[idx] = sm[i * SCAN_BLOCK + threadIdx.x];
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_BLOCK - 1) *total_out = pre;
}

// Exclusive scan out[i] = sum_{j<i} in[j]; optionally writes the grand total
// to the device word *d_total.  in and out may alias.
template <typename Tin, typename Tout>
void exclusive_scan(const Tin *in, Tout *out, size_t n, Tout *d_total, cudaStream_t s) {
  if (n == 0) {
    if (d_total) DG_CUDA(cudaMemsetAsync(d_total, 0, sizeof(Tout), s));
    return;
  }
  size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  const double nb = (double)n * (sizeof(Tin) + sizeof(Tout));
  if (tiles == 1) {
    ProfScope _prof("scan", nb);
    k_scan_tiles<Tin, Tout><<<1, SCAN_BLOCK, 0, s>>>(in, n, out, nullptr, d_total);
    DG_LAUNCH_CHECK();
    return;
  }
  DBuf<Tout> sums(tiles, s);
  {
    ProfScope _prof("scan_tile_sums", (double)n * sizeof(Tin));
    k_scan_tile_sums<Tin, Tout><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(in, n, sums.get());
    DG_LAUNCH_CHECK();
  }
  exclusive_scan<Tout, Tout>(sums.get(), sums.get(), tiles, (Tout *)nullptr, s);
  {
    ProfScope _prof("scan", nb);
    k_scan_tiles<Tin, Tout><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(in, n, out, sums.get(), d_total);
    DG_LAUNCH_CHECK();
  }
}

// ------------------------------------------------------------------------
// compaction: out[rank] = in[i] for flags[i] != 0 (stable); returns count
// ------------------------------------------------------------------------
template <typename T>
__global__ void k_scatter_flagged(const T *__restrict__ in, const uint32_t *__restrict__ flags,
                                  const uint64_t *__restrict__ pos, size_t n, T *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flags[i]) out[pos[i]] = in[i];
}

template <typename T>
size_t compact(Context &ctx, const T *in, const uint32_t *flags, size_t n, T *out) {
  if (n == 0) return 0;
  DBuf<uint64_t> pos(n, ctx.stream);
  uint64_t *d_total = reinterpret_cast<uint64_t *>(ctx.d_scratch);
  exclusive_scan<uint32_t, uint64_t>(flags, pos.get(), n, d_total, ctx.stream);
  {
    ProfScope _prof(ctx, "compact", (double)n * (4 + 8) + (double)n * sizeof(T) * 2);
    k_scatter_flagged<T><<<grid_for(n, 256), 256, 0, ctx.stream>>>(in, flags, pos.get(), n, out);
  DG_LAUNCH_CHECK();
    }
  return (size_t)read_scalar(ctx, d_total);
}

// ------------------------------------------------------------------------
// OR / AND of all keys (bits that vary across the array = OR ^ AND)
// ------------------------------------------------------------------------
template <typename K>
__global__ void k_key_or_and(const K *__restrict__ keys, size_t n, unsigned long long *orand) {
  // orand[0..1] = OR (lo, hi), orand[2..3] = AND (lo, hi)
  uint64_t olo = 0, ohi = 0, alo = ~0ull, ahi = ~0ull;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    K k = keys[i];
    if constexpr (sizeof(K) == 16) {
      const Key128 &q = reinterpret_cast<const Key128 &>(k);
      olo |= q.lo;
      ohi |= q.hi;
      alo &= q.lo;
      ahi &= q.hi;
    } else {
      const uint64_t &q = reinterpret_cast<const uint64_t &>(k);
      olo |= q;
      alo &= q;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    olo |= __shfl_xor_sync(0xffffffffu, olo, o);
    ohi |= __shfl_xor_sync(0xffffffffu, ohi, o);
    alo &= __shfl_xor_sync(0xffffffffu, alo, o);
    ahi &= __shfl_xor_sync(0xffffffffu, ahi, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicOr(&orand[0], (unsigned long long)olo);
    atomicOr(&orand[1], (unsigned long long)ohi);
    atomicAnd(&orand[2], (unsigned long long)alo);
    atomicAnd(&orand[3], (unsigned long long)ahi);
  }
}

// ------------------------------------------------------------------------
// radix sort
// ------------------------------------------------------------------------
constexpr int RS_BLOCK = 256;
constexpr int RS_WARPS = RS_BLOCK / 32;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_BLOCK * RS_ITEMS;
constexpr int RS_WARP_KEYS = RS_TILE / RS_WARPS;

template <typename K>
__global__ void __launch_bounds__(RS_BLOCK) k_rs_hist(const K *__restrict__ keys, size_t n, int shift,
                                                      uint32_t *__restrict__ hist, size_t ntiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * RS_TILE;
#pragma unroll
  for (int i = 0; i < RS_ITEMS; i++) {
    size_t idx = base + (size_t)i * RS_BLOCK + threadIdx.x;
    if (idx < n) atomicAdd(&h[KeyOps<K>::digit(keys[idx], shift)], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

template <typename K>
__global__ void __launch_bounds__(RS_BLOCK) k_rs_scatter(const K *__restrict__ in, K *__restrict__ out, size_t n,
                                                         int shift, const uint32_t *__restrict__ offs,
                                                         size_t ntiles) {
  __shared__ K tk[RS_TILE];
  __shared__ uint32_t wh[RS_WARPS][256];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const size_t base = (size_t)blockIdx.x * RS_TILE;
#pragma unroll
  for (int i = 0; i < RS_ITEMS; i++) {
    size_t idx = base + (size_t)i * RS_BLOCK + threadIdx.x;
    if (idx < n) tk[i * RS_BLOCK + threadIdx.x] = in[idx];
  }
#pragma unroll
  for (int i = 0; i < 256 / 32; i++) wh[wid][i * 32 + lane] = 0;
  __syncthreads();
  const unsigned lt_mask = (1u << lane) - 1u;
  // phase A: per-warp digit counts over the warp's contiguous key range
#pragma unroll
  for (int r = 0; r < RS_WARP_KEYS / 32; r++) {
    int t = wid * RS_WARP_KEYS + r * 32 + lane;
    bool valid = base + (size_t)t < n;
    unsigned d = valid ? KeyOps<K>::digit(tk[t], shift) : 256u + lane;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    if (valid && (peers & lt_mask) == 0) wh[wid][d] += __popc(peers);
  }
  __syncthreads();
  // phase B: turn counts into global write positions, warp order within tile
  {
    unsigned d = threadIdx.x;
    uint32_t run = offs[(size_t)d * ntiles + blockIdx.x];
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
      uint32_t c = wh[w][d];
      wh[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  // phase C: stable ranks, scatter
#pragma unroll
  for (int r = 0; r < RS_WARP_KEYS / 32; r++) {
    int t = wid * RS_WARP_KEYS + r * 32 + lane;
    bool valid = base + (size_t)t < n;
    K k;
    unsigned d;
    if (valid) {
      k = tk[t];
      d = KeyOps<K>::digit(k, shift);
    } else {
      d = 256u + lane;
    }
    unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t pos = 0;
    if (valid) pos = wh[wid][d] + __popc(peers & lt_mask);
    __syncwarp();
    if (valid && (peers & lt_mask) == 0) wh[wid][d] += __popc(peers);
    __syncwarp();
    if (valid) out[pos] = k;
  }
}

// Sort n keys (stable).  Only digits of bits [0, end_bit) on which the keys
// differ are processed.  Returns the buffer that holds the result (keys or
// tmp).  n must be < 2^32.
template <typename K>
K *radix_sort(Context &ctx, K *keys, K *tmp, size_t n, int end_bit) {
  if (n < 2) return keys;
  cudaStream_t s = ctx.stream;
  unsigned long long init[4] = {0ull, 0ull, ~0ull, ~0ull};
  unsigned long long *d_oa = ctx.d_scratch + 4;
  DG_CUDA(cudaMemcpyAsync(d_oa, init, sizeof(init), cudaMemcpyHostToDevice, s));
  unsigned g = grid_for(n, 256, (unsigned)(ctx.num_sms * 8));
  {
    ProfScope _prof(ctx, "key_or_and", (double)n * sizeof(K));
    k_key_or_and<K><<<g, 256, 0, s>>>(keys, n, d_oa);
    DG_LAUNCH_CHECK();
  }
  DG_CUDA(cudaMemcpyAsync(ctx.h_scratch + 4, d_oa, sizeof(init), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  uint64_t vary_lo = ctx.h_scratch[4] ^ ctx.h_scratch[6];
  uint64_t vary_hi = ctx.h_scratch[5] ^ ctx.h_scratch[7];

  size_t ntiles = (n + RS_TILE - 1) / RS_TILE;
  DBuf<uint32_t> hist(256 * ntiles, s);
  K *src = keys, *dst = tmp;
  for (int shift = 0; shift < end_bit && shift < KeyOps<K>::BITS; shift += 8) {
    uint64_t mlo = 0, mhi = 0;
    for (int b = shift; b < shift + 8 && b < end_bit; b++) {
      if (b < 64) mlo |= 1ull << b;
      else mhi |= 1ull << (b - 64);
    }
    if (!((vary_lo & mlo) | (vary_hi & mhi))) continue;
    {
    ProfScope _prof(ctx, "rs_hist", (double)n * sizeof(K));
    k_rs_hist<K><<<(unsigned)ntiles, RS_BLOCK, 0, s>>>(src, n, shift, hist.get(), ntiles);
    DG_LAUNCH_CHECK();
    }
    exclusive_scan<uint32_t, uint32_t>(hist.get(), hist.get(), 256 * ntiles, (uint32_t *)nullptr, s);
    {
    ProfScope _prof(ctx, "rs_scatter", (double)n * sizeof(K) * 2);
    k_rs_scatter<K><<<(unsigned)ntiles, RS_BLOCK, 0, s>>>(src, dst, n, shift, hist.get(), ntiles);
    DG_LAUNCH_CHECK();
    }
    K *t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// flags[i] = (i == 0 || keys[i] != keys[i-1])
template <typename K>
__global__ void k_flag_unique(const K *__restrict__ keys, size_t n, uint32_t *__restrict__ flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = (i == 0 || !KeyOps<K>::eq(keys[i], keys[i - 1])) ? 1u : 0u;
}

// sort + unique.  The unique keys end up in whichever of keys/tmp does not
// hold the sorted sequence; *result points at them.  Returns their count.
template <typename K>
size_t sort_unique(Context &ctx, K *keys, K *tmp, size_t n, int end_bit, K **result) {
  if (n == 0) {
    *result = keys;
    return 0;
  }
  K *sorted = radix_sort<K>(ctx, keys, tmp, n, end_bit);
  K *out = (sorted == keys) ? tmp : keys;
  DBuf<uint32_t> flags(n, ctx.stream);
  {
    ProfScope _prof(ctx, "flag_unique", (double)n * (sizeof(K) + 4));
    k_flag_unique<K><<<grid_for(n, 256), 256, 0, ctx.stream>>>(sorted, n, flags.get());
  DG_LAUNCH_CHECK();
    }
  *result = out;
  return compact<K>(ctx, sorted, flags.get(), n, out);
}

}  // namespace dg
