// Device-wide primitives: exclusive scan, stream compaction and a stable
// LSD radix sort of 64- or 128-bit keys that skips the digits on which all
// keys agree.
//
// Radix sort, per 8-bit digit: (1) per-tile 256-bin histograms (shared
// atomics), (2) one exclusive scan of the digit-major histogram matrix,
// (3) a stable scatter in which each warp ranks its keys in order with
// __match_any_sync and per-warp running digit counters in shared memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <utility>
#include <vector>

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

// ------------------------------------------------------------------------
// single-pass-per-digit ("onesweep") radix sort
//   1. one read of all keys builds the 256-bin histogram of every digit
//      position that is sorted; digits with a single occupied bin are
//      skipped; the digit offsets come from these histograms
//   2. per digit, one kernel: a block takes the next tile (ticket order),
//      counts its digits, publishes the counts, looks back over the
//      preceding tiles' published counts (decoupled look-back) for its
//      global offsets, and scatters its keys stably
// Look-back waits are bounded: a wait that exceeds the bound sets
// DGF_TIMEOUT and the host reports DG_ERR_TIMEOUT.
// ------------------------------------------------------------------------
constexpr int OS_MAX_PASSES = 16;
constexpr uint64_t OS_FLAG_AGG = 1ull << 62;
constexpr uint64_t OS_FLAG_INCL = 2ull << 62;
constexpr uint64_t OS_VALUE = (1ull << 62) - 1;
constexpr unsigned OS_SPIN_LIMIT = 1u << 22;

// tile of one onesweep block: ITEMS keys per thread (the default; the
// autotuner also tries OsAlt<K>::ITEMS)
template <typename K>
struct OsCfg {
  static constexpr int ITEMS = sizeof(K) == 16 ? 8 : 16;
  static constexpr int TILE = RS_BLOCK * ITEMS;
  static constexpr int WARP_KEYS = TILE / RS_WARPS;
};
template <typename K>
struct OsAlt {
  static constexpr int ITEMS = OsCfg<K>::ITEMS / 2;
};
constexpr size_t OS_TUNE_MIN = size_t(1) << 16;  // smaller sorts use the default tile

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint64_t *p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Histograms of every sorted digit position in one read of the keys.  Two
// shared copies (even / odd lanes) halve the same-address contention that
// skewed high digits cause.
template <typename K>
__global__ void __launch_bounds__(RS_BLOCK) k_rs_digit_hists(const K *__restrict__ keys, size_t n, int npass,
                                                              const int *__restrict__ shifts,
                                                              unsigned long long *__restrict__ ghist) {
  __shared__ uint32_t h[2][OS_MAX_PASSES * 256];
  __shared__ int sh[OS_MAX_PASSES];
  for (int i = threadIdx.x; i < 2 * OS_MAX_PASSES * 256; i += blockDim.x) (&h[0][0])[i] = 0;
  if (threadIdx.x < npass) sh[threadIdx.x] = shifts[threadIdx.x];
  __syncthreads();
  uint32_t *mine = h[threadIdx.x & 1];
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    K k = keys[i];
    for (int p = 0; p < npass; p++) atomicAdd(&mine[p * 256 + KeyOps<K>::digit(k, sh[p])], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < npass * 256; i += blockDim.x) {
    uint32_t v = h[0][i] + h[1][i];
    if (v) atomicAdd(&ghist[i], (unsigned long long)v);
  }
}

// One digit pass.  Keys are ranked in registers (warp-striped tile layout:
// match_any gives the rank among equal digits of a warp round, per-warp
// running counters order the rounds), placed in shared memory in digit
// order, then written out so that consecutive threads write consecutive
// addresses of each digit's run.
// MINB: blocks per SM the kernel is compiled for (register budget); the
// autotuner picks the tile and MINB per size class.
template <typename K, int ITEMS = OsCfg<K>::ITEMS, int MINB = 4>
__global__ void __launch_bounds__(RS_BLOCK, MINB) k_rs_onesweep(const K *__restrict__ in, K *__restrict__ out, size_t n,
                                                          int shift, const uint64_t *__restrict__ digit_off,
                                                          uint64_t *__restrict__ status, unsigned *tile_counter,
                                                          uint32_t *flags) {
  constexpr int TILE = RS_BLOCK * ITEMS, WK = TILE / RS_WARPS;
  __shared__ K tk[TILE];
  __shared__ uint32_t wh[RS_WARPS][256];
  __shared__ uint32_t s_local[256];
  __shared__ uint64_t s_glob[256];
  __shared__ unsigned s_tile;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
#pragma unroll
  for (int i = 0; i < 256 / 32; i++) wh[wid][i * 32 + lane] = 0;
  __syncthreads();
  const unsigned tile = s_tile;
  const size_t base = (size_t)tile * TILE;
  const unsigned lt_mask = (1u << lane) - 1u;
  K k[ITEMS];
  unsigned d[ITEMS];
  uint32_t rank[ITEMS];
#pragma unroll
  for (int r = 0; r < ITEMS; r++) {
    size_t idx = base + (size_t)(wid * WK + r * 32 + lane);
    if (idx < n) {
      k[r] = in[idx];
      d[r] = KeyOps<K>::digit(k[r], shift);
    } else {
      d[r] = 256u + lane;
    }
  }
  // rank within the warp's part of the tile, in key order
#pragma unroll
  for (int r = 0; r < ITEMS; r++) {
    const bool valid = d[r] < 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d[r]);
    uint32_t cur = valid ? wh[wid][d[r]] : 0u;
    __syncwarp();
    if (valid && (peers & lt_mask) == 0) wh[wid][d[r]] = cur + __popc(peers);
    __syncwarp();
    rank[r] = cur + __popc(peers & lt_mask);
  }
  __syncthreads();
  {
    const unsigned dg = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
      uint32_t c = wh[w][dg];
      wh[w][dg] = run;
      run += c;
    }
    uint32_t total_unused;
    const uint32_t local = block_excl_scan<uint32_t, RS_BLOCK>(run, total_unused);
    s_local[dg] = local;
    uint64_t *my = status + (size_t)tile * 256 + dg;
    uint64_t excl = 0;
    if (tile == 0) {
      st_relaxed(my, OS_FLAG_INCL | (uint64_t)run);
    } else {
      st_relaxed(my, OS_FLAG_AGG | (uint64_t)run);
      // look back four predecessors per round trip: their words are read
      // together, then summed newest first until an inclusive one; a word
      // not yet published is waited for (bounded) and the walk resumes there
      long t = (long)tile - 1;
      unsigned spins = 0;
      while (t >= 0) {
        uint64_t v[4];
#pragma unroll
        for (int q = 0; q < 4; q++) v[q] = (t - q >= 0) ? ld_relaxed(status + (size_t)(t - q) * 256 + dg) : 0;
        int q = 0;
        bool done = false;
        for (; q < 4 && t - q >= 0; q++) {
          if ((v[q] & ~OS_VALUE) == 0) break;
          excl += v[q] & OS_VALUE;
          if (v[q] & OS_FLAG_INCL) {
            done = true;
            break;
          }
        }
        if (done) break;
        t -= q;
        if (q < 4 && t >= 0) {  // tile t has not published yet
          if (++spins > OS_SPIN_LIMIT) {
            atomicOr(flags, DGF_TIMEOUT);
            break;
          }
          __nanosleep(32);
        }
      }
      st_relaxed(my, OS_FLAG_INCL | (excl + run));
    }
    s_glob[dg] = digit_off[dg] + excl - (uint64_t)local;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < ITEMS; r++)
    if (d[r] < 256u) tk[s_local[d[r]] + wh[wid][d[r]] + rank[r]] = k[r];
  __syncthreads();
  const size_t tile_n = (n - base < (size_t)TILE) ? n - base : (size_t)TILE;
#pragma unroll
  for (int i = 0; i < ITEMS; i++) {
    const int p = i * RS_BLOCK + threadIdx.x;
    if ((size_t)p < tile_n) {
      K key = tk[p];
      out[s_glob[KeyOps<K>::digit(key, shift)] + (uint64_t)p] = key;
    }
  }
}

// Sort n keys (stable) on the digits of bits [0, end_bit) (8-bit digits;
// end_bit must not cut into bits that vary above it).  Digits on which all
// keys agree are skipped.  Returns the buffer that holds the result (keys or
// tmp).
template <typename K>
K *radix_sort(Context &ctx, K *keys, K *tmp, size_t n, int end_bit) {
  if (n < 2 || end_bit <= 0) return keys;
  cudaStream_t s = ctx.stream;
  int shifts[OS_MAX_PASSES];
  int npass = 0;
  for (int sh = 0; sh < end_bit && sh < KeyOps<K>::BITS && npass < OS_MAX_PASSES; sh += 8) shifts[npass++] = sh;
  // histograms of every digit position, one read of the keys
  DBuf<unsigned long long> ghist(npass * 256, s);
  DBuf<int> dshifts(npass, s);
  DG_CUDA(cudaMemcpyAsync(dshifts.get(), shifts, npass * sizeof(int), cudaMemcpyHostToDevice, s));
  // launch shape of this size class: the context's decision, else the
  // disk cache's, else tuned below
  const int width = sizeof(K) == 16 ? 1 : 0;
  int bucket = 0;
  while (bucket < 63 && ((size_t)2 << bucket) <= n) bucket++;
  Context::Tune &tn = ctx.tune[width][bucket];
  const bool tunable = n >= OS_TUNE_MIN;
  if (tunable && tn.items == 0 && tune_cache_get(ctx.device, width, bucket, &tn)) {
    char line[160];
    std::snprintf(line, sizeof(line), "onesweep %d-byte keys, 2^%d: %d keys/thread, %d blocks/SM, histogram %d "
                  "blocks/SM (disk cache)\n", (int)sizeof(K), bucket, tn.items, tn.minb, tn.hist_mul);
    ctx.tune_log += line;
  }
  const bool tuning = tunable && tn.items == 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (tuning) {
    DG_CUDA(cudaEventCreate(&e0));
    DG_CUDA(cudaEventCreate(&e1));
  }
  // best of two timings: other streams sharing the GPU can slow any one
  auto time2 = [&](auto &&launch) {
    float best = 0.f;
    for (int rep = 0; rep < 2; rep++) {
      float t = 0.f;
      DG_CUDA(cudaEventRecord(e0, s));
      launch();
      DG_CUDA(cudaEventRecord(e1, s));
      DG_CUDA(cudaEventSynchronize(e1));
      DG_CUDA(cudaEventElapsedTime(&t, e0, e1));
      best = rep == 0 ? t : std::min(best, t);
    }
    return best;
  };
  auto hists = [&](int mul) {
    DG_CUDA(cudaMemsetAsync(ghist.get(), 0, npass * 256 * sizeof(unsigned long long), s));
    ProfScope _prof(ctx, "rs_digit_hists", (double)n * sizeof(K));
    unsigned g = grid_for(n, RS_BLOCK, (unsigned)(ctx.num_sms * mul));
    k_rs_digit_hists<K><<<g, RS_BLOCK, 0, s>>>(keys, n, npass, dshifts.get(), ghist.get());
    DG_LAUNCH_CHECK();
  };
  float hist_ms[3] = {0.f, 0.f, 0.f};
  const int hist_cand[3] = {2, 4, 8};
  if (tuning) {
    for (int c = 0; c < 3; c++) hist_ms[c] = time2([&]() { hists(hist_cand[c]); });
    int b = 0;
    for (int c = 1; c < 3; c++)
      if (hist_ms[c] < hist_ms[b]) b = c;
    tn.hist_mul = hist_cand[b];
  }
  hists(tn.hist_mul ? tn.hist_mul : 4);
  std::vector<unsigned long long> h(npass * 256);
  DG_CUDA(cudaMemcpyAsync(h.data(), ghist.get(), h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  std::vector<int> active;
  std::vector<uint64_t> offs;
  for (int p = 0; p < npass; p++) {
    int occupied = 0;
    for (int d = 0; d < 256; d++) occupied += h[p * 256 + d] != 0;
    if (occupied <= 1) continue;  // every key has the same digit here
    active.push_back(p);
    uint64_t run = 0;
    for (int d = 0; d < 256; d++) {
      offs.push_back(run);
      run += h[p * 256 + d];
    }
  }
  if (active.empty()) {
    if (tuning) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      tn = Context::Tune();  // nothing to sort here: decide on a later sort of this size
    }
    return keys;
  }
  DBuf<uint64_t> doffs(offs.size(), s);
  DG_CUDA(cudaMemcpyAsync(doffs.get(), offs.data(), offs.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  const size_t max_tiles = (n + RS_BLOCK * OsAlt<K>::ITEMS - 1) / (RS_BLOCK * OsAlt<K>::ITEMS);
  if (max_tiles >= 0xffffffffull) fail(DG_ERR_INVALID_ARG, "radix sort: too many keys");
  DBuf<uint64_t> status(max_tiles * 256, s);
  unsigned *d_counter = reinterpret_cast<unsigned *>(ctx.d_scratch + 12);
  // one digit pass with `items` keys per thread, compiled for `minb` blocks
  // per SM
  auto pass = [&](int items, int minb, const K *src, K *dst, size_t a) {
    if (items != OsCfg<K>::ITEMS) items = OsAlt<K>::ITEMS;  // the two compiled tiles
    const size_t tile = (size_t)RS_BLOCK * items, ntiles = (n + tile - 1) / tile;
    DG_CUDA(cudaMemsetAsync(status.get(), 0, ntiles * 256 * sizeof(uint64_t), s));
    DG_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s));
    ProfScope _prof(ctx, "rs_onesweep", (double)n * sizeof(K) * 2);
    const int sh = shifts[active[a]];
    const uint64_t *off = doffs.get() + 256 * a;
    const unsigned g = (unsigned)ntiles;
    if (items == OsCfg<K>::ITEMS && minb == 3)
      k_rs_onesweep<K, OsCfg<K>::ITEMS, 3><<<g, RS_BLOCK, 0, s>>>(src, dst, n, sh, off, status.get(), d_counter,
                                                                  ctx.d_flags);
    else if (items == OsCfg<K>::ITEMS && minb == 5)
      k_rs_onesweep<K, OsCfg<K>::ITEMS, 5><<<g, RS_BLOCK, 0, s>>>(src, dst, n, sh, off, status.get(), d_counter,
                                                                  ctx.d_flags);
    else if (items == OsCfg<K>::ITEMS)
      k_rs_onesweep<K, OsCfg<K>::ITEMS, 4><<<g, RS_BLOCK, 0, s>>>(src, dst, n, sh, off, status.get(), d_counter,
                                                                  ctx.d_flags);
    else
      k_rs_onesweep<K, OsAlt<K>::ITEMS, 4><<<g, RS_BLOCK, 0, s>>>(src, dst, n, sh, off, status.get(), d_counter,
                                                                  ctx.d_flags);
    DG_LAUNCH_CHECK();
  };
  // autotuner: the first sort of each size class (log2 of the key count)
  // times every onesweep shape on its first digit pass (the pass is stable,
  // so every run writes the same output) and keeps the fastest for every
  // later pass and sort of that class
  K *src = keys, *dst = tmp;
  size_t a0 = 0;
  if (tuning) {
    struct Cand {
      int items, minb;
    };
    const Cand cand[4] = {{OsCfg<K>::ITEMS, 4}, {OsAlt<K>::ITEMS, 4}, {OsCfg<K>::ITEMS, 3}, {OsCfg<K>::ITEMS, 5}};
    float ms[4];
    int b = 0;
    for (int c = 0; c < 4; c++) {
      ms[c] = time2([&]() { pass(cand[c].items, cand[c].minb, src, dst, 0); });
      if (ms[c] < ms[b]) b = c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tn.items = cand[b].items;
    tn.minb = cand[b].minb;
    char line[320];
    std::snprintf(line, sizeof(line),
                  "onesweep %d-byte keys, 2^%d: keys/thread x blocks/SM %dx%d %.3f ms, %dx%d %.3f, %dx%d %.3f, "
                  "%dx%d %.3f -> %dx%d; histogram blocks/SM 2/4/8 %.3f/%.3f/%.3f ms -> %d\n",
                  (int)sizeof(K), bucket, cand[0].items, cand[0].minb, ms[0], cand[1].items, cand[1].minb, ms[1],
                  cand[2].items, cand[2].minb, ms[2], cand[3].items, cand[3].minb, ms[3], tn.items, tn.minb,
                  hist_ms[0], hist_ms[1], hist_ms[2], tn.hist_mul);
    ctx.tune_log += line;
    tune_cache_put(ctx.device, width, bucket, tn);
    std::swap(src, dst);
    a0 = 1;
  }
  const int use = tn.items ? tn.items : OsCfg<K>::ITEMS, use_minb = tn.minb ? tn.minb : 4;
  for (size_t a = a0; a < active.size(); a++) {
    pass(use, use_minb, src, dst, a);
    K *t = src;
    src = dst;
    dst = t;
  }
  check_device_flags(ctx, "radix sort");
  return src;
}

// flags[i] = (i == 0 || keys[i] != keys[i-1])
template <typename K>
__global__ void k_flag_unique(const K *__restrict__ keys, size_t n, uint32_t *__restrict__ flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = (i == 0 || !KeyOps<K>::eq(keys[i], keys[i - 1])) ? 1u : 0u;
}

// Small sorts in one CTA: up to SMALL_SORT_MAX keys are sorted in shared
// memory (bitonic network, padded with the largest key), repeated keys are
// dropped and the rest written in order with their count.  Keys agree on
// every bit above the sorted ones, so whole-key order is the radix order.
// Used by sort_unique below the size where the radix sort's passes, each a
// launch, and its histogram read-back cost more than the keys themselves
// (the deep and coarse levels of a balance, most multigrid levels).
constexpr int SMALL_SORT_MAX = 4096;
constexpr int SMALL_SORT_BLOCK = 1024;

__device__ __forceinline__ bool key_less(uint64_t a, uint64_t b) { return a < b; }
__device__ __forceinline__ bool key_less(const Key128 &a, const Key128 &b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
template <typename K>
__device__ __forceinline__ K key_max();
template <>
__device__ __forceinline__ uint64_t key_max<uint64_t>() {
  return ~0ull;
}
template <>
__device__ __forceinline__ Key128 key_max<Key128>() {
  return Key128{~0ull, ~0ull};
}

template <typename K>
__global__ void __launch_bounds__(SMALL_SORT_BLOCK) k_small_sort_unique(const K *__restrict__ in, int n, int n2,
                                                                         K *__restrict__ out,
                                                                         unsigned long long *count) {
  extern __shared__ __align__(16) unsigned char ss_raw[];
  K *sk = reinterpret_cast<K *>(ss_raw);
  __shared__ int wsum[SMALL_SORT_BLOCK / 32];
  const int tid = threadIdx.x;
  for (int i = tid; i < n2; i += SMALL_SORT_BLOCK) sk[i] = i < n ? in[i] : key_max<K>();
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < n2; i += SMALL_SORT_BLOCK) {
        const int l = i ^ j;
        if (l > i) {
          const K a = sk[i], b = sk[l];
          const bool up = (i & k) == 0;
          if (up ? key_less(b, a) : key_less(a, b)) {
            sk[i] = b;
            sk[l] = a;
          }
        }
      }
      __syncthreads();
    }
  // thread t owns the consecutive items [4t, 4t + 4); first of each run kept
  constexpr int PER = SMALL_SORT_MAX / SMALL_SORT_BLOCK;
  int keep[PER], c = 0;
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int i = tid * PER + q;
    keep[q] = i < n && (i == 0 || key_less(sk[i - 1], sk[i]));
    c += keep[q];
  }
  // block exclusive scan of the counts
  const int lane = tid & 31, w = tid >> 5;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    int v = lane < SMALL_SORT_BLOCK / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane < SMALL_SORT_BLOCK / 32) wsum[lane] = v;  // inclusive per warp
  }
  __syncthreads();
  int pos = (w > 0 ? wsum[w - 1] : 0) + incl - c;
#pragma unroll
  for (int q = 0; q < PER; q++)
    if (keep[q]) out[pos++] = sk[tid * PER + q];
  if (tid == SMALL_SORT_BLOCK - 1) *count = (unsigned long long)(pos);
}

// sort + unique.  The unique keys end up in whichever of keys/tmp does not
// hold the sorted sequence; *result points at them.  Returns their count.
template <typename K>
size_t sort_unique(Context &ctx, K *keys, K *tmp, size_t n, int end_bit, K **result) {
  if (n == 0) {
    *result = keys;
    return 0;
  }
  if (n <= (size_t)SMALL_SORT_MAX) {
    int n2 = 2;
    while (n2 < (int)n) n2 <<= 1;
    const int smem = n2 * (int)sizeof(K);
    ensure_smem_attr(ctx, k_small_sort_unique<K>, SMALL_SORT_MAX * (int)sizeof(K));
    unsigned long long *d_count = ctx.d_scratch + 8;
    {
      ProfScope _prof(ctx, "sort_unique_small", (double)n * sizeof(K) * 2);
      k_small_sort_unique<K><<<1, SMALL_SORT_BLOCK, smem, ctx.stream>>>(keys, (int)n, n2, tmp, d_count);
      DG_LAUNCH_CHECK();
    }
    *result = tmp;
    return (size_t)read_scalar(ctx, d_count);
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
