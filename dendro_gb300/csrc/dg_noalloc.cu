// dg_sort_unique_points_noalloc: the points -> sorted unique point octants
// step (par::sampleSort + par::removeDuplicates at one rank,
// include/parUtils.h:424,437) without any device allocation in the call.
//
// Every scratch byte lives in one file-scope static device array of fixed
// size.  Its address is taken once per device (cudaGetSymbolAddress, with
// that device current) on the first call there, then reused.  The pipeline
// is the one dg_sort_unique_points runs -- quantise, one histogram read of
// every digit, the onesweep digit passes (digits shared by all keys skipped),
// flag first-of-run, scan, compact -- with the same radix-sort kernels
// instantiated here on scratch slices instead of pooled buffers.
//
// Capacity: DG_NOALLOC_MAX_POINTS points.  Scratch: two 16-byte key arrays,
// two 4-byte arrays (flags and positions) of that length, the look-back
// status words of one digit pass, 2 x 16 x 256 histogram / offset words and
// a small header; about 41 MB.
//
// The scratch is shared by every call on a device: overlapping calls on one
// device race; the caller serialises them.
#include <mutex>

#include "dendro_gb300.h"
#include "dg_octree.cuh"

namespace dg {
namespace {

constexpr size_t NA_MAX = DG_NOALLOC_MAX_POINTS;
constexpr size_t NA_ALIGN = 256;
constexpr size_t na_round(size_t b) { return (b + NA_ALIGN - 1) / NA_ALIGN * NA_ALIGN; }

constexpr size_t NA_TILES = (NA_MAX + OsCfg<Key128>::TILE - 1) / OsCfg<Key128>::TILE;
constexpr size_t NA_SCAN_TILES = (NA_MAX + SCAN_TILE - 1) / SCAN_TILE;

// header words (first 256 bytes)
struct NaHeader {
  uint32_t flags;         // DGF_* raised by the kernels
  uint32_t active;        // bit p: digit pass p has more than one occupied bin
  uint32_t count;         // unique keys
  unsigned tile_counter;  // onesweep tile tickets
  int shifts[OS_MAX_PASSES];
};
static_assert(sizeof(NaHeader) <= NA_ALIGN, "header fits its slot");

// byte offsets of the scratch slices
constexpr size_t NA_OFF_HIST = NA_ALIGN;
constexpr size_t NA_OFF_OFFS = NA_OFF_HIST + na_round(OS_MAX_PASSES * 256 * sizeof(unsigned long long));
constexpr size_t NA_OFF_SUMS = NA_OFF_OFFS + na_round(OS_MAX_PASSES * 256 * sizeof(uint64_t));
constexpr size_t NA_OFF_STATUS = NA_OFF_SUMS + na_round(NA_SCAN_TILES * sizeof(uint32_t));
constexpr size_t NA_OFF_KEYS_A = NA_OFF_STATUS + na_round(NA_TILES * 256 * sizeof(uint64_t));
constexpr size_t NA_OFF_KEYS_B = NA_OFF_KEYS_A + na_round(NA_MAX * sizeof(Key128));
constexpr size_t NA_OFF_FLAGS = NA_OFF_KEYS_B + na_round(NA_MAX * sizeof(Key128));
constexpr size_t NA_OFF_POS = NA_OFF_FLAGS + na_round(NA_MAX * sizeof(uint32_t));
constexpr size_t NA_BYTES = NA_OFF_POS + na_round(NA_MAX * sizeof(uint32_t));

__device__ __align__(256) unsigned char g_na_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
struct NaDevice {
  std::mutex mu;
  bool ready = false;  // set only once the set-up succeeded
  unsigned char *base = nullptr;
  int num_sms = 0;
};
NaDevice g_na_dev[NA_MAX_DEVICES];

// The scratch address of device `dev` (current): looked up on the first
// successful call there.  A failed look-up (for example a transient error
// while the module loads) is not remembered: the next call tries again.
bool na_setup(NaDevice &nd, int dev) {
  std::lock_guard<std::mutex> lock(nd.mu);
  if (nd.ready) return true;
  unsigned char *base = nullptr;
  int sms = 0;
  if (cudaGetSymbolAddress((void **)&base, g_na_scratch) != cudaSuccess || !base ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  nd.base = base;
  nd.num_sms = sms;
  nd.ready = true;
  return true;
}

// The quantisation rule of points2OctreeSeq (src/construct.cpp:930-942):
// multiply by 2^D, divide by gLen, truncate; a point is valid iff the
// truncated value lies in [0, 2^D) on every axis.
__global__ void k_na_quantize(const double *__restrict__ xyz, size_t n, double scale, double gx, double gy, double gz,
                              unsigned D, Key128 *__restrict__ keys, uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double qx = __ddiv_rn(__dmul_rn(xyz[3 * i], scale), gx);
  const double qy = __ddiv_rn(__dmul_rn(xyz[3 * i + 1], scale), gy);
  const double qz = __ddiv_rn(__dmul_rn(xyz[3 * i + 2], scale), gz);
  const bool ok = (qx > -1.0) && (qx < scale) && (qy > -1.0) && (qy < scale) && (qz > -1.0) && (qz < scale);
  uint32_t ux = 0, uy = 0, uz = 0;
  if (ok) {
    ux = (uint32_t)__double2uint_rz(qx);
    uy = (uint32_t)__double2uint_rz(qy);
    uz = (uint32_t)__double2uint_rz(qz);
  } else {
    atomicOr(flags, DGF_DOMAIN);
  }
  keys[i] = make_tagged(morton3(ux, uy, uz), D);
}

__global__ void k_na_shifts(int *shifts, int npass) {
  if ((int)threadIdx.x < npass) shifts[threadIdx.x] = 8 * (int)threadIdx.x;
}

// per digit pass: exclusive scan of the 256 bins into digit offsets, and the
// pass is active when more than one bin is occupied (one block of 256)
__global__ void __launch_bounds__(256) k_na_plan(const unsigned long long *__restrict__ ghist, int npass,
                                                 uint64_t *__restrict__ offs, uint32_t *active) {
  uint32_t mask = 0;
  for (int p = 0; p < npass; p++) {
    const unsigned long long v = ghist[p * 256 + threadIdx.x];
    const int occupied = __syncthreads_count(v != 0ull);
    unsigned long long total;
    const unsigned long long ex = block_excl_scan<unsigned long long, 256>(v, total);
    offs[p * 256 + threadIdx.x] = ex;
    if (occupied > 1) mask |= 1u << p;
  }
  if (threadIdx.x == 0) *active = mask;
}

__global__ void k_na_emit(const Key128 *__restrict__ keys, const uint32_t *__restrict__ flags,
                          const uint32_t *__restrict__ pos, size_t n, uint4 *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flags[i]) return;
  uint32_t x, y, z;
  demorton3(tag_anchor(keys[i]), x, y, z);
  out[pos[i]] = make_uint4(x, y, z, tag_level(keys[i]));
}

// device memory of device `dev` (or managed memory) that the kernels may read
bool device_pointer(const void *p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace dg

#define NA_TRY(call)                        \
  do {                                      \
    if ((call) != cudaSuccess) {            \
      cudaGetLastError();                   \
      return DG_ERR_CUDA;                   \
    }                                       \
  } while (0)

extern "C" int dg_sort_unique_points_noalloc(const double *xyz, size_t n, const double gLens[3], unsigned maxDepth,
                                             uint32_t *out_xyzl, size_t *n_unique, void *cuda_stream) {
  using namespace dg;
  if (!gLens || !n_unique || (n && (!xyz || !out_xyzl)) || maxDepth > 30) return DG_ERR_INVALID_ARG;
  if (n > NA_MAX) return DG_ERR_CAPACITY;
  if (n == 0) {
    *n_unique = 0;
    return DG_OK;
  }
  if ((uintptr_t)xyz % 8 || (uintptr_t)out_xyzl % 16) return DG_ERR_INVALID_ARG;
  int dev = -1;
  NA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NA_MAX_DEVICES) return DG_ERR_UNSUPPORTED;
  NaDevice &nd = g_na_dev[dev];
  // set-up, once per device, with that device current
  if (!na_setup(nd, dev)) return DG_ERR_CUDA;
  if (!device_pointer(xyz, dev) || !device_pointer(out_xyzl, dev)) return DG_ERR_INVALID_ARG;

  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  unsigned char *b = nd.base;
  NaHeader *hdr = reinterpret_cast<NaHeader *>(b);
  auto *ghist = reinterpret_cast<unsigned long long *>(b + NA_OFF_HIST);
  auto *offs = reinterpret_cast<uint64_t *>(b + NA_OFF_OFFS);
  auto *sums = reinterpret_cast<uint32_t *>(b + NA_OFF_SUMS);
  auto *status = reinterpret_cast<uint64_t *>(b + NA_OFF_STATUS);
  auto *keys_a = reinterpret_cast<Key128 *>(b + NA_OFF_KEYS_A);
  auto *keys_b = reinterpret_cast<Key128 *>(b + NA_OFF_KEYS_B);
  auto *flags = reinterpret_cast<uint32_t *>(b + NA_OFF_FLAGS);
  auto *pos = reinterpret_cast<uint32_t *>(b + NA_OFF_POS);

  // what must start at zero: the header words and the digit histograms
  NA_TRY(cudaMemsetAsync(hdr, 0, NA_ALIGN, s));
  NA_TRY(cudaMemsetAsync(ghist, 0, OS_MAX_PASSES * 256 * sizeof(unsigned long long), s));
  const double scale = (double)(1u << maxDepth);
  k_na_quantize<<<grid_for(n, 256), 256, 0, s>>>(xyz, n, scale, gLens[0], gLens[1], gLens[2], maxDepth, keys_a,
                                                 &hdr->flags);
  NA_TRY(cudaGetLastError());
  // digits of the anchor bits [0, 3D); the level byte is D for every key
  const int npass = (3 * (int)maxDepth + 7) / 8;
  if (npass > 0) {
    k_na_shifts<<<1, 32, 0, s>>>(hdr->shifts, npass);
    NA_TRY(cudaGetLastError());
    k_rs_digit_hists<Key128><<<grid_for(n, RS_BLOCK, (unsigned)(nd.num_sms * 4)), RS_BLOCK, 0, s>>>(
        keys_a, n, npass, hdr->shifts, ghist);
    NA_TRY(cudaGetLastError());
    k_na_plan<<<1, 256, 0, s>>>(ghist, npass, offs, &hdr->active);
    NA_TRY(cudaGetLastError());
  }
  uint32_t h2[2] = {0, 0};  // flags, active
  NA_TRY(cudaMemcpyAsync(h2, hdr, sizeof(h2), cudaMemcpyDeviceToHost, s));
  NA_TRY(cudaStreamSynchronize(s));
  if (h2[0] & DGF_DOMAIN) return DG_ERR_DOMAIN;

  const size_t ntiles = (n + OsCfg<Key128>::TILE - 1) / OsCfg<Key128>::TILE;
  Key128 *src = keys_a, *dst = keys_b;
  for (int p = 0; p < npass; p++) {
    if (!(h2[1] >> p & 1u)) continue;
    // look-back status words and the tile ticket start at zero in every pass
    NA_TRY(cudaMemsetAsync(status, 0, ntiles * 256 * sizeof(uint64_t), s));
    NA_TRY(cudaMemsetAsync(&hdr->tile_counter, 0, sizeof(unsigned), s));
    k_rs_onesweep<Key128><<<(unsigned)ntiles, RS_BLOCK, 0, s>>>(src, dst, n, 8 * p, offs + 256 * p, status,
                                                                &hdr->tile_counter, &hdr->flags);
    NA_TRY(cudaGetLastError());
    Key128 *t = src;
    src = dst;
    dst = t;
  }
  // first key of each run of equal keys, then its rank among them
  k_flag_unique<Key128><<<grid_for(n, 256), 256, 0, s>>>(src, n, flags);
  NA_TRY(cudaGetLastError());
  const size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 1) {
    k_scan_tiles<uint32_t, uint32_t><<<1, SCAN_BLOCK, 0, s>>>(flags, n, pos, nullptr, &hdr->count);
    NA_TRY(cudaGetLastError());
  } else {
    k_scan_tile_sums<uint32_t, uint32_t><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(flags, n, sums);
    NA_TRY(cudaGetLastError());
    // tiles <= SCAN_TILE, so the tile sums scan in one block (in place)
    k_scan_tiles<uint32_t, uint32_t><<<1, SCAN_BLOCK, 0, s>>>(sums, tiles, sums, nullptr, nullptr);
    NA_TRY(cudaGetLastError());
    k_scan_tiles<uint32_t, uint32_t><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(flags, n, pos, sums, &hdr->count);
    NA_TRY(cudaGetLastError());
  }
  k_na_emit<<<grid_for(n, 256), 256, 0, s>>>(src, flags, pos, n, reinterpret_cast<uint4 *>(out_xyzl));
  NA_TRY(cudaGetLastError());
  uint32_t h3[3] = {0, 0, 0};  // flags, active, count
  NA_TRY(cudaMemcpyAsync(h3, hdr, sizeof(h3), cudaMemcpyDeviceToHost, s));
  NA_TRY(cudaStreamSynchronize(s));
  if (h3[0] & DGF_TIMEOUT) return DG_ERR_TIMEOUT;
  if (h3[0]) return DG_ERR_INTERNAL;
  *n_unique = h3[2];
  return DG_OK;
}
