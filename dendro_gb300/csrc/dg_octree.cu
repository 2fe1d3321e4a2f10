// Octree construction (points2Octree) and 2:1 balance (balanceOctree) on
// the GPU.  All data stays in HBM; the host only reads sizes.
//
// Batches: several clouds ("segments") are processed by the same launches;
// segment s lives in key bits [3D, 3D + seg_bits) (dg_octree.cuh), so every
// sort, NCA and gap computation below stays inside its own cloud.
//
// Construction (unique points, reference p2oLocal, src/construct.cpp:976):
// the leaf that holds point i is the child of its deepest ancestor that
// contains more than maxPts points.  With the points in Morton order that
// ancestor's level is max_j NCA(p_j, p_{j+m}) over the windows j in
// [i-m, i] (m = maxPts), so every point's leaf is computed independently;
// the empty leaves between consecutive point leaves are the maximal aligned
// Morton blocks of the gap.  Inputs with repeated points take the
// reference's sequential walk verbatim (a single-thread kernel), because its
// point bookkeeping then departs from the rule above.
//
// Balance (reference comboRipple, src/balance.cpp:801): the coarsest 2:1
// balanced refinement is unique.  With I_l the internal nodes at level l,
//   I_{l-1} = parent(input leaves at level l) U parents of the 3x3x3 blocks
//             around every q in I_l (8 octants per q, clipped to the domain)
// and the balanced leaves at level l are children(I_{l-1}) \ I_l.  Each
// level is one generate + radix sort + unique; the leaves are then placed in
// Morton order by a bottom-up leaf count and a top-down offset pass.
#include "dg_octree.cuh"
#include "dg_walk.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

namespace dg {

__device__ __forceinline__ void set_flag(uint32_t *flags, uint32_t f) { atomicOr(flags, f); }

// key with only the Morton bits of one cloud (bits [0, 3D))
__host__ __device__ __forceinline__ Key128 morton_part(Key128 k, unsigned D) {
  Key128 a = tag_anchor(k);
  if (3 * D < 64) {
    a.lo &= (3 * D) ? ((1ull << (3 * D)) - 1) : 0ull;
    a.hi = 0;
  } else {
    a.hi &= (1ull << (3 * D - 64)) - 1;
  }
  return a;
}
__host__ __device__ __forceinline__ uint64_t seg_of(Key128 k, unsigned D) {
  return to_u128(tag_anchor(k)) >> (3 * D) & 0xffffffffffull;
}
__host__ __device__ __forceinline__ Key128 seg_key(uint64_t seg, unsigned D) {
  return from_u128((u128)seg << (3 * D));
}

// ------------------------------------------------------------------------
// quantize + Morton key (construct.cpp:930-942)
// ------------------------------------------------------------------------
// (unsigned int)(x * (double)(1u << D) / gLen): multiply, divide, truncate.
// When every gLen is a power of two (the unit cube of the workloads), its
// reciprocal is exact and x * 2^D * (1 / gLen) is the same correctly rounded
// value as the division (both round the same exact quotient), without the
// FP64 divide.
template <bool POW2>
__global__ void k_quantize(const double *__restrict__ xyz, size_t n, double scale, double gx, double gy, double gz,
                           unsigned D, const uint64_t *__restrict__ seg_start, size_t nseg, Key128 *__restrict__ keys,
                           uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  double qx, qy, qz;
  if constexpr (POW2) {  // gx, gy, gz hold the exact reciprocals here
    qx = __dmul_rn(__dmul_rn(x, scale), gx);
    qy = __dmul_rn(__dmul_rn(y, scale), gy);
    qz = __dmul_rn(__dmul_rn(z, scale), gz);
  } else {
    qx = __ddiv_rn(__dmul_rn(x, scale), gx);
    qy = __ddiv_rn(__dmul_rn(y, scale), gy);
    qz = __ddiv_rn(__dmul_rn(z, scale), gz);
  }
  // valid iff the truncated value lies in [0, 2^D): q in (-1, 2^D); NaN fails
  bool ok = (qx > -1.0) && (qx < scale) && (qy > -1.0) && (qy < scale) && (qz > -1.0) && (qz < scale);
  uint32_t ux = 0, uy = 0, uz = 0;
  if (ok) {
    ux = (uint32_t)__double2uint_rz(qx);
    uy = (uint32_t)__double2uint_rz(qy);
    uz = (uint32_t)__double2uint_rz(qz);
  } else {
    set_flag(flags, DGF_DOMAIN);
  }
  Key128 k = morton3(ux, uy, uz);
  if (seg_start) {  // segment of point i: last s with seg_start[s] <= i
    size_t lo = 0, hi = nseg;
    while (hi - lo > 1) {
      size_t mid = (lo + hi) / 2;
      if (seg_start[mid] <= i) lo = mid;
      else hi = mid;
    }
    k = key_or(k, seg_key(lo, D));
  }
  keys[i] = make_tagged(k, D);
}

// NCA level of two points of the same cloud; -1 across clouds
__device__ __forceinline__ int nca_level(Key128 a, Key128 b, unsigned D) {
  Key128 x = key_xor(tag_anchor(a), tag_anchor(b));
  if (!x.lo && !x.hi) return (int)D;
  int lz = key_clz(x, 3 * (int)D);
  return lz < 0 ? -1 : lz / 3;
}

// dupseg[s] = 1 when cloud s holds a repeated point
__global__ void k_flag_dups(const Key128 *__restrict__ p, size_t n, unsigned D, uint32_t *dupseg, uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 1 && i < n && key_eq(p[i], p[i - 1])) {
    dupseg[seg_of(p[i], D)] = 1u;
    set_flag(flags, 0x100u);
  }
}

__device__ __forceinline__ unsigned leaf_level(const Key128 *__restrict__ p, size_t n, size_t i, unsigned m,
                                               unsigned D) {
  size_t lo = (i >= m) ? i - m : 0;
  size_t hi = (i + m < n) ? i : (n > m ? n - 1 - m : 0);
  int best = -1;
  if (n > m)
    for (size_t j = lo; j <= hi; j++) best = max(best, nca_level(p[j], p[j + m], D));
  return (unsigned)min(best + 1, (int)D);
}

// leaf of every point and the flag "first point of its leaf"
__global__ void k_p2o_seeds(const Key128 *__restrict__ p, size_t n, unsigned m, unsigned D,
                            Key128 *__restrict__ seeds, uint32_t *__restrict__ first) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned L = leaf_level(p, n, i, m, D);
  Key128 a = key_shl(key_shr(tag_anchor(p[i]), 3 * (D - L)), 3 * (D - L));
  seeds[i] = make_tagged(a, L);
  bool f = true;
  if (i > 0) {
    unsigned L2 = leaf_level(p, n, i - 1, m, D);
    Key128 a2 = key_shl(key_shr(tag_anchor(p[i - 1]), 3 * (D - L2)), 3 * (D - L2));
    f = !(L2 == L && key_eq(a2, a));
  }
  first[i] = f ? 1u : 0u;
}

__device__ __forceinline__ u128 kpos(Key128 k) { return to_u128(tag_anchor(k)); }

__device__ __forceinline__ int ctz128(u128 v) {
  uint64_t lo = (uint64_t)v;
  if (lo) return __ffsll((long long)lo) - 1;
  uint64_t hi = (uint64_t)(v >> 64);
  return hi ? 64 + __ffsll((long long)hi) - 1 : 128;
}
__device__ __forceinline__ int log2_128(u128 v) {  // v > 0
  uint64_t hi = (uint64_t)(v >> 64);
  if (hi) return 127 - __clzll((long long)hi);
  return 63 - __clzll((long long)(uint64_t)v);
}

// largest k <= D with s % 8^k == 0 and s + 8^k <= e (s < e); blocks never
// cross a cloud boundary because clouds are aligned 8^D ranges
__device__ __forceinline__ int block_exp(u128 s, u128 e, unsigned D) {
  int k1 = (s == 0) ? (int)D : min((int)D, ctz128(s) / 3);
  int k2 = log2_128(e - s) / 3;
  return min(k1, k2);
}

__device__ unsigned gap_count(u128 s, u128 e, unsigned D) {
  unsigned c = 0;
  while (s < e) {
    int k = block_exp(s, e, D);
    s += (u128)1 << (3 * k);
    c++;
  }
  return c;
}

__device__ size_t gap_emit(u128 s, u128 e, unsigned D, Key128 *out, size_t w) {
  while (s < e) {
    int k = block_exp(s, e, D);
    out[w++] = make_tagged(from_u128(s), D - (unsigned)k);
    s += (u128)1 << (3 * k);
  }
  return w;
}

__device__ __forceinline__ u128 seed_end(Key128 s, unsigned D) {
  return kpos(s) + ((u128)1 << (3 * (D - tag_level(s))));
}

__global__ void k_fill_count(const Key128 *__restrict__ seeds, size_t ns, unsigned D, u128 total,
                             uint32_t *__restrict__ cnt) {
  size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ns) return;
  u128 e = (j + 1 < ns) ? kpos(seeds[j + 1]) : total;
  unsigned c = 1 + gap_count(seed_end(seeds[j], D), e, D);
  if (j == 0) c += gap_count(0, kpos(seeds[0]), D);
  cnt[j] = c;
}

__global__ void k_fill_emit(const Key128 *__restrict__ seeds, size_t ns, unsigned D, u128 total,
                            const uint64_t *__restrict__ off, Key128 *__restrict__ out) {
  size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ns) return;
  size_t w = off[j];
  if (j == 0) w = gap_emit(0, kpos(seeds[0]), D, out, w);
  out[w++] = seeds[j];
  u128 e = (j + 1 < ns) ? kpos(seeds[j + 1]) : total;
  gap_emit(seed_end(seeds[j], D), e, D, out, w);
}

// ------------------------------------------------------------------------
// the reference walk for clouds with repeated points (dg_walk.cuh): one
// block per such cloud, thread 0 walks it; count pass then emit pass
// ------------------------------------------------------------------------
__global__ void k_p2o_walk_segments(const Key128 *__restrict__ pk, const uint64_t *__restrict__ pt_start,
                                    const uint32_t *__restrict__ dup_list, unsigned m, unsigned D,
                                    const uint64_t *__restrict__ out_off, Key128 *__restrict__ out,
                                    unsigned long long *counts, bool batched) {
  if (threadIdx.x != 0) return;
  const uint32_t s = dup_list[blockIdx.x];
  const size_t b = pt_start[s], e = pt_start[s + 1];
  bool outside = false;
  size_t c = p2o_walk(pk + b, e - b, m, D, out ? out + out_off[blockIdx.x] : nullptr, seg_key(s, D), &outside);
  counts[blockIdx.x] = c;
  if (outside && batched) counts[blockIdx.x] = (unsigned long long)P2O_WALK_OUTSIDE;
}

// first index of each cloud in a sorted key array (lower bound of s << 3D)
__global__ void k_seg_bounds(const Key128 *__restrict__ keys, size_t n, unsigned D, size_t nseg,
                             uint64_t *__restrict__ off) {
  size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s > nseg) return;
  Key128 v = seg_key(s, D);
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (key_lt(tag_anchor(keys[mid]), v)) lo = mid + 1;
    else hi = mid;
  }
  off[s] = lo;
}

// place each cloud's octants at their final offsets: clouds with repeated
// points take the walk's output, the others the parallel construction's.
// The walk outputs are stored cloud after cloud in dup-list order; a walk
// octant's cloud is found from its position (its key may lie outside the
// cloud's domain, see dg_walk.cuh).
__global__ void k_assemble(const Key128 *__restrict__ par, size_t npar, const uint64_t *__restrict__ par_off,
                           const Key128 *__restrict__ walk, const uint64_t *__restrict__ walk_off, size_t nd,
                           const uint32_t *__restrict__ dup_list, const uint32_t *__restrict__ dupseg, size_t nseg,
                           const uint64_t *__restrict__ final_off, unsigned D, Key128 *__restrict__ out,
                           size_t nwalk_total) {
  size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < npar) {
    uint64_t s = seg_of(par[j], D);
    if (s < nseg && !dupseg[s]) out[final_off[s] + (j - par_off[s])] = par[j];
  }
  if (j < nwalk_total) {
    size_t lo = 0, hi = nd;  // last slot with walk_off[slot] <= j
    while (hi - lo > 1) {
      size_t mid = (lo + hi) / 2;
      if (walk_off[mid] <= j) lo = mid;
      else hi = mid;
    }
    uint32_t s = dup_list[lo];
    out[final_off[s] + (j - walk_off[lo])] = walk[j];
  }
}

// ------------------------------------------------------------------------
// host: point sort and construction
// ------------------------------------------------------------------------
void check_device_flags(Context &ctx, const char *where) {
  uint32_t f = read_scalar(ctx, ctx.d_flags);
  if (f) {
    DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), ctx.stream));
    if (f & DGF_DOMAIN) fail(DG_ERR_DOMAIN, std::string(where) + ": input outside the domain");
    if (f & DGF_NOT_BALANCED) fail(DG_ERR_NOT_BALANCED, std::string(where) + ": input is not a complete 2:1 balanced octree");
    if (f & DGF_TIMEOUT) fail(DG_ERR_TIMEOUT, std::string(where) + ": a device wait timed out");
    if (f & DGF_INTERNAL) fail(DG_ERR_INTERNAL, std::string(where) + ": internal consistency check failed");
    if (f & DGF_ORDER) fail(DG_ERR_INVALID_ARG, std::string(where) + ": input is not sorted / unique as declared");
  }
}

static void quantize_sorted(Context &ctx, const double *d_xyz, size_t n, const double g[3], unsigned D,
                            const uint64_t *d_seg_start, size_t nseg, unsigned seg_bits, DBuf<Key128> &keys,
                            DBuf<Key128> &tmp, Key128 **sorted) {
  keys.alloc(n, ctx.stream);
  tmp.alloc(n, ctx.stream);
  {
    ProfScope _prof(ctx, "quantize", (double)n * 40);
    // a power of two whose reciprocal is a normal double
    auto pow2 = [](double v) {
      int e = 0;
      return std::frexp(v, &e) == 0.5 && e > -1020 && e < 1020;
    };
    if (pow2(g[0]) && pow2(g[1]) && pow2(g[2]))
      k_quantize<true><<<grid_for(n, 256), 256, 0, ctx.stream>>>(d_xyz, n, (double)(1u << D), 1.0 / g[0], 1.0 / g[1],
                                                                 1.0 / g[2], D, d_seg_start, nseg, keys.get(),
                                                                 ctx.d_flags);
    else
      k_quantize<false><<<grid_for(n, 256), 256, 0, ctx.stream>>>(d_xyz, n, (double)(1u << D), g[0], g[1], g[2], D,
                                                                  d_seg_start, nseg, keys.get(), ctx.d_flags);
    DG_LAUNCH_CHECK();
  }
  check_device_flags(ctx, "points2Octree");
  *sorted = radix_sort<Key128>(ctx, keys.get(), tmp.get(), n, 3 * (int)D + (int)seg_bits);
}

size_t sort_points(Context &ctx, const double *d_xyz, size_t n, const double g[3], unsigned D, Key128 *d_out,
                   bool *has_dups) {
  if (n == 0) return 0;
  DBuf<Key128> keys, tmp;
  Key128 *sorted;
  quantize_sorted(ctx, d_xyz, n, g, D, nullptr, 1, 0, keys, tmp, &sorted);
  DBuf<uint32_t> flags(n, ctx.stream);
  {
    ProfScope _prof(ctx, "flag_unique", (double)n * 20);
    k_flag_unique<Key128><<<grid_for(n, 256), 256, 0, ctx.stream>>>(sorted, n, flags.get());
    DG_LAUNCH_CHECK();
  }
  size_t nu = compact<Key128>(ctx, sorted, flags.get(), n, d_out);
  if (has_dups) *has_dups = nu != n;
  return nu;
}

void points_to_octree(Context &ctx, const double *d_xyz, size_t n, const double g[3], unsigned D, unsigned m,
                      Octree &out, const uint64_t *h_seg_start, size_t nseg) {
  if (m == 0 || D > 30) fail(DG_ERR_INVALID_ARG, "points2Octree: maxNumPts must be >= 1 and maxDepth <= 30");
  if (n >= 0x7fffffffull) fail(DG_ERR_INVALID_ARG, "points2Octree: too many points");
  if (nseg == 0) fail(DG_ERR_INVALID_ARG, "points2Octree: no clouds");
  const unsigned SB = bits_for(nseg);
  if (3 * D + SB > 120) fail(DG_ERR_INVALID_ARG, "points2Octree: too many clouds for maxDepth");
  if (h_seg_start) {
    if (h_seg_start[0] != 0 || h_seg_start[nseg] != n)
      fail(DG_ERR_INVALID_ARG, "points2Octree: cloud offsets must run from 0 to n");
    for (size_t s = 0; s < nseg; s++)
      if (h_seg_start[s + 1] < h_seg_start[s]) fail(DG_ERR_INVALID_ARG, "points2Octree: cloud offsets decrease");
  }
  out.max_depth = D;
  out.nseg = nseg;
  out.seg_bits = SB;
  cudaStream_t s = ctx.stream;
  const u128 total = (u128)nseg << (3 * D);
  DBuf<uint64_t> d_seg_start;
  if (nseg > 1) {
    d_seg_start.alloc(nseg + 1, s);
    DG_CUDA(cudaMemcpyAsync(d_seg_start.get(), h_seg_start, (nseg + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  }
  if (D == 0 || n == 0 || (nseg == 1 && n <= m)) {
    // construct.cpp:916-920, 948-952: a cloud with at most maxPts points is
    // the root alone (still validate the points like the quantize loop)
    if (n && D) {
      DBuf<Key128> keys(n, s);
      {
        ProfScope _prof(ctx, "quantize", (double)n * 40);
        k_quantize<false><<<grid_for(n, 256), 256, 0, s>>>(d_xyz, n, (double)(1u << D), g[0], g[1], g[2], D, nullptr,
                                                           1, keys.get(), ctx.d_flags);
        DG_LAUNCH_CHECK();
      }
      check_device_flags(ctx, "points2Octree");
    }
    std::vector<Key128> roots(nseg);
    for (size_t i = 0; i < nseg; i++) roots[i] = make_tagged(seg_key(i, D), 0);
    out.n = nseg;
    DG_CUDA(cudaMallocAsync((void **)&out.keys, nseg * sizeof(Key128), s));
    DG_CUDA(cudaMemcpyAsync(out.keys, roots.data(), nseg * sizeof(Key128), cudaMemcpyHostToDevice, s));
    if (nseg > 1) {
      std::vector<uint64_t> off(nseg + 1);
      for (size_t i = 0; i <= nseg; i++) off[i] = i;
      DG_CUDA(cudaMallocAsync((void **)&out.seg_off, (nseg + 1) * sizeof(uint64_t), s));
      DG_CUDA(cudaMemcpyAsync(out.seg_off, off.data(), (nseg + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    }
    DG_CUDA(cudaStreamSynchronize(s));
    return;
  }
  DBuf<Key128> keys, tmp;
  Key128 *p;
  quantize_sorted(ctx, d_xyz, n, g, D, d_seg_start.get(), nseg, SB, keys, tmp, &p);
  Key128 *other = (p == keys.get()) ? tmp.get() : keys.get();

  // clouds with repeated points
  DBuf<uint32_t> dupseg(nseg, s);
  DG_CUDA(cudaMemsetAsync(dupseg.get(), 0, nseg * sizeof(uint32_t), s));
  DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
  {
    ProfScope _prof(ctx, "flag_dups", (double)n * 16);
    k_flag_dups<<<grid_for(n, 256), 256, 0, s>>>(p, n, D, dupseg.get(), ctx.d_flags);
    DG_LAUNCH_CHECK();
  }
  uint32_t dupflag = read_scalar(ctx, ctx.d_flags);
  DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));

  // parallel construction over all points (clouds with repeated points are
  // replaced below)
  DBuf<uint32_t> first(n, s);
  {
    ProfScope _prof(ctx, "p2o_seeds", (double)n * 36);
    k_p2o_seeds<<<grid_for(n, 256), 256, 0, s>>>(p, n, m, D, other, first.get());
    DG_LAUNCH_CHECK();
  }
  DBuf<Key128> walk_keys;  // keeps p alive for the walk when needed
  Key128 *seeds = other;
  if (dupflag) {
    // the walk needs the sorted points: compact the seeds into a new buffer
    walk_keys.alloc(n, s);
    seeds = walk_keys.get();
  }
  size_t ns = compact<Key128>(ctx, other, first.get(), n, dupflag ? seeds : p);
  if (!dupflag) seeds = p;
  first.release();
  DBuf<uint32_t> cnt(ns, s);
  {
    ProfScope _prof(ctx, "fill_count", (double)ns * 20);
    k_fill_count<<<grid_for(ns, 256), 256, 0, s>>>(seeds, ns, D, total, cnt.get());
    DG_LAUNCH_CHECK();
  }
  DBuf<uint64_t> off(ns, s);
  uint64_t *d_total = reinterpret_cast<uint64_t *>(ctx.d_scratch);
  exclusive_scan<uint32_t, uint64_t>(cnt.get(), off.get(), ns, d_total, s);
  size_t npar = (size_t)read_scalar(ctx, d_total);
  DBuf<Key128> res(npar, s);
  {
    ProfScope _prof(ctx, "fill_emit", (double)ns * 24);
    k_fill_emit<<<grid_for(ns, 256), 256, 0, s>>>(seeds, ns, D, total, off.get(), res.get());
    DG_LAUNCH_CHECK();
  }
  cnt.release();
  off.release();

  DBuf<uint64_t> seg_off;
  if (nseg > 1 || dupflag) {
    seg_off.alloc(nseg + 1, s);
    {
      ProfScope _prof(ctx, "seg_bounds", (double)(nseg + 1) * 16);
      k_seg_bounds<<<grid_for(nseg + 1, 256), 256, 0, s>>>(res.get(), npar, D, nseg, seg_off.get());
      DG_LAUNCH_CHECK();
    }
  }
  if (!dupflag) {
    out.n = npar;
    out.keys = res.release_ptr();
    out.seg_off = nseg > 1 ? seg_off.release_ptr() : nullptr;
    DG_CUDA(cudaStreamSynchronize(s));
    return;
  }

  // walk every cloud with repeated points
  std::vector<uint32_t> h_dup(nseg);
  DG_CUDA(cudaMemcpyAsync(h_dup.data(), dupseg.get(), nseg * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  std::vector<uint64_t> h_par_off(nseg + 1);
  DG_CUDA(cudaMemcpyAsync(h_par_off.data(), seg_off.get(), (nseg + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  std::vector<uint32_t> dup_list, walk_slot(nseg, 0xffffffffu);
  for (size_t i = 0; i < nseg; i++)
    if (h_dup[i]) {
      walk_slot[i] = (uint32_t)dup_list.size();
      dup_list.push_back((uint32_t)i);
    }
  const size_t nd = dup_list.size();
  std::vector<uint64_t> h_pt_start(nseg + 1);
  if (h_seg_start) {
    for (size_t i = 0; i <= nseg; i++) h_pt_start[i] = h_seg_start[i];
  } else {
    h_pt_start[0] = 0;
    h_pt_start[1] = n;
  }
  DBuf<uint64_t> d_pt_start(nseg + 1, s), d_walk_off(nd + 1, s);
  DBuf<uint32_t> d_dup_list(nd, s);
  DBuf<unsigned long long> d_counts(nd, s);
  DG_CUDA(cudaMemcpyAsync(d_pt_start.get(), h_pt_start.data(), (nseg + 1) * 8, cudaMemcpyHostToDevice, s));
  DG_CUDA(cudaMemcpyAsync(d_dup_list.get(), dup_list.data(), nd * 4, cudaMemcpyHostToDevice, s));
  {
    ProfScope _prof(ctx, "p2o_walk_serial", (double)n * 16);
    k_p2o_walk_segments<<<(unsigned)nd, 32, 0, s>>>(p, d_pt_start.get(), d_dup_list.get(), m, D, nullptr, nullptr,
                                                    d_counts.get(), nseg > 1);
    DG_LAUNCH_CHECK();
  }
  std::vector<unsigned long long> h_counts(nd);
  DG_CUDA(cudaMemcpyAsync(h_counts.data(), d_counts.get(), nd * 8, cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  std::vector<uint64_t> h_walk_off(nd + 1, 0);
  for (size_t i = 0; i < nd; i++) {
    if (h_counts[i] == (unsigned long long)P2O_WALK_NO_END)
      fail(DG_ERR_INVALID_ARG,
           "points2Octree: with these repeated points the reference construction walk never terminates");
    if (h_counts[i] == (unsigned long long)P2O_WALK_OUTSIDE)
      fail(DG_ERR_DOMAIN,
           "points2Octree: with these repeated points the reference construction emits octants outside the domain, "
           "which a batch can not hold (build this cloud alone)");
    h_walk_off[i + 1] = h_walk_off[i] + h_counts[i];
  }
  const size_t nwalk = h_walk_off[nd];
  DG_CUDA(cudaMemcpyAsync(d_walk_off.get(), h_walk_off.data(), (nd + 1) * 8, cudaMemcpyHostToDevice, s));
  DBuf<Key128> walk_out(nwalk ? nwalk : 1, s);
  {
    ProfScope _prof(ctx, "p2o_walk_serial", (double)n * 16 + (double)nwalk * 16);
    k_p2o_walk_segments<<<(unsigned)nd, 32, 0, s>>>(p, d_pt_start.get(), d_dup_list.get(), m, D, d_walk_off.get(),
                                                    walk_out.get(), d_counts.get(), nseg > 1);
    DG_LAUNCH_CHECK();
  }
  // final offsets
  std::vector<uint64_t> h_final(nseg + 1, 0);
  for (size_t i = 0; i < nseg; i++) {
    uint64_t c = h_dup[i] ? h_counts[walk_slot[i]] : (h_par_off[i + 1] - h_par_off[i]);
    h_final[i + 1] = h_final[i] + c;
  }
  const size_t nfinal = h_final[nseg];
  DBuf<uint64_t> d_final(nseg + 1, s);
  DG_CUDA(cudaMemcpyAsync(d_final.get(), h_final.data(), (nseg + 1) * 8, cudaMemcpyHostToDevice, s));
  DBuf<Key128> fin(nfinal ? nfinal : 1, s);
  {
    ProfScope _prof(ctx, "p2o_assemble", (double)(npar + nwalk) * 32);
    k_assemble<<<grid_for(std::max(npar, nwalk), 256), 256, 0, s>>>(res.get(), npar, seg_off.get(), walk_out.get(),
                                                                    d_walk_off.get(), nd, d_dup_list.get(),
                                                                    dupseg.get(), nseg, d_final.get(), D, fin.get(),
                                                                    nwalk);
    DG_LAUNCH_CHECK();
  }
  out.n = nfinal;
  out.keys = fin.release_ptr();
  if (nseg > 1) {
    out.seg_off = d_final.release_ptr();
  }
  DG_CUDA(cudaStreamSynchronize(s));
}

void octree_segment_offsets(Context &ctx, const Octree &o, uint64_t *h_off) {
  if (o.nseg == 1 || !o.seg_off) {
    h_off[0] = 0;
    h_off[1] = o.n;
    return;
  }
  DG_CUDA(cudaMemcpyAsync(h_off, o.seg_off, (o.nseg + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream));
  DG_CUDA(cudaStreamSynchronize(ctx.stream));
}

// ------------------------------------------------------------------------
// balance
// ------------------------------------------------------------------------
// level histogram; flags octants that are not aligned octants of the
// domain of their cloud (the reference asserts on those,
// octFunctions.cpp:310)
__global__ void k_level_hist(const Key128 *__restrict__ k, size_t n, unsigned D, uint64_t nseg,
                             unsigned long long *hist, uint32_t *flags) {
  __shared__ unsigned int h[32];
  if (threadIdx.x < 32) h[threadIdx.x] = 0;
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    Key128 ki = k[i];
    unsigned l = tag_level(ki);
    Key128 a = morton_part(ki, D);
    bool ok = l <= D && seg_of(ki, D) < nseg;
    if (ok && l < D) ok = key_eq(key_shl(key_shr(a, 3 * (D - l)), 3 * (D - l)), a);
    if (!ok) atomicOr(flags, DGF_DOMAIN);
    atomicAdd(&h[l & 31u], 1u);
  }
  __syncthreads();
  if (threadIdx.x < 32 && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], (unsigned long long)h[threadIdx.x]);
}

// level-(l-1) index (cloud bits included) of the parent of every input leaf
// at level l
__device__ __forceinline__ void put_key(Key128 *out, size_t i, Key128 v) { out[i] = v; }
__device__ __forceinline__ void put_key(uint64_t *out, size_t i, Key128 v) { out[i] = v.lo; }

template <typename K>
__global__ void k_leaf_parents(const Key128 *__restrict__ k, size_t n, unsigned D, unsigned l, K *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) put_key(out, i, key_shr(tag_anchor(k[i]), 3 * (D - l + 1)));
}

// for q at level l: the 8 level-(l-1) parents of q's 3x3x3 block; parents
// outside the domain are replaced by q's own parent (removed by the unique).
// Without corners (balanceOctree's incCorner = false: faces and edges only,
// the 18 directions of TreeNode::addBalancingDescendants,
// src/TreeNode.cpp:160-190) the parent that only q's corner neighbours
// reach (outward on all three axes) is replaced the same way.
template <typename K>
__global__ void k_block_parents(const Key128 *__restrict__ q, size_t nq, unsigned l, bool inc_corner,
                                K *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const Key128 qi = q[i];
  const Key128 segk = key_shl(key_shr(qi, 3 * l), 3 * (l - 1));  // cloud bits at level l-1
  Key128 idx = qi;
  if (3 * l < 64) {
    idx.lo &= (1ull << (3 * l)) - 1;
    idx.hi = 0;
  } else {
    idx.hi &= (1ull << (3 * l - 64)) - 1;
  }
  uint32_t c[3];
  demorton3(idx, c[0], c[1], c[2]);  // level-l integer coordinates
  const int64_t side = (int64_t)1 << (l - 1);  // parents per axis
  int64_t opt[3][2];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    int64_t par = c[a] >> 1;
    opt[a][0] = par;
    opt[a][1] = (c[a] & 1) ? par + 1 : par - 1;
  }
#pragma unroll
  for (int t = 0; t < 8; t++) {
    int64_t p0 = opt[0][t & 1], p1 = opt[1][(t >> 1) & 1], p2 = opt[2][(t >> 2) & 1];
    if (p0 < 0 || p1 < 0 || p2 < 0 || p0 >= side || p1 >= side || p2 >= side || (t == 7 && !inc_corner)) {
      p0 = opt[0][0];
      p1 = opt[1][0];
      p2 = opt[2][0];
    }
    put_key(out, 8 * i + t, key_or(morton3((uint32_t)p0, (uint32_t)p1, (uint32_t)p2), segk));
  }
}

__global__ void k_widen(const uint64_t *__restrict__ in, size_t n, Key128 *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = Key128{in[i], 0};
}

__device__ __forceinline__ size_t lower_bound_key(const Key128 *a, size_t n, Key128 v) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (key_lt(a[mid], v)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// rank map: R[8*parent_index + child] = index of the internal child in I_l
__global__ void k_mark_internal(const Key128 *__restrict__ Il, size_t nl, const Key128 *__restrict__ Ip, size_t np,
                                uint32_t *__restrict__ R, uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nl) return;
  Key128 par = key_shr(Il[i], 3);
  size_t p = lower_bound_key(Ip, np, par);
  if (p >= np || !key_eq(Ip[p], par)) {
    atomicOr(flags, DGF_INTERNAL);
    return;
  }
  R[8 * p + (Il[i].lo & 7u)] = (uint32_t)i;
}

// clouds whose root is internal: Rtop[cloud] = index of its root in I_0
__global__ void k_mark_roots(const Key128 *__restrict__ I0, size_t n0, size_t nseg, uint32_t *__restrict__ Rtop,
                             uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n0) return;
  uint64_t sg = I0[i].lo;
  if (I0[i].hi || sg >= nseg) {
    atomicOr(flags, DGF_INTERNAL);
    return;
  }
  Rtop[sg] = (uint32_t)i;
}

__global__ void k_subtree_count(const uint32_t *__restrict__ R, size_t np, const uint64_t *__restrict__ sub_child,
                                uint64_t *__restrict__ sub) {
  size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= np) return;
  uint64_t c = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    uint32_t x = R ? R[8 * r + q] : 0xffffffffu;
    c += (x == 0xffffffffu) ? 1ull : sub_child[x];
  }
  sub[r] = c;
}

// leaf count of every cloud (1 when its root is a leaf)
__global__ void k_cloud_count(const uint32_t *__restrict__ Rtop, size_t nseg, const uint64_t *__restrict__ sub0,
                              uint64_t *__restrict__ cnt) {
  size_t sg = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= nseg) return;
  uint32_t x = Rtop[sg];
  cnt[sg] = (x == 0xffffffffu) ? 1ull : sub0[x];
}

// place cloud roots: a leaf root is written out, an internal one passes its
// offset to level 0
__global__ void k_place_roots(const uint32_t *__restrict__ Rtop, size_t nseg, const uint64_t *__restrict__ cloud_off,
                              unsigned D, uint64_t *__restrict__ off0, Key128 *__restrict__ out) {
  size_t sg = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= nseg) return;
  uint32_t x = Rtop[sg];
  if (x == 0xffffffffu) out[cloud_off[sg]] = make_tagged(from_u128((u128)sg << (3 * D)), 0);
  else off0[x] = cloud_off[sg];
}

__global__ void k_place(const Key128 *__restrict__ Ip, size_t np, unsigned l, unsigned D, const uint32_t *__restrict__ R,
                        const uint64_t *__restrict__ sub_child, const uint64_t *__restrict__ off,
                        uint64_t *__restrict__ off_child, Key128 *__restrict__ out) {
  size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= np) return;
  uint64_t run = off[r];
  Key128 base = key_shl(Ip[r], 3);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    uint32_t x = R ? R[8 * r + q] : 0xffffffffu;
    if (x == 0xffffffffu) {
      Key128 ch = base;
      ch.lo |= (uint64_t)q;
      out[run] = make_tagged(key_shl(ch, 3 * (D - l - 1)), l + 1);
      run += 1;
    } else {
      off_child[x] = run;
      run += sub_child[x];
    }
  }
}

void balance_octree(Context &ctx, const Octree &in, Octree &out, bool inc_corner) {
  cudaStream_t s = ctx.stream;
  const unsigned D = in.max_depth;
  const size_t nseg = in.nseg;
  const unsigned SB = in.seg_bits;
  out.max_depth = D;
  out.nseg = nseg;
  out.seg_bits = SB;
  const size_t n = in.n;
  if (n == 0) fail(DG_ERR_INVALID_ARG, "balanceOctree: empty input");
  // level histogram + domain validation
  unsigned long long *d_hist = ctx.d_scratch + 16;
  DG_CUDA(cudaMemsetAsync(d_hist, 0, 32 * sizeof(unsigned long long), s));
  DG_CUDA(cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), s));
  {
    ProfScope _prof(ctx, "bal_level_hist", (double)n * 16);
    k_level_hist<<<grid_for(n, 256, ctx.num_sms * 4), 256, 0, s>>>(in.keys, n, D, nseg, d_hist, ctx.d_flags);
    DG_LAUNCH_CHECK();
  }
  check_device_flags(ctx, "balanceOctree (octant outside the domain or misaligned)");
  unsigned long long hcnt[32];
  DG_CUDA(cudaMemcpyAsync(ctx.h_scratch + 16, d_hist, sizeof(hcnt), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  std::memcpy(hcnt, ctx.h_scratch + 16, sizeof(hcnt));
  unsigned maxL = 0;
  for (unsigned l = 0; l < 32; l++)
    if (hcnt[l]) maxL = l;

  // bucket the leaves by level (one stable radix pass on the level byte);
  // every bucket stays in (cloud, Morton) order
  DBuf<Key128> bucketed(n, s);
  {
    size_t ntiles = (n + RS_TILE - 1) / RS_TILE;
    DBuf<uint32_t> hist(256 * ntiles, s);
    {
      ProfScope _prof(ctx, "rs_hist", (double)n * 16);
      k_rs_hist<Key128><<<(unsigned)ntiles, RS_BLOCK, 0, s>>>(in.keys, n, 120, hist.get(), ntiles);
      DG_LAUNCH_CHECK();
    }
    exclusive_scan<uint32_t, uint32_t>(hist.get(), hist.get(), 256 * ntiles, (uint32_t *)nullptr, s);
    {
      ProfScope _prof(ctx, "rs_scatter", (double)n * 32);
      k_rs_scatter<Key128><<<(unsigned)ntiles, RS_BLOCK, 0, s>>>(in.keys, bucketed.get(), n, 120, hist.get(), ntiles);
      DG_LAUNCH_CHECK();
    }
  }
  std::vector<size_t> boff(33, 0);
  for (unsigned l = 0; l < 32; l++) boff[l + 1] = boff[l] + hcnt[l];

  std::vector<DBuf<Key128>> I(maxL + 1);
  std::vector<size_t> nI(maxL + 1, 0);
  for (int l = (int)maxL; l >= 1; l--) {
    size_t nt = hcnt[l], nq = nI[l];
    size_t nc = nt + 8 * nq;
    if (nc == 0) continue;
    const int kbits = 3 * (l - 1) + (int)SB;
    if (kbits <= 64) {
      // level-(l-1) indices fit one word: sort 8-byte keys
      DBuf<uint64_t> cand(nc, s), ctmp(nc, s);
      if (nt) {
        ProfScope _prof(ctx, "bal_leaf_parents", (double)nt * 24);
        k_leaf_parents<uint64_t><<<grid_for(nt, 256), 256, 0, s>>>(bucketed.get() + boff[l], nt, D, (unsigned)l,
                                                                   cand.get());
        DG_LAUNCH_CHECK();
      }
      if (nq) {
        ProfScope _prof(ctx, "bal_block_parents", (double)nq * 80);
        k_block_parents<uint64_t><<<grid_for(nq, 256), 256, 0, s>>>(I[l].get(), nq, (unsigned)l, inc_corner, cand.get() + nt);
        DG_LAUNCH_CHECK();
      }
      uint64_t *res;
      size_t nu = sort_unique<uint64_t>(ctx, cand.get(), ctmp.get(), nc, kbits, &res);
      DBuf<Key128> Il(nu, s);
      {
        ProfScope _prof(ctx, "bal_widen", (double)nu * 24);
        k_widen<<<grid_for(nu, 256), 256, 0, s>>>(res, nu, Il.get());
        DG_LAUNCH_CHECK();
      }
      I[l - 1] = std::move(Il);
      nI[l - 1] = nu;
    } else {
      DBuf<Key128> cand(nc, s), ctmp(nc, s);
      if (nt) {
        ProfScope _prof(ctx, "bal_leaf_parents", (double)nt * 32);
        k_leaf_parents<Key128><<<grid_for(nt, 256), 256, 0, s>>>(bucketed.get() + boff[l], nt, D, (unsigned)l,
                                                                 cand.get());
        DG_LAUNCH_CHECK();
      }
      if (nq) {
        ProfScope _prof(ctx, "bal_block_parents", (double)nq * 144);
        k_block_parents<Key128><<<grid_for(nq, 256), 256, 0, s>>>(I[l].get(), nq, (unsigned)l, inc_corner, cand.get() + nt);
        DG_LAUNCH_CHECK();
      }
      Key128 *res;
      size_t nu = sort_unique<Key128>(ctx, cand.get(), ctmp.get(), nc, kbits, &res);
      DBuf<Key128> Il(nu, s);
      DG_CUDA(cudaMemcpyAsync(Il.get(), res, nu * sizeof(Key128), cudaMemcpyDeviceToDevice, s));
      I[l - 1] = std::move(Il);
      nI[l - 1] = nu;
    }
  }
  bucketed.release();

  // rank maps R_l (l = 0..maxL-1): children of I_l that are internal
  std::vector<DBuf<uint32_t>> R(maxL + 1);
  for (unsigned l = 0; l + 1 <= maxL; l++) {
    if (!nI[l] || !nI[l + 1]) continue;
    R[l].alloc(8 * nI[l], s);
    DG_CUDA(cudaMemsetAsync(R[l].get(), 0xff, 8 * nI[l] * sizeof(uint32_t), s));
    {
      ProfScope _prof(ctx, "bal_mark_internal", (double)nI[l + 1] * 20);
      k_mark_internal<<<grid_for(nI[l + 1], 256), 256, 0, s>>>(I[l + 1].get(), nI[l + 1], I[l].get(), nI[l],
                                                               R[l].get(), ctx.d_flags);
      DG_LAUNCH_CHECK();
    }
  }
  DBuf<uint32_t> Rtop(nseg, s);
  DG_CUDA(cudaMemsetAsync(Rtop.get(), 0xff, nseg * sizeof(uint32_t), s));
  if (maxL > 0 && nI[0]) {
    k_mark_roots<<<grid_for(nI[0], 256), 256, 0, s>>>(I[0].get(), nI[0], nseg, Rtop.get(), ctx.d_flags);
    DG_LAUNCH_CHECK();
  }
  check_device_flags(ctx, "balanceOctree");
  // bottom-up leaf counts
  std::vector<DBuf<uint64_t>> sub(maxL + 1);
  for (int l = (int)maxL - 1; l >= 0; l--) {
    if (!nI[l]) continue;
    sub[l].alloc(nI[l], s);
    {
      ProfScope _prof(ctx, "bal_subtree_count", (double)nI[l] * 72);
      k_subtree_count<<<grid_for(nI[l], 256), 256, 0, s>>>(R[l].get(), nI[l], sub[l + 1].get(), sub[l].get());
      DG_LAUNCH_CHECK();
    }
  }
  DBuf<uint64_t> ccnt(nseg, s), coff(nseg + 1, s);
  k_cloud_count<<<grid_for(nseg, 256), 256, 0, s>>>(Rtop.get(), nseg, sub[0].get(), ccnt.get());
  DG_LAUNCH_CHECK();
  uint64_t *d_total = reinterpret_cast<uint64_t *>(ctx.d_scratch);
  exclusive_scan<uint64_t, uint64_t>(ccnt.get(), coff.get(), nseg, d_total, s);
  size_t total = (size_t)read_scalar(ctx, d_total);
  DG_CUDA(cudaMemcpyAsync(coff.get() + nseg, d_total, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
  DBuf<Key128> res(total, s);
  // top-down placement
  DBuf<uint64_t> off_cur(nI[0] ? nI[0] : 1, s);
  k_place_roots<<<grid_for(nseg, 256), 256, 0, s>>>(Rtop.get(), nseg, coff.get(), D, off_cur.get(), res.get());
  DG_LAUNCH_CHECK();
  for (unsigned l = 0; l < maxL; l++) {
    if (!nI[l]) break;
    DBuf<uint64_t> off_next(nI[l + 1] ? nI[l + 1] : 1, s);
    {
      ProfScope _prof(ctx, "bal_place", (double)nI[l] * 24);
      k_place<<<grid_for(nI[l], 256), 256, 0, s>>>(I[l].get(), nI[l], l, D, R[l].get(), sub[l + 1].get(),
                                                   off_cur.get(), off_next.get(), res.get());
      DG_LAUNCH_CHECK();
    }
    off_cur = std::move(off_next);
  }
  DG_CUDA(cudaStreamSynchronize(s));
  out.n = total;
  out.keys = res.release_ptr();
  out.seg_off = nseg > 1 ? coff.release_ptr() : nullptr;
}

// ------------------------------------------------------------------------
// coarsenOctree (src/coarsen.cpp:53): every complete family of 8 sibling
// leaves is replaced by its parent.  On a sorted, linear, complete octree
// the reference's rule (a first child followed by 7 octants that are not
// first children) is exactly "the 8 octants from a first child are the 8
// children of one parent"; a batch never merges across clouds because the
// parent test includes the cloud bits.
// ------------------------------------------------------------------------
__device__ __forceinline__ unsigned key_child(Key128 k, unsigned D) {
  unsigned l = tag_level(k);
  if (l == 0) return 0;
  return (unsigned)(key_shr(tag_anchor(k), 3 * (D - l)).lo & 7u);
}
__device__ __forceinline__ Key128 key_parent(Key128 k, unsigned D) {
  unsigned l = tag_level(k);
  unsigned sh = 3 * (D - l + 1);
  return make_tagged(key_shl(key_shr(tag_anchor(k), sh), sh), l - 1);
}

__global__ void k_coarsen_mark(const Key128 *__restrict__ k, size_t n, unsigned D, uint32_t *__restrict__ fam) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Key128 ki = k[i];
  const unsigned l = tag_level(ki);
  bool start = l >= 1 && key_child(ki, D) == 0 && i + 7 < n;
  if (start) {
    const Key128 par = key_parent(ki, D);
    for (int j = 1; j < 8 && start; j++) {
      Key128 kj = k[i + j];
      start = tag_level(kj) == l && key_eq(key_parent(kj, D), par);
    }
  }
  fam[i] = start ? 1u : 0u;
}

__global__ void k_coarsen_apply(const Key128 *__restrict__ k, size_t n, unsigned D, const uint32_t *__restrict__ fam,
                                Key128 *__restrict__ val, uint32_t *__restrict__ keep) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Key128 ki = k[i];
  const unsigned c = key_child(ki, D);
  const bool member = c >= 1 && i >= c && fam[i - c];
  keep[i] = member ? 0u : 1u;
  val[i] = fam[i] ? key_parent(ki, D) : ki;
}

void coarsen_octree(Context &ctx, const Octree &in, Octree &out) {
  cudaStream_t s = ctx.stream;
  const size_t n = in.n;
  out.max_depth = in.max_depth;
  out.nseg = in.nseg;
  out.seg_bits = in.seg_bits;
  if (in.nseg != 1) fail(DG_ERR_UNSUPPORTED, "coarsenOctree: one cloud per call");
  DBuf<Key128> res(n ? n : 1, s);
  if (n < 8) {  // coarsen.cpp:66-70
    if (n) DG_CUDA(cudaMemcpyAsync(res.get(), in.keys, n * sizeof(Key128), cudaMemcpyDeviceToDevice, s));
    DG_CUDA(cudaStreamSynchronize(s));
    out.n = n;
    out.keys = res.release_ptr();
    return;
  }
  DBuf<uint32_t> fam(n, s), keep(n, s);
  DBuf<Key128> val(n, s);
  {
    ProfScope _prof(ctx, "coarsen_mark", (double)n * 20);
    k_coarsen_mark<<<grid_for(n, 256), 256, 0, s>>>(in.keys, n, in.max_depth, fam.get());
    DG_LAUNCH_CHECK();
  }
  {
    ProfScope _prof(ctx, "coarsen_apply", (double)n * 40);
    k_coarsen_apply<<<grid_for(n, 256), 256, 0, s>>>(in.keys, n, in.max_depth, fam.get(), val.get(), keep.get());
    DG_LAUNCH_CHECK();
  }
  out.n = compact<Key128>(ctx, val.get(), keep.get(), n, res.get());
  out.keys = res.release_ptr();
}

// ------------------------------------------------------------------------
// completeOctree (src/construct.cpp:518).  At one rank the reference runs its
// general path (:534-700): the tree sort's sort + duplicate + ancestor
// removal when the input is not declared unique (include/sfcSort.h:532-575),
// a plain sort when it is unique but not declared sorted, then
// appendCompleteRegion (:1077) between consecutive octants, an octant that is
// followed by its own descendant being left out.  The filled gaps are the
// maximal aligned Morton blocks between consecutive leaves (the same blocks
// appendCompleteRegion emits), so the construction's gap kernels apply.
// ------------------------------------------------------------------------
// sort form: the Morton anchor above the 5 level bits, so that a radix sort
// over the low 3D + 5 bits gives the reference's order (on equal anchors the
// coarser octant first)
__global__ void k_to_sortform(const Key128 *__restrict__ in, size_t n, Key128 *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = key_or(key_shl(tag_anchor(in[i]), 5), Key128{(uint64_t)tag_level(in[i]), 0});
}

__global__ void k_from_sortform(const Key128 *__restrict__ in, size_t n, Key128 *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_tagged(key_shr(in[i], 5), (unsigned)(in[i].lo & 31u));
}

// octant i is kept unless its successor is its descendant; an order that
// breaks the caller's declaration raises DGF_ORDER
__global__ void k_complete_leaves(const Key128 *__restrict__ s, size_t n, unsigned D, bool strict,
                                  Key128 *__restrict__ val, uint32_t *__restrict__ keep, uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Key128 a = s[i];
  const unsigned la = (unsigned)(a.lo & 31u);
  bool k = true;
  if (i + 1 < n) {
    const Key128 b = s[i + 1];
    if (key_lt(b, a) || (strict && key_eq(a, b))) atomicOr(flags, DGF_ORDER);
    const unsigned lb = (unsigned)(b.lo & 31u);
    if (la < lb) {
      const unsigned sh = 5 + 3 * (D - la);
      k = !key_eq(key_shr(a, sh), key_shr(b, sh));
    }
  }
  val[i] = make_tagged(key_shr(a, 5), la);
  keep[i] = k ? 1u : 0u;
}

// ------------------------------------------------------------------------
// one cloud of a batch as its own octree (cloud bits cleared)
// ------------------------------------------------------------------------
__global__ void k_strip_cloud(const Key128 *__restrict__ in, size_t n, unsigned D, Key128 *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_tagged(morton_part(in[i], D), tag_level(in[i]));
}

void octree_extract(Context &ctx, const Octree &in, size_t seg, Octree &out) {
  if (seg >= in.nseg) fail(DG_ERR_INVALID_ARG, "octree: cloud index out of range");
  uint64_t off[2] = {0, in.n};
  if (in.nseg > 1)
    DG_CUDA(cudaMemcpyAsync(off, in.seg_off + seg, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream));
  DG_CUDA(cudaStreamSynchronize(ctx.stream));
  const size_t n = off[1] - off[0];
  out = Octree();
  out.max_depth = in.max_depth;
  out.n = n;
  DBuf<Key128> k(n ? n : 1, ctx.stream);
  if (n) {
    ProfScope _prof(ctx, "strip_cloud", (double)n * 32);
    k_strip_cloud<<<grid_for(n, 256), 256, 0, ctx.stream>>>(in.keys + off[0], n, in.max_depth, k.get());
    DG_LAUNCH_CHECK();
  }
  out.keys = k.release_ptr();
}

// ------------------------------------------------------------------------
// conversions
// ------------------------------------------------------------------------
// (a single cloud may hold octants just outside its domain: the reference's
// construction emits them for some inputs with repeated points; their
// anchor bits then run past 3D and are decoded as is)
__global__ void k_to_xyzl(const Key128 *__restrict__ k, size_t n, unsigned D, bool batched, uint4 *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t x, y, z;
  demorton3(batched ? morton_part(k[i], D) : tag_anchor(k[i]), x, y, z);
  out[i] = make_uint4(x, y, z, tag_level(k[i]));
}

__global__ void k_from_xyzl(const uint4 *__restrict__ in, size_t n, unsigned D, Key128 *__restrict__ out,
                            uint32_t *flags) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint4 v = in[i];
  unsigned lev = v.w & 31u;
  uint64_t len = 1ull << (D - min(lev, D));
  uint64_t dom = 1ull << D;
  bool ok = lev <= D && v.x % len == 0 && v.y % len == 0 && v.z % len == 0 && v.x < dom && v.y < dom && v.z < dom;
  if (!ok) atomicOr(flags, DGF_DOMAIN);
  out[i] = make_tagged(morton3(v.x, v.y, v.z), lev);
}

// ------------------------------------------------------------------------
// Hilbert order (the reference's default build, -DHILBERT_ORDERING:
// TreeNode::operator< include/TreeNode.tcc:130-210 with the tables of
// src/hcurvedata.cpp:329-520).  The curve is self-similar: a cell's 8
// children are visited in the order HIL_BASE_ORDER, transformed by the
// cell's own symmetry, and each child's cell carries its parent's symmetry
// composed with HIL_CHILD_SYM of its base position.  A state table of the
// reachable symmetries (24) is generated from these two rows; an octant's
// key is its child ranks root to leaf (3 bits per level), padded to maxDepth,
// above its level, which orders octants as the reference's comparison does
// (an ancestor before its descendants).
// ------------------------------------------------------------------------
namespace {
// corner index c = x | y << 1 | z << 2
constexpr uint8_t HIL_BASE_ORDER[8] = {0, 2, 3, 1, 5, 7, 6, 4};
// child symmetry per base corner: new bit i = old bit perm[i] ^ bit i of flip
struct CubeSym {
  uint8_t perm[3];
  uint8_t flip;
};
constexpr CubeSym HIL_CHILD_SYM[8] = {{{0, 2, 1}, 0}, {{2, 0, 1}, 6}, {{2, 1, 0}, 0}, {{0, 1, 2}, 0},
                                      {{0, 2, 1}, 6}, {{2, 0, 1}, 3}, {{2, 1, 0}, 5}, {{0, 1, 2}, 0}};
constexpr int HIL_MAX_STATES = 32;

struct HilbertTable {
  uint8_t e[HIL_MAX_STATES * 8];  // [state][corner]: rank | next state << 3
};

HilbertTable build_hilbert_table() {
  using Map = std::array<uint8_t, 8>;  // a symmetry as its action on corners
  auto sym_map = [](const CubeSym &g) {
    Map m{};
    for (unsigned c = 0; c < 8; c++) {
      unsigned r = 0;
      for (unsigned i = 0; i < 3; i++) r |= (((c >> g.perm[i]) & 1u) ^ ((g.flip >> i) & 1u)) << i;
      m[c] = (uint8_t)r;
    }
    return m;
  };
  uint8_t rank0[8];
  for (unsigned k = 0; k < 8; k++) rank0[HIL_BASE_ORDER[k]] = (uint8_t)k;
  std::vector<Map> states;
  Map id{};
  for (unsigned c = 0; c < 8; c++) id[c] = (uint8_t)c;
  states.push_back(id);
  HilbertTable t{};
  for (size_t s = 0; s < states.size(); s++) {
    const Map g = states[s];
    Map ginv{};
    for (unsigned c = 0; c < 8; c++) ginv[g[c]] = (uint8_t)c;
    for (unsigned c = 0; c < 8; c++) {
      const unsigned c0 = ginv[c];
      const Map tc = sym_map(HIL_CHILD_SYM[c0]);
      Map child{};
      for (unsigned q = 0; q < 8; q++) child[q] = g[tc[q]];
      size_t id2 = std::find(states.begin(), states.end(), child) - states.begin();
      if (id2 == states.size()) {
        if (states.size() == HIL_MAX_STATES) fail(DG_ERR_INTERNAL, "Hilbert table: too many states");
        states.push_back(child);
      }
      t.e[s * 8 + c] = (uint8_t)(rank0[c0] | (id2 << 3));
    }
  }
  return t;
}

const HilbertTable &hilbert_table() {
  static const HilbertTable t = build_hilbert_table();
  return t;
}
}  // namespace

// key[i] = (Hilbert rank path << 5 | level) << 32 | i for the octants of
// one cloud (i < 2^32)
__global__ void k_hilbert_keys(const Key128 *__restrict__ k, size_t n, unsigned D, bool batched, HilbertTable tab,
                               Key128 *__restrict__ out) {
  __shared__ uint8_t t[HIL_MAX_STATES * 8];
  for (int i = threadIdx.x; i < HIL_MAX_STATES * 8; i += blockDim.x) t[i] = tab.e[i];
  __syncthreads();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t x, y, z;
  demorton3(batched ? morton_part(k[i], D) : tag_anchor(k[i]), x, y, z);
  const unsigned lev = tag_level(k[i]);
  u128 h = 0;
  unsigned st = 0;
  for (unsigned l = 0; l < lev; l++) {
    const unsigned b = D - 1 - l;
    const unsigned c = ((x >> b) & 1u) | (((y >> b) & 1u) << 1) | (((z >> b) & 1u) << 2);
    const unsigned e = t[st * 8 + c];
    h = (h << 3) | (e & 7u);
    st = e >> 3;
  }
  h <<= 3 * (D - lev);
  out[i] = from_u128((((h << 5) | lev) << 32) | (u128)(uint32_t)i);
}

__global__ void k_gather_xyzl(const Key128 *__restrict__ k, const Key128 *__restrict__ order, size_t n, unsigned D,
                              bool batched, uint4 *__restrict__ out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Key128 v = k[(uint32_t)order[i].lo];
  uint32_t x, y, z;
  demorton3(batched ? morton_part(v, D) : tag_anchor(v), x, y, z);
  out[i] = make_uint4(x, y, z, tag_level(v));
}

// records of o in Hilbert order, cloud by cloud
static void octree_to_xyzl_hilbert(Context &ctx, const Octree &o, uint32_t *d_xyzl) {
  cudaStream_t s = ctx.stream;
  const unsigned D = o.max_depth;
  std::vector<uint64_t> off{0, (uint64_t)o.n};
  if (o.nseg > 1) {
    off.resize(o.nseg + 1);
    DG_CUDA(cudaMemcpyAsync(off.data(), o.seg_off, (o.nseg + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    DG_CUDA(cudaStreamSynchronize(s));
  }
  const HilbertTable &tab = hilbert_table();
  DBuf<Key128> a(o.n, s), b(o.n, s);
  for (size_t g = 0; g + 1 < off.size(); g++) {
    const size_t n = off[g + 1] - off[g];
    if (!n) continue;
    if (n > 0xffffffffull) fail(DG_ERR_UNSUPPORTED, "Hilbert order: more than 2^32 octants in one cloud");
    ProfScope _prof(ctx, "hilbert_order", (double)n * 16 * 36);
    k_hilbert_keys<<<grid_for(n, 256), 256, 0, s>>>(o.keys + off[g], n, D, o.nseg > 1, tab, a.get() + off[g]);
    DG_LAUNCH_CHECK();
    Key128 *srt = radix_sort<Key128>(ctx, a.get() + off[g], b.get() + off[g], n, 3 * (int)D + 5 + 32);
    k_gather_xyzl<<<grid_for(n, 256), 256, 0, s>>>(o.keys + off[g], srt, n, D, o.nseg > 1,
                                                   reinterpret_cast<uint4 *>(d_xyzl) + off[g]);
    DG_LAUNCH_CHECK();
  }
}

void octree_to_xyzl(Context &ctx, const Octree &o, uint32_t *d_xyzl) {
  if (!o.n) return;
  if (ctx.order == 1) {
    octree_to_xyzl_hilbert(ctx, o, d_xyzl);
    return;
  }
  {
    ProfScope _prof("to_xyzl", (double)o.n * 32);
    k_to_xyzl<<<grid_for(o.n, 256), 256, 0, ctx.stream>>>(o.keys, o.n, o.max_depth, o.nseg > 1,
                                                          reinterpret_cast<uint4 *>(d_xyzl));
    DG_LAUNCH_CHECK();
  }
}

void octree_from_xyzl(Context &ctx, const uint32_t *d_xyzl, size_t n, unsigned D, Octree &out) {
  out.max_depth = D;
  out.n = n;
  DBuf<Key128> k(n, ctx.stream);
  if (n) {
    {
      ProfScope _prof("from_xyzl", (double)n * 32);
      k_from_xyzl<<<grid_for(n, 256), 256, 0, ctx.stream>>>(reinterpret_cast<const uint4 *>(d_xyzl), n, D, k.get(),
                                                            ctx.d_flags);
      DG_LAUNCH_CHECK();
    }
    check_device_flags(ctx, "octree upload");
    if (ctx.order == 1) {  // records in Hilbert order: the device keeps Morton order
      DBuf<Key128> a(n, ctx.stream), b(n, ctx.stream);
      k_to_sortform<<<grid_for(n, 256), 256, 0, ctx.stream>>>(k.get(), n, a.get());
      DG_LAUNCH_CHECK();
      Key128 *srt = radix_sort<Key128>(ctx, a.get(), b.get(), n, 3 * (int)D + 5);
      k_from_sortform<<<grid_for(n, 256), 256, 0, ctx.stream>>>(srt, n, k.get());
      DG_LAUNCH_CHECK();
    }
  }
  out.keys = k.release_ptr();
}

void octree_free(Context &ctx, Octree &o) {
  if (o.keys) cudaFreeAsync(o.keys, ctx.stream);
  if (o.seg_off) cudaFreeAsync(o.seg_off, ctx.stream);
  o = Octree();
}

void complete_octree(Context &ctx, const uint32_t *d_xyzl, size_t n, unsigned D, bool is_unique, bool is_sorted,
                     Octree &out) {
  cudaStream_t s = ctx.stream;
  out = Octree();
  out.max_depth = D;
  if (n == 0) return;  // construct.cpp:587: nothing to complete
  DBuf<Key128> a(n, s), b(n, s);
  {
    ProfScope _prof(ctx, "complete_sortform", (double)n * 48);
    k_from_xyzl<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const uint4 *>(d_xyzl), n, D, b.get(),
                                                 ctx.d_flags);
    DG_LAUNCH_CHECK();
    k_to_sortform<<<grid_for(n, 256), 256, 0, s>>>(b.get(), n, a.get());
    DG_LAUNCH_CHECK();
  }
  check_device_flags(ctx, "completeOctree");  // domain and alignment of the records
  const int bits = 3 * (int)D + 5;
  if (ctx.order == 1) is_sorted = false;  // records in Hilbert order: sorted into Morton order here
  Key128 *sorted = a.get();
  size_t m = n;
  if (!is_unique) m = sort_unique<Key128>(ctx, a.get(), b.get(), n, bits, &sorted);
  else if (!is_sorted) sorted = radix_sort<Key128>(ctx, a.get(), b.get(), n, bits);
  Key128 *other = (sorted == a.get()) ? b.get() : a.get();
  DBuf<uint32_t> keep(m, s);
  {
    ProfScope _prof(ctx, "complete_leaves", (double)m * 36);
    k_complete_leaves<<<grid_for(m, 256), 256, 0, s>>>(sorted, m, D, is_unique, other, keep.get(), ctx.d_flags);
    DG_LAUNCH_CHECK();
  }
  check_device_flags(ctx, "completeOctree");
  const size_t ns = compact<Key128>(ctx, other, keep.get(), m, sorted);
  keep.release();
  const u128 total = (u128)1 << (3 * D);
  DBuf<uint32_t> cnt(ns, s);
  {
    ProfScope _prof(ctx, "fill_count", (double)ns * 20);
    k_fill_count<<<grid_for(ns, 256), 256, 0, s>>>(sorted, ns, D, total, cnt.get());
    DG_LAUNCH_CHECK();
  }
  DBuf<uint64_t> off(ns, s);
  uint64_t *d_total = reinterpret_cast<uint64_t *>(ctx.d_scratch);
  exclusive_scan<uint32_t, uint64_t>(cnt.get(), off.get(), ns, d_total, s);
  const size_t nout = (size_t)read_scalar(ctx, d_total);
  DBuf<Key128> res(nout, s);
  {
    ProfScope _prof(ctx, "fill_emit", (double)ns * 24);
    k_fill_emit<<<grid_for(ns, 256), 256, 0, s>>>(sorted, ns, D, total, off.get(), res.get());
    DG_LAUNCH_CHECK();
  }
  out.n = nout;
  out.keys = res.release_ptr();
}

// par::sampleSort (include/parUtils.h:424; at one rank a local sort,
// src/parUtils.tcc:1868-1875) and par::removeDuplicates (parUtils.h:437) of
// octant records: sorted in the octant order (ancestor first on equal
// anchors), repeated records removed when asked (mode 1).  Mode 2 is the
// TS_REMOVE_DUPLICATES output of SFC::seqSort::SFC_treeSort
// (include/sfcSort.h:532-575): sorted, repeated records removed, and every
// octant followed by one of its descendants removed (the descendants of an
// octant follow it contiguously in any space-filling-curve order).
void sort_octants(Context &ctx, const uint32_t *d_xyzl, size_t n, unsigned D, int mode, Octree &out) {
  const bool unique = mode != 0;
  cudaStream_t s = ctx.stream;
  out = Octree();
  out.max_depth = D;
  if (n == 0) return;
  DBuf<Key128> a(n, s), b(n, s);
  {
    ProfScope _prof(ctx, "sort_octants_keys", (double)n * 48);
    k_from_xyzl<<<grid_for(n, 256), 256, 0, s>>>(reinterpret_cast<const uint4 *>(d_xyzl), n, D, b.get(),
                                                 ctx.d_flags);
    DG_LAUNCH_CHECK();
    k_to_sortform<<<grid_for(n, 256), 256, 0, s>>>(b.get(), n, a.get());
    DG_LAUNCH_CHECK();
  }
  check_device_flags(ctx, "sortOctants");
  const int bits = 3 * (int)D + 5;
  Key128 *srt = a.get();
  size_t m = n;
  if (unique) m = sort_unique<Key128>(ctx, a.get(), b.get(), n, bits, &srt);
  else srt = radix_sort<Key128>(ctx, a.get(), b.get(), n, bits);
  if (mode == 2) {
    // tagged keys of the octants not followed by a descendant
    Key128 *other = (srt == a.get()) ? b.get() : a.get();
    DBuf<uint32_t> keep(m, s);
    {
      ProfScope _prof(ctx, "treesort_leaves", (double)m * 36);
      k_complete_leaves<<<grid_for(m, 256), 256, 0, s>>>(srt, m, D, true, other, keep.get(), ctx.d_flags);
      DG_LAUNCH_CHECK();
    }
    DBuf<Key128> res(m, s);
    const size_t nk = compact<Key128>(ctx, other, keep.get(), m, res.get());
    check_device_flags(ctx, "SFC_treeSort");
    out.n = nk;
    out.keys = res.release_ptr();
    return;
  }
  DBuf<Key128> res(m, s);
  k_from_sortform<<<grid_for(m, 256), 256, 0, s>>>(srt, m, res.get());
  DG_LAUNCH_CHECK();
  out.n = m;
  out.keys = res.release_ptr();
}

// ------------------------------------------------------------------------
namespace {
__global__ void k_selftest_keys(uint64_t *k, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) k[i] = (i * 0x9E3779B97F4A7C15ull) >> 7;  // every low digit occurs
}
}  // namespace

void lookback_timeout_selftest(Context &ctx, size_t n, unsigned skipped) {
  using K = uint64_t;
  constexpr size_t TILE = (size_t)RS_BLOCK * OsCfg<K>::ITEMS;
  const size_t ntiles = (n + TILE - 1) / TILE;
  if (skipped == 0 || ntiles <= skipped || ntiles > (1u << 20))
    fail(DG_ERR_INVALID_ARG, "look-back self-test: need 1 <= skipped < tiles <= 2^20");
  cudaStream_t s = ctx.stream;
  DBuf<K> in(n, s), out(n, s);
  DBuf<uint64_t> status(ntiles * 256, s), doffs(256, s);
  k_selftest_keys<<<grid_for(n, 256), 256, 0, s>>>(in.get(), n);
  DG_LAUNCH_CHECK();
  // digit offsets of the low byte (exclusive scan of its histogram), so
  // every write of the pass stays inside [0, n)
  std::vector<uint64_t> h(256, 0), offs(256, 0);
  std::vector<K> keys(n);
  DG_CUDA(cudaMemcpyAsync(keys.data(), in.get(), n * sizeof(K), cudaMemcpyDeviceToHost, s));
  DG_CUDA(cudaStreamSynchronize(s));
  for (K k : keys) h[k & 255]++;
  for (int d = 1; d < 256; d++) offs[d] = offs[d - 1] + h[d - 1];
  DG_CUDA(cudaMemcpyAsync(doffs.get(), offs.data(), 256 * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  DG_CUDA(cudaMemsetAsync(status.get(), 0, ntiles * 256 * sizeof(uint64_t), s));
  // the tile tickets start at `skipped`: tiles [0, skipped) are never
  // processed and their status words stay unpublished
  unsigned *d_counter = reinterpret_cast<unsigned *>(ctx.d_scratch + 12);
  const unsigned start = skipped;
  DG_CUDA(cudaMemcpyAsync(d_counter, &start, sizeof(unsigned), cudaMemcpyHostToDevice, s));
  k_rs_onesweep<K, OsCfg<K>::ITEMS><<<(unsigned)(ntiles - skipped), RS_BLOCK, 0, s>>>(
      in.get(), out.get(), n, 0, doffs.get(), status.get(), d_counter, ctx.d_flags);
  DG_LAUNCH_CHECK();
  check_device_flags(ctx, "look-back self-test");
}

}  // namespace dg
