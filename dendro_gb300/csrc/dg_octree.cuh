// Device-resident linear octrees and the construction / balance pipelines.
#pragma once

#include "dg_prims.cuh"

namespace dg {

// An octant is one 16-byte tagged key: the Morton index of its anchor at the
// finest level D in bits [0, 3D) and its level in the top byte (bits
// 120..127).  A linear octree is a sorted array of tagged keys; ordering
// compares the anchor bits only.
constexpr uint64_t TAG_MASK = 0x00ffffffffffffffull;

__host__ __device__ __forceinline__ unsigned tag_level(Key128 k) { return (unsigned)(k.hi >> 56); }
__host__ __device__ __forceinline__ Key128 tag_anchor(Key128 k) { return Key128{k.lo, k.hi & TAG_MASK}; }
__host__ __device__ __forceinline__ Key128 make_tagged(Key128 anchor, unsigned lev) {
  return Key128{anchor.lo, (anchor.hi & TAG_MASK) | ((uint64_t)lev << 56)};
}

// A batch of independent octrees ("segments", one per point cloud) shares
// one key array: segment s occupies keys [seg_off[s], seg_off[s+1]) and its
// keys carry s in bits [3D, 3D + seg_bits), so one sort orders the whole
// batch by cloud, then by Morton order within each cloud.
struct Octree {
  unsigned max_depth = 0;
  size_t n = 0;
  Key128 *keys = nullptr;      // tagged, sorted
  size_t nseg = 1;
  unsigned seg_bits = 0;
  uint64_t *seg_off = nullptr;  // device, nseg + 1 (null for one segment)
};

inline unsigned bits_for(size_t nseg) {
  unsigned b = 0;
  while (b < 40 && ((size_t)1 << b) < nseg) b++;
  return b;
}

void octree_free(Context &ctx, Octree &o);

// ot::points2Octree (src/construct.cpp:759) on device-resident FP64 xyz, for
// a batch of clouds: cloud s holds points [h_seg_start[s], h_seg_start[s+1])
// (host array of nseg + 1 entries; null for a single cloud).  Each cloud's
// octree is the one the reference builds for that cloud alone.
void points_to_octree(Context &ctx, const double *d_xyz, size_t n, const double glens[3], unsigned max_depth,
                      unsigned max_pts, Octree &out, const uint64_t *h_seg_start = nullptr, size_t nseg = 1);

// per-segment output offsets of a batched octree, on the host
void octree_segment_offsets(Context &ctx, const Octree &o, uint64_t *h_off);

// Morton sort of level-D point anchors (par::sampleSort / removeDuplicates
// step); returns sorted tagged keys in d_out and the number of distinct
// points.
size_t sort_points(Context &ctx, const double *d_xyz, size_t n, const double glens[3], unsigned max_depth,
                   Key128 *d_out, bool *has_duplicates);

// ot::balanceOctree (src/balance.cpp:31): 2:1 balance across faces, edges
// and corners (inc_corner) or across faces and edges only.
void balance_octree(Context &ctx, const Octree &in, Octree &out, bool inc_corner = true);

// cloud `seg` of a batched octree as a single-cloud octree
void octree_extract(Context &ctx, const Octree &in, size_t seg, Octree &out);

// ot::coarsenOctree (src/coarsen.cpp:53), one cloud.
void coarsen_octree(Context &ctx, const Octree &in, Octree &out);

// ot::completeOctree (src/construct.cpp:518), one cloud: the octants of
// d_xyzl (n records x y z level at max_depth), sorted and made unique and
// linear unless declared so, completed with the coarsest octants.
void complete_octree(Context &ctx, const uint32_t *d_xyzl, size_t n, unsigned max_depth, bool is_unique,
                     bool is_sorted, Octree &out);

// par::sampleSort / par::removeDuplicates (include/parUtils.h:424,437) of
// n octant records at max_depth: mode 0 sorts, mode 1 also removes repeated
// octants, mode 2 also removes every octant that has a descendant in the
// set (SFC_treeSort with TS_REMOVE_DUPLICATES, include/sfcSort.h:532-575)
void sort_octants(Context &ctx, const uint32_t *d_xyzl, size_t n, unsigned max_depth, int mode, Octree &out);

// conversions between tagged keys and {x, y, z, level} u32 records
void octree_to_xyzl(Context &ctx, const Octree &o, uint32_t *d_xyzl);
void octree_from_xyzl(Context &ctx, const uint32_t *d_xyzl, size_t n, unsigned max_depth, Octree &out);

// Self-test of the radix sort's bounded look-back wait: one digit pass over
// n_keys keys in which the first `skipped` tiles never run, so the next
// tile waits for a predecessor that never publishes.  The wait gives up
// after its spin limit and the pass raises DGF_TIMEOUT (DG_ERR_TIMEOUT).
void lookback_timeout_selftest(Context &ctx, size_t n_keys, unsigned skipped);

}  // namespace dg
