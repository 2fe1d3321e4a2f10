// The reference's p2oLocal walk (src/construct.cpp:976-1076), step for step,
// for inputs with repeated points; host and device (one thread).
#pragma once

#include "dg_octree.cuh"

namespace dg {

// ------------------------------------------------------------------------
// the reference walk, verbatim, for inputs with repeated points
// (construct.cpp:976-1076); one thread; count pass then emit pass
// ------------------------------------------------------------------------
struct WOct {
  uint32_t x, y, z, lev;
};
// the point's anchor within its cloud (segment bits above 3D dropped)
__host__ __device__ __forceinline__ WOct wo_from_key(Key128 k, unsigned D) {
  WOct o;
  Key128 a = tag_anchor(k);
  if (3 * D < 64) {
    a.lo &= (1ull << (3 * D)) - 1;
    a.hi = 0;
  } else {
    a.hi &= (1ull << (3 * D - 64)) - 1;
  }
  demorton3(a, o.x, o.y, o.z);
  o.lev = tag_level(k);
  return o;
}
__host__ __device__ __forceinline__ u128 wo_key(const WOct &o) {
  return (to_u128(morton3(o.x, o.y, o.z)) << 5) | (u128)(o.lev & 31u);
}
__host__ __device__ __forceinline__ bool wo_is_anc(const WOct &a, const WOct &b, unsigned D) {
  if (!(a.lev < b.lev)) return false;
  uint64_t la = 1ull << (D - a.lev), lb = 1ull << (D - b.lev);
  return b.x >= a.x && b.y >= a.y && b.z >= a.z && (uint64_t)b.x + lb <= (uint64_t)a.x + la &&
         (uint64_t)b.y + lb <= (uint64_t)a.y + la && (uint64_t)b.z + lb <= (uint64_t)a.z + la;
}
__host__ __device__ __forceinline__ WOct wo_next(WOct m, unsigned D) {
  uint32_t mask = 1u << (D - m.lev);
  int i;
  for (i = (int)m.lev; i >= 0; --i) {
    m.x ^= mask;
    if (m.x & mask) break;
    m.y ^= mask;
    if (m.y & mask) break;
    m.z ^= mask;
    if (m.z & mask) break;
    mask <<= 1;
  }
  m.lev = (uint32_t)i;
  return m;
}
__host__ __device__ __forceinline__ WOct wo_dld(const WOct &a, unsigned D) {
  uint32_t l = 1u << (D - a.lev);
  return WOct{a.x + l - 1, a.y + l - 1, a.z + l - 1, D};
}

// The walk's getNext climbs above the root when it runs past the last
// octant; at level "-1" getNext no longer moves and the reference loops
// forever (repeated points at a coarse maxDepth reach that state).  The walk
// below stops there, and also after a step bound no terminating walk reaches.
constexpr size_t P2O_WALK_NO_END = ~(size_t)0;
// count reported for a batched cloud whose walk leaves the cloud's domain
constexpr size_t P2O_WALK_OUTSIDE = ~(size_t)0 - 1;

// Runs the walk over the n sorted level-D point keys of one cloud; writes the
// octants (with the cloud's segment key `seg` or-ed in) to out when not null
// and returns their count, or P2O_WALK_NO_END.
__host__ __device__ inline size_t p2o_walk(const Key128 *pk, size_t n, unsigned m, unsigned D, Key128 *out,
                                           Key128 seg = Key128{0, 0}, bool *outside = nullptr) {
  const uint32_t num_pts = (uint32_t)n;
  WOct curr{0, 0, 0, 0};
  WOct last = wo_dld(curr, D);
  WOct next = wo_next(curr, D);
  uint32_t curr_pt = 0, next_pt = curr_pt + m;
  size_t w = 0;
  u128 prev_key = ~(u128)0;
  auto push = [&](const WOct &o) {
    u128 k = wo_key(o);
    if (k == prev_key) return;  // std::list::unique
    prev_key = k;
    if (outside && (o.x >> D || o.y >> D || o.z >> D)) *outside = true;
    if (out) out[w] = make_tagged(key_or(morton3(o.x, o.y, o.z), seg), o.lev);
    w++;
  };
  const uint64_t max_steps = 64ull * ((uint64_t)n + 1) * (D + 2);
  uint64_t steps = 0;
  while (next_pt < num_pts) {
    if (curr.lev > D || ++steps > max_steps) return P2O_WALK_NO_END;
    for (;;) {
      WOct a = wo_from_key(pk[next_pt - 1], D), b = wo_from_key(pk[next_pt], D);
      if (!(wo_is_anc(curr, a, D) && wo_is_anc(curr, b, D) && curr.lev < D)) break;
      curr.lev++;
      next = wo_next(curr, D);
    }
    uint32_t inc = m;
    while (curr.lev == D - 1) {
      inc <<= 1;
      next_pt += inc;
      if (next_pt > num_pts) {
        next_pt = num_pts - 1;
        break;
      }
    }
    // lower_bound(pts[curr_pt..next_pt), next, less_equal)
    u128 nk = wo_key(next);
    uint32_t lo = curr_pt, hi = next_pt;
    while (lo < hi) {
      uint32_t mid = lo + (hi - lo) / 2;
      if (wo_key(wo_from_key(pk[mid], D)) <= nk) lo = mid + 1;
      else hi = mid;
    }
    int found_pt = (int)(lo - curr_pt);
    next_pt = curr_pt + (uint32_t)found_pt;
    push(curr);
    curr = next;
    next = wo_next(curr, D);
    if (next_pt > curr_pt) curr_pt = next_pt;
    next_pt = curr_pt + m;
  }
  u128 lastk = wo_key(last);
  while (wo_key(curr) <= lastk) {
    if (curr.lev > D || ++steps > max_steps) return P2O_WALK_NO_END;
    while (wo_key(wo_dld(curr, D)) > lastk && curr.lev < D) curr.lev++;
    push(curr);
    if (wo_key(wo_dld(curr, D)) == lastk) break;
    curr = wo_next(curr, D);
  }
  return w;
}


}  // namespace dg
