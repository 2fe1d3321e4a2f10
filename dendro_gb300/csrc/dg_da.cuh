// Octree mesh (the reference's ot::DA at one rank) and the element-loop
// operators that run on it.
#pragma once

#include "dg_octree.cuh"

namespace dg {

// Element e of the mesh is octant e of the balanced octree.  Storage (SoA,
// coalesced by element):
//   meta[e]    = level | child << 8 | hanging mask << 16 | element type << 24
//   conn[k][e] = node id of vertex k (k = x + 2y + 4z); a hanging vertex k
//                refers to vertex k of the element's parent
// Nodes are the mesh vertices that are not hanging, coordinates in
// [0, 2^D]^3.  Node ids follow element order: the non-hanging anchor of
// every element, then its vertices on the positive domain boundary.
struct Mesh {
  unsigned max_depth = 0;
  size_t n_elem = 0;
  size_t n_node = 0;
  uint32_t *meta = nullptr;
  uint32_t *conn = nullptr;      // 8 * n_elem, vertex-major
  uint32_t *node_xyz = nullptr;  // 3 * n_node, coordinate-major
  // element loop tables (dg_elem.cuh): n_patch patches of PATCH elements
  size_t n_patch = 0;
  uint16_t *pinc = nullptr;   // PATCH_ENT per patch, node-sorted pairs
  uint16_t *pexc = nullptr;   // PATCH per patch: runs starting before pair 8t
  uint32_t *pmeta = nullptr;  // PATCH per patch: meta in the patch's element order,
                              // bits 16..23 = the element's stencil key index
  uint16_t *pkeys = nullptr;  // PKEY_MAX per patch: (type << 5 | level) of each key
  uint16_t *pkcount = nullptr;  // keys per patch (> PKEY_MAX: per-element L, M path)
  uint32_t *pnode = nullptr;  // node of each run, patch after patch
  uint64_t *poff = nullptr;   // n_patch + 1 run offsets into pnode
  // pperm maps a patch's (type, level) order back to its element order
  uint16_t *pperm = nullptr;  // PATCH per patch
  // run form of the FP32 element loop (dg_elem.cuh, k_patch_matvec_runs):
  // per (type, level) position the 8 patch-local run indices of its
  // vertices in the canonical stencil order (8 x 16 bits), and per run its
  // node with bit 31 set when the run holds all the node's pairs
  uint4 *plid = nullptr;      // PATCH per patch
  uint32_t *prun = nullptr;   // one per run, at poff
  // compressed mode (the reference's compressLut): conn is released once the
  // patch tables exist and decoded from them on demand (mesh_conn)
  bool compressed = false;
};

void mesh_build(Context &ctx, const Octree &bal, Mesh &m, bool compress = false);
// the 8 x n_elem vertex-major node ids: m.conn, or decoded from the patch
// tables into tmp when the mesh is compressed
const uint32_t *mesh_conn(Context &ctx, const Mesh &m, DBuf<uint32_t> &tmp);
// device bytes the mesh holds
size_t mesh_bytes(const Mesh &m);
void mesh_free(Context &ctx, Mesh &m);

// y = (lapFac * Laplacian + massFac * mass) x over all elements
// (examples/src/backend/odaJac.C:294-377, block :275-292)
template <typename T>
void mesh_matvec(Context &ctx, const Mesh &m, const T *x, T *y, double lap_fac, double mass_fac);
// the same with per-element factors: coef[2e] scales element e's Laplacian,
// coef[2e + 1] its mass (Jacobian2MatMult, examples/src/backend/omgJac.C:1666-1735)
template <typename T>
void mesh_matvec_coef(Context &ctx, const Mesh &m, const double *coef, const T *x, T *y);
// diagonal of lap_fac K + mass_fac M, or with coef the per-element form
// (Jacobian1MatGetDiagonal odaJac.C:160-222, Jacobian2MatGetDiagonal omgJac.C:1641)
void mesh_diagonal(Context &ctx, const Mesh &m, const double *coef, double lap_fac, double mass_fac, double *diag);

// index of the leaf whose anchor is the largest anchor <= pos in a sorted
// tagged-key array (0 when pos precedes every leaf; callers verify)
__device__ __forceinline__ size_t find_leaf(const Key128 *__restrict__ keys, size_t n, Key128 pos) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    size_t mid = lo + (hi - lo) / 2;
    if (key_le(tag_anchor(keys[mid]), pos)) lo = mid + 1;
    else hi = mid;
  }
  return lo ? lo - 1 : 0;
}

// the same index as find_leaf, searched outward from `hint` (doubling steps,
// then bisection): a leaf near the hint in Morton order costs a few nearby
// probes instead of a bisection of the whole array
__device__ __forceinline__ size_t find_leaf_from(const Key128 *__restrict__ keys, size_t n, Key128 pos, size_t hint) {
  size_t lo, hi;  // keys[lo] <= pos < keys[hi] (hi == n: past the end)
  if (key_le(tag_anchor(keys[hint]), pos)) {
    lo = hint;
    hi = n;
    for (size_t step = 1; hint + step < n; step <<= 1) {
      if (key_le(tag_anchor(keys[hint + step]), pos)) {
        lo = hint + step;
      } else {
        hi = hint + step;
        break;
      }
    }
  } else {
    hi = hint;
    lo = n;  // none found yet
    for (size_t step = 1; step <= hint; step <<= 1) {
      if (key_le(tag_anchor(keys[hint - step]), pos)) {
        lo = hint - step;
        break;
      }
      hi = hint - step;
    }
    if (lo == n) {
      if (!key_le(tag_anchor(keys[0]), pos)) return 0;  // pos precedes every leaf
      lo = 0;
    }
  }
  while (hi - lo > 1) {
    const size_t mid = lo + (hi - lo) / 2;
    if (key_le(tag_anchor(keys[mid]), pos)) lo = mid;
    else hi = mid;
  }
  return lo;
}

// device stencil layout: for each (child, type) a 128-entry block, 64
// Laplacian then 64 mass entries, row-major 8x8
constexpr int STEN_ENTRIES = 8 * 18 * 128;

// stencil tables on the device, generated on first use
void ensure_stencils(Context &ctx);
// the combined-stencil table of the element loop for these factors
// (rebuilt on ctx's stream when they differ from the last call's)
template <typename T>
const T *comb_table(Context &ctx, double lap_fac, double mass_fac);

// the double-single run-form loop (FP64 vectors, FP32-pair arithmetic; x
// scaled by 2^scale_exp inside, the result by 2^-scale_exp)
template <bool DIR>
void launch_matvec_runs_ds(Context &ctx, const Mesh &m, const double *x, double *y, double lap_fac,
                           double mass_fac, int scale_exp, const char *name, double bytes);
// the run-form element loop on a mesh with run tables (m.plid)
template <typename T, bool DIR>
void launch_matvec_runs(Context &ctx, const Mesh &m, const T *x, T *y, double lap_fac,
                        double mass_fac, const char *name, double bytes);

// host-side generators (same mathematics as the reference's .inp tables)
void gen_etype_masks(uint8_t masks[8 * 18]);
void gen_stencils(double *lap, double *mass);

}  // namespace dg
