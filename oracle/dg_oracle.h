/*
 * dg_oracle — CPU restatement of the reference (Dendro4) octree hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the parity tests,
 * smoke() and the CPU-baseline leg of bench.py compare the CUDA library
 * against.  The shipped library never links, loads or calls it.
 *
 * Octants are {x, y, z, level} at a given maxDepth D (anchor coordinates in
 * [0, 2^D), level 0 = root).  Arrays of octants are always sorted in the
 * reference's Morton order: by the bit-interleaved anchor (z above y above x
 * at every bit), ties broken by level, ancestor first
 * (include/TreeNode.tcc:122-237, Morton branch :211-236).
 *
 * Every function returns 0 on success and a negative DGO_E* code otherwise.
 * Output arrays are malloc'd by the callee and released with dgo_free().
 */
#ifndef DG_ORACLE_H
#define DG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGO_OK 0
#define DGO_EINVAL (-1)
#define DGO_ENOMEM (-2)
#define DGO_EINTERNAL (-3)
#define DGO_ENOTERM (-4) /* the reference's walk would never terminate */

typedef struct {
  uint32_t x, y, z, lev;
} dgo_oct;

void dgo_free(void *p);

/* Quantize FP64 points to level-D anchors exactly as points2OctreeSeq does
 * (src/construct.cpp:930-942): (unsigned)(x * 2^D / gLen), then sort them in
 * Morton order (construct.cpp:955, omp_par::merge_sort).  Duplicates kept. */
int dgo_quantize_sort(const double *xyz, size_t n, const double gLens[3], unsigned maxDepth, dgo_oct **out);

/* ot::points2Octree at one rank (src/construct.cpp:759-770 -> 911-970),
 * including the p2oLocal walk (construct.cpp:976-1076) with all its
 * data-dependent behaviour. */
int dgo_points_to_octree(const double *xyz, size_t n, const double gLens[3], unsigned maxDepth, unsigned maxPts,
                         dgo_oct **out, size_t *nout);

/* p2oLocal from the root over already-sorted level-D points. */
int dgo_p2o_local(const dgo_oct *pts, size_t n, unsigned maxDepth, unsigned maxPts, dgo_oct **out, size_t *nout);

/* ot::balanceOctree(incCorner=1) at one rank (src/balance.cpp:31-63): the
 * coarsest 2:1 (faces, edges and corners) balanced refinement of a sorted,
 * linear, complete octree.  That octree is unique; this restatement computes
 * it as the closure "every neighbour of the parent of a node is a node"
 * rather than by the reference's block + ripple procedure
 * (balance.cpp:801-1338, TreeNode.cpp:884-1342). */
int dgo_balance(const dgo_oct *in, size_t n, unsigned maxDepth, dgo_oct **out, size_t *nout);
/* incCorner = 0: balanced across faces and edges only */
int dgo_balance_ex(const dgo_oct *in, size_t n, unsigned maxDepth, int incCorner, dgo_oct **out, size_t *nout);

/* ot::coarsenOctree, sequential form (src/coarsen.cpp:53): every complete
 * family of 8 sibling leaves of a sorted, linear, complete octree is
 * replaced by its parent. */
int dgo_coarsen(const dgo_oct *in, size_t n, unsigned maxDepth, dgo_oct **out, size_t *nout);

/* Checkers mirroring src/test/testUtils.C:18 (isLinear), :28 (isComplete)
 * and :82 (isBalanced with corners, maxLevDiff 1).  Return 1 / 0. */
/* completeOctree (src/construct.cpp:518) at one rank, input in any order
 * unless declared sorted / unique. */
int dgo_complete(const dgo_oct *in, size_t n, unsigned maxDepth, int isUnique, int isSorted, dgo_oct **out,
                 size_t *nout);

/* the octants in the order of the reference's Hilbert build
 * (TreeNode::operator<, include/TreeNode.tcc:130-210), in place; and the
 * number of curve states the generated tables hold (24) */
int dgo_hilbert_sort(dgo_oct *a, size_t n, unsigned maxDepth);
int dgo_hilbert_states(void);

int dgo_is_sorted_unique(const dgo_oct *a, size_t n, unsigned maxDepth);
int dgo_is_linear(const dgo_oct *a, size_t n, unsigned maxDepth);
int dgo_is_complete(const dgo_oct *a, size_t n, unsigned maxDepth);
int dgo_is_balanced(const dgo_oct *a, size_t n, unsigned maxDepth);
int dgo_is_balanced_ex(const dgo_oct *a, size_t n, unsigned maxDepth, int incCorner);

/* Element-type tables (include/oda/cnumEtypes.h, include/oda/odaUtils.tcc:14):
 * masks[c*18 + t] is the 8-bit hanging-vertex mask of element type t for
 * Morton child number c. */
void dgo_etype_masks(uint8_t masks[8 * 18]);

/* Type-2 Laplacian and mass stencils on the reference element [-1,1]^3,
 * indexed [c][t][k][j] (8*18*8*8 doubles each), the tables the reference
 * reads from Stencils/LapType2Stencils.inp and MassType2Stencils.inp
 * (examples/src/backend/handleType2Stencils.C:519,754).  Restated from the
 * mathematics: S = P^T K P with K the trilinear element matrix and P the
 * hanging-vertex interpolation of element type t. */
void dgo_stencils(double *lap, double *mass);

/* DA built from a balanced octree (src/oda/oda.cpp:250 at one rank).
 * Elements are the input octants in order.  Per element: child number,
 * hanging-vertex mask (bit k: vertex k lies inside a face or edge of a
 * coarser neighbour), element type, and 8 node ids; a hanging vertex k is
 * replaced by vertex k of the parent (odaJac.C:352-355).  Nodes are the
 * non-hanging vertices, numbered in Morton order of their coordinates;
 * node coordinates are in [0, 2^D]. */
typedef struct {
  size_t n_elem;
  size_t n_node;
  uint8_t *child;   /* n_elem */
  uint8_t *hmask;   /* n_elem */
  uint8_t *etype;   /* n_elem */
  uint8_t *level;   /* n_elem */
  uint32_t *nodes;  /* 8 * n_elem, element-major */
  uint32_t *node_xyz; /* 3 * n_node */
} dgo_da;

int dgo_da_build(const dgo_oct *bal, size_t n, unsigned maxDepth, dgo_da *da);
void dgo_da_free(dgo_da *da);

/* One Laplacian + mass element loop in FP64 (examples/src/backend/odaJac.C:
 * 275-292, 294-377): out[id[k]] += sum_j (lapFac*h/2*L[c][t][k][j] +
 * massFac*h^3/8*M[c][t][k][j]) * in[id[j]], with h the element's side in the
 * unit cube.  out is overwritten (zeroed first). */
int dgo_matvec(const dgo_da *da, unsigned maxDepth, const double *in, double *out, double lapFac, double massFac);

/* Multigrid building blocks.  Boundary nodes are the nodes on the boundary
 * of the unit cube (assignBoundaryFlags, src/oda/odaUtils.cpp:2464).
 * dgo_dirichlet_matvec: DirichletJacobianMatMult (examples/src/backend/
 * omgJac.C:958-1057); dgo_dirichlet_diag: its diagonal; dgo_prolong_map: 8
 * (coarse node, weight) pairs per fine node, the transpose of
 * restrictMatVecType1 (src/omg/restrictMatVec.cpp:74-146). */
int dgo_dirichlet_matvec(const dgo_da *da, unsigned maxDepth, const double *in, double *out);
int dgo_dirichlet_diag(const dgo_da *da, unsigned maxDepth, double *diag);
int dgo_prolong_map(const dgo_da *fine, const dgo_oct *coarse_oct, size_t nc, const dgo_da *coarse, unsigned maxDepth,
                    uint32_t *ids, double *w);

/* Restriction stencil tables (Stencils/RmatType1Stencils.inp, 8*8*18*64
 * doubles; RmatType2Stencils.inp, 8*18*64 doubles), from the mathematics. */
void dgo_rmat_tables(double *r1, double *r2);

/* FNV-1a over the {x,y,z,lev} records (u32 little-endian). */
uint64_t dgo_fnv1a(const dgo_oct *a, size_t n);

#ifdef __cplusplus
}
#endif
#endif
