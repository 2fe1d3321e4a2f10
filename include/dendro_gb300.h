/*
 * dendro_gb300 — C ABI of the GB300 octree hot path.
 *
 * One library, one GPU, no inter-GPU communication.  Each entry point
 * replaces one function of the reference (Dendro4) C++ API at one MPI rank;
 * the reference function is cited beside it (paths inside the Dendro4
 * source tree).  Plain pointers and sizes only.
 *
 * Conventions
 *   - Every function returns int: DG_OK (0) on success, a DG_ERR_* code
 *     otherwise; dg_ctx_last_error() returns the message of the last failure
 *     on that context.  (The reference returns 1 from ot::/par:: functions
 *     and asserts on errors; the C++ mirror in include/dendro_gb300.hpp maps
 *     back to that convention.)
 *   - Pointer arguments flagged `*_on_device` are CUDA device pointers when
 *     the flag is nonzero, host pointers otherwise.  Host pointers may be
 *     pageable or pinned; pinned memory gives the full link bandwidth.
 *   - Octants are exchanged as 4 x uint32 records {x, y, z, level} (the
 *     anchor and level fields of ot::TreeNode, include/TreeNode.h:42) in the
 *     reference's Morton order.
 *   - A context owns a CUDA stream; calls on one context are serialised on
 *     it and return once their results are complete.  Handles (octrees,
 *     meshes) keep their data resident in device memory until freed.
 *   - The reference's MPI_Comm parameters are represented by `comm_size`
 *     where an entry point takes one: only 1 is accepted (DG_ERR_COMM_SIZE
 *     otherwise).
 */
#ifndef DENDRO_GB300_H
#define DENDRO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DG_OK 0
#define DG_ERR_INVALID_ARG 1
#define DG_ERR_OUT_OF_MEMORY 2
#define DG_ERR_CUDA 3
#define DG_ERR_DOMAIN 4       /* a point outside [0, gLen)^3, or NaN */
#define DG_ERR_NOT_BALANCED 5 /* mesh input is not a complete 2:1 balanced octree */
#define DG_ERR_TIMEOUT 6
#define DG_ERR_INTERNAL 7
#define DG_ERR_COMM_SIZE 8
#define DG_ERR_UNSUPPORTED 9
#define DG_ERR_CAPACITY 10 /* input larger than a fixed-capacity entry point accepts */

typedef struct dg_ctx_s *dg_ctx;
typedef struct dg_octree_s *dg_octree;
typedef struct dg_da_s *dg_da;
typedef struct dg_mg_s *dg_mg;
typedef struct dg_csr_s *dg_csr;

/* ---- context ------------------------------------------------------------
 * Replaces the per-rank global state the reference sets up in
 * _InitializeHcurve (src/hcurvedata.cpp:23) and ot::DA_Initialize
 * (src/oda/odaUtils.cpp:3352): here the SFC is always Morton and the
 * stencil tables are generated on the device on first use. */
int dg_ctx_create(int device, dg_ctx *out);
int dg_ctx_destroy(dg_ctx ctx);
/* Run subsequent calls on an external cudaStream_t (NULL: the context's own). */
int dg_ctx_set_stream(dg_ctx ctx, void *cuda_stream);
const char *dg_ctx_last_error(dg_ctx ctx);
/* Choices the context's autotuner made so far, one line each (the radix
 * sort's tile: each size class's first sort times both tiles on its first
 * digit pass and keeps the faster).  No counterpart in the reference. */
const char *dg_ctx_autotune_log(dg_ctx ctx);
/* Order of octant records at the boundary: DG_ORDER_MORTON (default, the
 * reference built without HILBERT_ORDERING) or DG_ORDER_HILBERT (the
 * reference's default build, CMakeLists.txt:48; TreeNode::operator<
 * include/TreeNode.tcc:130-210 with the tables of src/hcurvedata.cpp).
 * Records leave the library (octree downloads, sortUniquePoints, MG level
 * octrees, octree files) in this order and octant records given to it
 * (octree uploads, completeOctree, octree files) are read in any order and
 * sorted.  The same octrees result in both orders; only the records' order
 * differs.  dg_sort_unique_points_noalloc has no context and stays Morton. */
#define DG_ORDER_MORTON 0
#define DG_ORDER_HILBERT 1
int dg_ctx_set_order(dg_ctx ctx, int order);
int dg_ctx_get_order(dg_ctx ctx, int *order);
const char *dg_status_string(int status);
int dg_version(void);

/* Form of the element loop (dg_matvec, dg_mg_matvec, the V-cycle and the
 * CG operator, FP32 and FP64): DG_MATVEC_RUNS (the default) sums each
 * element's results into patch-local node slots, DG_MATVEC_PAIRS sums them
 * through per-pair slots and a segmented scan.  Both give the same operator
 * (to the rounding of the precision); a compressed DA and the
 * per-element-factor loop always use the pair form.  No counterpart in the
 * reference. */
#define DG_MATVEC_RUNS 0
#define DG_MATVEC_PAIRS 1
int dg_ctx_set_matvec_form(dg_ctx ctx, int form);

/* ---- ot::points2Octree ---------------------------------------------------
 * include/octUtils.h:633 / src/construct.cpp:759 (1-rank branch :767-770 ->
 * points2OctreeSeq :911).  xyz holds n points, x y z interleaved (FP64).
 * Unlike the reference, xyz is not cleared.  A point whose quantised
 * coordinate falls outside [0, 2^maxDepth) is rejected (DG_ERR_DOMAIN); the
 * reference would produce an octant outside the domain. */
int dg_points_to_octree(dg_ctx ctx, const double *xyz, size_t n, const double gLens[3], unsigned maxDepth,
                        unsigned maxNumPtsPerOctant, int comm_size, int xyz_on_device, dg_octree *out);

/* ---- batches of clouds ------------------------------------------------------
 * points2Octree for nseg independent clouds in one pass: cloud s holds the
 * points [seg_start[s], seg_start[s+1]) of xyz (seg_start: host array of
 * nseg + 1 offsets, seg_start[0] = 0, seg_start[nseg] = n).  The resulting
 * handle holds the nseg octrees back to back, each identical to what
 * dg_points_to_octree returns for that cloud alone; dg_balance_octree on it
 * balances every cloud independently.  dg_octree_segments reports where each
 * cloud's octants start.  No counterpart in the reference (one cloud per
 * call, construct.cpp:759). */
int dg_points_to_octree_batch(dg_ctx ctx, const double *xyz, size_t n, const uint64_t *seg_start, size_t nseg,
                              const double gLens[3], unsigned maxDepth, unsigned maxNumPtsPerOctant,
                              int xyz_on_device, dg_octree *out);
/* offsets: host array of nseg + 1 entries (may be NULL to query nseg) */
int dg_octree_segments(dg_ctx ctx, dg_octree o, size_t *nseg, uint64_t *offsets);
/* cloud `seg` of a batch as its own octree handle (device copy) */
int dg_octree_extract(dg_ctx ctx, dg_octree o, size_t seg, dg_octree *out);

/* ---- par::sampleSort + par::removeDuplicates of point octants -------------
 * include/parUtils.h:424,437 (1-rank branch parUtils.tcc:1868-1875): the
 * points quantised to level maxDepth, sorted in Morton order, duplicates
 * removed.  Writes up to n records {x, y, z, maxDepth} to out_xyzl and the
 * count to *n_unique. */
int dg_sort_unique_points(dg_ctx ctx, const double *xyz, size_t n, const double gLens[3], unsigned maxDepth,
                          int xyz_on_device, uint32_t *out_xyzl, int out_on_device, size_t *n_unique);

/* ---- sort + unique of points, allocating nothing --------------------------
 * No counterpart in the reference.  dg_sort_unique_points for callers that
 * must not allocate device memory during the call: a process whose device
 * memory is wholly reserved by another allocator (a framework's caching
 * allocator, or a fixed pool sized at start-up), and steady-state loops that
 * may not call cudaMalloc / cudaFree because those can synchronise the whole
 * device.  Same inputs, same results bit for bit.  Differences:
 *   - xyz and out_xyzl are device (or managed) memory of the current device,
 *     xyz 8-byte and out_xyzl 16-byte aligned (DG_ERR_INVALID_ARG otherwise,
 *     checked before any work);
 *   - n <= DG_NOALLOC_MAX_POINTS, else DG_ERR_CAPACITY before any work;
 *   - records are in Morton order whatever order other calls use (it has
 *     no context);
 *   - all scratch (about 41 MB) is one static device array of the library,
 *     reserved on a device when the runtime loads the library's device code
 *     there (its first kernel launch on that device under lazy module
 *     loading, the default; context creation under
 *     CUDA_MODULE_LOADING=EAGER); the first call on each device looks up its
 *     address (cudaGetSymbolAddress with that device current; a failed
 *     look-up is retried by the next call): make that first call before any
 *     stream capture begins;
 *   - the work runs on cuda_stream (a cudaStream_t of the current device;
 *     NULL: the legacy default stream), which the call synchronises before
 *     it returns;
 *   - the scratch is shared by every call on one device: calls that overlap
 *     in time there (two host threads, or two streams) race, and the caller
 *     must serialise them. */
#define DG_NOALLOC_MAX_POINTS ((size_t)1 << 20)
int dg_sort_unique_points_noalloc(const double *xyz, size_t n, const double gLens[3], unsigned maxDepth,
                                  uint32_t *out_xyzl, size_t *n_unique, void *cuda_stream);

/* ---- ot::balanceOctree ------------------------------------------------------
 * include/octUtils.h:692 / src/balance.cpp:31 (1-rank branch :54-63): the
 * coarsest refinement that is 2:1 balanced across faces, edges and corners
 * (incCorner != 0) or across faces and edges only (incCorner = 0, the 18
 * directions of TreeNode::addBalancingDescendants, src/TreeNode.cpp:138).
 * The input must be sorted, linear and complete (the reference's
 * assumption).  The input handle is left intact (the reference clears
 * `in`). */
int dg_balance_octree(dg_ctx ctx, dg_octree in, int incCorner, int comm_size, dg_octree *out);

/* ---- ot::coarsenOctree -----------------------------------------------------
 * include/octUtils.h:825 / src/coarsen.cpp:53 (sequential form): every
 * complete family of 8 sibling leaves of a sorted, linear, complete octree is
 * replaced by its parent.  One cloud per call. */
int dg_coarsen_octree(dg_ctx ctx, dg_octree in, dg_octree *out);

/* ---- par::sampleSort / par::removeDuplicates of octants ---------------------
 * include/parUtils.h:424,437 (at one rank a local sort, src/parUtils.tcc:
 * 1868-1875): the n octant records xyzl ({x, y, z, level} at maxDepth) in
 * the octant order of the context (Morton unless dg_ctx_set_order chose
 * Hilbert; an ancestor before its descendants), repeated records removed
 * when removeDuplicates is set.  out_xyzl holds n records; *n_out is the
 * count written.  Records outside the domain or not aligned to their level:
 * DG_ERR_DOMAIN. */
int dg_sort_octants(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, int removeDuplicates,
                    int src_on_device, uint32_t *out_xyzl, int dst_on_device, size_t *n_out);

/* ---- SFC::parSort::SFC_treeSort --------------------------------------------
 * include/sfcSort.h:1378 (one rank: SFC::seqSort::SFC_treeSort :418), the
 * tree sort the reference's DA factory and completeOctree call
 * (src/oda/private/odaFactory.cpp:186, src/construct.cpp:541,553): the n
 * octant records xyzl sorted in the context's octant order.  options
 * DG_TS_SORT_ONLY: all n records, sorted (the reference sorts pNodes in
 * place); DG_TS_REMOVE_DUPLICATES: sorted, repeated octants removed and every
 * octant that has a descendant in the input removed (the reference's
 * pOutSorted, sfcSort.h:532-575).  *n_out is the count written to out_xyzl
 * (room for n records).  DG_TS_CONSTRUCT_OCTREE / DG_TS_BALANCE_OCTREE give
 * DG_ERR_UNSUPPORTED: completeOctree and balanceOctree are
 * dg_complete_octree and dg_balance_octree.  Differences: one input record
 * with DG_TS_REMOVE_DUPLICATES gives that record (the reference leaves
 * pOutSorted unchanged below two records, sfcSort.h:532). */
#define DG_TS_SORT_ONLY 0u
#define DG_TS_REMOVE_DUPLICATES 1u
#define DG_TS_CONSTRUCT_OCTREE 2u
#define DG_TS_BALANCE_OCTREE 4u
int dg_tree_sort(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, unsigned options, int src_on_device,
                 uint32_t *out_xyzl, int dst_on_device, size_t *n_out);

/* ---- ot::completeOctree ----------------------------------------------------
 * include/octUtils.h:813 / src/construct.cpp:518 at one rank: the n octants
 * xyzl ({x, y, z, level} records at maxDepth, host or device memory) are
 * sorted and made unique when isUnique is 0 (duplicates and every octant
 * that has a descendant in the input are dropped, include/sfcSort.h:532-575),
 * sorted when isUnique is 1 and isSorted is 0, and the gaps are filled with
 * the coarsest octants (appendCompleteRegion, construct.cpp:1077), giving a
 * sorted, linear, complete octree.  n = 0 gives an empty octree.  Records
 * outside the domain or not aligned to their level: DG_ERR_DOMAIN.  Input
 * that breaks its declared order (isSorted = 1 but not sorted, isUnique = 1
 * with repeated octants): DG_ERR_INVALID_ARG, where the reference returns an
 * unspecified list. */
int dg_complete_octree(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, int isUnique, int isSorted,
                       int src_on_device, dg_octree *out);

/* ---- octree handles --------------------------------------------------------
 * Materialise / import the std::vector<ot::TreeNode> of the reference as
 * {x, y, z, level} records. */
int dg_octree_size(dg_octree o, size_t *n, unsigned *maxDepth);
/* DA handles accept single-cloud octrees only (DG_ERR_UNSUPPORTED otherwise). */
int dg_octree_download(dg_ctx ctx, dg_octree o, uint32_t *xyzl, int dst_on_device);
int dg_octree_upload(dg_ctx ctx, const uint32_t *xyzl, size_t n, unsigned maxDepth, int src_on_device, dg_octree *out);
int dg_octree_free(dg_ctx ctx, dg_octree o);

/* ---- point and octree files ------------------------------------------------
 * The reference's formats (src/octFunctions.cpp).  Point files
 * (readPtsFromFile :319, writePtsToFile :380): a uint32 count, then x y z per
 * point in FP64; no points -> an empty file.  Octree text files
 * (readNodesFromFile :452, writeNodesToFile :496): "3 maxDepth", the count,
 * then "x y z level" per octant, one per line, byte for byte as the reference
 * writes them.  Binary octree files (readNodesFromFile_binary :435,
 * writeNodesToFile_binary :482): 28-byte records x y z level weight dim
 * maxDepth.  Differences: the binary reader returns the file's records (the
 * reference's repeats the last one), malformed files get DG_ERR_INVALID_ARG
 * instead of undefined values, and writers take one cloud per octree.  Device
 * buffers and octree handles are filled through pinned staging buffers;
 * octree text is formatted and parsed on the GPU.  The order of the file's
 * octants is kept. */
int dg_pts_file_count(const char *path, size_t *n);
int dg_pts_file_read(dg_ctx ctx, const char *path, double *xyz, size_t capacity, int dst_on_device, size_t *n);
int dg_pts_file_write(dg_ctx ctx, const char *path, const double *xyz, size_t n, int src_on_device);
int dg_octree_write_text(dg_ctx ctx, dg_octree o, const char *path);
int dg_octree_read_text(dg_ctx ctx, const char *path, dg_octree *out);
int dg_octree_write_binary(dg_ctx ctx, dg_octree o, const char *path);
int dg_octree_read_binary(dg_ctx ctx, const char *path, dg_octree *out);

/* ---- ot::DA ----------------------------------------------------------------
 * include/oda/oda.h:622 / src/oda/oda.cpp:250 at one rank: element -> node
 * map with hanging vertices resolved to the parent's vertex
 * (getNodeIndices, include/oda/oda.tcc:1304), child numbers
 * (getChildNumber, oda.tcc:1273), hanging masks (getHangingNodeIndex,
 * src/oda/oda.cpp:1038) and element types (GET_ETYPE_BLOCK,
 * include/oda/odaUtils.h:379).  Node numbering differs from the
 * reference's buffer layout; nodes are identified by coordinates
 * (dg_da_download node_xyz). */
int dg_da_build(dg_ctx ctx, dg_octree balanced, dg_da *out);
/* ot::DA with compressLut (include/oda/oda.h:622, decoded by
 * getNodeIndices, include/oda/oda.tcc:1304-1420): compressLut = 1 keeps only
 * the element loop's per-patch tables (16-bit slots per element vertex and
 * one node id per node run) and releases the plain 8 x u32 node list; the
 * node list is decoded from the tables when a call needs it
 * (dg_da_download, dg_da_assemble).  Results are identical in both modes.
 * dg_da_memory: device bytes the DA holds. */
int dg_da_build_ex(dg_ctx ctx, dg_octree balanced, int compressLut, dg_da *out);
int dg_da_memory(dg_da da, size_t *bytes);
int dg_da_sizes(dg_da da, size_t *n_elem, size_t *n_node);
/* Any output pointer may be NULL.  meta[e] = level | child<<8 | hmask<<16 |
 * etype<<24; nodes is 8*n_elem, element-major (nodes[8e+k]); node_xyz is
 * 3*n_node, point-major (x y z per node), coordinates at the octree's
 * maxDepth scale, vertices in [0, 2^maxDepth]. */
int dg_da_download(dg_ctx ctx, dg_da da, uint32_t *meta, uint32_t *nodes, uint32_t *node_xyz, int dst_on_device);
int dg_da_free(dg_ctx ctx, dg_da da);

/* ---- Jacobian1MatMult ------------------------------------------------------
 * examples/src/backend/odaJac.C:294-377 (element block :275-292, the
 * PETSc MatShell MATOP_MULT callback of examples/include/odaJac.h:35):
 * out = (lapFac * Laplacian + massFac * mass) in, nodal vectors of n_node
 * entries in dg_da node order.  precision 64: FP64 in/out (double*);
 * precision 32: FP32 in/out (float*).  lapFac and massFac play the role of
 * the -lapMatPropFac / -massMatPropFac options (odaJac.C:302-306). */
int dg_matvec(dg_ctx ctx, dg_da da, const void *in, void *out, int precision, double lapFac, double massFac,
              int on_device);
/* Per-element factors: coef holds 2 FP64 values per element (element i =
 * octant i of the balanced octree): coef[2i] scales its Laplacian and
 * coef[2i + 1] its mass; the operator of Jacobian2MatMult
 * (examples/src/backend/omgJac.C:1666-1735, its matProp vector). coef and
 * the vectors are all host or all device memory (on_device). */
int dg_matvec_coef(dg_ctx ctx, dg_da da, const double *coef, const void *in, void *out, int precision, int on_device);
/* Diagonals (FP64): dg_da_diagonal of lapFac K + massFac M, or of the
 * per-element form when coef is given (Jacobian1MatGetDiagonal
 * odaJac.C:160-222, Jacobian2MatGetDiagonal omgJac.C:1641); dg_mg_diagonal of
 * a level's Dirichlet operator, 1 on boundary nodes
 * (DirichletJacobianMatGetDiagonal omgJac.C:1111). */
int dg_da_diagonal(dg_ctx ctx, dg_da da, const double *coef, double lapFac, double massFac, double *diag,
                   int on_device);
int dg_mg_diagonal(dg_ctx ctx, dg_mg mg, size_t level, double *diag, int on_device);

/* ---- geometric multigrid (omg) ---------------------------------------------
 * The reference's DAMG hierarchy and solve for -lap(u) + u = f, u = 0 on the
 * boundary of the unit cube (src/omg/blockDiag.cpp:1312 DAMGCreateAndSetDA,
 * :1122 DAMGSolve; operators examples/src/backend/omgJac.C:958
 * DirichletJacobianMatMult; transfers src/omg/restrictMatVec.cpp,
 * prolongMatVec.cpp; solver options bin/options:48-206).  Levels are made by
 * coarsenOctree + balanceOctree until a level holds at most
 * max_coarse_elems elements; the coarsest level is solved with a dense
 * inverse.  Level 0 is the input octree; its node numbering equals
 * dg_da_build's on the same octree. */
int dg_mg_setup(dg_ctx ctx, dg_octree balanced, size_t max_coarse_elems, dg_mg *out);
int dg_mg_levels(dg_mg mg, size_t *nlevels);
int dg_mg_level_sizes(dg_mg mg, size_t level, size_t *n_elem, size_t *n_node);
/* node coordinates of a level, x y z per node (3 * n_node) */
int dg_mg_level_nodes(dg_ctx ctx, dg_mg mg, size_t level, uint32_t *node_xyz, int dst_on_device);
/* the level's balanced octree as {x, y, z, level} records */
int dg_mg_level_octree(dg_ctx ctx, dg_mg mg, size_t level, uint32_t *xyzl, int dst_on_device);
/* DirichletJacobianMatMult on a level: boundary rows identity, boundary
 * columns skipped.  precision 32 / 64 as dg_matvec; 48: FP64 vectors in
 * double-single arithmetic (the CG operator of dg_mg_set_cg_operator 48). */
int dg_mg_matvec(dg_ctx ctx, dg_mg mg, size_t level, const void *in, void *out, int precision, int on_device);
/* restrictMatVecType1: out (level+1) = R in (level); prolongMatVecType1:
 * out (level) = P in (level+1), P = R^T. */
int dg_mg_restrict(dg_ctx ctx, dg_mg mg, size_t fine_level, const void *in, void *out, int precision, int on_device);
int dg_mg_prolong(dg_ctx ctx, dg_mg mg, size_t fine_level, const void *in, void *out, int precision, int on_device);
/* damped-Jacobi smoother (default omega 0.667, bin/options:190) and sweeps
 * per V-cycle side (default 2 and 2) */
int dg_mg_set_smoother(dg_mg mg, double omega, int nu_pre, int nu_post);
/* The CG's own operator application q = A p when the V-cycle runs in FP32
 * (precision 32 of dg_mg_solve).  48 (the default): A p on the FP64
 * vectors in double-single arithmetic (stencil entries and x as FP32 pairs,
 * each element row exact to about 2^-46 of its terms, summed across
 * elements in FP64; GB300's FP64 pipe issues 2 multiply-adds per clock per
 * SM).  64: A p in FP64 every iteration.  32: A p in FP32
 * (the FP32 element loop), and the recurrence
 * residual replaced by the FP64 residual b - A x whenever it has fallen by
 * reliable_delta since the last replacement, and before the stopping test
 * accepts it ("reliable updates"); residual, dot products, updates and the
 * stopping test stay FP64.  No counterpart in the reference (PETSc's CG
 * runs one precision). */
int dg_mg_set_cg_operator(dg_mg mg, int precision, double reliable_delta);
/* load vector of a nodal field on level 0: b = M f, boundary entries 0 */
int dg_mg_rhs(dg_ctx ctx, dg_mg mg, const double *f, double *b, int on_device);
/* CG preconditioned by one V-cycle per iteration, to ||b - A x|| <= rtol
 * ||b||.  Residual, dot products and updates are FP64; the V-cycle runs in
 * FP32 (precision 32) or FP64 (precision 64).  *relres is the final FP64
 * relative residual recomputed from x. */
int dg_mg_solve(dg_ctx ctx, dg_mg mg, const double *b, double *x, int precision, double rtol, int maxit, int on_device,
                int *iterations, double *relres);
int dg_mg_free(dg_ctx ctx, dg_mg mg);

/* ---- assembled sparse matrices -------------------------------------------
 * The element operators as CSR matrices on the device, rows and columns in
 * this library's node numbering (DA node ids, dg_da_download /
 * dg_mg_level_nodes give each node's coordinates), columns sorted within a
 * row.  The reference assembles them into a PETSc Mat through
 * DA::computeLocalToGlobalMappings (src/oda/oda.cpp:77) and
 * DA::setValuesInMatrix (oda.cpp:139).
 * dg_da_assemble: lapFac K + massFac M, the matrix of dg_matvec:
 *   CreateAndComputeFullJacobian1 (examples/src/backend/odaJac.C:470), the
 *   -buildFullMatAll / -buildFullCoarseMat matrices (omgJac.C:1333).
 * dg_mg_assemble: the Dirichlet operator of a multigrid level (the matrix of
 *   dg_mg_matvec): ComputeDirichletJacobian (omgJac.C:383); boundary rows
 *   are the identity, boundary columns are dropped.
 * dg_csr_download: row_ptr (n_rows + 1), col (nnz), val (nnz), host or
 * device arrays.  dg_csr_spmv: y = A x (FP64). */
int dg_da_assemble(dg_ctx ctx, dg_da da, double lapFac, double massFac, dg_csr *out);
int dg_mg_assemble(dg_ctx ctx, dg_mg mg, size_t level, dg_csr *out);
/* with per-element factors (coef as for dg_matvec_coef):
 * BUILD_FULL_JAC_TYPE2_BLOCK (omgJac.C:1804-1858) */
int dg_da_assemble_coef(dg_ctx ctx, dg_da da, const double *coef, int coef_on_device, dg_csr *out);
int dg_csr_sizes(dg_csr a, size_t *n_rows, size_t *nnz, unsigned *max_row_len);
int dg_csr_download(dg_ctx ctx, dg_csr a, int64_t *row_ptr, uint32_t *col, double *val, int dst_on_device);
int dg_csr_spmv(dg_ctx ctx, dg_csr a, const double *x, double *y, int on_device);
int dg_csr_free(dg_ctx ctx, dg_csr a);

/* ---- timing ---------------------------------------------------------------
 * Milliseconds of device time spent by the last completed call on ctx
 * (CUDA events on the context's stream). */
int dg_ctx_last_device_ms(dg_ctx ctx, double *ms);

/* Per-kernel timing: while enabled, every kernel launch of the library is
 * bracketed by CUDA events on the context's stream and accumulated by kernel
 * name (total device ms, launch count, algorithmic bytes moved).  Enabling
 * or disabling clears the statistics.  No counterpart in the reference (it
 * logs PETSc events, src/sys.cpp:19). */
int dg_ctx_profile(dg_ctx ctx, int enable);
int dg_ctx_profile_count(dg_ctx ctx, int *count);
int dg_ctx_profile_entry(dg_ctx ctx, int index, char *name, size_t name_len, double *total_ms,
                         unsigned long long *launches, double *bytes);

/* ---- self-test of the bounded device waits -----------------------------
 * No counterpart in the reference (it has no device code).  Runs one digit
 * pass of the radix sort over n_keys synthetic keys in which the first
 * skipped_tiles tiles are never processed, so the next tile's look-back
 * waits for a predecessor that never publishes its count.  The wait gives
 * up after its spin limit (2^22 polls, a fraction of a second), the kernel
 * returns, and the call reports DG_ERR_TIMEOUT; the context stays usable.
 * Needs 1 <= skipped_tiles < tiles (4096 keys per tile) <= 2^20. */
int dg_debug_lookback_timeout(dg_ctx ctx, size_t n_keys, unsigned skipped_tiles);

/* In-place FP32 inverse of a symmetric positive definite n x n row-major
 * matrix in device memory (n <= 20000), the routine that inverts the
 * coarsest multigrid operator: block Gauss-Jordan without pivoting, the
 * rank-64 trailing updates on the tensor cores (3xTF32).  Replaces the
 * coarse LU the reference's PCMG configuration asks PETSc for
 * (bin/options:206); no direct counterpart in Dendro itself. */
int dg_dense_spd_inverse(dg_ctx ctx, float *X, size_t n);

#ifdef __cplusplus
}
#endif
#endif
