/*
 * Oracle driver around the REFERENCE's own code (Dendro4), compiled from the
 * reference sources by oracle/Makefile into oracle/_ref/ref_driver.  Test
 * infrastructure only: it produces golden outputs for the parity tests and
 * times the reference CPU path.  Nothing in the shipped library uses it.
 *
 * Modes (all files are little-endian raw binary):
 *   p2o   PTS MAXDEPTH MAXPTS OUT.oct
 *         ot::points2Octree (src/construct.cpp:759) at 1 rank.
 *   bal   IN.oct MAXDEPTH INCCORNER PATCHED OUT.oct
 *         ot::balanceOctree (src/balance.cpp:31).  PATCHED=1 calls the same
 *         1-rank body (copy + ot::comboRipple, balance.cpp:54-63) with a
 *         maxNum of 4e9 instead of the default _COMBO_RIPPLE_FACTOR_
 *         (include/octUtils.h:477), which works around the empty-output
 *         defect of comboRipple above 1e7 octants (balance.cpp:821-900).
 *   coarsen IN.oct MAXDEPTH OUT.oct
 *         ot::coarsenOctree, sequential form (src/coarsen.cpp:53).
 *   complete IN.oct MAXDEPTH ISUNIQUE ISSORTED OUT.oct
 *         ot::completeOctree (src/construct.cpp:518) at 1 rank, with the
 *         input octants in file order.
 *   treesort IN.oct MAXDEPTH OPTIONS OUT.oct
 *         SFC::parSort::SFC_treeSort (include/sfcSort.h:1378) at 1 rank:
 *         OPTIONS 0 writes the input sorted in place, TS_REMOVE_DUPLICATES
 *         (1) writes the sorted output without duplicates and ancestors.
 *   check IN.oct MAXDEPTH
 *         ot::test::isLinear / isComplete / isBalanced (src/test/testUtils.C).
 *   da    BAL.oct MAXDEPTH STENCILDIR VEC_IN|- OUT_PREFIX
 *         ot::DA (src/oda/oda.cpp:250) then one Laplacian+mass element loop
 *         (examples/src/backend/odaJac.C:275-292, hFac as odaJac.C:311-313).
 *         Writes OUT_PREFIX.elem (per element: x y z level child hmask etype
 *         and the 8 node indices as node coordinates) and, when VEC_IN is
 *         given, OUT_PREFIX.mv (node coordinates + output value).  A 7th
 *         argument "mat" also writes OUT_PREFIX.mat: the assembled
 *         K + M of CreateAndComputeFullJacobian1
 *         (examples/src/backend/odaJac.C:470-535, lapFac = massFac = 1) with
 *         every element's records added in element order, as
 *         (row x y z, column x y z, value) by node coordinates.
 *
 *   transfer FINE.oct MAXDEPTH STENCILDIR VEC_F VEC_C OUT_PREFIX
 *         the reference's inter-grid transfers between FINE (a balanced
 *         octree) and its next coarser level, made as DAMGCreateAndSetDA
 *         makes it at one rank (src/omg/blockDiag.cpp:1384-1425: coarsen,
 *         then balance with incCorner): the two ot::DAs, the Dirichlet
 *         flags of SetDirichletJacContexts (examples/src/backend/
 *         omgJac.C:509-575) as the suppressed DOFs, the TransferOpData of
 *         createInterpolationType1 (blockDiag.cpp:2254-2303) with its dummy
 *         pass, then one restrictMatVecType1 of VEC_F
 *         (src/omg/restrictMatVec.cpp) and one prolongMatVecType1 of VEC_C
 *         (src/omg/prolongMatVec.cpp).  Writes OUT_PREFIX.coarse (the
 *         coarse octree), OUT_PREFIX.r (R VEC_F by coarse node coordinates)
 *         and OUT_PREFIX.p (P VEC_C by fine node coordinates).
 *   dirichlet BAL.oct MAXDEPTH STENCILDIR VEC_IN OUT_PREFIX
 *         the multigrid level operator at one rank: the ot::DA of BAL, the
 *         DirichletJacData of SetDirichletJacContexts
 *         (examples/src/backend/omgJac.C:509-575), then one
 *         DirichletJacobianMatMult of VEC_IN (omgJac.C:958) and
 *         DirichletJacobianMatGetDiagonal (omgJac.C:1111), through a
 *         MatShell as the reference registers them.  Writes OUT_PREFIX.mv
 *         (A VEC_IN) and OUT_PREFIX.diag by node coordinates.
 *   jac   BAL.oct MAXDEPTH STENCILDIR VEC_IN COEF_IN OUT_PREFIX
 *         the element-loop MatShell callbacks at one rank on the ot::DA of
 *         BAL, registered as the reference registers them:
 *         Jacobian1MatMult, Jacobian1MatGetDiagonal, MassMatMult and
 *         MassMatGetDiagonal (examples/src/backend/odaJac.C:294,160,399,229;
 *         context Jac1MFreeData) and Jacobian2MatMult / Jacobian2MatGetDiagonal
 *         (examples/src/backend/omgJac.C:1776,1641; a one-level DAMG whose
 *         Jac2MFreeData holds the per-element (lap, mass) factors of COEF_IN,
 *         an elemental 2-dof vector).  Writes OUT_PREFIX.{j1,j1d,m,md,j2,j2d}
 *         by node coordinates.
 *   assemble BAL.oct MAXDEPTH STENCILDIR COEF_IN OUT_PREFIX
 *         the reference's assembled matrices at one rank on the ot::DA of
 *         BAL (after DA::computeLocalToGlobalMappings, src/oda/oda.cpp:77;
 *         entries through DA::setValuesInMatrix, oda.cpp:139, into the
 *         shim's recording MatSetValues): CreateAndComputeFullJacobian1
 *         (examples/src/backend/odaJac.C:470, -fullJacMatType aij),
 *         ComputeDirichletJacobian (omgJac.C:383, the boundary flags of
 *         SetDirichletJacContexts) and ComputeJacobian2 (omgJac.C:1861,
 *         BUILD_FULL_JAC_TYPE2_BLOCK with the per-element factors of
 *         COEF_IN).  Writes OUT_PREFIX.{k,kd,k2} in the mat format.
 *
 * Formats
 *   coef : u64 n, then n*(u32 x, u32 y, u32 z, u32 level, f64 lap, f64 mass),
 *          one record per octant of BAL (octree level)
 *   .pts : u64 n, then n*3 f64 (x,y,z interleaved)
 *   .oct : u64 n, then n*(u32 x, u32 y, u32 z, u32 level)
 *   mat  : u64 n, then n*(u32 rx, ry, rz, cx, cy, cz, f64 value)
 *   vec  : u64 n, then n*(u32 x, u32 y, u32 z, u32 pad, f64 value), node
 *          coordinates at the octree's maxDepth scale (vertices in [0,2^D]).
 */
#include <chrono>
#include <map>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "TreeNode.h"
#include "handleStencils.h"
#include "omg.h"
#include "odaJac.h"
#include "omgJac.h"
#include "octUtils.h"
#include "oda.h"
#include "odaUtils.h"
#include "parUtils.h"
#include "sfcSort.h"
#include "testUtils.h"

double ****LaplacianType2Stencil = nullptr;
double ****MassType2Stencil = nullptr;
/* the type-1 tables of omgJac.C's Jacobian3 (never called here) */
double *****LaplacianType1Stencil = nullptr;
double *****MassType1Stencil = nullptr;
namespace ot {
double ****ShapeFnCoeffs = nullptr;
/* the restriction tables and vertex maps (defined in src/omg/blockDiag.cpp,
 * which is not compiled here; loaded by the transfer mode) */
double *****RmatType1Stencil = nullptr;
double ****RmatType2Stencil = nullptr;
unsigned short ****VtxMap1 = nullptr;
unsigned short *****VtxMap2 = nullptr;
unsigned short *****VtxMap3 = nullptr;
unsigned short ******VtxMap4 = nullptr;
int readRmatType1Stencil(double *****&lut);
int readRmatType2Stencil(double ****&lut);
int readVtxMaps(unsigned short ****&map1, unsigned short *****&map2, unsigned short *****&map3,
                unsigned short ******&map4);
/* the scatter of the type-2 transfers (blockDiag.cpp), which only run where
 * a level has an auxiliary mesh: never at one rank */
int scatterValues(Vec, Vec, PetscInt, PetscInt, int *&, int *&, int *&, int *&, MPI_Comm) {
  std::fprintf(stderr, "scatterValues: type-2 transfers are not used at one rank\n");
  std::abort();
}
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static FILE *xopen(const char *p, const char *m) {
  FILE *f = std::fopen(p, m);
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", p);
    std::exit(2);
  }
  return f;
}

static std::vector<ot::TreeNode> read_oct(const char *path, unsigned maxDepth) {
  FILE *f = xopen(path, "rb");
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) std::exit(3);
  std::vector<uint32_t> buf(4 * n);
  if (n && std::fread(buf.data(), 4, 4 * n, f) != 4 * n) std::exit(3);
  std::fclose(f);
  std::vector<ot::TreeNode> out;
  out.reserve(n);
  for (uint64_t i = 0; i < n; i++)
    out.push_back(ot::TreeNode(buf[4 * i], buf[4 * i + 1], buf[4 * i + 2], buf[4 * i + 3], 3, maxDepth));
  return out;
}

static void write_oct(const char *path, const std::vector<ot::TreeNode> &v) {
  FILE *f = xopen(path, "wb");
  uint64_t n = v.size();
  std::fwrite(&n, 8, 1, f);
  std::vector<uint32_t> buf(4 * n);
  for (uint64_t i = 0; i < n; i++) {
    buf[4 * i] = v[i].getX();
    buf[4 * i + 1] = v[i].getY();
    buf[4 * i + 2] = v[i].getZ();
    buf[4 * i + 3] = v[i].getLevel();
  }
  if (n) std::fwrite(buf.data(), 4, 4 * n, f);
  std::fclose(f);
}

static int mode_p2o(int argc, char **argv) {
  if (argc < 6) return 1;
  unsigned maxDepth = std::atoi(argv[3]), maxPts = std::atoi(argv[4]);
  FILE *f = xopen(argv[2], "rb");
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) return 3;
  std::vector<double> pts(3 * n);
  if (n && std::fread(pts.data(), 8, 3 * n, f) != 3 * n) return 3;
  std::fclose(f);
  double gLens[3] = {1.0, 1.0, 1.0};
  std::vector<ot::TreeNode> nodes;
  double t0 = now_s();
  ot::points2Octree(pts, gLens, nodes, 3, maxDepth, maxPts, MPI_COMM_WORLD);
  double t1 = now_s();
  write_oct(argv[5], nodes);
  std::printf("{\"op\":\"p2o\",\"n_pts\":%llu,\"n_oct\":%zu,\"seconds\":%.6f}\n", (unsigned long long)n,
              nodes.size(), t1 - t0);
  return 0;
}

static int mode_bal(int argc, char **argv) {
  if (argc < 7) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  bool incCorner = std::atoi(argv[4]) != 0;
  bool patched = std::atoi(argv[5]) != 0;
  std::vector<ot::TreeNode> in = read_oct(argv[2], maxDepth), out;
  size_t nin = in.size();
  double t0 = now_s();
  if (patched) {
    out = in;
    in.clear();
    ot::comboRipple(out, incCorner, 4000000000u);
  } else {
    ot::balanceOctree(in, out, 3, maxDepth, incCorner, MPI_COMM_WORLD, NULL, NULL);
  }
  double t1 = now_s();
  write_oct(argv[6], out);
  std::printf("{\"op\":\"bal\",\"n_in\":%zu,\"n_out\":%zu,\"patched\":%d,\"seconds\":%.6f}\n", nin, out.size(),
              (int)patched, t1 - t0);
  return 0;
}

static int mode_coarsen(int argc, char **argv) {
  if (argc < 5) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  std::vector<ot::TreeNode> in = read_oct(argv[2], maxDepth), out;
  double t0 = now_s();
  ot::coarsenOctree(in, out);
  double t1 = now_s();
  write_oct(argv[4], out);
  std::printf("{\"op\":\"coarsen\",\"n_in\":%zu,\"n_out\":%zu,\"seconds\":%.6f}\n", in.size(), out.size(), t1 - t0);
  return 0;
}

static int mode_complete(int argc, char **argv) {
  if (argc < 7) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  bool isUnique = std::atoi(argv[4]) != 0, isSorted = std::atoi(argv[5]) != 0;
  std::vector<ot::TreeNode> in = read_oct(argv[2], maxDepth), out;
  double t0 = now_s();
  ot::completeOctree(in, out, 3, maxDepth, isUnique, isSorted, false, MPI_COMM_WORLD);
  double t1 = now_s();
  write_oct(argv[6], out);
  std::printf("{\"op\":\"complete\",\"n_in\":%zu,\"n_out\":%zu,\"seconds\":%.6f}\n", in.size(), out.size(),
              t1 - t0);
  return 0;
}

// treesort IN.oct MAXDEPTH OPTIONS OUT.oct: SFC::parSort::SFC_treeSort
// (include/sfcSort.h:1378; one rank: the sequential sort :418) with the
// arguments its callers pass (src/construct.cpp:541,553, odaFactory.cpp:186:
// root parent, rotation 0, k = 1).  OPTIONS 0 writes the input sorted in
// place; TS_REMOVE_DUPLICATES (1) writes pOutSorted.
static int mode_treesort(int argc, char **argv) {
  if (argc < 6) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  unsigned options = std::atoi(argv[4]);
  std::vector<ot::TreeNode> in = read_oct(argv[2], maxDepth), tmp;
  ot::TreeNode root(3, maxDepth);
  double t0 = now_s();
  SFC::parSort::SFC_treeSort(in, tmp, tmp, tmp, 0.1, maxDepth, root, 0, 1, options, NUM_NPES_THRESHOLD,
                             MPI_COMM_WORLD);
  double t1 = now_s();
  write_oct(argv[5], options & TS_REMOVE_DUPLICATES ? tmp : in);
  std::printf("{\"op\":\"treesort\",\"n_in\":%zu,\"n_out\":%zu,\"seconds\":%.6f}\n", in.size(),
              (options & TS_REMOVE_DUPLICATES ? tmp : in).size(), t1 - t0);
  return 0;
}

static int mode_check(int argc, char **argv) {
  if (argc < 4) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  std::vector<ot::TreeNode> v = read_oct(argv[2], maxDepth);
  bool s = seq::test::isUniqueAndSorted(v);
  bool l = ot::test::isLinear(v);
  bool c = ot::test::isComplete(v);
  bool b = ot::test::isBalanced(3, maxDepth, (char *)"_ref_check_fail", v, true, 1);
  std::printf("{\"op\":\"check\",\"sorted\":%d,\"linear\":%d,\"complete\":%d,\"balanced\":%d}\n", (int)s, (int)l,
              (int)c, (int)b);
  return 0;
}

/* node coordinate key (coordinates at the octree's maxDepth scale, < 2^31) */
static inline unsigned __int128 ckey(uint32_t x, uint32_t y, uint32_t z) {
  return ((unsigned __int128)x << 64) | ((unsigned __int128)y << 32) | (unsigned __int128)z;
}
struct CKeyHash {
  size_t operator()(unsigned __int128 k) const noexcept {
    uint64_t a = (uint64_t)k, b = (uint64_t)(k >> 64);
    return (size_t)((a * 0x9E3779B97F4A7C15ull) ^ (b + 0x632BE59BD9B4E019ull + (a << 6) + (a >> 2)));
  }
};

static int mode_da(int argc, char **argv) {
  if (argc < 7) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  std::string stencilDir = argv[4];
  const char *vecIn = argv[5];
  std::string prefix = argv[6];
  std::vector<ot::TreeNode> bal = read_oct(argv[2], maxDepth);
  size_t nb = bal.size();
  {
    /* DA_Initialize and the stencil loaders read their tables from the CWD */
    char oldcwd[4096];
    if (!getcwd(oldcwd, sizeof(oldcwd))) return 4;
    if (chdir(stencilDir.c_str()) != 0) return 4;
    ot::DA_Initialize(MPI_COMM_WORLD);
    createLmatType2(LaplacianType2Stencil);
    createMmatType2(MassType2Stencil);
    if (chdir(oldcwd) != 0) return 4;
  }

  double t0 = now_s();
  ot::DA da(bal, MPI_COMM_WORLD, MPI_COMM_WORLD, 0.3, false);
  double t1 = now_s();
  const unsigned maxD = da.getMaxDepth(); /* DA maxDepth = maxDepth + 1 */

  /* Element sweep: record element data and the geometric position of every
   * node index (vertex k of the element, or vertex k of its parent when the
   * vertex is hanging).  A conflict would mean the hanging-vertex rule
   * assumed here is wrong, so it is reported. */
  std::vector<uint32_t> rec;
  std::vector<uint32_t> idxPos; /* 3 per buffer slot */
  std::vector<unsigned char> idxSeen;
  size_t bufSize = da.getLocalBufferSize();
  idxPos.assign(3 * bufSize, 0);
  idxSeen.assign(bufSize, 0);
  long conflicts = 0;
  size_t nel = 0;
  for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
    Point pt = da.getCurrentOffset();
    unsigned lev = da.getLevel(da.curr());
    unsigned idx[8];
    da.getNodeIndices(idx);
    unsigned char cn = da.getChildNumber();
    unsigned char hm = da.getHangingNodeIndex(da.curr());
    unsigned char et = 0;
    GET_ETYPE_BLOCK(et, hm, cn)
    uint32_t x = pt.xint(), y = pt.yint(), z = pt.zint();
    uint32_t h = 1u << (maxD - lev);
    uint32_t px = x - ((cn & 1) ? h : 0), py = y - ((cn & 2) ? h : 0), pz = z - ((cn & 4) ? h : 0);
    rec.push_back(x);
    rec.push_back(y);
    rec.push_back(z);
    rec.push_back(lev | (cn << 8) | (hm << 16) | (et << 24));
    for (int k = 0; k < 8; k++) {
      uint32_t vx, vy, vz;
      if (hm & (1u << k)) {
        vx = px + ((k & 1) ? 2 * h : 0);
        vy = py + ((k & 2) ? 2 * h : 0);
        vz = pz + ((k & 4) ? 2 * h : 0);
      } else {
        vx = x + ((k & 1) ? h : 0);
        vy = y + ((k & 2) ? h : 0);
        vz = z + ((k & 4) ? h : 0);
      }
      rec.push_back(vx);
      rec.push_back(vy);
      rec.push_back(vz);
      if (idxSeen[idx[k]]) {
        if (idxPos[3 * idx[k]] != vx || idxPos[3 * idx[k] + 1] != vy || idxPos[3 * idx[k] + 2] != vz) conflicts++;
      } else {
        idxSeen[idx[k]] = 1;
        idxPos[3 * idx[k]] = vx;
        idxPos[3 * idx[k] + 1] = vy;
        idxPos[3 * idx[k] + 2] = vz;
      }
    }
    nel++;
  }
  {
    std::string p = prefix + ".elem";
    FILE *f = xopen(p.c_str(), "wb");
    uint64_t n = nel;
    std::fwrite(&n, 8, 1, f);
    if (n) std::fwrite(rec.data(), 4, rec.size(), f);
    std::fclose(f);
  }
  size_t nNodesUsed = 0;
  for (size_t i = 0; i < bufSize; i++) nNodesUsed += idxSeen[i];

  double tmv = -1.0;
  if (std::strcmp(vecIn, "-") != 0) {
    /* input vector by node coordinate (node coordinates at the DA scale are
     * the octree coordinates: the DA keeps anchors and adds one level) */
    FILE *f = xopen(vecIn, "rb");
    uint64_t nv = 0;
    if (std::fread(&nv, 8, 1, f) != 1) return 3;
    std::unordered_map<unsigned __int128, double, CKeyHash> val;
    val.reserve(2 * nv);
    for (uint64_t i = 0; i < nv; i++) {
      uint32_t c[4];
      double v;
      if (std::fread(c, 4, 4, f) != 4 || std::fread(&v, 8, 1, f) != 1) return 3;
      val[ckey(c[0], c[1], c[2])] = v;
    }
    std::fclose(f);

    std::vector<double> in, out;
    da.createVector(in, false, false, 1);
    da.createVector(out, false, false, 1);
    for (size_t i = 0; i < in.size(); i++) in[i] = out[i] = 0.0;
    double *inArr = NULL, *outArr = NULL;
    da.vecGetBuffer<double>(in, inArr, false, false, true, 1);
    da.vecGetBuffer<double>(out, outArr, false, false, false, 1);
    /* the buffers are indexed like getNodeIndices: fill the input by node
     * coordinate, zero the output */
    long missing = 0;
    for (size_t i = 0; i < bufSize; i++) {
      outArr[i] = 0.0;
      if (!idxSeen[i]) continue;
      auto it = val.find(ckey(idxPos[3 * i], idxPos[3 * i + 1], idxPos[3 * i + 2]));
      if (it == val.end())
        missing++;
      else
        inArr[i] = it->second;
    }
    da.ReadFromGhostsBegin<double>(inArr, 1);
    da.ReadFromGhostsEnd<double>(inArr);
    double hFac = 1.0 / ((double)(1u << (maxD - 1)));
    double t2 = now_s();
    for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
      unsigned lev = da.getLevel(da.curr());
      double h = hFac * (1u << (maxD - lev));
      double fac1 = h / 2.0, fac2 = h * h * h / 8.0;
      unsigned idx[8];
      da.getNodeIndices(idx);
      unsigned char cn = da.getChildNumber();
      unsigned char hm = da.getHangingNodeIndex(da.curr());
      unsigned char et = 0;
      GET_ETYPE_BLOCK(et, hm, cn)
      for (int k = 0; k < 8; k++)
        for (int j = 0; j < 8; j++)
          outArr[idx[k]] += (fac1 * LaplacianType2Stencil[cn][et][k][j] + fac2 * MassType2Stencil[cn][et][k][j]) *
                            inArr[idx[j]];
    }
    double t3 = now_s();
    tmv = t3 - t2;
    std::vector<double> res(bufSize, 0.0);
    for (size_t i = 0; i < bufSize; i++) res[i] = outArr[i];
    da.vecRestoreBuffer<double>(in, inArr, false, false, true, 1);
    da.vecRestoreBuffer<double>(out, outArr, false, false, false, 1);
    std::string p = prefix + ".mv";
    FILE *g = xopen(p.c_str(), "wb");
    uint64_t n = nNodesUsed;
    std::fwrite(&n, 8, 1, g);
    for (size_t i = 0; i < bufSize; i++) {
      if (!idxSeen[i]) continue;
      uint32_t c[4] = {idxPos[3 * i], idxPos[3 * i + 1], idxPos[3 * i + 2], 0};
      std::fwrite(c, 4, 4, g);
      std::fwrite(&res[i], 8, 1, g);
    }
    std::fclose(g);
    if (missing) std::fprintf(stderr, "warning: %ld node values missing from input vector\n", missing);
  }
  if (argc > 7 && std::strcmp(argv[7], "mat") == 0) {
    /* the records of CreateAndComputeFullJacobian1, summed per (row, col) in
     * the order the loop visits them (ADD_VALUES) */
    std::map<std::pair<unsigned, unsigned>, double> mat;
    double hFac = 1.0 / ((double)(1u << (maxD - 1)));
    for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
      unsigned lev = da.getLevel(da.curr());
      double h = hFac * (1u << (maxD - lev));
      double fac1 = 1.0 * h / 2.0, fac2 = 1.0 * h * h * h / 8.0;
      unsigned idx[8];
      da.getNodeIndices(idx);
      unsigned char cn = da.getChildNumber();
      unsigned char hm = da.getHangingNodeIndex(da.curr());
      unsigned char et = 0;
      GET_ETYPE_BLOCK(et, hm, cn)
      for (int k = 0; k < 8; k++)
        for (int j = 0; j < 8; j++)
          mat[std::make_pair(idx[k], idx[j])] +=
              (fac1 * LaplacianType2Stencil[cn][et][k][j]) + (fac2 * MassType2Stencil[cn][et][k][j]);
    }
    std::string p = prefix + ".mat";
    FILE *g = xopen(p.c_str(), "wb");
    uint64_t n = mat.size();
    std::fwrite(&n, 8, 1, g);
    for (const auto &kv : mat) {
      unsigned r = kv.first.first, c = kv.first.second;
      uint32_t rc[6] = {idxPos[3 * r], idxPos[3 * r + 1], idxPos[3 * r + 2],
                        idxPos[3 * c], idxPos[3 * c + 1], idxPos[3 * c + 2]};
      std::fwrite(rc, 4, 6, g);
      std::fwrite(&kv.second, 8, 1, g);
    }
    std::fclose(g);
  }
  std::printf(
      "{\"op\":\"da\",\"n_bal\":%zu,\"n_elem\":%zu,\"n_nodes_da\":%u,\"n_nodes_used\":%zu,\"conflicts\":%ld,"
      "\"t_da\":%.6f,\"t_matvec\":%.6f}\n",
      nb, nel, da.getNodeSize(), nNodesUsed, conflicts, t1 - t0, tmv);
  return conflicts ? 5 : 0;
}

/* node coordinates of every buffer index of a DA (vertex k of an element, or
 * vertex k of its parent where the vertex is hanging); returns the number of
 * indices seen at two positions (0 when the hanging-vertex rule holds) */
static long node_positions(ot::DA &da, std::vector<uint32_t> &pos, std::vector<unsigned char> &seen) {
  const unsigned maxD = da.getMaxDepth();
  const size_t nb = da.getLocalBufferSize();
  pos.assign(3 * nb, 0);
  seen.assign(nb, 0);
  long conflicts = 0;
  for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
    Point pt = da.getCurrentOffset();
    unsigned lev = da.getLevel(da.curr());
    unsigned idx[8];
    da.getNodeIndices(idx);
    unsigned char cn = da.getChildNumber();
    unsigned char hm = da.getHangingNodeIndex(da.curr());
    uint32_t x = pt.xint(), y = pt.yint(), z = pt.zint();
    uint32_t h = 1u << (maxD - lev);
    uint32_t px = x - ((cn & 1) ? h : 0), py = y - ((cn & 2) ? h : 0), pz = z - ((cn & 4) ? h : 0);
    for (int k = 0; k < 8; k++) {
      uint32_t v[3];
      if (hm & (1u << k)) {
        v[0] = px + ((k & 1) ? 2 * h : 0);
        v[1] = py + ((k & 2) ? 2 * h : 0);
        v[2] = pz + ((k & 4) ? 2 * h : 0);
      } else {
        v[0] = x + ((k & 1) ? h : 0);
        v[1] = y + ((k & 2) ? h : 0);
        v[2] = z + ((k & 4) ? h : 0);
      }
      if (seen[idx[k]]) {
        if (pos[3 * idx[k]] != v[0] || pos[3 * idx[k] + 1] != v[1] || pos[3 * idx[k] + 2] != v[2]) conflicts++;
      } else {
        seen[idx[k]] = 1;
        for (int a = 0; a < 3; a++) pos[3 * idx[k] + a] = v[a];
      }
    }
  }
  return conflicts;
}

static bool read_vec(const char *path, std::unordered_map<unsigned __int128, double, CKeyHash> &val) {
  FILE *f = xopen(path, "rb");
  uint64_t nv = 0;
  if (std::fread(&nv, 8, 1, f) != 1) return false;
  val.reserve(2 * nv);
  for (uint64_t i = 0; i < nv; i++) {
    uint32_t c[4];
    double v;
    if (std::fread(c, 4, 4, f) != 4 || std::fread(&v, 8, 1, f) != 1) return false;
    val[ckey(c[0], c[1], c[2])] = v;
  }
  std::fclose(f);
  return true;
}

/* a nodal PETSc vector of da filled by node coordinate (through the DA's own
 * buffer, as the reference moves data between vectors and buffers) */
static long fill_vec(ot::DA &da, Vec v, const std::vector<uint32_t> &pos, const std::vector<unsigned char> &seen,
                     const std::unordered_map<unsigned __int128, double, CKeyHash> &val) {
  PetscScalar *arr = NULL;
  da.vecGetBuffer(v, arr, false, false, false, 1);
  long missing = 0;
  for (size_t i = 0; i < seen.size(); i++) {
    arr[i] = 0.0;
    if (!seen[i]) continue;
    auto it = val.find(ckey(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    if (it == val.end())
      missing++;
    else
      arr[i] = it->second;
  }
  da.vecRestoreBuffer(v, arr, false, false, false, 1);
  return missing;
}

static void write_vec(ot::DA &da, Vec v, const std::vector<uint32_t> &pos, const std::vector<unsigned char> &seen,
                      const std::string &path) {
  PetscScalar *arr = NULL;
  da.vecGetBuffer(v, arr, false, false, true, 1);
  FILE *g = xopen(path.c_str(), "wb");
  uint64_t n = 0;
  for (size_t i = 0; i < seen.size(); i++) n += seen[i];
  std::fwrite(&n, 8, 1, g);
  for (size_t i = 0; i < seen.size(); i++) {
    if (!seen[i]) continue;
    uint32_t c[4] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0};
    std::fwrite(c, 4, 4, g);
    std::fwrite(&arr[i], 8, 1, g);
  }
  std::fclose(g);
  da.vecRestoreBuffer(v, arr, false, false, true, 1);
}

/* the Dirichlet flags of SetDirichletJacContexts (omgJac.C:509-575) as a
 * suppressed-DOF array indexed like the DA's buffers */
static std::vector<unsigned char> suppressed_dofs(ot::DA &da) {
  std::vector<unsigned char> flags;
  ot::assignBoundaryFlags(&da, flags);
  unsigned char *bdy = NULL;
  da.vecGetBuffer<unsigned char>(flags, bdy, false, false, true, 1);
  std::vector<unsigned char> sup(da.getLocalBufferSize(), 0);
  for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
    unsigned idx[8];
    da.getNodeIndices(idx);
    for (int k = 0; k < 8; k++) sup[idx[k]] = bdy[idx[k]];
  }
  da.vecRestoreBuffer<unsigned char>(flags, bdy, false, false, true, 1);
  return sup;
}

static int mode_transfer(int argc, char **argv) {
  if (argc < 8) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  std::string stencilDir = argv[4];
  std::string prefix = argv[7];
  std::vector<ot::TreeNode> fine = read_oct(argv[2], maxDepth), coarse;
  {
    /* the next coarser level: coarsen, then balance (blockDiag.cpp:1384-1425) */
    std::vector<ot::TreeNode> tmp, in = fine;
    ot::coarsenOctree(in, tmp);
    ot::balanceOctree(tmp, coarse, 3, maxDepth, true, MPI_COMM_WORLD, NULL, NULL);
  }
  write_oct((prefix + ".coarse").c_str(), coarse);
  {
    /* the tables are read from the working directory */
    char oldcwd[4096];
    if (!getcwd(oldcwd, sizeof(oldcwd))) return 4;
    if (chdir(stencilDir.c_str()) != 0) return 4;
    ot::DA_Initialize(MPI_COMM_WORLD);
    ot::readRmatType1Stencil(ot::RmatType1Stencil);
    ot::readRmatType2Stencil(ot::RmatType2Stencil);
    ot::readVtxMaps(ot::VtxMap1, ot::VtxMap2, ot::VtxMap3, ot::VtxMap4);
    if (chdir(oldcwd) != 0) return 4;
  }
  const size_t nFine = fine.size(), nCoarse = coarse.size();
  /* the coarse DA first; the fine DA takes its blocks (blockDiag.cpp:2005-2007) */
  std::vector<ot::TreeNode> cIn = coarse, fIn = fine;
  ot::DA dac(cIn, MPI_COMM_WORLD, MPI_COMM_WORLD, 0.3, false);
  std::vector<ot::TreeNode> blocks = dac.getBlocks();
  ot::DA daf(fIn, MPI_COMM_WORLD, MPI_COMM_WORLD, 0.3, false, &blocks, NULL);
  std::vector<uint32_t> posC, posF;
  std::vector<unsigned char> seenC, seenF;
  long conflicts = node_positions(dac, posC, seenC) + node_positions(daf, posF, seenF);
  std::vector<unsigned char> supC = suppressed_dofs(dac), supF = suppressed_dofs(daf);

  /* createInterpolationType1 (blockDiag.cpp:2254-2303) at one rank */
  ot::TransferOpData data;
  std::memset(&data, 0, sizeof(data));
  data.dac = &dac;
  data.daf = &daf;
  data.minIndependentSize = dac.getIndependentSize();
  data.suppressedDOFc = supC.data();
  data.suppressedDOFf = supF.data();
  data.comm = MPI_COMM_WORLD;
  data.dof = 1;
  data.fineTouchedFlags = new std::vector<ot::FineTouchedStatus>;
  Mat R;
  MatCreateShell(MPI_COMM_WORLD, dac.getNodeSize(), daf.getNodeSize(), PETSC_DETERMINE, PETSC_DETERMINE,
                 (void *)&data, &R);
  MatShellSetOperation(R, MATOP_MULT, (void (*)(void))ot::restrictMatVecType1);
  MatShellSetOperation(R, MATOP_MULT_TRANSPOSE, (void (*)(void))ot::prolongMatVecType1);
  daf.createVector<ot::FineTouchedStatus>(*data.fineTouchedFlags, false, false, 1);
  ot::dummyRestrictMatVecType1(&data);

  std::unordered_map<unsigned __int128, double, CKeyHash> vf, vc;
  if (!read_vec(argv[5], vf) || !read_vec(argv[6], vc)) return 3;
  Vec f, c, pf;
  daf.createVector(f, false, false, 1);
  daf.createVector(pf, false, false, 1);
  dac.createVector(c, false, false, 1);
  long missing = fill_vec(daf, f, posF, seenF, vf);
  Vec rc;
  dac.createVector(rc, false, false, 1);
  if (MatMult(R, f, rc) != 0) return 6;
  write_vec(dac, rc, posC, seenC, prefix + ".r");
  missing += fill_vec(dac, c, posC, seenC, vc);
  if (MatMultTranspose(R, c, pf) != 0) return 6;
  write_vec(daf, pf, posF, seenF, prefix + ".p");
  if (missing) std::fprintf(stderr, "warning: %ld node values missing from the input vectors\n", missing);
  std::printf("{\"op\":\"transfer\",\"n_fine\":%zu,\"n_coarse\":%zu,\"fine_nodes\":%u,\"coarse_nodes\":%u,"
              "\"conflicts\":%ld,\"missing\":%ld}\n",
              nFine, nCoarse, daf.getNodeSize(), dac.getNodeSize(), conflicts, missing);
  return conflicts ? 5 : 0;
}

static int mode_dirichlet(int argc, char **argv) {
  if (argc < 7) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  std::string stencilDir = argv[4];
  std::string prefix = argv[6];
  std::vector<ot::TreeNode> bal = read_oct(argv[2], maxDepth);
  const size_t nb = bal.size();
  {
    /* the tables are read from the working directory */
    char oldcwd[4096];
    if (!getcwd(oldcwd, sizeof(oldcwd))) return 4;
    if (chdir(stencilDir.c_str()) != 0) return 4;
    ot::DA_Initialize(MPI_COMM_WORLD);
    createLmatType2(LaplacianType2Stencil);
    createMmatType2(MassType2Stencil);
    if (chdir(oldcwd) != 0) return 4;
  }
  ot::DA da(bal, MPI_COMM_WORLD, MPI_COMM_WORLD, 0.3, false);
  std::vector<uint32_t> pos;
  std::vector<unsigned char> seen;
  long conflicts = node_positions(da, pos, seen);
  /* one level of the DAMG, as DAMGCreateAndSetDA and DAMGCreateSuppressedDOFs
   * (src/omg/blockDiag.cpp:1836-1860, 46-60) leave it at one rank */
  ot::DAMG damg[1];
  damg[0] = new ot::_p_DAMG();
  damg[0]->da = &da;
  damg[0]->dof = 1;
  damg[0]->nlevels = 1;
  damg[0]->totalLevels = 1;
  damg[0]->comm = MPI_COMM_WORLD;
  std::vector<unsigned char> sup(da.getLocalBufferSize(), 0);
  damg[0]->suppressedDOF = sup.data();
  SetDirichletJacContexts(damg);
  Mat J;
  MatCreateShell(MPI_COMM_WORLD, da.getNodeSize(), da.getNodeSize(), PETSC_DETERMINE, PETSC_DETERMINE,
                 (void *)damg[0], &J);
  MatShellSetOperation(J, MATOP_MULT, (void (*)(void))DirichletJacobianMatMult);
  MatShellSetOperation(J, MATOP_GET_DIAGONAL, (void (*)(void))DirichletJacobianMatGetDiagonal);
  std::unordered_map<unsigned __int128, double, CKeyHash> val;
  if (!read_vec(argv[5], val)) return 3;
  Vec in, out, diag;
  da.createVector(in, false, false, 1);
  da.createVector(out, false, false, 1);
  da.createVector(diag, false, false, 1);
  long missing = fill_vec(da, in, pos, seen, val);
  if (MatMult(J, in, out) != 0 || MatGetDiagonal(J, diag) != 0) return 6;
  write_vec(da, out, pos, seen, prefix + ".mv");
  write_vec(da, diag, pos, seen, prefix + ".diag");
  size_t nbdy = 0;
  for (unsigned char b : sup) nbdy += b != 0;
  if (missing) std::fprintf(stderr, "warning: %ld node values missing from the input vector\n", missing);
  std::printf("{\"op\":\"dirichlet\",\"n_bal\":%zu,\"nodes\":%u,\"boundary_nodes\":%zu,\"conflicts\":%ld,"
              "\"missing\":%ld}\n",
              nb, da.getNodeSize(), nbdy, conflicts, missing);
  return conflicts ? 5 : 0;
}

static int mode_jac(int argc, char **argv) {
  if (argc < 8) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  std::string stencilDir = argv[4];
  std::string prefix = argv[7];
  std::vector<ot::TreeNode> bal = read_oct(argv[2], maxDepth);
  const size_t nb = bal.size();
  {
    /* the tables are read from the working directory */
    char oldcwd[4096];
    if (!getcwd(oldcwd, sizeof(oldcwd))) return 4;
    if (chdir(stencilDir.c_str()) != 0) return 4;
    ot::DA_Initialize(MPI_COMM_WORLD);
    createLmatType2(LaplacianType2Stencil);
    createMmatType2(MassType2Stencil);
    if (chdir(oldcwd) != 0) return 4;
  }
  /* per-element factors by (anchor, octree level) */
  std::map<std::pair<unsigned __int128, unsigned>, std::pair<double, double>> coef;
  {
    FILE *f = xopen(argv[6], "rb");
    uint64_t n = 0;
    if (std::fread(&n, 8, 1, f) != 1) return 3;
    for (uint64_t i = 0; i < n; i++) {
      uint32_t c[4];
      double v[2];
      if (std::fread(c, 4, 4, f) != 4 || std::fread(v, 8, 2, f) != 2) return 3;
      coef[std::make_pair(ckey(c[0], c[1], c[2]), c[3])] = std::make_pair(v[0], v[1]);
    }
    std::fclose(f);
  }
  ot::DA da(bal, MPI_COMM_WORLD, MPI_COMM_WORLD, 0.3, false);
  std::vector<uint32_t> pos;
  std::vector<unsigned char> seen;
  long conflicts = node_positions(da, pos, seen);
  /* the elemental, ghosted 2-dof factor vector (lap, mass per element) */
  std::vector<double> matProp;
  da.createVector<double>(matProp, true, true, 2);
  long missing = 0;
  {
    double *arr = NULL;
    da.vecGetBuffer<double>(matProp, arr, true, true, false, 2);
    for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
      Point pt = da.getCurrentOffset();
      unsigned lev = da.getLevel(da.curr()) - 1; /* the DA adds one level */
      auto it = coef.find(std::make_pair(ckey(pt.xint(), pt.yint(), pt.zint()), lev));
      if (it == coef.end()) {
        missing++;
        continue;
      }
      arr[2 * da.curr()] = it->second.first;
      arr[2 * da.curr() + 1] = it->second.second;
    }
    da.vecRestoreBuffer<double>(matProp, arr, true, true, false, 2);
  }
  Jac1MFreeData jd;
  jd.da = &da;
  jd.isFinestLevel = false;
  jd.Jmat_private = NULL;
  jd.inTmp = NULL;
  jd.outTmp = NULL;
  Mat J1, M;
  MatCreateShell(MPI_COMM_WORLD, da.getNodeSize(), da.getNodeSize(), PETSC_DETERMINE, PETSC_DETERMINE, (void *)&jd,
                 &J1);
  MatShellSetOperation(J1, MATOP_MULT, (void (*)(void))Jacobian1MatMult);
  MatShellSetOperation(J1, MATOP_GET_DIAGONAL, (void (*)(void))Jacobian1MatGetDiagonal);
  MatCreateShell(MPI_COMM_WORLD, da.getNodeSize(), da.getNodeSize(), PETSC_DETERMINE, PETSC_DETERMINE, (void *)&jd,
                 &M);
  MatShellSetOperation(M, MATOP_MULT, (void (*)(void))MassMatMult);
  MatShellSetOperation(M, MATOP_GET_DIAGONAL, (void (*)(void))MassMatGetDiagonal);
  Jac2MFreeData j2d;
  j2d.matProp = &matProp;
  j2d.isFinestLevel = false;
  j2d.Jmat_private = NULL;
  j2d.inTmp = NULL;
  j2d.outTmp = NULL;
  ot::DAMG damg = new ot::_p_DAMG();
  damg->da = &da;
  damg->dof = 1;
  damg->nlevels = 1;
  damg->totalLevels = 1;
  damg->comm = MPI_COMM_WORLD;
  damg->user = &j2d;
  Mat J2;
  MatCreateShell(MPI_COMM_WORLD, da.getNodeSize(), da.getNodeSize(), PETSC_DETERMINE, PETSC_DETERMINE, (void *)damg,
                 &J2);
  MatShellSetOperation(J2, MATOP_MULT, (void (*)(void))Jacobian2MatMult);
  MatShellSetOperation(J2, MATOP_GET_DIAGONAL, (void (*)(void))Jacobian2MatGetDiagonal);

  std::unordered_map<unsigned __int128, double, CKeyHash> val;
  if (!read_vec(argv[5], val)) return 3;
  Vec in, out;
  da.createVector(in, false, false, 1);
  da.createVector(out, false, false, 1);
  missing += fill_vec(da, in, pos, seen, val);
  const struct {
    Mat m;
    const char *ext;
  } ops[3] = {{J1, ".j1"}, {M, ".m"}, {J2, ".j2"}};
  for (const auto &op : ops) {
    if (MatMult(op.m, in, out) != 0) return 6;
    write_vec(da, out, pos, seen, prefix + op.ext);
    if (MatGetDiagonal(op.m, out) != 0) return 6;
    write_vec(da, out, pos, seen, prefix + op.ext + "d");
  }
  if (missing) std::fprintf(stderr, "warning: %ld values missing from the inputs\n", missing);
  std::printf("{\"op\":\"jac\",\"n_bal\":%zu,\"nodes\":%u,\"conflicts\":%ld,\"missing\":%ld}\n", nb,
              da.getNodeSize(), conflicts, missing);
  return conflicts ? 5 : 0;
}

/* per-element (lap, mass) factors of a coef file into the DA's elemental,
 * ghosted 2-dof vector; returns the elements without a record */
static long read_coef(const char *path, ot::DA &da, std::vector<double> &matProp) {
  std::map<std::pair<unsigned __int128, unsigned>, std::pair<double, double>> coef;
  FILE *f = xopen(path, "rb");
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) return -1;
  for (uint64_t i = 0; i < n; i++) {
    uint32_t c[4];
    double v[2];
    if (std::fread(c, 4, 4, f) != 4 || std::fread(v, 8, 2, f) != 2) return -1;
    coef[std::make_pair(ckey(c[0], c[1], c[2]), c[3])] = std::make_pair(v[0], v[1]);
  }
  std::fclose(f);
  da.createVector<double>(matProp, true, true, 2);
  long missing = 0;
  double *arr = NULL;
  da.vecGetBuffer<double>(matProp, arr, true, true, false, 2);
  for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
    Point pt = da.getCurrentOffset();
    unsigned lev = da.getLevel(da.curr()) - 1; /* the DA adds one level */
    auto it = coef.find(std::make_pair(ckey(pt.xint(), pt.yint(), pt.zint()), lev));
    if (it == coef.end()) {
      missing++;
      continue;
    }
    arr[2 * da.curr()] = it->second.first;
    arr[2 * da.curr() + 1] = it->second.second;
  }
  da.vecRestoreBuffer<double>(matProp, arr, true, true, false, 2);
  return missing;
}

/* the recorded entries of an assembled matrix, by node coordinates (global
 * index -> buffer index through the DA's local-to-global map) */
static long write_entries(ot::DA &da, Mat m, const std::vector<uint32_t> &pos, const std::vector<unsigned char> &seen,
                          const std::string &path) {
  const DendroIntL *l2g = da.getLocalToGlobalMap();
  std::unordered_map<DendroIntL, size_t> g2b;
  for (size_t i = 0; i < seen.size(); i++)
    if (seen[i]) g2b[l2g[i]] = i;
  FILE *g = xopen(path.c_str(), "wb");
  uint64_t n = m->entries ? m->entries->size() : 0;
  std::fwrite(&n, 8, 1, g);
  long unmapped = 0;
  if (m->entries)
    for (const auto &kv : *m->entries) {
      auto r = g2b.find(kv.first.first), c = g2b.find(kv.first.second);
      if (r == g2b.end() || c == g2b.end()) {
        unmapped++;
        continue;
      }
      uint32_t rc[6] = {pos[3 * r->second], pos[3 * r->second + 1], pos[3 * r->second + 2],
                        pos[3 * c->second], pos[3 * c->second + 1], pos[3 * c->second + 2]};
      std::fwrite(rc, 4, 6, g);
      std::fwrite(&kv.second, 8, 1, g);
    }
  std::fclose(g);
  return unmapped;
}

static int mode_assemble(int argc, char **argv) {
  if (argc < 7) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  std::string stencilDir = argv[4];
  std::string prefix = argv[6];
  std::vector<ot::TreeNode> bal = read_oct(argv[2], maxDepth);
  const size_t nb = bal.size();
  {
    /* the tables are read from the working directory */
    char oldcwd[4096];
    if (!getcwd(oldcwd, sizeof(oldcwd))) return 4;
    if (chdir(stencilDir.c_str()) != 0) return 4;
    ot::DA_Initialize(MPI_COMM_WORLD);
    createLmatType2(LaplacianType2Stencil);
    createMmatType2(MassType2Stencil);
    if (chdir(oldcwd) != 0) return 4;
  }
  ot::DA da(bal, MPI_COMM_WORLD, MPI_COMM_WORLD, 0.3, false);
  std::vector<uint32_t> pos;
  std::vector<unsigned char> seen;
  long conflicts = node_positions(da, pos, seen);
  da.computeLocalToGlobalMappings();
  std::vector<double> matProp;
  long missing = read_coef(argv[5], da, matProp);
  if (missing < 0) return 3;

  dg_shim_options()["-fullJacMatType"] = MATAIJ;
  Mat K = NULL;
  if (CreateAndComputeFullJacobian1(&da, &K) != 0) return 6;

  /* one level of the DAMG (as in the dirichlet mode) for the Dirichlet
   * matrix, and one with the Jacobian2 context */
  ot::DAMG damg[1];
  damg[0] = new ot::_p_DAMG();
  damg[0]->da = &da;
  damg[0]->dof = 1;
  damg[0]->nlevels = 1;
  damg[0]->totalLevels = 1;
  damg[0]->comm = MPI_COMM_WORLD;
  std::vector<unsigned char> sup(da.getLocalBufferSize(), 0);
  damg[0]->suppressedDOF = sup.data();
  SetDirichletJacContexts(damg);
  Mat KD = NULL;
  da.createMatrix(KD, MATAIJ, 1);
  if (ComputeDirichletJacobian(damg[0], KD, KD) != 0) return 6;

  Jac2MFreeData j2d;
  j2d.matProp = &matProp;
  j2d.isFinestLevel = false;
  j2d.Jmat_private = NULL;
  j2d.inTmp = NULL;
  j2d.outTmp = NULL;
  ot::DAMG damg2 = new ot::_p_DAMG();
  damg2->da = &da;
  damg2->dof = 1;
  damg2->nlevels = 1;
  damg2->totalLevels = 1;
  damg2->comm = MPI_COMM_WORLD;
  damg2->user = &j2d;
  Mat K2 = NULL;
  da.createMatrix(K2, MATAIJ, 1);
  if (ComputeJacobian2(damg2, K2, K2) != 0) return 6;

  long unmapped = write_entries(da, K, pos, seen, prefix + ".k") + write_entries(da, KD, pos, seen, prefix + ".kd") +
                  write_entries(da, K2, pos, seen, prefix + ".k2");
  std::printf("{\"op\":\"assemble\",\"n_bal\":%zu,\"nodes\":%u,\"nnz\":[%zu,%zu,%zu],\"conflicts\":%ld,"
              "\"missing\":%ld,\"unmapped\":%ld}\n",
              nb, da.getNodeSize(), K->entries ? K->entries->size() : (size_t)0,
              KD->entries ? KD->entries->size() : (size_t)0, K2->entries ? K2->entries->size() : (size_t)0, conflicts,
              missing, unmapped);
  return (conflicts || unmapped) ? 5 : 0;
}

// io PTS D OUTPREFIX: the reference's own file writers on one cloud --
// writePtsToFile (OUTPREFIX.pts), and for its balanced octree writeNodesToFile
// (OUTPREFIX.ot, text) and writeNodesToFile_binary (OUTPREFIX.otb); then its
// readers on those files, reporting what they return
static int mode_io(int argc, char **argv) {
  if (argc < 5) return 1;
  unsigned maxDepth = std::atoi(argv[3]);
  FILE *f = xopen(argv[2], "rb");
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) return 3;
  std::vector<double> pts(3 * n);
  if (n && std::fread(pts.data(), 8, 3 * n, f) != 3 * n) return 3;
  std::fclose(f);
  std::string pre = argv[4];
  std::string fp = pre + ".pts", ft = pre + ".ot", fb = pre + ".otb";
  ot::writePtsToFile(&fp[0], pts);
  std::vector<double> back;
  ot::readPtsFromFile(&fp[0], back);
  const bool pts_same = back == pts;
  double gLens[3] = {1.0, 1.0, 1.0};
  std::vector<ot::TreeNode> lin, bal;
  ot::points2Octree(pts, gLens, lin, 3, maxDepth, 1, MPI_COMM_WORLD);
  ot::balanceOctree(lin, bal, 3, maxDepth, true, MPI_COMM_WORLD, NULL, NULL);
  ot::writeNodesToFile(&ft[0], bal);
  ot::writeNodesToFile_binary(&fb[0], bal);
  std::vector<ot::TreeNode> rt, rb;
  ot::readNodesFromFile(&ft[0], rt);
  ot::readNodesFromFile_binary(&fb[0], rb);
  bool text_same = rt.size() == bal.size();
  for (size_t i = 0; text_same && i < rt.size(); i++) text_same = rt[i] == bal[i] && rt[i].getLevel() == bal[i].getLevel();
  bool bin_prefix_same = rb.size() >= bal.size();
  for (size_t i = 0; bin_prefix_same && i < bal.size(); i++)
    bin_prefix_same = rb[i] == bal[i] && rb[i].getLevel() == bal[i].getLevel();
  std::printf("{\"op\":\"io\",\"n_pts\":%llu,\"n_bal\":%zu,\"pts_roundtrip\":%d,\"text_read\":%zu,"
              "\"text_same\":%d,\"binary_read\":%zu,\"binary_prefix_same\":%d,\"treenode_bytes\":%zu}\n",
              (unsigned long long)n, bal.size(), (int)pts_same, rt.size(), (int)text_same, rb.size(),
              (int)bin_prefix_same, sizeof(ot::TreeNode));
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: ref_driver p2o|bal|check|da ...\n");
    return 1;
  }
  _InitializeHcurve(3);
  std::string m = argv[1];
  int rc = 1;
  if (m == "p2o") rc = mode_p2o(argc, argv);
  if (m == "bal") rc = mode_bal(argc, argv);
  if (m == "check") rc = mode_check(argc, argv);
  if (m == "coarsen") rc = mode_coarsen(argc, argv);
  if (m == "complete") rc = mode_complete(argc, argv);
  if (m == "da") rc = mode_da(argc, argv);
  if (m == "io") rc = mode_io(argc, argv);
  if (m == "treesort") rc = mode_treesort(argc, argv);
  if (m == "transfer") rc = mode_transfer(argc, argv);
  if (m == "dirichlet") rc = mode_dirichlet(argc, argv);
  if (m == "jac") rc = mode_jac(argc, argv);
  if (m == "assemble") rc = mode_assemble(argc, argv);
  return rc;
}
