// dendro_gb300.hpp — C++ drop-in mirror of the reference's octree API over
// the C ABI of dendro_gb300.h (header only).
//
// Signatures follow Dendro4 (include/octUtils.h:633,692,813,825,
// include/parUtils.h:424,437, include/sfcSort.h:1378, include/oda/oda.h:622)
// with the octant type as a template parameter, so a caller keeps its own
// ot::TreeNode: any type constructible as TN(x, y, z, level, dim, maxDepth)
// with getX/getY/getZ/getLevel/getMaxDepth works (include/TreeNode.h:39).
//
// Communicators: when <mpi.h> is included first (MPI_VERSION defined), the
// comm parameters are MPI_Comm, as in the reference, and the library asks
// MPI_Comm_size; only a single-rank communicator is accepted.  Without MPI a
// communicator is represented by its size (dg::cxx::comm_t, default 1).
//
// Namespaces: everything lives in dg::ot, dg::par, dg::SFC::parSort and
// dg::omg, and is also visible as ot::, par::, SFC::parSort:: and omg::
// (using-directives), so reference call sites compile unchanged; define
// DG_NO_REFERENCE_NAMESPACES to keep only the dg:: names.
//
// Return values follow the reference: 1 on success (PROF_*_END expands to
// `return 1`, include/octUtils.h:419-428).  Failures throw dg::cxx::Error
// carrying the C ABI status, where the reference would assert.
#ifndef DENDRO_GB300_HPP
#define DENDRO_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "dendro_gb300.h"

namespace dg {
namespace cxx {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(dg_ctx ctx, int st, const char *what) {
  if (st != DG_OK) {
    std::string m = std::string(what) + ": " + dg_status_string(st);
    if (ctx && dg_ctx_last_error(ctx)[0]) m += std::string(" (") + dg_ctx_last_error(ctx) + ")";
    throw Error(st, m);
  }
}

#if defined(MPI_VERSION)
typedef MPI_Comm comm_t;
inline int comm_size(comm_t c) {
  int n = 0;
  MPI_Comm_size(c, &n);
  return n;
}
inline comm_t default_comm() { return MPI_COMM_WORLD; }
#else
// without MPI a communicator is its number of ranks
struct comm_t {
  int size;
  comm_t(int s = 1) : size(s) {}
};
inline int comm_size(comm_t c) { return c.size; }
inline comm_t default_comm() { return comm_t(1); }
#endif

// process-wide context on one device (the reference keeps per-rank globals)
inline dg_ctx context(int device = 0) {
  static dg_ctx c = nullptr;
  if (!c) check(nullptr, dg_ctx_create(device, &c), "dg_ctx_create");
  return c;
}

template <class TN>
inline void records_to_nodes(const std::vector<uint32_t> &r, unsigned maxDepth, std::vector<TN> &out) {
  out.clear();
  out.reserve(r.size() / 4);
  for (size_t i = 0; i < r.size() / 4; i++) out.push_back(TN(r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3], 3, maxDepth));
}

template <class TN>
inline std::vector<uint32_t> nodes_to_records(const std::vector<TN> &v) {
  std::vector<uint32_t> r(4 * v.size());
  for (size_t i = 0; i < v.size(); i++) {
    r[4 * i] = v[i].getX();
    r[4 * i + 1] = v[i].getY();
    r[4 * i + 2] = v[i].getZ();
    r[4 * i + 3] = v[i].getLevel();
  }
  return r;
}

inline std::vector<uint32_t> download(dg_ctx c, dg_octree o) {
  size_t n = 0;
  unsigned d = 0;
  check(c, dg_octree_size(o, &n, &d), "dg_octree_size");
  std::vector<uint32_t> r(4 * n);
  check(c, dg_octree_download(c, o, r.data(), 0), "dg_octree_download");
  return r;
}

inline void single_rank(comm_t comm, const char *what) {
  if (comm_size(comm) != 1) throw Error(DG_ERR_COMM_SIZE, std::string(what) + ": one rank only");
}

}  // namespace cxx

namespace ot {

using cxx::comm_t;

// ot::points2Octree (src/construct.cpp:759).  Like the reference, pts is
// cleared (construct.cpp:944).
template <class TN>
int points2Octree(std::vector<double> &pts, double *gLens, std::vector<TN> &nodes, unsigned int dim,
                  unsigned int maxDepth, unsigned int maxNumPts, comm_t comm = cxx::default_comm(),
                  double /*tol*/ = 0.1) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "points2Octree: only dim = 3");
  dg_ctx c = cxx::context();
  dg_octree o = nullptr;
  cxx::check(c, dg_points_to_octree(c, pts.data(), pts.size() / 3, gLens, maxDepth, maxNumPts, cxx::comm_size(comm), 0,
                                    &o),
             "points2Octree");
  std::vector<uint32_t> r = cxx::download(c, o);
  dg_octree_free(c, o);
  cxx::records_to_nodes(r, maxDepth, nodes);
  pts.clear();
  return 1;
}

// ot::balanceOctree (src/balance.cpp:31): incCorner balances across faces,
// edges and corners, otherwise across faces and edges.  Like the reference,
// in is cleared and out overwritten (balance.cpp:42,60-61); at one rank the
// new communicator is the input one and every rank is active.
template <class TN>
int balanceOctree(std::vector<TN> &in, std::vector<TN> &out, unsigned int dim, unsigned int maxDepth,
                  bool incCorner, comm_t comm = cxx::default_comm(), comm_t *newCommPtr = nullptr,
                  bool *iAmActive = nullptr) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "balanceOctree: only dim = 3");
  dg_ctx c = cxx::context();
  std::vector<uint32_t> r = cxx::nodes_to_records(in);
  dg_octree a = nullptr, b = nullptr;
  cxx::check(c, dg_octree_upload(c, r.data(), in.size(), maxDepth, 0, &a), "balanceOctree (upload)");
  int st = dg_balance_octree(c, a, incCorner ? 1 : 0, cxx::comm_size(comm), &b);
  dg_octree_free(c, a);
  cxx::check(c, st, "balanceOctree");
  r = cxx::download(c, b);
  dg_octree_free(c, b);
  cxx::records_to_nodes(r, maxDepth, out);
  in.clear();
  if (newCommPtr) *newCommPtr = comm;
  if (iAmActive) *iAmActive = true;
  return 1;
}

// ot::completeOctree (include/octUtils.h:813, src/construct.cpp:518) at one
// rank.  A declared order the input breaks throws DG_ERR_INVALID_ARG.
template <class TN>
int completeOctree(const std::vector<TN> &in, std::vector<TN> &out, unsigned int dim, unsigned int maxDepth,
                   bool isUnique, bool isSorted, bool /*assertNoEmptyProcs*/ = false,
                   comm_t comm = cxx::default_comm(), double /*tol*/ = 0.1) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "completeOctree: only dim = 3");
  cxx::single_rank(comm, "completeOctree");
  dg_ctx c = cxx::context();
  std::vector<uint32_t> r = cxx::nodes_to_records(in);
  dg_octree o = nullptr;
  cxx::check(c, dg_complete_octree(c, r.data(), in.size(), maxDepth, isUnique ? 1 : 0, isSorted ? 1 : 0, 0, &o),
             "completeOctree");
  r = cxx::download(c, o);
  dg_octree_free(c, o);
  cxx::records_to_nodes(r, maxDepth, out);
  return 1;
}

// ot::coarsenOctree (include/octUtils.h:825, sequential form src/coarsen.cpp:53):
// every complete family of 8 sibling leaves replaced by its parent.
template <class TN>
int coarsenOctree(const std::vector<TN> &in, std::vector<TN> &out, unsigned int dim, unsigned int maxDepth,
                  comm_t comm = cxx::default_comm(), bool /*skipPartition*/ = false, comm_t *newCommPtr = nullptr,
                  bool *iAmActive = nullptr) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "coarsenOctree: only dim = 3");
  cxx::single_rank(comm, "coarsenOctree");
  dg_ctx c = cxx::context();
  std::vector<uint32_t> r = cxx::nodes_to_records(in);
  dg_octree a = nullptr, b = nullptr;
  cxx::check(c, dg_octree_upload(c, r.data(), in.size(), maxDepth, 0, &a), "coarsenOctree (upload)");
  int st = dg_coarsen_octree(c, a, &b);
  dg_octree_free(c, a);
  cxx::check(c, st, "coarsenOctree");
  r = cxx::download(c, b);
  dg_octree_free(c, b);
  cxx::records_to_nodes(r, maxDepth, out);
  if (newCommPtr) *newCommPtr = comm;
  if (iAmActive) *iAmActive = true;
  return 1;
}

// par::removeDuplicates of point octants at level maxDepth
// (include/parUtils.h:437), from FP64 points.
template <class TN>
int sortUniquePoints(const std::vector<double> &pts, double *gLens, std::vector<TN> &nodes, unsigned int maxDepth) {
  dg_ctx c = cxx::context();
  std::vector<uint32_t> r(4 * (pts.size() / 3 + 1));
  size_t nu = 0;
  cxx::check(c, dg_sort_unique_points(c, pts.data(), pts.size() / 3, gLens, maxDepth, 0, r.data(), 0, &nu),
             "sortUniquePoints");
  r.resize(4 * nu);
  cxx::records_to_nodes(r, maxDepth, nodes);
  return 1;
}

// the loop types of ot::DA (include/oda/odaUtils.h:157)
namespace DA_FLAGS {
enum loopType { ALL, WRITABLE, DEPENDENT, INDEPENDENT, W_DEPENDENT, FROM_STORED };
}

// an element anchor as ot::DA::getCurrentOffset returns it (integer
// coordinates at the octree's maxDepth scale)
struct Point {
  unsigned int xi, yi, zi;
  Point(unsigned int x = 0, unsigned int y = 0, unsigned int z = 0) : xi(x), yi(y), zi(z) {}
  unsigned int xint() const { return xi; }
  unsigned int yint() const { return yi; }
  unsigned int zint() const { return zi; }
  double x() const { return xi; }
  double y() const { return yi; }
  double z() const { return zi; }
};

// ot::DA (include/oda/oda.h:622) built from a balanced octree, resident on the
// GPU, with the element loop of Jacobian1MatMult (odaJac.C:294) and the
// reference's per-element loop and vector surface at one rank.
//
// Indices: a node index (getNodeIndices) addresses this DA's nodal vectors
// (createVector / vecGetBuffer, getNodeSize() entries); the numbering is the
// library's own, not the reference's buffer layout.  curr() is the element
// index in octree order.  getLevel and getMaxDepth count levels of the DA's
// embedding, one deeper than the octree (src/oda/private/odaFactory.cpp:179).
// At one rank there are no ghosts: ALL, WRITABLE and INDEPENDENT loops visit
// every element, DEPENDENT and W_DEPENDENT none.
class DA {
 public:
  // compressLut: the reference's DA(in, comm, activeComm, tol, compressLut)
  // (include/oda/oda.h:622)
  template <class TN>
  explicit DA(const std::vector<TN> &in, unsigned maxDepth, bool compressLut = false) {
    build(in, maxDepth, compressLut);
  }
  // the reference's constructor: maxDepth from the octants (in must not be
  // empty)
  template <class TN>
  DA(std::vector<TN> &in, comm_t comm, comm_t /*inputActiveComm*/, double /*tol*/, bool compressLut = false,
     const std::vector<TN> * /*blocksPtr*/ = nullptr, bool *iAmActive = nullptr) {
    cxx::single_rank(comm, "DA");
    if (in.empty()) throw cxx::Error(DG_ERR_INVALID_ARG, "DA: empty octree");
    build(in, in[0].getMaxDepth(), compressLut);
    if (iAmActive) *iAmActive = true;
  }
  ~DA() {
    if (da_) dg_da_free(c_, da_);
  }
  DA(const DA &) = delete;
  DA &operator=(const DA &) = delete;

  unsigned int getElementSize() const { return (unsigned)ne_; }
  unsigned int getNodeSize() const { return (unsigned)nn_; }
  unsigned int getLocalBufferSize() const { return (unsigned)nn_; }
  unsigned int getIndependentSize() const { return (unsigned)ne_; }
  unsigned int getGhostedElementSize() const { return (unsigned)ne_; }
  unsigned int getMaxDepth() const { return maxDepth_ + 1; }
  unsigned int getDimension() const { return 3; }
  bool iAmActive() const { return true; }

  // node coordinates at the octree's maxDepth scale, x y z per node
  std::vector<uint32_t> getNodeCoordinates() const {
    std::vector<uint32_t> xyz(3 * nn_);
    cxx::check(c_, dg_da_download(c_, da_, nullptr, nullptr, xyz.data(), 0), "dg_da_download");
    return xyz;
  }
  // 8 node ids per element (getNodeIndices) and meta words
  void getElementData(std::vector<uint32_t> &nodes, std::vector<uint32_t> &meta) const {
    nodes.resize(8 * ne_);
    meta.resize(ne_);
    cxx::check(c_, dg_da_download(c_, da_, meta.data(), nodes.data(), nullptr, 0), "dg_da_download");
  }

  // ---- the element loop (include/oda/oda.tcc:255-660) ----
  template <DA_FLAGS::loopType type>
  void init() {
    load();
    cur_ = (type == DA_FLAGS::DEPENDENT || type == DA_FLAGS::W_DEPENDENT) ? ne_ : 0;
  }
  unsigned int curr() const { return (unsigned)cur_; }
  template <DA_FLAGS::loopType type>
  unsigned int end() const {
    return (unsigned)ne_;
  }
  template <DA_FLAGS::loopType type>
  unsigned int next() {
    return (unsigned)++cur_;
  }
  // the 8 node indices of the current element, vertex k at anchor + h *
  // (k & 1, k >> 1 & 1, k >> 2); a hanging vertex gives the node of the
  // parent's vertex k (include/oda/oda.tcc:1304)
  int getNodeIndices(unsigned int *nodes) const {
    for (int k = 0; k < 8; k++) nodes[k] = nodes_[8 * cur_ + k];
    return 1;
  }
  // Morton child number of the current element (oda.tcc:1273)
  unsigned char getChildNumber() const { return (unsigned char)(meta_[cur_] >> 8); }
  // hanging-vertex mask of element i (src/oda/oda.cpp:1038)
  unsigned char getHangingNodeIndex(unsigned int i) const { return (unsigned char)(meta_[i] >> 16); }
  bool isHanging(unsigned int i) const { return getHangingNodeIndex(i) != 0; }
  // element type 0-17 of element i (GET_ETYPE_BLOCK, include/oda/odaUtils.h:379)
  unsigned char getElementType(unsigned int i) const { return (unsigned char)(meta_[i] >> 24); }
  // level of element i in the DA's embedding (octree level + 1)
  unsigned char getLevel(unsigned int i) const { return (unsigned char)((meta_[i] & 255u) + 1); }
  // anchor of the current element (oda.h:699)
  Point getCurrentOffset() const { return Point(anchor_[3 * cur_], anchor_[3 * cur_ + 1], anchor_[3 * cur_ + 2]); }

  // ---- vectors (oda.h:1108-1197) ----
  template <typename T>
  int createVector(std::vector<T> &local, bool isElemental, bool /*isGhosted*/, unsigned int dof = 1) const {
    local.assign((isElemental ? ne_ : nn_) * dof, T());
    return 0;
  }
  // the vector's own storage: node indices address it directly, so nothing
  // is copied in or out (no ghosts at one rank)
  template <typename T>
  int vecGetBuffer(std::vector<T> &in, T *&out, bool isElemental, bool /*isGhosted*/, bool /*isReadOnly*/,
                   unsigned int dof = 1) const {
    if (in.size() != (isElemental ? ne_ : nn_) * dof)
      throw cxx::Error(DG_ERR_INVALID_ARG, "vecGetBuffer: vector not created by this DA");
    out = in.data();
    return 0;
  }
  template <typename T>
  int vecRestoreBuffer(std::vector<T> & /*in*/, T *&out, bool, bool, bool, unsigned int = 1) const {
    out = nullptr;
    return 0;
  }
  template <typename T>
  int ReadFromGhostsBegin(T *, unsigned int = 1) const { return 0; }
  template <typename T>
  int ReadFromGhostsEnd(T *) const { return 0; }
  template <typename T>
  int WriteToGhostsBegin(T *, unsigned int = 1) const { return 0; }
  template <typename T>
  int WriteToGhostsEnd(T *, unsigned int = 1) const { return 0; }

  // ---- operators ----
  // out = (lapFac L + massFac M) in  (Jacobian1MatMult); host arrays of
  // getNodeSize() values
  void matVec(const double *in, double *out, double lapFac = 1.0, double massFac = 1.0) const {
    cxx::check(c_, dg_matvec(c_, da_, in, out, 64, lapFac, massFac, 0), "Jacobian1MatMult");
  }
  void matVec(const std::vector<double> &in, std::vector<double> &out, double lapFac = 1.0,
              double massFac = 1.0) const {
    if (in.size() != nn_) throw cxx::Error(DG_ERR_INVALID_ARG, "Jacobian1MatMult: vector length != node count");
    out.resize(nn_);
    matVec(in.data(), out.data(), lapFac, massFac);
  }
  void matVec(const std::vector<float> &in, std::vector<float> &out, double lapFac = 1.0, double massFac = 1.0) const {
    if (in.size() != nn_) throw cxx::Error(DG_ERR_INVALID_ARG, "Jacobian1MatMult: vector length != node count");
    out.resize(nn_);
    cxx::check(c_, dg_matvec(c_, da_, in.data(), out.data(), 32, lapFac, massFac, 0), "Jacobian1MatMult");
  }
  // per-element factors, matProp[2e] (Laplacian) and matProp[2e + 1] (mass)
  // of element e in octree order (Jacobian2MatMult)
  void matVec(const std::vector<double> &matProp, const std::vector<double> &in, std::vector<double> &out) const {
    if (matProp.size() != 2 * ne_) throw cxx::Error(DG_ERR_INVALID_ARG, "matProp must hold 2 values per element");
    if (in.size() != nn_) throw cxx::Error(DG_ERR_INVALID_ARG, "Jacobian2MatMult: vector length != node count");
    out.resize(nn_);
    cxx::check(c_, dg_matvec_coef(c_, da_, matProp.data(), in.data(), out.data(), 64, 0), "Jacobian2MatMult");
  }
  // diagonal of lapFac L + massFac M (Jacobian1MatGetDiagonal)
  void getDiagonal(double *diag, double lapFac = 1.0, double massFac = 1.0) const {
    cxx::check(c_, dg_da_diagonal(c_, da_, nullptr, lapFac, massFac, diag, 0), "Jacobian1MatGetDiagonal");
  }
  void getDiagonal(std::vector<double> &diag, double lapFac = 1.0, double massFac = 1.0) const {
    diag.resize(nn_);
    getDiagonal(diag.data(), lapFac, massFac);
  }
  // the assembled lapFac L + massFac M as CSR arrays over node ids
  // (CreateAndComputeFullJacobian1)
  void assemble(std::vector<int64_t> &rowPtr, std::vector<uint32_t> &col, std::vector<double> &val,
                double lapFac = 1.0, double massFac = 1.0) const {
    dg_csr a = nullptr;
    cxx::check(c_, dg_da_assemble(c_, da_, lapFac, massFac, &a), "CreateAndComputeFullJacobian1");
    size_t n = 0, nnz = 0;
    dg_csr_sizes(a, &n, &nnz, nullptr);
    rowPtr.resize(n + 1);
    col.resize(nnz);
    val.resize(nnz);
    int st = dg_csr_download(c_, a, rowPtr.data(), col.data(), val.data(), 0);
    dg_csr_free(c_, a);
    cxx::check(c_, st, "dg_csr_download");
  }
  dg_da handle() const { return da_; }

 private:
  template <class TN>
  void build(const std::vector<TN> &in, unsigned maxDepth, bool compressLut) {
    c_ = cxx::context();
    maxDepth_ = maxDepth;
    std::vector<uint32_t> r = cxx::nodes_to_records(in);
    dg_octree o = nullptr;
    cxx::check(c_, dg_octree_upload(c_, r.data(), in.size(), maxDepth, 0, &o), "DA (upload)");
    int st = dg_da_build_ex(c_, o, compressLut ? 1 : 0, &da_);
    dg_octree_free(c_, o);
    cxx::check(c_, st, "DA");
    cxx::check(c_, dg_da_sizes(da_, &ne_, &nn_), "dg_da_sizes");
    anchor_.resize(3 * ne_);
    for (size_t e = 0; e < ne_; e++)
      for (int a = 0; a < 3; a++) anchor_[3 * e + a] = r[4 * e + a];
  }
  // the element data the loop reads, downloaded once
  void load() {
    if (loaded_) return;
    getElementData(nodes_, meta_);
    loaded_ = true;
  }
  dg_ctx c_ = nullptr;
  dg_da da_ = nullptr;
  size_t ne_ = 0, nn_ = 0, cur_ = 0;
  unsigned maxDepth_ = 0;
  bool loaded_ = false;
  std::vector<uint32_t> nodes_, meta_, anchor_;
};

}  // namespace ot

namespace par {

using cxx::comm_t;

// par::sampleSort (include/parUtils.h:424) at one rank: out = in sorted in
// the octant order (in is left unchanged).
template <class TN>
int sampleSort(std::vector<TN> &in, std::vector<TN> &out, comm_t comm = cxx::default_comm()) {
  cxx::single_rank(comm, "sampleSort");
  if (in.empty()) {
    out.clear();
    return 1;
  }
  dg_ctx c = cxx::context();
  const unsigned maxDepth = in[0].getMaxDepth();
  std::vector<uint32_t> r = cxx::nodes_to_records(in), o(r.size());
  size_t n = 0;
  cxx::check(c, dg_sort_octants(c, r.data(), in.size(), maxDepth, 0, 0, o.data(), 0, &n), "sampleSort");
  o.resize(4 * n);
  cxx::records_to_nodes(o, maxDepth, out);
  return 1;
}

// par::removeDuplicates (include/parUtils.h:437) at one rank: sorted, repeated
// octants removed, in place.
template <class TN>
int removeDuplicates(std::vector<TN> &v, bool /*isSorted*/, comm_t comm = cxx::default_comm()) {
  cxx::single_rank(comm, "removeDuplicates");
  if (v.empty()) return 1;
  dg_ctx c = cxx::context();
  const unsigned maxDepth = v[0].getMaxDepth();
  std::vector<uint32_t> r = cxx::nodes_to_records(v), o(r.size());
  size_t n = 0;
  cxx::check(c, dg_sort_octants(c, r.data(), v.size(), maxDepth, 1, 0, o.data(), 0, &n), "removeDuplicates");
  o.resize(4 * n);
  cxx::records_to_nodes(o, maxDepth, v);
  return 1;
}

}  // namespace par

namespace SFC {
namespace parSort {

using cxx::comm_t;

// SFC::parSort::SFC_treeSort (include/sfcSort.h:1378) at one rank, with the
// options of sfcSort.h:125-128: pNodes is sorted in place in the octant
// order; with TS_REMOVE_DUPLICATES, pOutSorted receives the sorted octants
// without repeats and without octants that have a descendant in the input
// (sfcSort.h:532-575).  TS_CONSTRUCT_OCTREE / TS_BALANCE_OCTREE are served
// by ot::completeOctree / ot::balanceOctree and throw DG_ERR_UNSUPPORTED
// here.  loadFlexibility, parent, rot_id, k and sf_k only matter across
// ranks or for the construct options; the curve is the context's.
template <class TN>
void SFC_treeSort(std::vector<TN> &pNodes, std::vector<TN> &pOutSorted, std::vector<TN> & /*pOutConstruct*/,
                  std::vector<TN> & /*pOutBalanced*/, double /*loadFlexibility*/, unsigned int pMaxDepth,
                  TN & /*parent*/, unsigned int /*rot_id*/, unsigned int /*k*/, unsigned int options,
                  unsigned int /*sf_k*/, comm_t pcomm = cxx::default_comm()) {
  cxx::single_rank(pcomm, "SFC_treeSort");
  if (options & (DG_TS_CONSTRUCT_OCTREE | DG_TS_BALANCE_OCTREE))
    throw cxx::Error(DG_ERR_UNSUPPORTED, "SFC_treeSort: use completeOctree / balanceOctree");
  if (pNodes.empty()) return;  // sfcSort.h:421
  dg_ctx c = cxx::context();
  std::vector<uint32_t> r = cxx::nodes_to_records(pNodes), o(r.size());
  size_t n = 0;
  cxx::check(c, dg_tree_sort(c, r.data(), pNodes.size(), pMaxDepth, DG_TS_SORT_ONLY, 0, o.data(), 0, &n),
             "SFC_treeSort");
  std::vector<TN> sorted;
  cxx::records_to_nodes(o, pMaxDepth, sorted);
  if (options & DG_TS_REMOVE_DUPLICATES) {
    cxx::check(c, dg_tree_sort(c, o.data(), n, pMaxDepth, DG_TS_REMOVE_DUPLICATES, 0, r.data(), 0, &n),
               "SFC_treeSort");
    r.resize(4 * n);
    cxx::records_to_nodes(r, pMaxDepth, pOutSorted);
  }
  pNodes.swap(sorted);
}

}  // namespace parSort
}  // namespace SFC

namespace omg {

// The reference's DAMG hierarchy for -lap(u) + u = f with u = 0 on the
// boundary of the unit cube (src/omg/blockDiag.cpp:1312 DAMGCreateAndSetDA:
// coarsenOctree + balanceOctree until a level holds at most maxCoarseElems
// elements), its level operators (DirichletJacobianMatMult,
// examples/src/backend/omgJac.C:958), transfers (src/omg/restrictMatVec.cpp,
// prolongMatVec.cpp) and the CG + V-cycle solve the reference configures
// (bin/options:48-206).  Level 0 is the input octree.
class MultiGrid {
 public:
  template <class TN>
  MultiGrid(const std::vector<TN> &balanced, unsigned maxDepth, size_t maxCoarseElems = 4096) {
    c_ = cxx::context();
    std::vector<uint32_t> r = cxx::nodes_to_records(balanced);
    dg_octree o = nullptr;
    cxx::check(c_, dg_octree_upload(c_, r.data(), balanced.size(), maxDepth, 0, &o), "DAMG (upload)");
    int st = dg_mg_setup(c_, o, maxCoarseElems, &mg_);
    dg_octree_free(c_, o);
    cxx::check(c_, st, "DAMGCreateAndSetDA");
  }
  ~MultiGrid() {
    if (mg_) dg_mg_free(c_, mg_);
  }
  MultiGrid(const MultiGrid &) = delete;
  MultiGrid &operator=(const MultiGrid &) = delete;

  size_t levels() const {
    size_t n = 0;
    dg_mg_levels(mg_, &n);
    return n;
  }
  size_t nodes(size_t level) const {
    size_t e = 0, v = 0;
    cxx::check(c_, dg_mg_level_sizes(mg_, level, &e, &v), "dg_mg_level_sizes");
    return v;
  }
  // DirichletJacobianMatMult on a level (host arrays)
  void matVec(size_t level, const double *in, double *out) const {
    cxx::check(c_, dg_mg_matvec(c_, mg_, level, in, out, 64, 0), "DirichletJacobianMatMult");
  }
  // DirichletJacobianMatGetDiagonal (omgJac.C:1111)
  void getDiagonal(size_t level, double *diag) const {
    cxx::check(c_, dg_mg_diagonal(c_, mg_, level, diag, 0), "DirichletJacobianMatGetDiagonal");
  }
  // restrictMatVecType1 / prolongMatVecType1
  void restrict_(size_t fineLevel, const double *in, double *out) const {
    cxx::check(c_, dg_mg_restrict(c_, mg_, fineLevel, in, out, 64, 0), "restrictMatVecType1");
  }
  void prolong(size_t fineLevel, const double *in, double *out) const {
    cxx::check(c_, dg_mg_prolong(c_, mg_, fineLevel, in, out, 64, 0), "prolongMatVecType1");
  }
  // load vector of a nodal field on level 0
  void rhs(const double *f, double *b) const { cxx::check(c_, dg_mg_rhs(c_, mg_, f, b, 0), "dg_mg_rhs"); }
  // the CG's operator with an FP32 V-cycle: 48 double-single (the default),
  // 64 FP64, 32 FP32 with FP64 residual replacement (dg_mg_set_cg_operator)
  void setCgOperator(int precision, double reliableDelta = 1e-3) {
    cxx::check(c_, dg_mg_set_cg_operator(mg_, precision, reliableDelta), "dg_mg_set_cg_operator");
  }
  // CG with one V-cycle per iteration to rtol; precision 32 runs the V-cycle
  // in FP32 (FP64 vectors and residuals), 64 all in FP64; returns the
  // iterations
  int solve(const double *b, double *x, int precision, double rtol, int maxit, double *relres = nullptr) const {
    int it = 0;
    double rr = 0;
    cxx::check(c_, dg_mg_solve(c_, mg_, b, x, precision, rtol, maxit, 0, &it, &rr), "DAMGSolve");
    if (relres) *relres = rr;
    return it;
  }
  dg_mg handle() const { return mg_; }

 private:
  dg_ctx c_ = nullptr;
  dg_mg mg_ = nullptr;
};

}  // namespace omg
}  // namespace dg

#ifndef DG_NO_REFERENCE_NAMESPACES
// the tree-sort options of include/sfcSort.h:125-128
#ifndef TS_SORT_ONLY
#define TS_SORT_ONLY DG_TS_SORT_ONLY
#define TS_REMOVE_DUPLICATES DG_TS_REMOVE_DUPLICATES
#define TS_CONSTRUCT_OCTREE DG_TS_CONSTRUCT_OCTREE
#define TS_BALANCE_OCTREE DG_TS_BALANCE_OCTREE
#endif
namespace ot {
using namespace ::dg::ot;
}
namespace par {
using namespace ::dg::par;
}
namespace SFC {
namespace parSort {
using namespace ::dg::SFC::parSort;
}
}  // namespace SFC
namespace omg {
using namespace ::dg::omg;
}
#endif

#endif
