// dendro_gb300.hpp — C++ drop-in mirror of the reference's octree API over
// the C ABI of dendro_gb300.h (header only).
//
// Signatures follow Dendro4 (include/octUtils.h:633,692, include/oda/oda.h:622,
// examples/include/odaJac.h:35) with the octant type as a template parameter,
// so a caller keeps its own ot::TreeNode: any type constructible as
// TN(x, y, z, level, dim, maxDepth) with getX/getY/getZ/getLevel works
// (include/TreeNode.h:39).  The communicator is a template parameter too; only
// a single-rank communicator is accepted (the caller passes its size).
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

}  // namespace cxx

namespace ot {

// ot::points2Octree (src/construct.cpp:759).  Like the reference, pts is
// cleared (construct.cpp:944).
template <class TN>
int points2Octree(std::vector<double> &pts, double *gLens, std::vector<TN> &nodes, unsigned int dim,
                  unsigned int maxDepth, unsigned int maxNumPts, int comm_size = 1) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "points2Octree: only dim = 3");
  dg_ctx c = cxx::context();
  dg_octree o = nullptr;
  cxx::check(c, dg_points_to_octree(c, pts.data(), pts.size() / 3, gLens, maxDepth, maxNumPts, comm_size, 0, &o),
             "points2Octree");
  std::vector<uint32_t> r = cxx::download(c, o);
  dg_octree_free(c, o);
  cxx::records_to_nodes(r, maxDepth, nodes);
  pts.clear();
  return 1;
}

// ot::balanceOctree (src/balance.cpp:31).  Like the reference, in is
// cleared and out overwritten (balance.cpp:42,60-61).
template <class TN>
int balanceOctree(std::vector<TN> &in, std::vector<TN> &out, unsigned int dim, unsigned int maxDepth,
                  bool incCorner, int comm_size = 1) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "balanceOctree: only dim = 3");
  dg_ctx c = cxx::context();
  std::vector<uint32_t> r = cxx::nodes_to_records(in);
  dg_octree a = nullptr, b = nullptr;
  cxx::check(c, dg_octree_upload(c, r.data(), in.size(), maxDepth, 0, &a), "balanceOctree (upload)");
  int st = dg_balance_octree(c, a, incCorner ? 1 : 0, comm_size, &b);
  dg_octree_free(c, a);
  cxx::check(c, st, "balanceOctree");
  r = cxx::download(c, b);
  dg_octree_free(c, b);
  cxx::records_to_nodes(r, maxDepth, out);
  in.clear();
  return 1;
}

// ot::completeOctree (include/octUtils.h:813, src/construct.cpp:518) at one
// rank.  A declared order the input breaks throws DG_ERR_INVALID_ARG.
template <class TN>
int completeOctree(const std::vector<TN> &in, std::vector<TN> &out, unsigned int dim, unsigned int maxDepth,
                   bool isUnique, bool isSorted, bool /*assertNoEmptyProcs*/ = false, int /*comm_size*/ = 1) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "completeOctree: only dim = 3");
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
                  int /*comm_size*/ = 1) {
  if (dim != 3) throw cxx::Error(DG_ERR_UNSUPPORTED, "coarsenOctree: only dim = 3");
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

// ot::DA (include/oda/oda.h:622) built from a balanced octree, resident on the
// GPU, with the element loop of Jacobian1MatMult (odaJac.C:294).
class DA {
 public:
  // compressLut: the reference's DA(in, comm, activeComm, tol, compressLut)
  // (include/oda/oda.h:622)
  template <class TN>
  explicit DA(const std::vector<TN> &in, unsigned maxDepth, bool compressLut = false) {
    c_ = cxx::context();
    std::vector<uint32_t> r = cxx::nodes_to_records(in);
    dg_octree o = nullptr;
    cxx::check(c_, dg_octree_upload(c_, r.data(), in.size(), maxDepth, 0, &o), "DA (upload)");
    int st = dg_da_build_ex(c_, o, compressLut ? 1 : 0, &da_);
    dg_octree_free(c_, o);
    cxx::check(c_, st, "DA");
    cxx::check(c_, dg_da_sizes(da_, &ne_, &nn_), "dg_da_sizes");
  }
  ~DA() {
    if (da_) dg_da_free(c_, da_);
  }
  DA(const DA &) = delete;
  DA &operator=(const DA &) = delete;

  unsigned int getElementSize() const { return (unsigned)ne_; }
  unsigned int getNodeSize() const { return (unsigned)nn_; }
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
  // out = (lapFac L + massFac M) in  (Jacobian1MatMult)
  void matVec(const std::vector<double> &in, std::vector<double> &out, double lapFac = 1.0,
              double massFac = 1.0) const {
    out.resize(nn_);
    cxx::check(c_, dg_matvec(c_, da_, in.data(), out.data(), 64, lapFac, massFac, 0), "Jacobian1MatMult");
  }
  void matVec(const std::vector<float> &in, std::vector<float> &out, double lapFac = 1.0, double massFac = 1.0) const {
    out.resize(nn_);
    cxx::check(c_, dg_matvec(c_, da_, in.data(), out.data(), 32, lapFac, massFac, 0), "Jacobian1MatMult");
  }
  // per-element factors, matProp[2e] (Laplacian) and matProp[2e + 1] (mass)
  // of element e in octree order (Jacobian2MatMult)
  void matVec(const std::vector<double> &matProp, const std::vector<double> &in, std::vector<double> &out) const {
    if (matProp.size() != 2 * ne_) throw cxx::Error(DG_ERR_INVALID_ARG, "matProp must hold 2 values per element");
    out.resize(nn_);
    cxx::check(c_, dg_matvec_coef(c_, da_, matProp.data(), in.data(), out.data(), 64, 0), "Jacobian2MatMult");
  }
  // diagonal of lapFac L + massFac M (Jacobian1MatGetDiagonal)
  void getDiagonal(std::vector<double> &diag, double lapFac = 1.0, double massFac = 1.0) const {
    diag.resize(nn_);
    cxx::check(c_, dg_da_diagonal(c_, da_, nullptr, lapFac, massFac, diag.data(), 0), "Jacobian1MatGetDiagonal");
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

 private:
  dg_ctx c_ = nullptr;
  dg_da da_ = nullptr;
  size_t ne_ = 0, nn_ = 0;
};

}  // namespace ot

namespace par {

// par::sampleSort (include/parUtils.h:424) at one rank: out = in sorted in
// the octant order (in is left unchanged).
template <class TN>
int sampleSort(std::vector<TN> &in, std::vector<TN> &out, int /*comm_size*/ = 1) {
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
int removeDuplicates(std::vector<TN> &v, bool /*isSorted*/, int /*comm_size*/ = 1) {
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
}  // namespace dg

#endif
