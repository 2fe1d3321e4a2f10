// C++ caller of the drop-in mirror (include/dendro_gb300.hpp) with its own
// octant type shaped like the reference's ot::TreeNode constructor.
// Reads FP64 points (u64 n, then 3n doubles), runs points2Octree ->
// balanceOctree -> DA -> matVec, writes the balanced octree as {x,y,z,level}
// records and prints sizes; then coarsenOctree of the balanced octree and
// completeOctree of every 5th balanced octant in reverse order.  Driven by tests/test_gpu_cpp_dropin.py.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "dendro_gb300.hpp"

struct MyNode {
  unsigned x, y, z, lev, md;
  MyNode(unsigned x_, unsigned y_, unsigned z_, unsigned l_, unsigned /*dim*/, unsigned maxDepth)
      : x(x_), y(y_), z(z_), lev(l_), md(maxDepth) {}
  unsigned getMaxDepth() const { return md; }
  unsigned getX() const { return x; }
  unsigned getY() const { return y; }
  unsigned getZ() const { return z; }
  unsigned getLevel() const { return lev; }
};

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) return 2;
  std::vector<double> pts(3 * n);
  if (std::fread(pts.data(), 8, 3 * n, f) != 3 * n) return 2;
  std::fclose(f);
  double gLens[3] = {1.0, 1.0, 1.0};
  std::vector<MyNode> lin, bal;
  dg::ot::points2Octree(pts, gLens, lin, 3, 30, 1);
  size_t nlin = lin.size();
  dg::ot::balanceOctree(lin, bal, 3, 30, true);
  dg::ot::DA da(bal, 30);
  std::vector<double> x(da.getNodeSize(), 1.0), y;
  da.matVec(x, y);  // A * 1: the Laplacian part vanishes, mass rows remain
  double s = 0;
  for (double v : y) s += v;
  FILE *g = std::fopen(argv[2], "wb");
  uint64_t nb = bal.size();
  std::fwrite(&nb, 8, 1, g);
  for (auto &o : bal) {
    uint32_t r[4] = {o.x, o.y, o.z, o.lev};
    std::fwrite(r, 4, 4, g);
  }
  std::fclose(g);
  // assembled matrix times ones = the matVec of ones; the diagonal is the
  // matrix's; per-element factors (1, 1) give the plain operator
  std::vector<int64_t> rp;
  std::vector<uint32_t> col;
  std::vector<double> val, diag, ones(da.getNodeSize(), 1.0), yc;
  da.assemble(rp, col, val);
  da.getDiagonal(diag);
  da.matVec(std::vector<double>(2 * da.getElementSize(), 1.0), ones, yc);
  double mat_err = 0, diag_err = 0, coef_err = 0, ymax = 0, dmax = 0;
  for (double v : y) ymax = std::max(ymax, std::abs(v));
  for (double v : diag) dmax = std::max(dmax, std::abs(v));
  for (size_t r = 0; r + 1 < rp.size(); r++) {
    double acc = 0, dv = 0;
    for (int64_t q = rp[r]; q < rp[r + 1]; q++) {
      acc += val[q];
      if (col[q] == r) dv = val[q];
    }
    mat_err = std::max(mat_err, std::abs(acc - y[r]));
    diag_err = std::max(diag_err, std::abs(dv - diag[r]));
    coef_err = std::max(coef_err, std::abs(yc[r] - y[r]));
  }
  std::vector<MyNode> coarse, sub, comp, same;
  dg::ot::coarsenOctree(bal, coarse, 3, 30);
  for (size_t i = 0; i < bal.size(); i += 5) sub.push_back(bal[bal.size() - 1 - i]);
  dg::ot::completeOctree(sub, comp, 3, 30, false, false);
  dg::ot::completeOctree(bal, same, 3, 30, true, true);
  // par::sampleSort of the reversed subset gives it back in order;
  // par::removeDuplicates of it twice over keeps one copy of each
  std::vector<MyNode> srt, dup = sub;
  dg::par::sampleSort(sub, srt);
  bool sort_ok = srt.size() == sub.size();
  for (size_t i = 0; sort_ok && i < srt.size(); i++) {
    const MyNode &a = srt[i], &b = sub[sub.size() - 1 - i];
    sort_ok = a.x == b.x && a.y == b.y && a.z == b.z && a.lev == b.lev;
  }
  dup.insert(dup.end(), sub.begin(), sub.end());
  dg::par::removeDuplicates(dup, false);
  sort_ok = sort_ok && dup.size() == sub.size();
  bool same_ok = same.size() == bal.size();
  for (size_t i = 0; same_ok && i < bal.size(); i++)
    same_ok = same[i].x == bal[i].x && same[i].y == bal[i].y && same[i].z == bal[i].z && same[i].lev == bal[i].lev;
  // sum of the mass matrix applied to ones = volume of the unit cube
  std::printf("{\"n_lin\": %zu, \"n_bal\": %zu, \"n_elem\": %u, \"n_node\": %u, \"sum_A1\": %.15f, "
              "\"n_coarse\": %zu, \"n_complete_sub\": %zu, \"complete_bal_same\": %d, \"sort_ok\": %d, "
              "\"mat_err\": %.3e, \"diag_err\": %.3e, \"coef_err\": %.3e}\n",
              nlin, bal.size(), da.getElementSize(), da.getNodeSize(), s, coarse.size(), comp.size(), same_ok ? 1 : 0,
              sort_ok ? 1 : 0, mat_err / ymax, diag_err / dmax, coef_err / ymax);
  // error path: a communicator of size 2 is refused
  try {
    std::vector<double> p2 = {0.5, 0.5, 0.5, 0.25, 0.25, 0.25};
    std::vector<MyNode> o2;
    dg::ot::points2Octree(p2, gLens, o2, 3, 30, 1, 2);
    return 3;
  } catch (const dg::cxx::Error &e) {
    if (e.status != DG_ERR_COMM_SIZE) return 4;
  }
  return 0;
}
