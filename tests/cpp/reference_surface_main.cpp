// A caller written against the reference's own API surface, compiled with an
// MPI header (MPI_Comm parameters) and a PETSc header (MatShell callbacks):
// here the single-rank stand-ins of oracle/ref_shim.  Uses the reference's
// namespaces (ot::, par::, SFC::parSort::, omg::) through
// include/dendro_gb300_petsc.hpp.  Driven by tests/test_gpu_cpp_dropin.py.
//
//   reference_surface_main POINTS OUT_PREFIX
// reads FP64 points (u64 n, then 3n doubles) and writes
//   OUT_PREFIX.bal    balanceOctree(incCorner = true)  {x,y,z,level} records
//   OUT_PREFIX.bal18  balanceOctree(incCorner = false)
//   OUT_PREFIX.elem   per element, from the DA loop: x y z, level | child << 8 |
//                     hmask << 16 | etype << 24, then the 8 node coordinates
//                     (records as the reference driver writes them)
//   OUT_PREFIX.sorted SFC_treeSort(TS_REMOVE_DUPLICATES) of a shuffled,
//                     repeated copy of the balanced octree plus ancestors
// and prints a JSON line of checks.
#include <mpi.h>
#include <petsc.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "dendro_gb300_petsc.hpp"

struct Node {
  unsigned x, y, z, lev, md;
  Node(unsigned x_, unsigned y_, unsigned z_, unsigned l_, unsigned /*dim*/, unsigned maxDepth)
      : x(x_), y(y_), z(z_), lev(l_), md(maxDepth) {}
  unsigned getMaxDepth() const { return md; }
  unsigned getX() const { return x; }
  unsigned getY() const { return y; }
  unsigned getZ() const { return z; }
  unsigned getLevel() const { return lev; }
};

static void write_nodes(const char *path, const std::vector<Node> &v) {
  FILE *g = std::fopen(path, "wb");
  uint64_t n = v.size();
  std::fwrite(&n, 8, 1, g);
  for (auto &o : v) {
    uint32_t r[4] = {o.x, o.y, o.z, o.lev};
    std::fwrite(r, 4, 4, g);
  }
  std::fclose(g);
}

static Vec make_vec(size_t n, const double *v) {
  Vec x;
  VecCreate(MPI_COMM_WORLD, &x);
  VecSetSizes(x, (PetscInt)n, PETSC_DECIDE);
  VecSetType(x, VECSEQ);
  PetscScalar *a;
  VecGetArray(x, &a);
  for (size_t i = 0; i < n; i++) a[i] = v ? v[i] : 0.0;
  VecRestoreArray(x, &a);
  return x;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  uint64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) return 2;
  std::vector<double> pts(3 * n);
  if (std::fread(pts.data(), 8, 3 * n, f) != 3 * n) return 2;
  std::fclose(f);
  const std::string pre = argv[2];
  double gLens[3] = {1.0, 1.0, 1.0};
  MPI_Comm comm = MPI_COMM_WORLD, newComm;
  bool active = false;

  std::vector<Node> lin, bal, lin2, bal18;
  ot::points2Octree(pts, gLens, lin, 3, 30, 1, comm);
  lin2 = lin;
  ot::balanceOctree(lin, bal, 3, 30, true, comm, &newComm, &active);
  ot::balanceOctree(lin2, bal18, 3, 30, false, comm);
  write_nodes((pre + ".bal").c_str(), bal);
  write_nodes((pre + ".bal18").c_str(), bal18);

  // ---- the DA's element loop, as the reference's drivers write it ----
  std::vector<Node> balCopy = bal;
  ot::DA da(balCopy, comm, comm, 0.3, false);
  const unsigned maxD = da.getMaxDepth();
  std::vector<uint32_t> xyz = da.getNodeCoordinates();
  std::vector<double> cnt;
  da.createVector(cnt, false, false, 1);
  double *cntArr = nullptr;
  da.vecGetBuffer(cnt, cntArr, false, false, false, 1);
  std::vector<uint32_t> rec;
  double volume = 0.0;
  size_t nel = 0;
  for (da.init<ot::DA_FLAGS::ALL>(); da.curr() < da.end<ot::DA_FLAGS::ALL>(); da.next<ot::DA_FLAGS::ALL>()) {
    ot::Point pt = da.getCurrentOffset();
    unsigned lev = da.getLevel(da.curr());
    unsigned idx[8];
    da.getNodeIndices(idx);
    unsigned char cn = da.getChildNumber();
    unsigned char hm = da.getHangingNodeIndex(da.curr());
    unsigned char et = da.getElementType(da.curr());
    rec.push_back(pt.xint());
    rec.push_back(pt.yint());
    rec.push_back(pt.zint());
    rec.push_back(lev | (cn << 8) | (hm << 16) | ((unsigned)et << 24));
    for (int k = 0; k < 8; k++) {
      for (int a = 0; a < 3; a++) rec.push_back(xyz[3 * idx[k] + a]);
      cntArr[idx[k]] += 1.0;
    }
    const double h = std::ldexp(1.0, -(int)(lev - 1));  // element side in units of the domain
    volume += h * h * h;
    nel++;
  }
  da.vecRestoreBuffer(cnt, cntArr, false, false, false, 1);
  size_t dep = 0;
  for (da.init<ot::DA_FLAGS::DEPENDENT>(); da.curr() < da.end<ot::DA_FLAGS::DEPENDENT>();
       da.next<ot::DA_FLAGS::DEPENDENT>())
    dep++;
  {
    FILE *g = std::fopen((pre + ".elem").c_str(), "wb");
    uint64_t ne = nel;
    std::fwrite(&ne, 8, 1, g);
    std::fwrite(rec.data(), 4, rec.size(), g);
    std::fclose(g);
  }
  double cnt_total = 0;
  for (double c : cnt) cnt_total += c;

  // ---- MatShell callbacks against the direct calls ----
  const size_t nn = da.getNodeSize();
  std::vector<double> xin(nn), ydirect, ddirect;
  for (size_t i = 0; i < nn; i++) {
    double cx = xyz[3 * i] / 1073741824.0, cy = xyz[3 * i + 1] / 1073741824.0, cz = xyz[3 * i + 2] / 1073741824.0;
    xin[i] = std::sin(3 * cx) * std::cos(2 * cy) + cz * cz;
  }
  da.matVec(xin, ydirect, 1.0, 1.0);
  da.getDiagonal(ddirect);
  Jac1MFreeData data;
  data.da = &da;
  Mat J;
  MatCreateShell(comm, (PetscInt)nn, (PetscInt)nn, (PetscInt)nn, (PetscInt)nn, &data, &J);
  MatShellSetOperation(J, MATOP_MULT, (void (*)(void))Jacobian1MatMult);
  MatShellSetOperation(J, MATOP_GET_DIAGONAL, (void (*)(void))Jacobian1MatGetDiagonal);
  Vec vx = make_vec(nn, xin.data()), vy = make_vec(nn, nullptr), vd = make_vec(nn, nullptr);
  PetscErrorCode e1 = MatMult(J, vx, vy);
  PetscErrorCode e2 = MatGetDiagonal(J, vd);
  double shell_err = 0, diag_err = 0, ymax = 0;
  for (size_t i = 0; i < nn; i++) {
    shell_err = std::max(shell_err, std::abs(vy->a[i] - ydirect[i]));
    diag_err = std::max(diag_err, std::abs(vd->a[i] - ddirect[i]));
    ymax = std::max(ymax, std::abs(ydirect[i]));
  }
  // mass only: M 1 sums to the volume of the unit cube
  MatShellSetOperation(J, MATOP_MULT, (void (*)(void))MassMatMult);
  std::vector<double> ones(nn, 1.0);
  Vec v1 = make_vec(nn, ones.data());
  PetscErrorCode e3 = MatMult(J, v1, vy);
  double mass_sum = 0;
  for (size_t i = 0; i < nn; i++) mass_sum += vy->a[i];

  // ---- the multigrid level operator through its shell ----
  omg::MultiGrid mg(bal, 30, 512);
  dg::petsc::DirichletJacCtx dctx;
  dctx.mg = &mg;
  dctx.level = 0;
  Mat JD;
  MatCreateShell(comm, (PetscInt)nn, (PetscInt)nn, (PetscInt)nn, (PetscInt)nn, &dctx, &JD);
  MatShellSetOperation(JD, MATOP_MULT, (void (*)(void))DirichletJacobianMatMult);
  MatShellSetOperation(JD, MATOP_GET_DIAGONAL, (void (*)(void))DirichletJacobianMatGetDiagonal);
  std::vector<double> ymg(mg.nodes(0)), dmg(mg.nodes(0));
  mg.matVec(0, xin.data(), ymg.data());
  mg.getDiagonal(0, dmg.data());
  PetscErrorCode e4 = MatMult(JD, vx, vy);
  PetscErrorCode e5 = MatGetDiagonal(JD, vd);
  double dir_err = 0, dirdiag_err = 0;
  for (size_t i = 0; i < nn; i++) {
    dir_err = std::max(dir_err, std::abs(vy->a[i] - ymg[i]));
    dirdiag_err = std::max(dirdiag_err, std::abs(vd->a[i] - dmg[i]));
  }

  // ---- SFC_treeSort: shuffled, repeated, with ancestors ----
  std::vector<Node> messy;
  for (size_t i = 0; i < bal.size(); i++) messy.push_back(bal[(i * 7919) % bal.size()]);
  for (size_t i = 0; i < bal.size(); i += 3) messy.push_back(bal[i]);
  for (size_t i = 0; i < bal.size(); i += 97) {
    const Node &o = bal[i];
    if (o.lev > 2) {
      unsigned la = o.lev - 2, m = ~((1u << (30 - la)) - 1);
      messy.push_back(Node(o.x & m, o.y & m, o.z & m, la, 3, 30));
    }
  }
  std::vector<Node> sorted, unusedC, unusedB;
  const size_t nmessy = messy.size();
  Node root(0, 0, 0, 0, 3, 30);
  SFC::parSort::SFC_treeSort(messy, sorted, unusedC, unusedB, 0.1, 30, root, 0, 1, TS_REMOVE_DUPLICATES, 16, comm);
  write_nodes((pre + ".sorted").c_str(), sorted);
  bool inplace_sorted = messy.size() == nmessy;
  // par::sampleSort of the same input agrees with the in-place tree sort
  std::vector<Node> again = messy, viaSample;
  par::sampleSort(again, viaSample, comm);
  for (size_t i = 0; inplace_sorted && i < messy.size(); i++)
    inplace_sorted = messy[i].x == viaSample[i].x && messy[i].y == viaSample[i].y && messy[i].z == viaSample[i].z &&
                     messy[i].lev == viaSample[i].lev;

  std::printf(
      "{\"n_bal\": %zu, \"n_bal18\": %zu, \"active\": %d, \"n_elem_loop\": %zu, \"dependent_elems\": %zu, "
      "\"maxD\": %u, \"volume\": %.17g, \"node_refs\": %.1f, \"shell_err\": %.3e, \"diag_err\": %.3e, "
      "\"ymax\": %.6e, \"mass_sum\": %.15f, \"dir_err\": %.3e, \"dirdiag_err\": %.3e, \"petsc_rc\": %d, "
      "\"mg_levels\": %zu, \"n_messy\": %zu, \"n_sorted\": %zu, \"inplace_sorted\": %d}\n",
      bal.size(), bal18.size(), active ? 1 : 0, nel, dep, maxD, volume, cnt_total, shell_err, diag_err, ymax,
      mass_sum, dir_err, dirdiag_err, (int)(e1 | e2 | e3 | e4 | e5), mg.levels(), nmessy, sorted.size(),
      inplace_sorted ? 1 : 0);
  VecDestroy(&vx);
  VecDestroy(&vy);
  VecDestroy(&vd);
  VecDestroy(&v1);
  MatDestroy(&J);
  MatDestroy(&JD);
  return 0;
}
