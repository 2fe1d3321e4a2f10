// Geometric multigrid on octree meshes (the reference's omg module at one
// rank) for -lap(u) + u = f with u = 0 on the boundary of the unit cube:
// level hierarchy by coarsen + balance, Dirichlet element operators, the
// inter-grid transfers, a damped-Jacobi V-cycle and an FP64 preconditioned
// CG whose V-cycle runs in FP32 or FP64.
#pragma once

#include <vector>

#include "dg_da.cuh"

namespace dg {

struct MGLevel {
  Octree oct;  // balanced octree of this level (owned)
  Mesh mesh;
  uint8_t *bdy = nullptr;  // 1 for nodes on the domain boundary
  double *dinv64 = nullptr;  // inverse diagonal of the Dirichlet operator
  float *dinv32 = nullptr;
  // prolongation from the next coarser level onto this level's nodes, the
  // nonzero weights only, packed per chunk of 32 nodes (256 entries per
  // chunk): node v takes coarse nodes tid[e] with weights tw[e] / 64 for
  // e = (v / 32) * 256 + (tpos[v] & 255) + j, j < tpos[v] >> 8, in the
  // coarse element's vertex order (every weight is a multiple of 1/64)
  uint16_t *tpos = nullptr;
  uint32_t *tid = nullptr;
  uint8_t *tw = nullptr;
  size_t tnnz = 0;  // nonzero weights (the tables' algorithmic size)
};

struct MG {
  std::vector<MGLevel> lv;  // 0 = finest
  size_t nc = 0;            // nodes of the coarsest level
  double *ca64 = nullptr;    // the coarsest level's assembled operator (dense, FP64)
  float *cinv32 = nullptr;   // its inverse in FP32 (refined in FP64 when the FP64 V-cycle applies it)
  double omega = 0.667;  // Jacobi damping (bin/options:190)
  int nu_pre = 2, nu_post = 2;
  // CG operator with an FP32 V-cycle: 48 (the default) applies A p in
  // double-single arithmetic on FP64 vectors (about 2^-46 relative per
  // element row); 64 in FP64; 32 in FP32, with the recurrence residual
  // replaced by the FP64 residual b - A x whenever it has fallen by
  // reliable_delta since the last replacement (and before stopping)
  int cg_operator = 48;
  double reliable_delta = 1e-3;
};

struct MGResult {
  int iterations = 0;
  double relres = 0.0;  // final ||b - A x|| / ||b|| in FP64
};

// levels from a balanced octree: coarsen (src/coarsen.cpp:53) + balance
// until a level has at most max_coarse_elem elements
// (examples/src/omg/blockDiag.cpp:1384-1425 coarsens to < 500 octants)
void mg_setup(Context &ctx, const Octree &fine, size_t max_coarse_elem, MG &mg);
void mg_free(Context &ctx, MG &mg);
// in-place FP32 inverse of an SPD n x n row-major matrix on the device
// (block Gauss-Jordan, rank-64 updates on the tensor cores; dg_coarse.cu)
void coarse_inverse(Context &ctx, float *X, size_t n);

// PCG to ||r|| / ||b|| <= rtol; residual, dot products and updates in FP64,
// the V-cycle preconditioner in FP32 (precision 32) or FP64 (precision 64)
void mg_solve(Context &ctx, MG &mg, const double *b, double *x, int precision, double rtol, int maxit, MGResult &res);

// building blocks (level operators), exposed for tests and callers
template <typename T>
void dirichlet_matvec(Context &ctx, const MGLevel &L, const T *x, T *y);  // DirichletJacobianMatMult
// the same operator on FP64 vectors in double-single arithmetic (FP32
// pairs, about 2^-46 relative per element row; the FP64 loop where a mesh
// has no run tables)
// (scale_exp: x is multiplied by 2^scale_exp inside the loop, chosen so
// that x is of order one; DS_SCALE_AUTO takes it from x's largest entry)
constexpr int DS_SCALE_AUTO = -100000;
void dirichlet_matvec_ds(Context &ctx, const MGLevel &L, const double *x, double *y, int scale_exp = DS_SCALE_AUTO);
// DirichletJacobianMatGetDiagonal (omgJac.C:1111): 1 on boundary nodes
void dirichlet_diagonal(Context &ctx, const MGLevel &L, double *diag);
template <typename T>
void mg_restrict(Context &ctx, const MG &mg, int fine_level, const T *rf, T *bc);  // restrictMatVecType1
template <typename T>
void mg_prolong(Context &ctx, const MG &mg, int fine_level, const T *xc, T *xf);  // prolongMatVecType1 (xf = P xc)
template <typename T>
void mg_vcycle(Context &ctx, const MG &mg, const T *b, T *x);  // one V(nu_pre, nu_post) from x = 0

}  // namespace dg
