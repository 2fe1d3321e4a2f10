// Assembled sparse matrices of the element operators, in CSR form over this
// library's node numbering.
//
//   lapFac K + massFac M   the matrix of dg_matvec: the reference's
//                          CreateAndComputeFullJacobian1
//                          (examples/src/backend/odaJac.C:470-535), the
//                          matrix its -buildFullMatAll / -buildFullCoarseMat
//                          options build (omgJac.C:1333-1459)
//   Dirichlet form         ComputeDirichletJacobian (omgJac.C:383-490):
//                          K + M over interior rows and columns, boundary
//                          rows the identity
//
// Rows are sorted by column; every entry sums the element contributions of
// its row in element order, so the values do not depend on the schedule.
#pragma once

#include "dg_da.cuh"

namespace dg {

struct Csr {
  size_t n_rows = 0;
  size_t nnz = 0;
  int64_t *row_ptr = nullptr;  // n_rows + 1
  uint32_t *col = nullptr;     // nnz
  double *val = nullptr;       // nnz
  unsigned max_row = 0;        // longest row
};

// bdy == nullptr: lap_fac K + mass_fac M, or with coef (2 per element,
// device) each element's own factors (the matrix of Jacobian2MatMult:
// BUILD_FULL_JAC_TYPE2_BLOCK, omgJac.C:1804-1858); bdy given: the Dirichlet
// form of K + M with bdy[v] != 0 marking boundary nodes (factors ignored)
void assemble_csr(Context &ctx, const Mesh &m, const uint8_t *bdy, double lap_fac, double mass_fac, Csr &out,
                  const double *coef = nullptr);
void csr_free(Context &ctx, Csr &c);
// y = A x (FP64), rows split over groups of 4 lanes
void csr_spmv(Context &ctx, const Csr &c, const double *x, double *y);

}  // namespace dg
