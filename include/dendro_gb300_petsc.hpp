// dendro_gb300_petsc.hpp — the reference's PETSc MatShell callbacks over the
// GPU operators of dendro_gb300.hpp (header only).  Include PETSc's header
// (petsc.h, double-precision real scalars) before this one.
//
// A caller that builds its shell matrices as the reference's examples do
//   MatCreateShell(comm, n, n, N, N, data, &J);
//   MatShellSetOperation(J, MATOP_MULT, (void (*)(void))Jacobian1MatMult);
//   MatShellSetOperation(J, MATOP_GET_DIAGONAL, (void (*)(void))Jacobian1MatGetDiagonal);
// keeps doing so; the shell context becomes this header's Jac1MFreeData
// (same fields as examples/include/odaJac.h:20, with da an
// dg::ot::DA) or, for the multigrid level operators, DirichletJacCtx.
// The callbacks read the Vec arrays on the host and run the element loop on
// the GPU (a host-device copy each way per call).
//
// Reference callbacks replaced:
//   Jacobian1MatMult, Jacobian1MatGetDiagonal, MassMatMult
//     examples/include/odaJac.h:35-40, examples/src/backend/odaJac.C:160-222,294-377,399
//   DirichletJacobianMatMult, DirichletJacobianMatGetDiagonal
//     examples/src/backend/omgJac.C:958-1057,1111
#ifndef DENDRO_GB300_PETSC_HPP
#define DENDRO_GB300_PETSC_HPP

#include <type_traits>

#include "dendro_gb300.hpp"

#ifndef PETSC_ERR_LIB
#define PETSC_ERR_LIB 76 /* PETSc's "error in library called by PETSc" */
#endif

namespace dg {
namespace petsc {

static_assert(std::is_same<PetscScalar, double>::value, "the callbacks need a double-precision real PETSc");

// MatShell context of Jacobian1MatMult / Jacobian1MatGetDiagonal /
// MassMatMult (examples/include/odaJac.h:20).  lapFac and massFac stand for
// the -lapMatPropFac / -massMatPropFac options the reference reads
// (odaJac.C:302-306); both default to 1.
struct Jac1MFreeData {
  ::dg::ot::DA *da = nullptr;
  bool isFinestLevel = true;
  Mat Jmat_private = nullptr;
  Vec inTmp = nullptr;
  Vec outTmp = nullptr;
  double lapFac = 1.0;
  double massFac = 1.0;
};

// MatShell context of the multigrid level operator: the hierarchy and the
// level (the reference passes its ot::DAMG of that level, omgJac.C:962).
struct DirichletJacCtx {
  const ::dg::omg::MultiGrid *mg = nullptr;
  size_t level = 0;
};

namespace detail {
// y = op(x) over host Vec arrays; library errors become PETSC_ERR_LIB
template <class Op>
inline PetscErrorCode apply(Vec in, Vec out, Op op) {
  const PetscScalar *x = nullptr;
  PetscScalar *y = nullptr;
  PetscErrorCode ierr = VecGetArrayRead(in, &x);
  CHKERRQ(ierr);
  ierr = VecGetArray(out, &y);
  CHKERRQ(ierr);
  PetscErrorCode rc = 0;
  try {
    op(x, y);
  } catch (const ::dg::cxx::Error &) {
    rc = PETSC_ERR_LIB;
  }
  ierr = VecRestoreArray(out, &y);
  CHKERRQ(ierr);
  ierr = VecRestoreArrayRead(in, &x);
  CHKERRQ(ierr);
  return rc;
}
template <class Op>
inline PetscErrorCode fill(Vec v, Op op) {
  PetscScalar *d = nullptr;
  PetscErrorCode ierr = VecGetArray(v, &d);
  CHKERRQ(ierr);
  PetscErrorCode rc = 0;
  try {
    op(d);
  } catch (const ::dg::cxx::Error &) {
    rc = PETSC_ERR_LIB;
  }
  ierr = VecRestoreArray(v, &d);
  CHKERRQ(ierr);
  return rc;
}
}  // namespace detail

// out = (lapFac L + massFac M) in  (odaJac.C:294)
inline PetscErrorCode Jacobian1MatMult(Mat J, Vec in, Vec out) {
  Jac1MFreeData *data = nullptr;
  PetscErrorCode ierr = MatShellGetContext(J, (void **)&data);
  CHKERRQ(ierr);
  return detail::apply(in, out, [&](const double *x, double *y) { data->da->matVec(x, y, data->lapFac, data->massFac); });
}

// out = M in  (odaJac.C:399)
inline PetscErrorCode MassMatMult(Mat J, Vec in, Vec out) {
  Jac1MFreeData *data = nullptr;
  PetscErrorCode ierr = MatShellGetContext(J, (void **)&data);
  CHKERRQ(ierr);
  return detail::apply(in, out, [&](const double *x, double *y) { data->da->matVec(x, y, 0.0, data->massFac); });
}

// diag = diagonal of lapFac L + massFac M  (odaJac.C:160-222)
inline PetscErrorCode Jacobian1MatGetDiagonal(Mat J, Vec diag) {
  Jac1MFreeData *data = nullptr;
  PetscErrorCode ierr = MatShellGetContext(J, (void **)&data);
  CHKERRQ(ierr);
  return detail::fill(diag, [&](double *d) { data->da->getDiagonal(d, data->lapFac, data->massFac); });
}

// the level's Dirichlet operator: boundary rows identity, boundary columns
// skipped (omgJac.C:958-1057)
inline PetscErrorCode DirichletJacobianMatMult(Mat J, Vec in, Vec out) {
  DirichletJacCtx *c = nullptr;
  PetscErrorCode ierr = MatShellGetContext(J, (void **)&c);
  CHKERRQ(ierr);
  return detail::apply(in, out, [&](const double *x, double *y) { c->mg->matVec(c->level, x, y); });
}

// its diagonal, 1 on boundary nodes (omgJac.C:1111)
inline PetscErrorCode DirichletJacobianMatGetDiagonal(Mat J, Vec diag) {
  DirichletJacCtx *c = nullptr;
  PetscErrorCode ierr = MatShellGetContext(J, (void **)&c);
  CHKERRQ(ierr);
  return detail::fill(diag, [&](double *d) { c->mg->getDiagonal(c->level, d); });
}

}  // namespace petsc
}  // namespace dg

#ifndef DG_NO_REFERENCE_NAMESPACES
using dg::petsc::DirichletJacobianMatGetDiagonal;
using dg::petsc::DirichletJacobianMatMult;
using dg::petsc::Jac1MFreeData;
using dg::petsc::Jacobian1MatGetDiagonal;
using dg::petsc::Jacobian1MatMult;
using dg::petsc::MassMatMult;
#endif

#endif
