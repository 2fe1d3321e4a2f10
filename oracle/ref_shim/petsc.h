/*
 * Header-only stand-in for the handful of PETSc types, macros and Vec/Mat
 * calls that the reference's octree/DA/element-loop sources reference.  Used
 * only to compile the reference into the CPU oracle binary (oracle/_ref).
 * Vec is a plain heap array; Mat is a context holder with the shell
 * operations MATOP_MULT and MATOP_GET_DIAGONAL (the MatShell callbacks of
 * include/dendro_gb300_petsc.hpp are tested through them) and
 * MATOP_MULT_TRANSPOSE (the reference's prolongation shell).  No solver
 * exists here.
 */
#ifndef DG_ORACLE_PETSC_SHIM_H
#define DG_ORACLE_PETSC_SHIM_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>

#include "mpi.h"

typedef int PetscErrorCode;
typedef double PetscScalar;
typedef double PetscReal;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef long long PetscInt64;
typedef int PetscClassId;
typedef int PetscLogEvent;
typedef int PetscLogStage;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef PetscBool PetscTruth;
typedef const char *MatType;
typedef const char *VecType;
typedef const char *KSPType;
typedef const char *PCType;
typedef enum { NOT_SET_VALUES = 0, INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { SCATTER_FORWARD = 0, SCATTER_REVERSE = 1 } ScatterMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { SAME_NONZERO_PATTERN = 0, DIFFERENT_NONZERO_PATTERN = 1 } MatStructure;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_INFINITY = 3 } NormType;
typedef enum {
  MATOP_MULT,
  MATOP_MULT_ADD,
  MATOP_MULT_TRANSPOSE,
  MATOP_MULT_TRANSPOSE_ADD,
  MATOP_GET_DIAGONAL,
  MATOP_DESTROY
} MatOperation;

struct dg_shim_vec {
  size_t n;
  PetscScalar *a;
};
typedef dg_shim_vec *Vec;
struct dg_shim_mat;
typedef dg_shim_mat *Mat;
struct dg_shim_mat {
  void *ctx;
  /* shell operations (MatShellSetOperation) */
  PetscErrorCode (*mult)(Mat, Vec, Vec);
  PetscErrorCode (*diag)(Mat, Vec);
  PetscErrorCode (*multT)(Mat, Vec, Vec);
  const char *type;
  /* the entries of an assembled (non-shell) matrix, by global (row, column) */
  std::map<std::pair<PetscInt, PetscInt>, PetscScalar> *entries;
};
struct dg_shim_opaque {
  int unused;
};
typedef dg_shim_opaque *KSP;
typedef dg_shim_opaque *PC;
typedef dg_shim_opaque *VecScatter;
typedef dg_shim_opaque *IS;
typedef dg_shim_opaque *PetscViewer;
typedef dg_shim_opaque *PetscRandom;
typedef dg_shim_opaque *MatNullSpace;
typedef dg_shim_opaque *PetscObject;

#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_COMM_SELF MPI_COMM_SELF
#define PETSC_NULL 0
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_ERR_ARG_NULL 85
#define PETSC_ERR_SUP 56
#define MATSHELL "shell"
#define MATAIJ "aij"
#define MATSEQAIJ "seqaij"
#define MATMPIAIJ "mpiaij"
#define MATDAAD "daad"
#define MATMFFD "mffd"
#define VECSEQ "seq"
#define VECMPI "mpi"

#define CHKERRQ(e)      \
  do {                  \
    if (e) return (e);  \
  } while (0)
#define SETERRQ(c, e, m) return (e)
#define PetscFunctionBegin
#define PetscFunctionReturn(x) return (x)
#define PetscLogEventBegin(...)
#define PetscLogEventEnd(...)
#define PetscLogFlops(x) 0

inline PetscErrorCode VecCreate(MPI_Comm, Vec *v) {
  *v = new dg_shim_vec{0, nullptr};
  return 0;
}
inline PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt) {
  v->n = (size_t)(n > 0 ? n : 0);
  v->a = (PetscScalar *)std::calloc(v->n ? v->n : 1, sizeof(PetscScalar));
  return 0;
}
inline PetscErrorCode VecSetType(Vec, VecType) { return 0; }
inline PetscErrorCode VecGetLocalSize(Vec v, PetscInt *n) {
  *n = (PetscInt)v->n;
  return 0;
}
inline PetscErrorCode VecGetArray(Vec v, PetscScalar **a) {
  *a = v->a;
  return 0;
}
inline PetscErrorCode VecRestoreArray(Vec, PetscScalar **) { return 0; }
inline PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a) {
  *a = v->a;
  return 0;
}
inline PetscErrorCode VecRestoreArrayRead(Vec, const PetscScalar **) { return 0; }
inline PetscErrorCode VecDestroy(Vec *v) {
  if (*v) {
    std::free((*v)->a);
    delete *v;
    *v = nullptr;
  }
  return 0;
}
inline PetscErrorCode VecZeroEntries(Vec v) {
  std::memset(v->a, 0, v->n * sizeof(PetscScalar));
  return 0;
}
inline PetscErrorCode VecDuplicate(Vec v, Vec *w) {
  VecCreate(MPI_COMM_SELF, w);
  return VecSetSizes(*w, (PetscInt)v->n, PETSC_DETERMINE);
}
/* y = y + alpha x */
inline PetscErrorCode VecAXPY(Vec y, PetscScalar alpha, Vec x) {
  for (size_t i = 0; i < y->n; i++) y->a[i] += alpha * x->a[i];
  return 0;
}
/* w = alpha x + y */
inline PetscErrorCode VecWAXPY(Vec w, PetscScalar alpha, Vec x, Vec y) {
  for (size_t i = 0; i < w->n; i++) w->a[i] = alpha * x->a[i] + y->a[i];
  return 0;
}
inline PetscErrorCode VecSet(Vec v, PetscScalar s) {
  for (size_t i = 0; i < v->n; i++) v->a[i] = s;
  return 0;
}
/* options: string options without a prefix can be set by the caller
 * (dg_shim_options()); integer and real options are never set, so the
 * reference's defaults apply */
inline std::map<std::string, std::string> &dg_shim_options() {
  static std::map<std::string, std::string> opts;
  return opts;
}
inline PetscErrorCode PetscOptionsGetInt(void *, const char *, const char *, PetscInt *, PetscBool *set) {
  if (set) *set = PETSC_FALSE;
  return 0;
}
inline PetscErrorCode PetscOptionsGetReal(void *, const char *, const char *, PetscReal *, PetscBool *set) {
  if (set) *set = PETSC_FALSE;
  return 0;
}
inline PetscErrorCode PetscOptionsGetString(void *, const char *pre, const char *name, char *out, size_t len,
                                            PetscBool *set) {
  auto it = dg_shim_options().find(name);
  const bool found = pre == nullptr && it != dg_shim_options().end() && len > 0;
  if (found) {
    std::strncpy(out, it->second.c_str(), len - 1);
    out[len - 1] = 0;
  }
  if (set) *set = (PetscBool)found;
  return 0;
}
inline PetscErrorCode VecPlaceArray(Vec v, const PetscScalar *a) {
  v->a = (PetscScalar *)a;
  return 0;
}
inline PetscErrorCode VecResetArray(Vec) { return 0; }
inline PetscErrorCode PetscStrcmp(const char *a, const char *b, PetscBool *f) {
  *f = (PetscBool)(std::strcmp(a, b) == 0);
  return 0;
}
inline PetscErrorCode MatCreate(MPI_Comm, Mat *m) {
  *m = new dg_shim_mat{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  return 0;
}
inline PetscErrorCode MatCreateShell(MPI_Comm, PetscInt, PetscInt, PetscInt, PetscInt, void *ctx, Mat *m) {
  *m = new dg_shim_mat{ctx, nullptr, nullptr, nullptr, MATSHELL, nullptr};
  return 0;
}
inline PetscErrorCode MatShellGetContext(Mat m, void *ctx) {
  *(void **)ctx = m->ctx;
  return 0;
}
inline PetscErrorCode MatShellSetOperation(Mat m, MatOperation op, void (*f)(void)) {
  if (op == MATOP_MULT) m->mult = (PetscErrorCode(*)(Mat, Vec, Vec))f;
  if (op == MATOP_GET_DIAGONAL) m->diag = (PetscErrorCode(*)(Mat, Vec))f;
  if (op == MATOP_MULT_TRANSPOSE) m->multT = (PetscErrorCode(*)(Mat, Vec, Vec))f;
  return 0;
}
inline PetscErrorCode MatMult(Mat m, Vec x, Vec y) { return m->mult ? m->mult(m, x, y) : PETSC_ERR_SUP; }
inline PetscErrorCode MatGetDiagonal(Mat m, Vec d) { return m->diag ? m->diag(m, d) : PETSC_ERR_SUP; }
inline PetscErrorCode MatMultTranspose(Mat m, Vec x, Vec y) { return m->multT ? m->multT(m, x, y) : PETSC_ERR_SUP; }
inline PetscErrorCode MatDestroy(Mat *m) {
  if (*m) delete (*m)->entries;
  delete *m;
  *m = nullptr;
  return 0;
}
inline PetscErrorCode MatSetSizes(Mat, PetscInt, PetscInt, PetscInt, PetscInt) { return 0; }
/* the reference asks this of matrices only */
inline PetscErrorCode PetscObjectTypeCompare(PetscObject o, const char *type, PetscBool *same) {
  const dg_shim_mat *m = reinterpret_cast<const dg_shim_mat *>(o);
  *same = (PetscBool)(m && m->type && std::strcmp(m->type, type) == 0);
  return 0;
}
inline PetscErrorCode MatZeroEntries(Mat m) {
  if (m->entries) m->entries->clear();
  return 0;
}
inline PetscErrorCode MatCreateVecs(Mat, Vec *, Vec *) { return PETSC_ERR_SUP; }
inline PetscErrorCode MatSetType(Mat m, MatType t) {
  /* the name may live in the caller's stack: keep a copy */
  static std::map<std::string, int> names;
  m->type = names.emplace(t, 0).first->first.c_str();
  return 0;
}
inline PetscErrorCode MatSeqAIJSetPreallocation(Mat, PetscInt, const PetscInt *) { return 0; }
inline PetscErrorCode MatMPIAIJSetPreallocation(Mat, PetscInt, const PetscInt *, PetscInt, const PetscInt *) {
  return 0;
}
/* records the entries (ADD_VALUES adds, INSERT_VALUES overwrites) */
inline PetscErrorCode MatSetValues(Mat m, PetscInt nr, const PetscInt *rows, PetscInt nc, const PetscInt *cols,
                                   const PetscScalar *v, InsertMode mode) {
  if (!m->entries) m->entries = new std::map<std::pair<PetscInt, PetscInt>, PetscScalar>;
  for (PetscInt i = 0; i < nr; i++)
    for (PetscInt j = 0; j < nc; j++) {
      PetscScalar &e = (*m->entries)[std::make_pair(rows[i], cols[j])];
      e = mode == ADD_VALUES ? e + v[i * nc + j] : v[i * nc + j];
    }
  return 0;
}
inline PetscErrorCode MatZeroRows(Mat, PetscInt, const PetscInt *, PetscScalar, Vec, Vec) { return 0; }
inline PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
inline PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType) { return 0; }

#endif
