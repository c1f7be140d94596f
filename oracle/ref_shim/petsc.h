/*
 * Minimal stand-in for the PETSc/MPI declarations that the reference's
 * per-cell operators, grid loops, boundary loops and checkpoint schedule
 * use, so that those reference sources compile unmodified for the oracle
 * build (oracle/_ref).  Types and macros only; a Vec is a plain array.
 * Written for this project; it is not PETSc.
 */
#ifndef LBMGPU_REF_PETSC_SHIM_H
#define LBMGPU_REF_PETSC_SHIM_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <type_traits>
#include <utility>
#include <vector>

typedef double PetscScalar;
typedef double PetscReal;
typedef int PetscInt;
typedef int PetscErrorCode;
typedef int PetscMPIInt;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef int MPI_Comm;

#define MPI_COMM_NULL 0
#define PETSC_COMM_SELF 0
#define PETSC_COMM_WORLD 0
#define PETSC_RESTRICT __restrict__
#define PetscLikely(x) (x)
#define PetscUnlikely(x) (x)
#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscFunctionBeginUser
#define PetscFunctionReturn(x) return (x)
#define PETSC_ERR_SUP 56
#define PETSC_ERR_MEM 55
#define PETSC_ERROR_INITIAL 1
#define PETSC_FUNCTION_NAME_CXX __func__
#define SETERRQ(c, n, s) return (n)
#define SETERRQ1(c, n, s, a) return (n)
#define SETERRQ2(c, n, s, a, b) return (n)
#define CHKERRQ(x) \
  do {             \
    if (x) return (x); \
  } while (0)
#define CHKERRABORT(c, x) \
  do {                    \
    if (x) std::abort();  \
  } while (0)

inline PetscErrorCode PetscError(MPI_Comm, int, const char*, const char*, int n, int,
                                 const char*, ...) {
  return n;
}

struct _p_Vec {
  std::vector<PetscScalar> v;
};
typedef _p_Vec* Vec;
typedef void* PetscObject;

inline PetscErrorCode PetscObjectGetComm(PetscObject, MPI_Comm* c) {
  *c = 0;
  return 0;
}
template <class T>
inline PetscErrorCode PetscMalloc1(PetscInt n, T** p) {
  *p = new T[n > 0 ? n : 1];
  return 0;
}
template <class T>
inline PetscErrorCode PetscFree(T*& p) {
  delete[] p;
  p = nullptr;
  return 0;
}
inline PetscErrorCode VecCopy(Vec a, Vec b) {
  b->v = a->v;
  return 0;
}
inline PetscErrorCode VecDuplicateVecs(Vec a, PetscInt n, Vec** out) {
  *out = new Vec[n];
  for (PetscInt i = 0; i < n; ++i) {
    (*out)[i] = new _p_Vec;
    (*out)[i]->v.assign(a->v.size(), 0.);
  }
  return 0;
}
inline PetscErrorCode VecDestroyVecs(PetscInt n, Vec** vs) {
  for (PetscInt i = 0; i < n; ++i) delete (*vs)[i];
  delete[] * vs;
  *vs = nullptr;
  return 0;
}

/* One-rank vector algebra used by the reference's MMA (topOpt/MMA.cc). */
#define MPIU_SCALAR 0
#define MPI_SUM 1
#define MPI_MAX 2
inline int MPI_Allreduce(const void* in, void* out, int n, int, int, MPI_Comm) {
  if (in != out) std::memmove(out, in, sizeof(PetscScalar) * (size_t)n);
  return 0;
}
#define PetscAbsReal(x) std::fabs(x)
inline PetscErrorCode PetscPrintf(MPI_Comm, const char*, ...) { return 0; }
inline PetscErrorCode PetscErrorPrintf(const char*, ...) { return 0; }
inline PetscErrorCode VecDuplicate(Vec a, Vec* out) {
  *out = new _p_Vec;
  (*out)->v.assign(a->v.size(), 0.);
  return 0;
}
inline PetscErrorCode VecDestroy(Vec* a) {
  delete *a;
  *a = nullptr;
  return 0;
}
inline PetscErrorCode VecGetLocalSize(Vec a, PetscInt* n) {
  *n = (PetscInt)a->v.size();
  return 0;
}
inline PetscErrorCode VecGetSize(Vec a, PetscInt* n) { return VecGetLocalSize(a, n); }
inline PetscErrorCode VecGetArray(Vec a, PetscScalar** p) {
  *p = a->v.data();
  return 0;
}
inline PetscErrorCode VecRestoreArray(Vec, PetscScalar** p) {
  *p = nullptr;
  return 0;
}
inline PetscErrorCode VecGetArrayRead(Vec a, const PetscScalar** p) {
  *p = a->v.data();
  return 0;
}
inline PetscErrorCode VecRestoreArrayRead(Vec, const PetscScalar** p) {
  *p = nullptr;
  return 0;
}
inline PetscErrorCode VecGetArrays(const Vec* a, PetscInt n, PetscScalar*** p) {
  *p = new PetscScalar*[n > 0 ? n : 1];
  for (PetscInt i = 0; i < n; ++i) (*p)[i] = a[i]->v.data();
  return 0;
}
inline PetscErrorCode VecRestoreArrays(const Vec*, PetscInt, PetscScalar*** p) {
  delete[] * p;
  *p = nullptr;
  return 0;
}
inline PetscErrorCode VecSet(Vec a, PetscScalar v) {
  for (auto& x : a->v) x = v;
  return 0;
}
/* y = alpha x + y */
inline PetscErrorCode VecAXPY(Vec y, PetscScalar alpha, Vec x) {
  for (size_t i = 0; i < y->v.size(); ++i) y->v[i] = alpha * x->v[i] + y->v[i];
  return 0;
}
/* z = alpha x + beta y + gamma z */
inline PetscErrorCode VecAXPBYPCZ(Vec z, PetscScalar alpha, PetscScalar beta, PetscScalar gamma,
                                  Vec x, Vec y) {
  for (size_t i = 0; i < z->v.size(); ++i)
    z->v[i] = alpha * x->v[i] + beta * y->v[i] + gamma * z->v[i];
  return 0;
}

#endif
