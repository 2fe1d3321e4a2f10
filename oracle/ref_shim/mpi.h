/*
 * Single-rank MPI stand-in used only to compile the reference's own sources
 * into the CPU oracle binary (oracle/_ref).  Test infrastructure: nothing in
 * the product links it.
 *
 * Semantics: one process, rank 0 of a communicator of size 1.  A datatype is
 * represented by its size in bytes, so derived contiguous types compose by
 * multiplication.  Every collective degenerates to a copy from the send
 * buffer to the receive buffer at the rank-0 displacement; point-to-point
 * calls to "self" copy nothing (the reference never needs them at 1 rank).
 */
#ifndef DG_ORACLE_MPI_STUB_H
#define DG_ORACLE_MPI_STUB_H

#include <cstdlib>
#include <cstring>

#define MPI_VERSION 3 /* as an MPI library's mpi.h announces itself */
typedef int MPI_Comm;
typedef long MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Group;
typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
} MPI_Status;
typedef void(MPI_User_function)(void *, void *, int *, MPI_Datatype *);

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 1
#define MPI_COMM_NULL 0
#define MPI_SUCCESS 0
#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3
#define MPI_UNDEFINED (-32766)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

/* datatypes: value == byte size */
#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_SIGNED_CHAR ((MPI_Datatype)sizeof(signed char))
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_UNSIGNED_CHAR ((MPI_Datatype)sizeof(unsigned char))
#define MPI_SHORT ((MPI_Datatype)sizeof(short))
#define MPI_UNSIGNED_SHORT ((MPI_Datatype)sizeof(unsigned short))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_UNSIGNED ((MPI_Datatype)sizeof(unsigned))
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_UNSIGNED_LONG ((MPI_Datatype)sizeof(unsigned long))
#define MPI_LONG_LONG ((MPI_Datatype)sizeof(long long))
#define MPI_LONG_LONG_INT ((MPI_Datatype)sizeof(long long))
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)sizeof(unsigned long long))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_LONG_DOUBLE ((MPI_Datatype)sizeof(long double))
#define MPI_INT64_T ((MPI_Datatype)8)
#define MPI_UINT64_T ((MPI_Datatype)8)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROD 4
#define MPI_LAND 5
#define MPI_LOR 6
#define MPI_BAND 7
#define MPI_BOR 8

static inline size_t dg_mpi_bytes(int count, MPI_Datatype t) {
  return (size_t)count * (size_t)(t > 0 ? t : 1);
}
static inline void dg_mpi_copy(const void *s, void *r, size_t nb) {
  if (s != MPI_IN_PLACE && s != r && nb) std::memmove(r, s, nb);
}

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline double MPI_Wtime() { return 0.0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); return 0; }

inline int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *nt) {
  *nt = (MPI_Datatype)n * (old > 0 ? old : 1);
  return 0;
}
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
inline int MPI_Type_free(MPI_Datatype *) { return 0; }
inline int MPI_Op_create(MPI_User_function *, int, MPI_Op *op) { *op = 100; return 0; }
inline int MPI_Op_free(MPI_Op *) { return 0; }

inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  dg_mpi_copy(s, r, dg_mpi_bytes(n, t));
  return 0;
}
inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  dg_mpi_copy(s, r, dg_mpi_bytes(n, t));
  return 0;
}
inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  dg_mpi_copy(s, r, dg_mpi_bytes(n, t));
  return 0;
}
inline int MPI_Exscan(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Gather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm) {
  dg_mpi_copy(s, r, dg_mpi_bytes(n, t));
  return 0;
}
inline int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm) {
  dg_mpi_copy(s, r, dg_mpi_bytes(n, t));
  return 0;
}
inline int MPI_Allgatherv(const void *s, int n, MPI_Datatype t, void *r, const int *, const int *displs,
                          MPI_Datatype rt, MPI_Comm) {
  dg_mpi_copy(s, (char *)r + dg_mpi_bytes(displs[0], rt), dg_mpi_bytes(n, t));
  return 0;
}
inline int MPI_Alltoall(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm) {
  dg_mpi_copy(s, r, dg_mpi_bytes(n, t));
  return 0;
}
inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r, const int *,
                         const int *rd, MPI_Datatype rt, MPI_Comm) {
  dg_mpi_copy((const char *)s + dg_mpi_bytes(sd[0], st), (char *)r + dg_mpi_bytes(rd[0], rt),
              dg_mpi_bytes(sc[0], st));
  return 0;
}
inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return 0; }
inline int MPI_Issend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return 0; }
inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return 0; }
inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
inline int MPI_Sendrecv(const void *s, int sn, MPI_Datatype st, int, int, void *r, int, MPI_Datatype, int, int,
                        MPI_Comm, MPI_Status *) {
  dg_mpi_copy(s, r, dg_mpi_bytes(sn, st));
  return 0;
}
inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
inline int MPI_Get_count(const MPI_Status *, MPI_Datatype, int *c) { *c = 0; return 0; }
inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm *n) { *n = c; return 0; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *n) { *n = c; return 0; }
inline int MPI_Comm_free(MPI_Comm *) { return 0; }
inline int MPI_Comm_compare(MPI_Comm, MPI_Comm, int *r) { *r = MPI_IDENT; return 0; }
inline int MPI_Comm_group(MPI_Comm, MPI_Group *g) { *g = 1; return 0; }
inline int MPI_Group_incl(MPI_Group, int, const int *, MPI_Group *n) { *n = 1; return 0; }
inline int MPI_Group_excl(MPI_Group, int, const int *, MPI_Group *n) { *n = 1; return 0; }
inline int MPI_Group_free(MPI_Group *) { return 0; }
inline int MPI_Comm_create(MPI_Comm c, MPI_Group, MPI_Comm *n) { *n = c; return 0; }

#endif
