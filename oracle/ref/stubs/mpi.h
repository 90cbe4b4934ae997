/* Single-rank stand-in for <mpi.h>, used only to compile the reference
 * unbinding sources (src/subhalo_unbind.cpp and the files it needs) into the
 * oracle/_ref harness.  None of these functions is reached by Subhalo_t::Unbind;
 * they exist so that the translation units which declare MPI helpers compile.
 * Test infrastructure only. */
#ifndef HBTU_STUB_MPI_H
#define HBTU_STUB_MPI_H
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef long MPI_Aint;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_VERSION 3
#define MPI_COMM_WORLD 0
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_LONG 3
#define MPI_FLOAT 4
#define MPI_DOUBLE 5
#define MPI_LONG_INT 6
#define MPI_2INT 7
#define MPI_UNSIGNED 8
#define MPI_LONG_LONG 9
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_IN_PLACE ((void *)1)
#define MPI_BOTTOM ((void *)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Get_processor_name(char *name, int *len)
{ strcpy(name, "stub"); *len = 4; return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Finalized(int *f) { *f = 0; return 0; }
static inline int MPI_Type_free(MPI_Datatype *) { return 0; }
static inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
static inline int MPI_Get_address(const void *p, MPI_Aint *a) { *a = (MPI_Aint)p; return 0; }
static inline int MPI_Type_create_hindexed(int, const int *, const MPI_Aint *, MPI_Datatype, MPI_Datatype *t)
{ *t = 0; return 0; }
static inline int MPI_Type_create_struct(int, const int *, const MPI_Aint *, const MPI_Datatype *, MPI_Datatype *t)
{ *t = 0; return 0; }
static inline int MPI_Type_create_resized(MPI_Datatype, MPI_Aint, MPI_Aint, MPI_Datatype *t)
{ *t = 0; return 0; }
static inline int MPI_Type_contiguous(int, MPI_Datatype, MPI_Datatype *t) { *t = 0; return 0; }
static inline int MPI_Alltoall(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm) { return 0; }
static inline int MPI_Alltoallv(const void *, const int *, const int *, MPI_Datatype, void *, const int *,
                                const int *, MPI_Datatype, MPI_Comm) { return 0; }
static inline int MPI_Alltoallw(const void *, const int *, const int *, const MPI_Datatype *, void *,
                                const int *, const int *, const MPI_Datatype *, MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void *, void *, int, MPI_Datatype, MPI_Op, int, MPI_Comm) { return 0; }
static inline int MPI_Allgather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm) { return 0; }
static inline int MPI_Gather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Scan(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
#endif
