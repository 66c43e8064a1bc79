/* Single-process stand-in for <mpi.h>, used only to compile the reference's
 * sources for the oracle's cross-check library (oracle/_ref) and the drop-in
 * adaptor in the compile test.  It declares the MPI names those sources
 * mention; nothing in the cross-check calls them. */
#ifndef TG3_REF_MPI_SHIM_H
#define TG3_REF_MPI_SHIM_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Group;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_COMM_NULL (-1)
#define MPI_SUCCESS 0
#define MPI_SUM 1
#define MPI_IN_PLACE ((void*)1)
#define MPI_INT 1
#define MPI_LONG 2
#define MPI_FLOAT 3
#define MPI_DOUBLE 4
#define MPI_C_BOOL 5
#define MPI_COMPLEX 6
#define MPI_DOUBLE_COMPLEX 7
#ifdef __cplusplus
extern "C" {
#endif
int MPI_Init(int*, char***);
int MPI_Finalize(void);
int MPI_Barrier(MPI_Comm);
int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Ssend(const void*, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*);
int MPI_Get_count(const MPI_Status*, MPI_Datatype, int*);
int MPI_Type_size(MPI_Datatype, int*);
int MPI_Comm_size(MPI_Comm, int*);
int MPI_Comm_rank(MPI_Comm, int*);
int MPI_Comm_group(MPI_Comm, MPI_Group*);
int MPI_Comm_create(MPI_Comm, MPI_Group, MPI_Comm*);
int MPI_Group_incl(MPI_Group, int, const int*, MPI_Group*);
int MPI_Group_free(MPI_Group*);
#ifdef __cplusplus
}
#endif
#endif
