/*
 * Fake <mpi.h> for running the drop-in adaptor in a test without MPI.  TEST
 * INFRASTRUCTURE.  The driver defines the functions: the hemisphere behaves
 * as tg3_fake_ranks ranks that all hold the same data, so a sum over it
 * multiplies in place by that count, and every call is counted.
 */
#ifndef TG3_TEST_FAKE_MPI_H
#define TG3_TEST_FAKE_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_SUCCESS 0
#define MPI_SUM 1
#define MPI_FLOAT 3
#define MPI_IN_PLACE ((void*)1)
#ifdef __cplusplus
extern "C" {
#endif
int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
#ifdef __cplusplus
}
#endif
#endif
