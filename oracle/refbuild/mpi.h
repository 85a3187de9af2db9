/* mpi.h -- single-process stand-in for the MPI interface that the reference
 * PNFFT sources use (TEST INFRASTRUCTURE: only for building the reference's
 * own C code into oracle/_ref/ to pin the oracle; never linked into the
 * product).  One rank, a 1x1x1 Cartesian communicator; collectives copy. */
#ifndef ORACLE_REFBUILD_MPI_H
#define ORACLE_REFBUILD_MPI_H
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_SUCCESS 0

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)2)
#define MPI_UNSIGNED ((MPI_Datatype)3)
#define MPI_LONG ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)5)
#define MPI_DOUBLE ((MPI_Datatype)6)
#define MPI_LONG_DOUBLE ((MPI_Datatype)7)
#define MPI_LONG_LONG ((MPI_Datatype)8)

#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm *newcomm);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Cartdim_get(MPI_Comm comm, int *ndims);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int *dims, int *periods, int *coords);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
double MPI_Wtime(void);
#endif
