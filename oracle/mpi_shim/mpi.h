/*
 * mpi.h -- project-written MPI shim used ONLY to build the reference CPU solver
 * (the oracle under oracle/_ref/) in a machine without an MPI installation.
 *
 * Oracle/test infrastructure: nothing in the cacg_gb300 product links this.
 *
 * Ranks are POSIX threads inside one process (cacg_mpi_run() starts them).
 * Every collective the reference solver path calls is implemented with the
 * semantics of MPI on MPI_COMM_WORLD:
 *   MPI_Allreduce / MPI_Reduce  (SUM, MIN, MAX; DOUBLE, LONG, INT) -- the
 *       reduction is evaluated in rank order 0..np-1 on every rank, so results
 *       are deterministic and identical on all ranks;
 *   MPI_Allgatherv, MPI_Bcast, MPI_Alltoall, MPI_Alltoallv, MPI_Barrier;
 *   MPI_Wtime (CLOCK_MONOTONIC).
 * With one rank every collective degenerates to a copy, which is what a
 * single-rank `mpirun -np 1` run of the reference computes.
 */
#ifndef CACG_MPI_SHIM_H
#define CACG_MPI_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0

#define MPI_DOUBLE 1
#define MPI_LONG 2
#define MPI_INT 3
#define MPI_CHAR 4

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype datatype, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype datatype, MPI_Op op, int root, MPI_Comm comm);
int MPI_Bcast(void *buffer, int count, MPI_Datatype datatype, int root,
              MPI_Comm comm);
int MPI_Allgatherv(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                   void *recvbuf, const int *recvcounts, const int *displs,
                   MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Scatterv(const void *sendbuf, const int *sendcounts, const int *displs,
                 MPI_Datatype sendtype, void *recvbuf, int recvcount,
                 MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Alltoall(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype,
                 MPI_Comm comm);
int MPI_Alltoallv(const void *sendbuf, const int *sendcounts,
                  const int *sdispls, MPI_Datatype sendtype, void *recvbuf,
                  const int *recvcounts, const int *rdispls,
                  MPI_Datatype recvtype, MPI_Comm comm);

/* Shim control: run fn(rank, arg) on np threads acting as MPI ranks. */
typedef void (*cacg_mpi_rank_fn)(int rank, void *arg);
int cacg_mpi_run(int np, cacg_mpi_rank_fn fn, void *arg);

#ifdef __cplusplus
}
#endif
#endif
