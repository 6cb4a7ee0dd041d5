/*
 * mpi_threads.c -- project-written MPI shim: MPI ranks as POSIX threads.
 *
 * Oracle/test infrastructure only (see mpi.h).  Each collective publishes the
 * caller's buffer pointer in a per-rank slot, meets the other ranks at a
 * barrier, reads what it needs from the other ranks' slots, and meets them at
 * a second barrier so that no rank returns (and reuses or frees its buffer)
 * while another rank is still reading it.
 */
#include "mpi.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define CACG_MPI_MAX_RANKS 256

typedef struct {
    const void *send;
    void *recv;
    const int *counts;
    const int *displs;
    const int *rcounts;
    const int *rdispls;
    int count;
} slot_t;

static int g_np = 1;
static pthread_barrier_t g_bar;
static slot_t g_slot[CACG_MPI_MAX_RANKS];
static __thread int t_rank = 0;

static size_t type_size(MPI_Datatype t) {
    switch (t) {
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG: return sizeof(long);
    case MPI_INT: return sizeof(int);
    case MPI_CHAR: return 1;
    default:
        fprintf(stderr, "mpi shim: unsupported datatype %d\n", t);
        abort();
    }
}

static void bar(void) {
    if (g_np > 1) pthread_barrier_wait(&g_bar);
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = t_rank; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = g_np; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm c) { (void)c; bar(); return MPI_SUCCESS; }

double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#define REDUCE_LOOP(T)                                                        \
    do {                                                                      \
        T *out = (T *)recvbuf;                                                \
        for (int i = 0; i < count; i++) {                                     \
            T acc = ((const T *)g_slot[0].send)[i];                           \
            for (int r = 1; r < g_np; r++) {                                  \
                T v = ((const T *)g_slot[r].send)[i];                         \
                if (op == MPI_SUM) acc = acc + v;                             \
                else if (op == MPI_MIN) acc = (v < acc) ? v : acc;            \
                else acc = (v > acc) ? v : acc;                               \
            }                                                                 \
            out[i] = acc;                                                     \
        }                                                                     \
    } while (0)

static void reduce_into(void *recvbuf, int count, MPI_Datatype dt, MPI_Op op) {
    if (dt == MPI_DOUBLE) REDUCE_LOOP(double);
    else if (dt == MPI_LONG) REDUCE_LOOP(long);
    else if (dt == MPI_INT) REDUCE_LOOP(int);
    else { fprintf(stderr, "mpi shim: bad reduce type\n"); abort(); }
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype dt, MPI_Op op, MPI_Comm c) {
    (void)c;
    g_slot[t_rank].send = sendbuf;
    bar();
    reduce_into(recvbuf, count, dt, op);
    bar();
    return MPI_SUCCESS;
}

int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype dt,
               MPI_Op op, int root, MPI_Comm c) {
    (void)c;
    g_slot[t_rank].send = sendbuf;
    bar();
    if (t_rank == root) reduce_into(recvbuf, count, dt, op);
    bar();
    return MPI_SUCCESS;
}

int MPI_Bcast(void *buffer, int count, MPI_Datatype dt, int root, MPI_Comm c) {
    (void)c;
    g_slot[t_rank].send = buffer;
    bar();
    if (t_rank != root)
        memcpy(buffer, g_slot[root].send, (size_t)count * type_size(dt));
    bar();
    return MPI_SUCCESS;
}

int MPI_Allgatherv(const void *sendbuf, int sendcount, MPI_Datatype st,
                   void *recvbuf, const int *recvcounts, const int *displs,
                   MPI_Datatype rt, MPI_Comm c) {
    (void)c; (void)rt;
    size_t es = type_size(st);
    g_slot[t_rank].send = sendbuf;
    g_slot[t_rank].count = sendcount;
    bar();
    for (int r = 0; r < g_np; r++) {
        size_t n = (size_t)recvcounts[r];
        if ((int)n != g_slot[r].count) {
            fprintf(stderr, "mpi shim: Allgatherv count mismatch\n");
            abort();
        }
        memcpy((char *)recvbuf + (size_t)displs[r] * es, g_slot[r].send, n * es);
    }
    bar();
    return MPI_SUCCESS;
}

int MPI_Scatterv(const void *sendbuf, const int *sendcounts, const int *displs,
                 MPI_Datatype st, void *recvbuf, int recvcount,
                 MPI_Datatype rt, int root, MPI_Comm c) {
    (void)c; (void)rt;
    size_t es = type_size(st);
    g_slot[t_rank].send = sendbuf;
    g_slot[t_rank].counts = sendcounts;
    g_slot[t_rank].displs = displs;
    bar();
    const slot_t *s = &g_slot[root];
    memcpy(recvbuf, (const char *)s->send + (size_t)s->displs[t_rank] * es,
           (size_t)recvcount * es);
    bar();
    return MPI_SUCCESS;
}

int MPI_Alltoall(const void *sendbuf, int sendcount, MPI_Datatype st,
                 void *recvbuf, int recvcount, MPI_Datatype rt, MPI_Comm c) {
    (void)c; (void)rt; (void)sendcount;
    size_t es = type_size(st);
    g_slot[t_rank].send = sendbuf;
    g_slot[t_rank].count = sendcount;
    bar();
    for (int r = 0; r < g_np; r++)
        memcpy((char *)recvbuf + (size_t)r * recvcount * es,
               (const char *)g_slot[r].send + (size_t)t_rank * g_slot[r].count * es,
               (size_t)recvcount * es);
    bar();
    return MPI_SUCCESS;
}

int MPI_Alltoallv(const void *sendbuf, const int *sendcounts, const int *sdispls,
                  MPI_Datatype st, void *recvbuf, const int *recvcounts,
                  const int *rdispls, MPI_Datatype rt, MPI_Comm c) {
    (void)c; (void)rt;
    size_t es = type_size(st);
    g_slot[t_rank].send = sendbuf;
    g_slot[t_rank].counts = sendcounts;
    g_slot[t_rank].displs = sdispls;
    bar();
    for (int r = 0; r < g_np; r++) {
        const slot_t *s = &g_slot[r];
        memcpy((char *)recvbuf + (size_t)rdispls[r] * es,
               (const char *)s->send + (size_t)s->displs[t_rank] * es,
               (size_t)recvcounts[r] * es);
    }
    bar();
    return MPI_SUCCESS;
}

typedef struct {
    int rank;
    cacg_mpi_rank_fn fn;
    void *arg;
} rank_arg_t;

static void *rank_main(void *p) {
    rank_arg_t *a = (rank_arg_t *)p;
    t_rank = a->rank;
    a->fn(a->rank, a->arg);
    return NULL;
}

int cacg_mpi_run(int np, cacg_mpi_rank_fn fn, void *arg) {
    if (np < 1 || np > CACG_MPI_MAX_RANKS) return -1;
    g_np = np;
    if (np == 1) {
        t_rank = 0;
        fn(0, arg);
        return 0;
    }
    pthread_barrier_init(&g_bar, NULL, (unsigned)np);
    pthread_t th[CACG_MPI_MAX_RANKS];
    rank_arg_t ra[CACG_MPI_MAX_RANKS];
    for (int r = 0; r < np; r++) {
        ra[r].rank = r; ra[r].fn = fn; ra[r].arg = arg;
        pthread_create(&th[r], NULL, rank_main, &ra[r]);
    }
    for (int r = 0; r < np; r++) pthread_join(th[r], NULL);
    pthread_barrier_destroy(&g_bar);
    g_np = 1;
    return 0;
}
