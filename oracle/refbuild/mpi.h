/*
 * Single-rank stand-in for <mpi.h>, used only to compile the upstream htool
 * headers into the test oracle library (oracle/_ref).  It is test
 * infrastructure: nothing in the htool_gb300 product includes it.
 *
 * Every communicator has exactly one rank (rank 0).  Collectives therefore
 * reduce to local copies that honour counts and displacements; datatypes are
 * encoded as their size in bytes so the copies know how much to move.  The
 * symbol set is exactly what htool's hmatrix.hpp, cluster.hpp,
 * wrapper_mpi.hpp and blocks.hpp call.
 *
 * htgpu_stub_set_world(P, p) makes MPI_Comm_size / MPI_Comm_rank report a
 * world of P ranks seen from rank p, so that one process can replay what
 * rank p of a P-rank run computes locally (its cluster tree, local tasks,
 * leaves and mymvprod_global_to_local).  The collectives stay local copies:
 * only the rank-local steps are meaningful in that mode.
 */
#ifndef HTGPU_ORACLE_MPI_STUB_H
#define HTGPU_ORACLE_MPI_STUB_H

#include <stddef.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype; /* value = element size in bytes */
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_SUCCESS 0
#define MPI_ANY_TAG (-1)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_UNSIGNED_CHAR ((MPI_Datatype)1)
#define MPI_UNSIGNED_SHORT ((MPI_Datatype)2)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_UNSIGNED ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_UNSIGNED_LONG ((MPI_Datatype)8)
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_C_COMPLEX ((MPI_Datatype)8)
#define MPI_C_DOUBLE_COMPLEX ((MPI_Datatype)16)

#define MPI_SUM ((MPI_Op)0)
#define MPI_MAX ((MPI_Op)1)
#define MPI_MIN ((MPI_Op)2)

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static int htgpu_stub_world_size = 1, htgpu_stub_world_rank = 0;
static inline void htgpu_stub_set_world(int size, int rank) {
    htgpu_stub_world_size = size;
    htgpu_stub_world_rank = rank;
}
static inline int MPI_Comm_size(MPI_Comm, int *size) {
    *size = htgpu_stub_world_size;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_rank(MPI_Comm, int *rank) {
    *rank = htgpu_stub_world_rank;
    return MPI_SUCCESS;
}
static inline double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

/* one rank: a reduction is the identity, so only a copy is needed */
static inline int htgpu_stub_copy(const void *src, void *dst, size_t bytes) {
    if (src != MPI_IN_PLACE && src != dst && bytes)
        memmove(dst, src, bytes);
    return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    return htgpu_stub_copy(s, r, (size_t)n * (size_t)t);
}
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    return htgpu_stub_copy(s, r, (size_t)n * (size_t)t);
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) {
    return htgpu_stub_copy(s, r, (size_t)sn * (size_t)st);
}
static inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *displs, MPI_Datatype rt, MPI_Comm) {
    if (s == MPI_IN_PLACE)
        return MPI_SUCCESS;
    return htgpu_stub_copy(s, (char *)r + (size_t)displs[0] * (size_t)rt, (size_t)sn * (size_t)st);
}
static inline int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *displs, MPI_Datatype rt, int, MPI_Comm) {
    if (s == MPI_IN_PLACE)
        return MPI_SUCCESS;
    return htgpu_stub_copy(s, (char *)r + (size_t)displs[0] * (size_t)rt, (size_t)sn * (size_t)st);
}
static inline int MPI_Scatterv(const void *s, const int *scounts, const int *sdispls, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm) {
    if (r == MPI_IN_PLACE)
        return MPI_SUCCESS;
    return htgpu_stub_copy((const char *)s + (size_t)sdispls[0] * (size_t)st, r, (size_t)scounts[0] * (size_t)st);
}
static inline int MPI_Alltoallv(const void *s, const int *scounts, const int *sdispls, MPI_Datatype st, void *r, const int *, const int *rdispls, MPI_Datatype rt, MPI_Comm) {
    return htgpu_stub_copy((const char *)s + (size_t)sdispls[0] * (size_t)st, (char *)r + (size_t)rdispls[0] * (size_t)rt, (size_t)scounts[0] * (size_t)st);
}
/* point-to-point is only used by the (excluded) DDM solvers */
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return MPI_SUCCESS; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return MPI_SUCCESS; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }

#endif
