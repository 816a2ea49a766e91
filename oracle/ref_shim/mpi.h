/* mpi.h -- single-process stand-in for the MPI calls of the reference build (TEST
 * INFRASTRUCTURE: only oracle/_ref is compiled against it).
 *
 * The reference solver (MPI decomposition over radial rows) runs here as one rank, so every
 * collective is a local copy: Allreduce / Reduce / Alltoall copy the send buffer, Barrier and
 * Bcast do nothing, Send / Recv are never reached with one rank and abort if they are.
 * Datatypes carry their size in bytes. */
#ifndef GSREF_SHIM_MPI_H
#define GSREF_SHIM_MPI_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;   /* the element size in bytes */
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_CHAR 1
#define MPI_BYTE 1
#define MPI_INT 4
#define MPI_UNSIGNED 4
#define MPI_FLOAT 4
#define MPI_LONG 8
#define MPI_DOUBLE 8
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_IN_PLACE ((void*)1)

static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out) { (void)color; (void)key; *out = c; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int gsref_mpi_copy(const void* s, void* r, long n, MPI_Datatype t) {
    if (s != MPI_IN_PLACE && s != r) memmove(r, s, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    (void)op; (void)c; return gsref_mpi_copy(s, r, n, t);
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
    (void)op; (void)root; (void)c; return gsref_mpi_copy(s, r, n, t);
}
static inline int MPI_Alltoall(const void* s, int ns, MPI_Datatype ts, void* r, int nr, MPI_Datatype tr, MPI_Comm c) {
    (void)nr; (void)tr; (void)c; return gsref_mpi_copy(s, r, ns, ts);
}
static inline int MPI_Send(const void* b, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c) {
    (void)b; (void)n; (void)t; (void)dest; (void)tag; (void)c;
    fprintf(stderr, "MPI_Send with a single rank\n"); exit(3);
}
static inline int MPI_Recv(void* b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status* st) {
    (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; (void)st;
    fprintf(stderr, "MPI_Recv with a single rank\n"); exit(3);
}
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; fflush(stdout); exit(code ? code : 2); }
static inline double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
#endif
