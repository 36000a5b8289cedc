/*
 * Single-rank MPI stand-in, used ONLY by test infrastructure: to compile the
 * reference's hot-path C sources into the test oracle library
 * (oracle/_ref/libref.so) and the shim's MPI branch into the compat test
 * harness (tests/compat).  Nothing in the rajzel_gb300 product includes it.
 *
 * With one rank every collective the reference uses on this path is the
 * identity: MPI_Allreduce copies send->recv (grad_obj.c:60,
 * sum_grad_MPI.c:36), MPI_Barrier / MPI_Bcast do nothing, MPI_Abort exits
 * (util.c:15).
 */
#ifndef RZ_ORACLE_STUB_MPI_H
#define RZ_ORACLE_STUB_MPI_H

#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int dummy; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 5
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline size_t rz_stub_mpi_size(MPI_Datatype t) {
    switch (t) {
        case MPI_CHAR: return 1;
        case MPI_INT: return sizeof(int);
        case MPI_FLOAT: return sizeof(float);
        case MPI_DOUBLE: return sizeof(double);
        default: return 1;
    }
}

static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code); return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) {
    (void)b; (void)n; (void)t; (void)root; (void)c; return 0;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    (void)op; (void)c;
    memmove(r, s, (size_t)n * rz_stub_mpi_size(t));
    return 0;
}
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline double MPI_Wtime(void) { return 0.0; }

#endif
