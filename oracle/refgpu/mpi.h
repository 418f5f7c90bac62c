/*
 * mpi.h -- a one-process stand-in for the MPI calls the reference's program
 * mains make (sgpstd-qmodeling/acousticsgps4.c, visacousticsgps4.c): this image
 * has no MPI, and the mains run one rank on one GPU here.  TEST INFRASTRUCTURE:
 * it only lets the reference's own programs be built to pin the oracle and time
 * the reference (baseline B1); nothing in the library uses it.
 *
 * Semantics for a world of one rank: rank 0 of size 1, broadcasts leave the
 * buffer as it is (the root's data is already there), a reduction to the root
 * copies the send buffer to the receive buffer.
 */
#ifndef QPSTD_MPI_STUB_H
#define QPSTD_MPI_STUB_H
#include <stdio.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype; /* the element size in bytes */
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_SUM 0
#define MPI_SUCCESS 0
#define MPI_MAX_PROCESSOR_NAME 64

static inline int MPI_Init(int *argc, char ***argv) {
    (void)argc;
    (void)argv;
    return MPI_SUCCESS;
}
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int *rank) {
    (void)c;
    *rank = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_size(MPI_Comm c, int *size) {
    (void)c;
    *size = 1;
    return MPI_SUCCESS;
}
static inline int MPI_Get_processor_name(char *name, int *len) {
    snprintf(name, MPI_MAX_PROCESSOR_NAME, "localhost");
    *len = (int)strlen(name);
    return MPI_SUCCESS;
}
static inline int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm c) {
    (void)buf;
    (void)count;
    (void)t;
    (void)root;
    (void)c;
    return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm c) {
    (void)c;
    return MPI_SUCCESS;
}
static inline int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype t, MPI_Op op, int root,
                             MPI_Comm c) {
    (void)op;
    (void)root;
    (void)c;
    if (send != recv) memmove(recv, send, (size_t)count * (size_t)t);
    return MPI_SUCCESS;
}
#endif
