/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the unmodified
 * PaRGO reference sources (gpro/*.h, apps/.../*Operator.cpp) into the test
 * oracle under oracle/_ref/.  It is test infrastructure: nothing in the
 * product links it.
 *
 * Semantics: one process, rank 0 of 1.  Collectives copy send -> recv,
 * point-to-point calls are never reached with one rank (the reference only
 * exchanges halos between distinct ranks) and report an error if they are.
 */
#ifndef PARGO_ORACLE_MPI_SHIM_H
#define PARGO_ORACLE_MPI_SHIM_H

#include <string.h>
#include <stdio.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_CHAR 1
#define MPI_BYTE 2
#define MPI_INT 3
#define MPI_UNSIGNED 4
#define MPI_FLOAT 5
#define MPI_DOUBLE 6
#define MPI_LAND 1
#define MPI_SUM 2
#define MPI_MAX 3
#define MPI_MIN 4
#define MPI_BSEND_OVERHEAD 96
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

static inline size_t pargo_shim_mpi_size(MPI_Datatype t) {
    switch (t) {
        case MPI_CHAR: case MPI_BYTE: return 1;
        case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
        case MPI_DOUBLE: return 8;
        default: return 1;
    }
}

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline double MPI_Wtime() {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != r) memcpy(r, s, (size_t)n * pargo_shim_mpi_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int pargo_shim_mpi_p2p(const char* what) {
    fprintf(stderr, "mpi shim: %s called with a single rank\n", what);
    return 1;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return pargo_shim_mpi_p2p("MPI_Send"); }
static inline int MPI_Bsend(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return pargo_shim_mpi_p2p("MPI_Bsend"); }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return pargo_shim_mpi_p2p("MPI_Recv"); }
static inline int MPI_Pack_size(int n, MPI_Datatype t, MPI_Comm, int* size) {
    *size = n * (int)pargo_shim_mpi_size(t);
    return MPI_SUCCESS;
}
/* MPI semantics: detach hands back the buffer that attach registered. */
static inline void** pargo_shim_mpi_attached(int** size) {
    static void* buf = 0;
    static int bytes = 0;
    *size = &bytes;
    return &buf;
}
static inline int MPI_Buffer_attach(void* buf, int size) {
    int* s;
    *pargo_shim_mpi_attached(&s) = buf;
    *s = size;
    return MPI_SUCCESS;
}
static inline int MPI_Buffer_detach(void* buf, int* size) {
    int* s;
    void** b = pargo_shim_mpi_attached(&s);
    *(void**)buf = *b;
    *size = *s;
    *b = 0;
    *s = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Get_processor_name(char* name, int* len) {
    strcpy(name, "localhost");
    *len = 9;
    return MPI_SUCCESS;
}
static inline int MPI_Abort(MPI_Comm, int code) { return code; }

#endif
