/* mpi.h -- the GPU build runs as one process on one GPU: the MPI calls that
 * application mains make around Run() (barriers, timing, rank queries) are
 * provided here for a single rank.  Implemented in src/gpro.cpp. */
#ifndef PARGO_GPRO_MPI_H
#define PARGO_GPRO_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_INT 3
#define MPI_DOUBLE 6
#define MPI_LAND 1
#define MPI_MAX 2
#define MPI_SUM 3
#define MPI_MAX_PROCESSOR_NAME 256
#ifdef __cplusplus
extern "C" {
#endif
int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
#ifdef __cplusplus
}
#endif
#endif
