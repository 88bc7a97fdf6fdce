/*
 * Single-process stand-in for the MPI header -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference build in oracle/_ref runs as one rank (the GB300 engine it pins runs on one
 * GPU), so every call here is the one-rank case: rank 0 of a world of size 1, Allgather a
 * copy, point-to-point calls never reached (they report an error if they are).
 */
#ifndef IMPEC_REFSHIM_MPI_H
#define IMPEC_REFSHIM_MPI_H

#include <cstdio>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUCCESS 0

static inline size_t impec_mpi_shim_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(double); }
static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) {
    std::memcpy(r, s, (size_t)n * impec_mpi_shim_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) {
    std::fprintf(stderr, "mpi shim: MPI_Send in a one-rank run\n");
    return 1;
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
    std::fprintf(stderr, "mpi shim: MPI_Recv in a one-rank run\n");
    return 1;
}

#endif
