/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the unmodified
 * PT-ICM reference sources as a CPU checker (oracle/_ref).  It is test
 * infrastructure: nothing in the product links it.
 *
 * With one rank every point-to-point call in the reference is skipped by its
 * own `numw > 1` / `worker != 0` guards (src/solver.cc, src/replica_exchange.cc,
 * src/icm.cc, src/mpi_utils.cc), so Send/Recv abort if they are ever reached.
 * Collectives degenerate: Bcast and Barrier do nothing, Reduce copies.
 */
#ifndef PTICM_ORACLE_MPI_STUB_H
#define PTICM_ORACLE_MPI_STUB_H

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstddef>

typedef int MPI_Comm;
typedef int MPI_Op;
/* A datatype is its element size in bytes (enough for Reduce's copy). */
typedef int MPI_Datatype;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUM 0
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_CXX_BOOL ((MPI_Datatype)1)
#define MPI_UNSIGNED_LONG ((MPI_Datatype)8)
#define MPI_UINT64_T ((MPI_Datatype)8)
#define MPI_SIGNED_CHAR ((MPI_Datatype)1)
#define MPI_UNSIGNED_CHAR ((MPI_Datatype)1)
#define MPI_UNSIGNED ((MPI_Datatype)4)
#define MPI_INT ((MPI_Datatype)4)

static inline int MPI_Init(void*, void*) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    std::memcpy(r, s, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) {
    std::fprintf(stderr, "mpi stub: MPI_Send reached with a single rank\n");
    std::abort();
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
    std::fprintf(stderr, "mpi stub: MPI_Recv reached with a single rank\n");
    std::abort();
}
static inline double MPI_Wtime() {
    return std::chrono::duration<double>(
        std::chrono::steady_clock::now().time_since_epoch()).count();
}
static inline int MPI_Type_create_struct(int, const int*, const MPI_Aint*, const MPI_Datatype*, MPI_Datatype* t) {
    *t = 0;
    return 0;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }

#endif
