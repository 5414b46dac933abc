/*
 * Single-rank stand-in for <mpi.h>, written for building the reference's own engine as a test
 * oracle.  Rank 0 of a world of size 1: collectives copy, point-to-point calls are unreachable at
 * one rank (the reference guards them with partitions_num > 1 or skips them, core/graph.hpp:809,
 * :1556, :1666, :1733) and abort if reached.
 */
#ifndef EG_REF_MPI_SHIM_H
#define EG_REF_MPI_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

typedef int MPI_Datatype; /* (id << 8) | element size */
typedef int MPI_Comm;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR, count_; } MPI_Status;

#define MPI_CHAR ((1 << 8) | 1)
#define MPI_UNSIGNED_CHAR ((2 << 8) | 1)
#define MPI_INT ((3 << 8) | 4)
#define MPI_UNSIGNED ((4 << 8) | 4)
#define MPI_LONG ((5 << 8) | 8)
#define MPI_UNSIGNED_LONG ((6 << 8) | 8)
#define MPI_FLOAT ((7 << 8) | 4)
#define MPI_DOUBLE ((8 << 8) | 8)
#define MPI_COMM_WORLD 0
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_ANY_SOURCE (-1)
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3

static inline void eg_mpi_unreachable_(const char* what) {
    fprintf(stderr, "single-rank MPI stand-in: %s is unreachable at one rank\n", what);
    abort();
}
static inline int MPI_Init_thread(int*, char***, int, int* provided) { *provided = MPI_THREAD_MULTIPLE; return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime() { return omp_get_wtime(); }
static inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype dt, MPI_Op, MPI_Comm) {
    if (send != MPI_IN_PLACE && count > 0) memmove(recv, send, (size_t)count * (size_t)(dt & 0xff));
    return 0;
}
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { eg_mpi_unreachable_("MPI_Isend"); return 1; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { eg_mpi_unreachable_("MPI_Send"); return 1; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { eg_mpi_unreachable_("MPI_Recv"); return 1; }
static inline int MPI_Probe(int, int, MPI_Comm, MPI_Status*) { eg_mpi_unreachable_("MPI_Probe"); return 1; }
static inline int MPI_Get_count(const MPI_Status*, MPI_Datatype, int*) { eg_mpi_unreachable_("MPI_Get_count"); return 1; }
static inline int MPI_Request_free(MPI_Request*) { eg_mpi_unreachable_("MPI_Request_free"); return 1; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { eg_mpi_unreachable_("MPI_Waitall"); return 1; }

#endif
