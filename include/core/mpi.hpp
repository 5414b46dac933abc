// mpi.hpp — the MPI surface the toolkits call (core/mpi.hpp:25-87 of the reference), for one rank
// per GPU: rank 0 of a world of size 1.  Reductions copy their input; there is no point-to-point
// traffic because a single-GPU graph has no mirrors.
#ifndef EG_CORE_MPI_HPP
#define EG_CORE_MPI_HPP

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <type_traits>

typedef int MPI_Datatype;  // element size in bytes in the low byte
typedef int MPI_Comm;
typedef int MPI_Op;

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
#define MPI_THREAD_MULTIPLE 3

inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline double MPI_Wtime() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype dt, MPI_Op, MPI_Comm) {
    if (send != MPI_IN_PLACE && count > 0) memmove(recv, send, (size_t)count * (size_t)(dt & 0xff));
    return 0;
}

template <typename T>
MPI_Datatype get_mpi_data_type() {
    if (std::is_same<T, char>::value) return MPI_CHAR;
    if (std::is_same<T, unsigned char>::value) return MPI_UNSIGNED_CHAR;
    if (std::is_same<T, int>::value) return MPI_INT;
    if (std::is_same<T, unsigned>::value) return MPI_UNSIGNED;
    if (std::is_same<T, long>::value) return MPI_LONG;
    if (std::is_same<T, unsigned long>::value) return MPI_UNSIGNED_LONG;
    if (std::is_same<T, float>::value) return MPI_FLOAT;
    if (std::is_same<T, double>::value) return MPI_DOUBLE;
    fprintf(stderr, "get_mpi_data_type: type not supported\n");
    exit(-1);
}

class MPI_Instance {
   public:
    MPI_Instance(int*, char***) {}
    void pause() {}
};

#endif
