// Single-rank MPI stand-in for building the reference's include/dsgl.hpp in the
// oracle's reference harness (test infrastructure only).  Every collective is the
// identity a one-process MPI job would compute.
#pragma once
#include <cstddef>
#include <cstring>
#include <cstdint>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 5
#define MPI_LONG_LONG 8
#define MPI_UNSIGNED_LONG 9
#define MPI_DOUBLE 10
#define MPI_SUM 0
#define MPI_IN_PLACE ((void*)1)
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_THREAD_MULTIPLE 3

inline size_t shim_mpi_type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: case MPI_FLOAT: return 4;
    default: return 8;
  }
}
inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE) std::memcpy(r, s, (size_t)n * shim_mpi_type_size(t));
  return 0;
}
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Get_processor_name(char* n, int* l) { std::strcpy(n, "oracle"); *l = 6; return 0; }

template <typename T> inline MPI_Datatype get_mpi_data_type();
template <> inline MPI_Datatype get_mpi_data_type<char>() { return MPI_CHAR; }
template <> inline MPI_Datatype get_mpi_data_type<int>() { return MPI_INT; }
template <> inline MPI_Datatype get_mpi_data_type<float>() { return MPI_FLOAT; }
template <> inline MPI_Datatype get_mpi_data_type<size_t>() { return MPI_UNSIGNED_LONG; }
