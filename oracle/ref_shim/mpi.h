/*
 * mpi.h -- a one-rank stand-in for MPI, written for this project so that the
 * reference program mpi/mpi_lsbsort.cpp compiles unmodified from its own
 * source file (oracle/Makefile, target `ref`). It implements only the calls
 * that file makes. With one rank every collective is a local copy:
 * MPI_Alltoallv copies the rank's own segment, MPI_Exscan leaves its output
 * alone (the reference overwrites rank 0's result, mpi_lsbsort.cpp:415-417),
 * MPI_Gather copies, MPI_Barrier returns.
 *
 * TEST INFRASTRUCTURE: used only to build the checker under oracle/_ref/.
 */
#ifndef LSB_REF_SHIM_MPI_H
#define LSB_REF_SHIM_MPI_H

#include <algorithm> /* the reference relies on <algorithm> arriving transitively */
#include <cstddef>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_SUM 0
#define MPI_SUCCESS 0

/* predefined datatypes: handle -> byte size through lsb_shim_type_size */
#define MPI_INT 1
#define MPI_LONG_LONG 2
#define MPI_UNSIGNED_LONG_LONG 3

namespace lsb_shim {
inline std::size_t* type_table() {
  static std::size_t sizes[64] = {0, sizeof(int), sizeof(long long), sizeof(unsigned long long)};
  return sizes;
}
inline int* type_count() {
  static int next = 4;
  return &next;
}
inline std::size_t type_size(MPI_Datatype t) { return type_table()[t]; }
}  // namespace lsb_shim

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) {
  int h = (*lsb_shim::type_count())++;
  lsb_shim::type_table()[h] = (std::size_t)count * lsb_shim::type_size(old);
  *out = h;
  return MPI_SUCCESS;
}
inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

inline int MPI_Alltoallv(const void* sendbuf, const int* sendcounts, const int* sdispls,
                         MPI_Datatype sendtype, void* recvbuf, const int* recvcounts,
                         const int* rdispls, MPI_Datatype recvtype, MPI_Comm) {
  std::size_t ss = lsb_shim::type_size(sendtype), rs = lsb_shim::type_size(recvtype);
  std::size_t bytes = (std::size_t)sendcounts[0] * ss;
  if (bytes && (std::size_t)recvcounts[0] * rs >= bytes)
    std::memmove((char*)recvbuf + (std::size_t)rdispls[0] * rs,
                 (const char*)sendbuf + (std::size_t)sdispls[0] * ss, bytes);
  return MPI_SUCCESS;
}

inline int MPI_Exscan(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) {
  return MPI_SUCCESS;
}

inline int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                      int, MPI_Datatype, int, MPI_Comm) {
  std::size_t bytes = (std::size_t)sendcount * lsb_shim::type_size(sendtype);
  if (bytes) std::memmove(recvbuf, sendbuf, bytes);
  return MPI_SUCCESS;
}

#endif
