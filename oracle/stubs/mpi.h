/* Single-rank subset of the MPI C API, written for this project so that the
 * reference's sources compile and run as one process without an MPI
 * installation.  It is test infrastructure: the checker's build of the
 * reference (oracle/Makefile) is its only user.
 *
 * Semantics with one rank: rank 0 of a world of size 1; reductions and
 * broadcasts copy (a reduction over one rank is its input); barriers return;
 * point-to-point messages have no partner, so MPI_Send / MPI_Recv abort with a
 * message if they are ever reached (the reference only calls them towards
 * other ranks).  MPI_Wtime reads a steady clock. */
#ifndef KMPM_ORACLE_MPI_STUB_H
#define KMPM_ORACLE_MPI_STUB_H

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef std::intptr_t MPI_Aint;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

/* datatypes: the code is an index into the size table below; derived types
 * get codes from MPI_Type_create_struct */
#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_DOUBLE 3
#define MPI_LONG_LONG 4
#define MPI_INT64_T 5
#define MPI_UNSIGNED 6
#define MPI_FLOAT 7
#define MPI_LONG 8

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_LOR 4
#define MPI_LAND 5
#define MPI_PROD 6

namespace kmpm_mpi_stub {
inline std::size_t &derived_extent(int code) {
  static std::size_t ext[256] = {0};
  return ext[code & 255];
}
inline int &next_code() {
  static int c = 16;
  return c;
}
inline std::size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG_LONG: return sizeof(long long);
    case MPI_INT64_T: return sizeof(std::int64_t);
    case MPI_UNSIGNED: return sizeof(unsigned);
    case MPI_FLOAT: return sizeof(float);
    case MPI_LONG: return sizeof(long);
    default: return derived_extent(t);
  }
}
[[noreturn]] inline void no_partner(const char *what) {
  std::fprintf(stderr, "single-rank MPI stub: %s has no partner rank\n", what);
  std::abort();
}
}  // namespace kmpm_mpi_stub

inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int *rank) {
  *rank = 0;
  return MPI_SUCCESS;
}
inline int MPI_Comm_size(MPI_Comm, int *size) {
  *size = 1;
  return MPI_SUCCESS;
}
inline int MPI_Comm_free(MPI_Comm *) { return MPI_SUCCESS; }
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Abort(MPI_Comm, int code) {
  std::exit(code == 0 ? 1 : code);
}
inline double MPI_Wtime() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}
inline int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (send != MPI_IN_PLACE && send != recv) std::memmove(recv, send, (std::size_t)count * kmpm_mpi_stub::type_size(t));
  return MPI_SUCCESS;
}
inline int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype t, MPI_Op op, int, MPI_Comm c) {
  return MPI_Allreduce(send, recv, count, t, op, c);
}
inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { kmpm_mpi_stub::no_partner("MPI_Send"); }
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  kmpm_mpi_stub::no_partner("MPI_Recv");
}
inline int MPI_Get_address(const void *p, MPI_Aint *a) {
  *a = (MPI_Aint)p;
  return MPI_SUCCESS;
}
inline int MPI_Type_create_struct(int n, const int *blocklen, const MPI_Aint *disp, const MPI_Datatype *types,
                                  MPI_Datatype *out) {
  std::size_t ext = 0;
  for (int i = 0; i < n; i++) {
    const std::size_t end = (std::size_t)disp[i] + (std::size_t)blocklen[i] * kmpm_mpi_stub::type_size(types[i]);
    if (end > ext) ext = end;
  }
  const int code = kmpm_mpi_stub::next_code()++;
  kmpm_mpi_stub::derived_extent(code) = ext;
  *out = code;
  return MPI_SUCCESS;
}
inline int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
inline int MPI_Type_free(MPI_Datatype *) { return MPI_SUCCESS; }

#endif
