/* Single-rank stand-in for the subset of MPI that atrip's sources call.
 *
 * Test infrastructure only: this header lets the unmodified reference
 * sources (src/atrip/*.cxx) compile and run as ONE rank, so the reference's
 * own Atrip::run can be executed as a parity oracle.  With one rank every
 * slice is SelfSufficient (src/atrip/SliceUnion.cxx:137-155), no point-to-
 * point message is ever matched, and every collective degenerates to a copy
 * of the caller's own contribution.  Point-to-point calls abort loudly,
 * because reaching them would mean the one-rank assumption is broken.
 */
#ifndef ORACLE_MPI_SHIM_H
#define ORACLE_MPI_SHIM_H

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef std::ptrdiff_t MPI_Aint;
struct MPI_Status {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
};

#define MPI_COMM_WORLD 1
#define MPI_SUCCESS 0
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_MAX_ERROR_STRING 64
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

/* Datatype handles index a table of extents (bytes).  Built-ins first. */
#define MPI_CHAR 0
#define MPI_BYTE 1
#define MPI_INT 2
#define MPI_DOUBLE 3
#define MPI_DOUBLE_COMPLEX 4
#define MPI_UINT64_T 5

inline std::vector<std::size_t> &oracle_mpi_extents() {
  static std::vector<std::size_t> t = {1, 1, sizeof(int), sizeof(double),
                                       2 * sizeof(double), sizeof(std::uint64_t)};
  return t;
}
inline std::size_t oracle_mpi_extent(MPI_Datatype d) {
  return oracle_mpi_extents().at((std::size_t)d);
}
inline int oracle_mpi_new_type(std::size_t extent) {
  oracle_mpi_extents().push_back(extent);
  return (int)oracle_mpi_extents().size() - 1;
}
[[noreturn]] inline void oracle_mpi_unreachable(const char *what) {
  std::fprintf(stderr, "mpi shim: %s called with one rank; unsupported\n", what);
  std::abort();
}

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm *out) { *out = c; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Get_processor_name(char *name, int *len) {
  std::strcpy(name, "oracle-host");
  *len = (int)std::strlen(name);
  return 0;
}
inline int MPI_Error_string(int code, char *s, int *len) {
  *len = std::snprintf(s, MPI_MAX_ERROR_STRING, "mpi shim error %d", code);
  return 0;
}
inline int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype dt,
                      MPI_Op, int, MPI_Comm) {
  if (send != recv) std::memmove(recv, send, count * oracle_mpi_extent(dt));
  return 0;
}
inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Allgather(const void *send, int scount, MPI_Datatype sdt,
                         void *recv, int, MPI_Datatype, MPI_Comm) {
  std::memmove(recv, send, scount * oracle_mpi_extent(sdt));
  return 0;
}
inline int MPI_Allgatherv(const void *send, int scount, MPI_Datatype sdt,
                          void *recv, const int *, const int *displs,
                          MPI_Datatype rdt, MPI_Comm) {
  std::memmove((char *)recv + displs[0] * oracle_mpi_extent(rdt), send,
               scount * oracle_mpi_extent(sdt));
  return 0;
}
inline int MPI_Scatter(const void *send, int scount, MPI_Datatype sdt,
                       void *recv, int, MPI_Datatype, int, MPI_Comm) {
  std::memmove(recv, send, scount * oracle_mpi_extent(sdt));
  return 0;
}
inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm,
                     MPI_Request *) {
  oracle_mpi_unreachable("MPI_Isend");
}
inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm,
                     MPI_Request *) {
  oracle_mpi_unreachable("MPI_Irecv");
}
inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
inline int MPI_Request_free(MPI_Request *) { return 0; }
inline int MPI_Type_vector(int count, int blocklen, int stride,
                           MPI_Datatype old, MPI_Datatype *out) {
  *out = oracle_mpi_new_type(((count - 1) * (std::size_t)stride + blocklen) *
                             oracle_mpi_extent(old));
  return 0;
}
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
inline int MPI_Type_free(MPI_Datatype *) { return 0; }
inline int MPI_Get_address(const void *p, MPI_Aint *a) {
  *a = (MPI_Aint)(std::uintptr_t)p;
  return 0;
}
inline MPI_Aint MPI_Aint_diff(MPI_Aint a, MPI_Aint b) { return a - b; }
inline int MPI_Type_create_struct(int n, const int *lens, const MPI_Aint *displs,
                                  const MPI_Datatype *types, MPI_Datatype *out) {
  std::size_t end = 0, align = 1;
  for (int i = 0; i < n; ++i) {
    std::size_t e = oracle_mpi_extent(types[i]);
    std::size_t stop = (std::size_t)displs[i] + lens[i] * e;
    if (stop > end) end = stop;
    if (e > align && e <= 8) align = e;
  }
  *out = oracle_mpi_new_type((end + align - 1) / align * align);
  return 0;
}

#endif
