// Single-rank implementation of the MPI subset declared in mpi.h.
// Test infrastructure for the CPU oracle build only.
#include "mpi.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct TypeInfo {
  MPI_Aint size;    // bytes of data in one element
  MPI_Aint extent;  // stride between consecutive elements
};

std::vector<TypeInfo> &Types() {
  static std::vector<TypeInfo> t = {
      {0, 0},                                         // NULL
      {sizeof(int), sizeof(int)},                     // INT
      {sizeof(double), sizeof(double)},               // DOUBLE
      {1, 1},                                         // CHAR
      {1, 1},                                         // PACKED
      {sizeof(bool), sizeof(bool)},                   // C_BOOL
      {sizeof(bool), sizeof(bool)},                   // CXX_BOOL
  };
  return t;
}

const TypeInfo &Info(MPI_Datatype t) {
  auto &tab = Types();
  if (t < 0 || t >= static_cast<int>(tab.size())) {
    std::fprintf(stderr, "single-rank MPI: bad datatype handle %d\n", t);
    std::abort();
  }
  return tab[t];
}

MPI_Datatype NewType(MPI_Aint size, MPI_Aint extent) {
  Types().push_back({size, extent});
  return static_cast<MPI_Datatype>(Types().size() - 1);
}

[[noreturn]] void NoPeers(const char *fn) {
  std::fprintf(stderr,
               "single-rank MPI: %s needs a second rank, which never exists "
               "in the oracle build\n",
               fn);
  std::abort();
}

}  // namespace

extern "C" {

int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int *size) {
  *size = 1;
  return MPI_SUCCESS;
}
int MPI_Comm_rank(MPI_Comm, int *rank) {
  *rank = 0;
  return MPI_SUCCESS;
}
int MPI_Get_version(int *version, int *subversion) {
  *version = 3;
  *subversion = 0;
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype type, MPI_Op, int, MPI_Comm) {
  // one rank: the reduction of a single contribution is that contribution
  if (sendbuf != MPI_IN_PLACE && sendbuf != recvbuf) {
    std::memmove(recvbuf, sendbuf,
                 static_cast<size_t>(count) * Info(type).extent);
  }
  return MPI_SUCCESS;
}

int MPI_Scatter(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                void *recvbuf, int, MPI_Datatype, int, MPI_Comm) {
  if (sendbuf != MPI_IN_PLACE && sendbuf != recvbuf) {
    std::memmove(recvbuf, sendbuf,
                 static_cast<size_t>(sendcount) * Info(sendtype).extent);
  }
  return MPI_SUCCESS;
}

int MPI_Pack(const void *inbuf, int incount, MPI_Datatype type, void *outbuf,
             int outsize, int *position, MPI_Comm) {
  const auto bytes = static_cast<int>(incount * Info(type).extent);
  if (*position + bytes > outsize) {
    std::fprintf(stderr, "single-rank MPI: MPI_Pack overflow\n");
    std::abort();
  }
  std::memcpy(static_cast<char *>(outbuf) + *position, inbuf, bytes);
  *position += bytes;
  return MPI_SUCCESS;
}

int MPI_Unpack(const void *inbuf, int insize, int *position, void *outbuf,
               int outcount, MPI_Datatype type, MPI_Comm) {
  const auto bytes = static_cast<int>(outcount * Info(type).extent);
  if (*position + bytes > insize) {
    std::fprintf(stderr, "single-rank MPI: MPI_Unpack overflow\n");
    std::abort();
  }
  std::memcpy(outbuf, static_cast<const char *>(inbuf) + *position, bytes);
  *position += bytes;
  return MPI_SUCCESS;
}

int MPI_Pack_size(int incount, MPI_Datatype type, MPI_Comm, int *size) {
  *size = static_cast<int>(incount * Info(type).extent);
  return MPI_SUCCESS;
}

int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
  NoPeers("MPI_Send");
}
int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  NoPeers("MPI_Recv");
}
int MPI_Probe(int, int, MPI_Comm, MPI_Status *) { NoPeers("MPI_Probe"); }
int MPI_Get_count(const MPI_Status *, MPI_Datatype, int *) {
  NoPeers("MPI_Get_count");
}
int MPI_Sendrecv_replace(void *, int, MPI_Datatype, int, int, int, int,
                         MPI_Comm, MPI_Status *) {
  NoPeers("MPI_Sendrecv_replace");
}

int MPI_Get_address(const void *location, MPI_Aint *address) {
  *address = reinterpret_cast<MPI_Aint>(location);
  return MPI_SUCCESS;
}

int MPI_Type_contiguous(int count, MPI_Datatype oldtype,
                        MPI_Datatype *newtype) {
  const auto &o = Info(oldtype);
  *newtype = NewType(count * o.size, count * o.extent);
  return MPI_SUCCESS;
}

int MPI_Type_create_struct(int count, const int blocklengths[],
                           const MPI_Aint displacements[],
                           const MPI_Datatype types[],
                           MPI_Datatype *newtype) {
  MPI_Aint size = 0, extent = 0;
  for (int ii = 0; ii < count; ++ii) {
    const auto &t = Info(types[ii]);
    size += blocklengths[ii] * t.size;
    const auto end = displacements[ii] + blocklengths[ii] * t.extent;
    if (end > extent) extent = end;
  }
  *newtype = NewType(size, extent);
  return MPI_SUCCESS;
}

int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint, MPI_Aint extent,
                            MPI_Datatype *newtype) {
  *newtype = NewType(Info(oldtype).size, extent);
  return MPI_SUCCESS;
}

int MPI_Type_get_extent(MPI_Datatype type, MPI_Aint *lb, MPI_Aint *extent) {
  *lb = 0;
  *extent = Info(type).extent;
  return MPI_SUCCESS;
}

int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype *type) {
  *type = MPI_DATATYPE_NULL;
  return MPI_SUCCESS;
}
int MPI_Op_create(MPI_User_function *, int, MPI_Op *op) {
  *op = 2;
  return MPI_SUCCESS;
}
int MPI_Op_free(MPI_Op *op) {
  *op = 0;
  return MPI_SUCCESS;
}

}  // extern "C"
