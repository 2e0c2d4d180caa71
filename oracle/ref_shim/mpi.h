// mpi.h -- single-process stand-in for the MPI interface KaMSTa's headers use.
//
// Test infrastructure: it lets the reference's own single-rank hot path
// (include/algorithms/local_contraction/..., gbbs_reimplementation.hpp)
// compile and run as the oracle's "reference" build.  One process is rank 0
// of a world of size 1, so every collective is a local copy (or nothing):
//   Allreduce / Allgather(v) / Gather(v) / Alltoall(v) copy send to receive,
//   Bcast and Barrier do nothing, Comm_split returns the same world.
// Datatype handles are small integers; derived types record their byte
// size in a registry so copies know how many bytes one element holds.
// Written from the MPI standard's C bindings; no MPI library code.
#pragma once

#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef long MPI_Aint;
typedef long long MPI_Count;
typedef void(MPI_User_function)(void*, void*, int*, MPI_Datatype*);

struct MPI_Status {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int count_bytes;
};
typedef int MPI_Request;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_COMM_SELF ((MPI_Comm)2)
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_REQUEST_NULL ((MPI_Request)0)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_UNDEFINED (-32766)
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3
#define MPI_MAX_PROCESSOR_NAME 256

// predefined datatypes: handle = index into the size table below
#define MPI_DATATYPE_NULL ((MPI_Datatype)0)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CHAR ((MPI_Datatype)2)
#define MPI_C_BOOL ((MPI_Datatype)3)
#define MPI_INT8_T ((MPI_Datatype)4)
#define MPI_UINT8_T ((MPI_Datatype)5)
#define MPI_INT16_T ((MPI_Datatype)6)
#define MPI_UINT16_T ((MPI_Datatype)7)
#define MPI_INT32_T ((MPI_Datatype)8)
#define MPI_UINT32_T ((MPI_Datatype)9)
#define MPI_INT64_T ((MPI_Datatype)10)
#define MPI_UINT64_T ((MPI_Datatype)11)
#define MPI_INT ((MPI_Datatype)12)
#define MPI_UNSIGNED ((MPI_Datatype)13)
#define MPI_LONG ((MPI_Datatype)14)
#define MPI_UNSIGNED_LONG ((MPI_Datatype)15)
#define MPI_LONG_LONG ((MPI_Datatype)16)
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)17)
#define MPI_FLOAT ((MPI_Datatype)18)
#define MPI_DOUBLE ((MPI_Datatype)19)
#define MPI_LONG_LONG_INT MPI_LONG_LONG
#define MPI_CXX_BOOL MPI_C_BOOL
#define MPI_SIZE_T MPI_UINT64_T

#define MPI_OP_NULL ((MPI_Op)0)
#define MPI_MAX ((MPI_Op)1)
#define MPI_MIN ((MPI_Op)2)
#define MPI_SUM ((MPI_Op)3)
#define MPI_PROD ((MPI_Op)4)
#define MPI_LAND ((MPI_Op)5)
#define MPI_LOR ((MPI_Op)6)
#define MPI_BAND ((MPI_Op)7)
#define MPI_BOR ((MPI_Op)8)

namespace kamsta_mpi_stub {

struct Registry {
  std::mutex mu;
  std::vector<long> type_bytes;  // by handle
  int next_op = 100;
  bool initialized = false, finalized = false;
  Registry()
      : type_bytes{0, 1, 1, 1, 1, 1, 2, 2, 4, 4, 8, 8, (long)sizeof(int), (long)sizeof(unsigned),
                   (long)sizeof(long), (long)sizeof(unsigned long), (long)sizeof(long long),
                   (long)sizeof(unsigned long long), 4, 8} {}
};
inline Registry& reg() {
  static Registry r;
  return r;
}
inline long type_size(MPI_Datatype t) {
  std::lock_guard<std::mutex> lk(reg().mu);
  return (t >= 0 && static_cast<size_t>(t) < reg().type_bytes.size()) ? reg().type_bytes[t] : 0;
}
inline MPI_Datatype new_type(long bytes) {
  std::lock_guard<std::mutex> lk(reg().mu);
  reg().type_bytes.push_back(bytes);
  return static_cast<MPI_Datatype>(reg().type_bytes.size() - 1);
}
inline void copy(const void* src, void* dst, long count, MPI_Datatype t) {
  if (src == MPI_IN_PLACE || src == dst || count <= 0) return;
  std::memmove(dst, src, static_cast<size_t>(count) * static_cast<size_t>(type_size(t)));
}

}  // namespace kamsta_mpi_stub

inline int MPI_Init(int*, char***) {
  kamsta_mpi_stub::reg().initialized = true;
  return MPI_SUCCESS;
}
inline int MPI_Init_thread(int*, char***, int required, int* provided) {
  kamsta_mpi_stub::reg().initialized = true;
  if (provided) *provided = required < MPI_THREAD_MULTIPLE ? MPI_THREAD_MULTIPLE : required;
  return MPI_SUCCESS;
}
inline int MPI_Initialized(int* flag) {
  *flag = kamsta_mpi_stub::reg().initialized ? 1 : 0;
  return MPI_SUCCESS;
}
inline int MPI_Finalize() {
  kamsta_mpi_stub::reg().finalized = true;
  return MPI_SUCCESS;
}
inline int MPI_Finalized(int* flag) {
  *flag = kamsta_mpi_stub::reg().finalized ? 1 : 0;
  return MPI_SUCCESS;
}
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
inline int MPI_Comm_rank(MPI_Comm, int* rank) {
  *rank = 0;
  return MPI_SUCCESS;
}
inline int MPI_Comm_size(MPI_Comm, int* size) {
  *size = 1;
  return MPI_SUCCESS;
}
inline int MPI_Comm_split(MPI_Comm comm, int, int, MPI_Comm* out) {
  *out = comm;
  return MPI_SUCCESS;
}
inline int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* out) {
  *out = comm;
  return MPI_SUCCESS;
}
inline int MPI_Comm_free(MPI_Comm* comm) {
  *comm = MPI_COMM_NULL;
  return MPI_SUCCESS;
}
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline double MPI_Wtime() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
inline int MPI_Get_processor_name(char* name, int* len) {
  std::strcpy(name, "localhost");
  *len = 9;
  return MPI_SUCCESS;
}

// ---- datatypes and reduction operators
inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) {
  *out = kamsta_mpi_stub::new_type(static_cast<long>(count) * kamsta_mpi_stub::type_size(old));
  return MPI_SUCCESS;
}
inline int MPI_Type_create_struct(int count, const int* lengths, const MPI_Aint* displs,
                                  const MPI_Datatype* types, MPI_Datatype* out) {
  long end = 0;  // extent: the end of the furthest block
  for (int i = 0; i < count; ++i) {
    const long e = displs[i] + static_cast<long>(lengths[i]) * kamsta_mpi_stub::type_size(types[i]);
    if (e > end) end = e;
  }
  *out = kamsta_mpi_stub::new_type(end);
  return MPI_SUCCESS;
}
inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
inline int MPI_Type_free(MPI_Datatype* t) {
  *t = MPI_DATATYPE_NULL;
  return MPI_SUCCESS;
}
inline int MPI_Type_size(MPI_Datatype t, int* size) {
  *size = static_cast<int>(kamsta_mpi_stub::type_size(t));
  return MPI_SUCCESS;
}
inline int MPI_Type_get_extent(MPI_Datatype t, MPI_Aint* lb, MPI_Aint* extent) {
  *lb = 0;
  *extent = kamsta_mpi_stub::type_size(t);
  return MPI_SUCCESS;
}
inline int MPI_Op_create(MPI_User_function*, int, MPI_Op* op) {
  std::lock_guard<std::mutex> lk(kamsta_mpi_stub::reg().mu);
  *op = kamsta_mpi_stub::reg().next_op++;
  return MPI_SUCCESS;
}
inline int MPI_Op_free(MPI_Op* op) {
  *op = MPI_OP_NULL;
  return MPI_SUCCESS;
}

// ---- collectives over a world of one: the local contribution is the result
inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op,
                         MPI_Comm) {
  kamsta_mpi_stub::copy(send, recv, count, t);
  return MPI_SUCCESS;
}
inline int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op, int,
                      MPI_Comm) {
  kamsta_mpi_stub::copy(send, recv, count, t);
  return MPI_SUCCESS;
}
inline int MPI_Scan(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  kamsta_mpi_stub::copy(send, recv, count, t);
  return MPI_SUCCESS;
}
inline int MPI_Exscan(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) {
  return MPI_SUCCESS;  // rank 0's exclusive prefix is undefined by the standard
}
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Allgather(const void* send, int scount, MPI_Datatype st, void* recv, int,
                         MPI_Datatype, MPI_Comm) {
  kamsta_mpi_stub::copy(send, recv, scount, st);
  return MPI_SUCCESS;
}
inline int MPI_Allgatherv(const void* send, int scount, MPI_Datatype st, void* recv,
                          const int*, const int* displs, MPI_Datatype rt, MPI_Comm) {
  if (send == MPI_IN_PLACE) return MPI_SUCCESS;
  char* dst = static_cast<char*>(recv) + static_cast<long>(displs[0]) * kamsta_mpi_stub::type_size(rt);
  kamsta_mpi_stub::copy(send, dst, scount, st);
  return MPI_SUCCESS;
}
inline int MPI_Gather(const void* send, int scount, MPI_Datatype st, void* recv, int,
                      MPI_Datatype, int, MPI_Comm) {
  kamsta_mpi_stub::copy(send, recv, scount, st);
  return MPI_SUCCESS;
}
inline int MPI_Gatherv(const void* send, int scount, MPI_Datatype st, void* recv, const int*,
                       const int* displs, MPI_Datatype rt, int, MPI_Comm) {
  if (send == MPI_IN_PLACE) return MPI_SUCCESS;
  char* dst = static_cast<char*>(recv) + static_cast<long>(displs[0]) * kamsta_mpi_stub::type_size(rt);
  kamsta_mpi_stub::copy(send, dst, scount, st);
  return MPI_SUCCESS;
}
inline int MPI_Scatter(const void* send, int scount, MPI_Datatype st, void* recv, int,
                       MPI_Datatype, int, MPI_Comm) {
  kamsta_mpi_stub::copy(send, recv, scount, st);
  return MPI_SUCCESS;
}
inline int MPI_Alltoall(const void* send, int scount, MPI_Datatype st, void* recv, int,
                        MPI_Datatype, MPI_Comm) {
  kamsta_mpi_stub::copy(send, recv, scount, st);
  return MPI_SUCCESS;
}
inline int MPI_Alltoallv(const void* send, const int* scounts, const int* sdispls,
                         MPI_Datatype st, void* recv, const int*, const int* rdispls,
                         MPI_Datatype rt, MPI_Comm) {
  const char* src = static_cast<const char*>(send) +
                    static_cast<long>(sdispls[0]) * kamsta_mpi_stub::type_size(st);
  char* dst = static_cast<char*>(recv) + static_cast<long>(rdispls[0]) * kamsta_mpi_stub::type_size(rt);
  kamsta_mpi_stub::copy(src, dst, scounts[0], st);
  return MPI_SUCCESS;
}
