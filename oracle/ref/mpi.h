/*
 * Single-rank MPI stand-in used only to compile the reference's header-only
 * C++ TPB path on a machine without an MPI installation.
 *
 * Test infrastructure: this header is part of the oracle build recipe
 * (oracle/Makefile) and is never linked into the product library.
 *
 * Semantics: every communicator has exactly one rank (rank 0).  Collectives
 * copy send buffers into receive buffers (or do nothing for MPI_IN_PLACE);
 * point-to-point messages go to a process-local FIFO keyed by tag, which is
 * enough for the reference's self-send "2-D slide" (framework/mpi_utility.h,
 * Mpi2dSlide) at communicator size 1.
 */
#ifndef SBDGB_ORACLE_MPI_SHIM_H
#define SBDGB_ORACLE_MPI_SHIM_H

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <deque>
#include <vector>
#include <stdexcept>

#define MPI_VERSION 3
#define MPI_SUBVERSION 1

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef long MPI_Aint;
typedef long long MPI_Count;
typedef int MPI_Request;
struct MPI_Status { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; long count_bytes; };

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_SUCCESS 0
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_REQUEST_NULL (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

/* datatype codes encode the element size in their low byte */
#define SBDGB_MPI_T(code, size) (((code) << 8) | (size))
#define MPI_CHAR SBDGB_MPI_T(1, 1)
#define MPI_BYTE SBDGB_MPI_T(2, 1)
#define MPI_UNSIGNED_CHAR SBDGB_MPI_T(3, 1)
#define MPI_C_BOOL SBDGB_MPI_T(4, 1)
#define MPI_UNSIGNED_SHORT SBDGB_MPI_T(5, 2)
#define MPI_INT SBDGB_MPI_T(6, 4)
#define MPI_UNSIGNED SBDGB_MPI_T(7, 4)
#define MPI_INT32_T SBDGB_MPI_T(8, 4)
#define MPI_UINT32_T SBDGB_MPI_T(9, 4)
#define MPI_FLOAT SBDGB_MPI_T(10, 4)
#define MPI_LONG SBDGB_MPI_T(11, 8)
#define MPI_UNSIGNED_LONG SBDGB_MPI_T(12, 8)
#define MPI_UNSIGNED_LONG_LONG SBDGB_MPI_T(13, 8)
#define MPI_UINT64_T SBDGB_MPI_T(14, 8)
#define MPI_INT64_T SBDGB_MPI_T(15, 8)
#define MPI_DOUBLE SBDGB_MPI_T(16, 8)
#define MPI_CXX_FLOAT_COMPLEX SBDGB_MPI_T(17, 8)
#define MPI_CXX_DOUBLE_COMPLEX SBDGB_MPI_T(18, 16)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_LAND 4
#define MPI_LOR 5
#define MPI_PROD 6

namespace sbdgb_mpi_shim {
inline size_t type_size(MPI_Datatype t) {
  /* derived struct types created by MPI_Type_create_struct carry their extent */
  if (t >= (1 << 20)) return (size_t)(t - (1 << 20));
  return (size_t)(t & 0xff);
}
struct Msg { int tag; std::vector<char> bytes; };
inline std::deque<Msg> &fifo() { static std::deque<Msg> q; return q; }
struct Pending { void *buf; size_t bytes; int tag; bool active; };
inline std::vector<Pending> &pending() { static std::vector<Pending> p; return p; }
inline void deliver(const void *buf, size_t bytes, int tag) {
  Msg m; m.tag = tag; m.bytes.resize(bytes);
  if (bytes) std::memcpy(m.bytes.data(), buf, bytes);
  fifo().push_back(std::move(m));
}
inline bool take(void *buf, size_t bytes, int tag) {
  auto &q = fifo();
  for (auto it = q.begin(); it != q.end(); ++it) {
    if (tag == MPI_ANY_TAG || it->tag == tag) {
      size_t n = bytes < it->bytes.size() ? bytes : it->bytes.size();
      if (n) std::memcpy(buf, it->bytes.data(), n);
      q.erase(it);
      return true;
    }
  }
  return false;
}
inline void copy_if_distinct(const void *s, void *r, size_t bytes) {
  if (s != MPI_IN_PLACE && s != r && bytes) std::memmove(r, s, bytes);
}
}  // namespace sbdgb_mpi_shim

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Init_thread(int *, char ***, int req, int *prov) { if (prov) *prov = req; return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Initialized(int *f) { *f = 1; return 0; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code == 0 ? 1 : code); }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm *n) { *n = c ? c : MPI_COMM_WORLD; return 0; }
inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *n) { *n = c; return 0; }
inline int MPI_Comm_free(MPI_Comm *c) { *c = MPI_COMM_NULL; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline double MPI_Wtime() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}
inline int MPI_Get_processor_name(char *name, int *len) {
  std::strcpy(name, "localhost"); *len = 9; return 0;
}
inline int MPI_Get_address(const void *p, MPI_Aint *a) { *a = (MPI_Aint)(intptr_t)p; return 0; }
inline int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *disp,
                                  const MPI_Datatype *types, MPI_Datatype *nt) {
  size_t extent = 0;
  for (int i = 0; i < n; ++i) {
    size_t end = (size_t)disp[i] + (size_t)bl[i] * sbdgb_mpi_shim::type_size(types[i]);
    if (end > extent) extent = end;
  }
  *nt = (1 << 20) + (int)extent;
  return 0;
}
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
inline int MPI_Type_free(MPI_Datatype *) { return 0; }

inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)n * sbdgb_mpi_shim::type_size(t)); return 0;
}
inline int MPI_Allreduce_c(const void *s, void *r, MPI_Count n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)n * sbdgb_mpi_shim::type_size(t)); return 0;
}
inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)n * sbdgb_mpi_shim::type_size(t)); return 0;
}
inline int MPI_Exscan(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)n * sbdgb_mpi_shim::type_size(t)); return 0;
}
inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm) {
  sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)sn * sbdgb_mpi_shim::type_size(st)); return 0;
}
inline int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *displs,
                       MPI_Datatype rt, int, MPI_Comm) {
  char *rr = (char *)r + (size_t)displs[0] * sbdgb_mpi_shim::type_size(rt);
  sbdgb_mpi_shim::copy_if_distinct(s, rr, (size_t)sn * sbdgb_mpi_shim::type_size(st)); return 0;
}
inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) {
  sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)sn * sbdgb_mpi_shim::type_size(st)); return 0;
}
inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *displs,
                          MPI_Datatype rt, MPI_Comm) {
  char *rr = (char *)r + (size_t)displs[0] * sbdgb_mpi_shim::type_size(rt);
  sbdgb_mpi_shim::copy_if_distinct(s, rr, (size_t)sn * sbdgb_mpi_shim::type_size(st)); return 0;
}
inline int MPI_Scatter(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm) {
  if (s) sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)sn * sbdgb_mpi_shim::type_size(st));
  return 0;
}
inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) {
  sbdgb_mpi_shim::copy_if_distinct(s, r, (size_t)sn * sbdgb_mpi_shim::type_size(st)); return 0;
}
inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r,
                         const int *, const int *rd, MPI_Datatype rt, MPI_Comm) {
  const char *ss = (const char *)s + (size_t)sd[0] * sbdgb_mpi_shim::type_size(st);
  char *rr = (char *)r + (size_t)rd[0] * sbdgb_mpi_shim::type_size(rt);
  sbdgb_mpi_shim::copy_if_distinct(ss, rr, (size_t)sc[0] * sbdgb_mpi_shim::type_size(st)); return 0;
}

inline int MPI_Send(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm) {
  sbdgb_mpi_shim::deliver(b, (size_t)n * sbdgb_mpi_shim::type_size(t), tag); return 0;
}
inline int MPI_Recv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Status *) {
  if (!sbdgb_mpi_shim::take(b, (size_t)n * sbdgb_mpi_shim::type_size(t), tag))
    throw std::runtime_error("mpi shim: receive without a matching self-send");
  return 0;
}
inline int MPI_Sendrecv(const void *sb, int sn, MPI_Datatype st, int, int stag, void *rb, int rn,
                        MPI_Datatype rt, int, int rtag, MPI_Comm c, MPI_Status *s) {
  MPI_Send(sb, sn, st, 0, stag, c);
  return MPI_Recv(rb, rn, rt, 0, rtag, c, s);
}
inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  sbdgb_mpi_shim::deliver(b, (size_t)n * sbdgb_mpi_shim::type_size(t), tag);
  *req = MPI_REQUEST_NULL; return 0;
}
inline int MPI_Isend_c(const void *b, MPI_Count n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  sbdgb_mpi_shim::deliver(b, (size_t)n * sbdgb_mpi_shim::type_size(t), tag);
  *req = MPI_REQUEST_NULL; return 0;
}
inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  auto &p = sbdgb_mpi_shim::pending();
  p.push_back({b, (size_t)n * sbdgb_mpi_shim::type_size(t), tag, true});
  *req = (int)p.size() - 1; return 0;
}
inline int MPI_Irecv_c(void *b, MPI_Count n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  auto &p = sbdgb_mpi_shim::pending();
  p.push_back({b, (size_t)n * sbdgb_mpi_shim::type_size(t), tag, true});
  *req = (int)p.size() - 1; return 0;
}
inline int MPI_Wait(MPI_Request *req, MPI_Status *) {
  if (*req >= 0) {
    auto &p = sbdgb_mpi_shim::pending();
    if (p[*req].active) {
      if (!sbdgb_mpi_shim::take(p[*req].buf, p[*req].bytes, p[*req].tag))
        throw std::runtime_error("mpi shim: wait on a receive without a matching self-send");
      p[*req].active = false;
    }
    bool any = false;
    for (auto &e : p) any = any || e.active;
    if (!any) p.clear();
  }
  *req = MPI_REQUEST_NULL;
  return 0;
}
inline int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *) {
  for (int i = 0; i < n; ++i) MPI_Wait(&reqs[i], nullptr);
  return 0;
}

#endif
