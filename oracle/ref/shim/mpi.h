/*
 * Single-rank MPI stand-in used only to compile the reference sources into the oracle
 * (oracle/build_ref.sh).  Rank 0 of 1; collectives copy; point-to-point messages go
 * through an in-process loopback queue (the loader's self-send, src/Graph.cpp:500-578).
 * Test infrastructure, not product code.
 */
#ifndef ZGREF_SHIM_MPI_H
#define ZGREF_SHIM_MPI_H

#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
#include <deque>
#include <mutex>
#include <vector>
#include <condition_variable>
#endif

typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; int count; } MPI_Status;

/* datatype handles encode their size in bytes */
#define MPI_CHAR            1
#define MPI_UNSIGNED_CHAR   0x101
#define MPI_INT             4
#define MPI_UNSIGNED        0x104
#define MPI_FLOAT           0x204
#define MPI_LONG            8
#define MPI_UNSIGNED_LONG   0x108
#define MPI_DOUBLE          0x208

#define MPI_COMM_WORLD      0
#define MPI_SUM             1
#define MPI_MAX             2
#define MPI_MIN             3
#define MPI_ANY_SOURCE      (-1)
#define MPI_THREAD_MULTIPLE 3
#define MPI_IN_PLACE        ((void*)1)
#define MPI_STATUS_IGNORE   ((MPI_Status*)0)

static inline int zgref_mpi_size(MPI_Datatype t) { return t & 0xff; }

static inline int MPI_Init_thread(int*, char***, int, int* provided) {
  if (provided) *provided = MPI_THREAD_MULTIPLE;
  return 0;
}
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op,
                                MPI_Comm) {
  if (send != MPI_IN_PLACE) memcpy(recv, send, (size_t)count * zgref_mpi_size(t));
  return 0;
}

#ifdef __cplusplus
/* loopback queue for self-sends */
struct zgref_msg { int tag; std::vector<char> data; };
struct zgref_loopback {
  std::mutex mu;
  std::condition_variable cv;
  std::deque<zgref_msg> q;
};
static inline zgref_loopback& zgref_lb() { static zgref_loopback lb; return lb; }

static inline int MPI_Send(const void* buf, int count, MPI_Datatype t, int, int tag, MPI_Comm) {
  zgref_msg m;
  m.tag = tag;
  m.data.assign((const char*)buf, (const char*)buf + (size_t)count * zgref_mpi_size(t));
  std::lock_guard<std::mutex> g(zgref_lb().mu);
  zgref_lb().q.push_back(m);
  zgref_lb().cv.notify_all();
  return 0;
}
static inline int MPI_Probe(int, int tag, MPI_Comm, MPI_Status* st) {
  std::unique_lock<std::mutex> g(zgref_lb().mu);
  zgref_lb().cv.wait(g, [] { return !zgref_lb().q.empty(); });
  if (st) {
    st->MPI_SOURCE = 0;
    st->MPI_TAG = zgref_lb().q.front().tag;
    st->count = (int)zgref_lb().q.front().data.size();
  }
  (void)tag;
  return 0;
}
static inline int MPI_Get_count(const MPI_Status* st, MPI_Datatype t, int* c) {
  *c = st->count / zgref_mpi_size(t);
  return 0;
}
static inline int MPI_Recv(void* buf, int count, MPI_Datatype t, int, int, MPI_Comm,
                           MPI_Status* st) {
  std::unique_lock<std::mutex> g(zgref_lb().mu);
  zgref_lb().cv.wait(g, [] { return !zgref_lb().q.empty(); });
  zgref_msg m = zgref_lb().q.front();
  zgref_lb().q.pop_front();
  size_t n = (size_t)count * zgref_mpi_size(t);
  if (n > m.data.size()) n = m.data.size();
  memcpy(buf, m.data.data(), n);
  if (st) { st->MPI_SOURCE = 0; st->MPI_TAG = m.tag; st->count = (int)n; }
  return 0;
}
#endif

#endif
