/* Single-rank stand-in for the MPI API, used only to compile the reference
 * MURaM hot-path sources on a machine without an MPI installation.
 *
 * Test infrastructure: this header is part of the oracle build and is never
 * linked into the product library.
 *
 * Semantics for one rank:
 *  - reductions copy send to receive buffers (identity on one rank);
 *  - Cartesian topology: rank 0 at coords (0,0,0), every neighbour is rank 0;
 *  - point-to-point: MPI_Irecv posts a (buffer, count, tag) receive, MPI_Isend
 *    delivers into the matching posted receive immediately (the reference's
 *    exchange posts each receive before the matching send), Waitall is a no-op.
 */
#ifndef GPUMHD_ORACLE_MPI_STUB_H
#define GPUMHD_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_NULL (-1)
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_PROC_NULL (-2)
#define MPI_ORDER_FORTRAN 1
#define MPI_ORDER_C 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SINGLE 0

/* Datatype handles encode the element size in bytes. */
#define MPI_BYTE 1
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 1004
#define MPI_DOUBLE 8
#define MPI_LONG 1008

#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3

static inline int gpumhd_stub_typesize(MPI_Datatype t) {
  if (t == MPI_FLOAT) return 4;
  if (t == MPI_LONG) return 8;
  if (t > 0 && t < 1000) return t;
  if (t >= 2000) return t - 2000; /* derived contiguous types */
  return 1;
}

static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Init_thread(int*, char***, int, int* p) { if (p) *p = MPI_THREAD_FUNNELED; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) {
  fprintf(stderr, "MPI_Abort(%d) called by the reference code\n", code);
  exit(code == 0 ? 3 : code);
}
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_split(MPI_Comm, int, int, MPI_Comm* c) { *c = 0; return 0; }
static inline int MPI_Comm_free(MPI_Comm*) { return 0; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != r) memmove(r, s, (size_t)n * gpumhd_stub_typesize(t));
  return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != r && r) memmove(r, s, (size_t)n * gpumhd_stub_typesize(t));
  return 0;
}
static inline int MPI_Type_contiguous(int n, MPI_Datatype t, MPI_Datatype* nt) {
  *nt = 2000 + n * gpumhd_stub_typesize(t);
  return 0;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline int MPI_Type_free(MPI_Datatype*) { return 0; }
static inline int MPI_Type_create_subarray(int, const int*, const int*, const int*, int,
                                           MPI_Datatype t, MPI_Datatype* nt) { *nt = t; return 0; }
static inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* c) { *c = 0; return 0; }
static inline int MPI_Cart_coords(MPI_Comm, int, int n, int* coords) {
  for (int i = 0; i < n; i++) coords[i] = 0;
  return 0;
}
static inline int MPI_Cart_shift(MPI_Comm, int, int, int* src, int* dst) { *src = 0; *dst = 0; return 0; }

/* Self-messaging mailbox for the one-rank halo exchange. */
struct gpumhd_stub_recv { void* buf; size_t bytes; int tag; int used; };
#define GPUMHD_STUB_MAXRECV 64
static struct gpumhd_stub_recv gpumhd_stub_posted[GPUMHD_STUB_MAXRECV];

static inline int MPI_Irecv(void* buf, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request* rq) {
  for (int i = 0; i < GPUMHD_STUB_MAXRECV; i++) {
    if (!gpumhd_stub_posted[i].used) {
      gpumhd_stub_posted[i].buf = buf;
      gpumhd_stub_posted[i].bytes = (size_t)n * gpumhd_stub_typesize(t);
      gpumhd_stub_posted[i].tag = tag;
      gpumhd_stub_posted[i].used = 1;
      if (rq) *rq = i;
      return 0;
    }
  }
  fprintf(stderr, "mpi stub: too many posted receives\n");
  exit(4);
}
static inline int MPI_Isend(const void* buf, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request* rq) {
  size_t bytes = (size_t)n * gpumhd_stub_typesize(t);
  for (int i = 0; i < GPUMHD_STUB_MAXRECV; i++) {
    if (gpumhd_stub_posted[i].used && gpumhd_stub_posted[i].tag == tag) {
      size_t m = bytes < gpumhd_stub_posted[i].bytes ? bytes : gpumhd_stub_posted[i].bytes;
      memcpy(gpumhd_stub_posted[i].buf, buf, m);
      gpumhd_stub_posted[i].used = 0;
      if (rq) *rq = -1;
      return 0;
    }
  }
  fprintf(stderr, "mpi stub: send with tag %d has no posted receive\n", tag);
  exit(4);
}
static inline int MPI_Send(const void* buf, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  return MPI_Isend(buf, n, t, d, tag, c, 0);
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }

#endif
