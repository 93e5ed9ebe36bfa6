/*
 * Single-process stand-in for the handful of MPI calls the lbmminiapp CPU
 * sources make.  It exists only so the reference's serial C++ path can be
 * compiled as a test oracle on a machine without an MPI installation.
 *
 * Semantics are those of a world of exactly one rank:
 *   - rank 0, size 1;
 *   - Bcast / Barrier are no-ops;
 *   - Allreduce copies send -> recv (or does nothing for MPI_IN_PLACE);
 *   - point-to-point calls are never reached with a neighbour on one rank
 *     (the reference's Communication::exchange loops over zero neighbours),
 *     so they only complete immediately;
 *   - Wtime is a monotonic wall clock in seconds.
 *
 * Test infrastructure only: nothing in the product library includes this.
 */
#ifndef LBM_ORACLE_MPI_STUB_H
#define LBM_ORACLE_MPI_STUB_H

#include <string.h>
#include <time.h>
#include <stdint.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0

#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_INT64_T 3
#define MPI_FLOAT 4

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

static inline size_t lbm_stub_type_size(MPI_Datatype t)
{
   switch (t) {
      case MPI_INT: return sizeof(int);
      case MPI_DOUBLE: return sizeof(double);
      case MPI_INT64_T: return sizeof(int64_t);
      case MPI_FLOAT: return sizeof(float);
      default: return 1;
   }
}

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

static inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t,
                                MPI_Op, MPI_Comm)
{
   if (send != MPI_IN_PLACE && send != recv) {
      memcpy(recv, send, (size_t)count * lbm_stub_type_size(t));
   }
   return MPI_SUCCESS;
}

static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r)
{
   *r = 0;
   return MPI_SUCCESS;
}

static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r)
{
   *r = 0;
   return MPI_SUCCESS;
}

static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }

static inline double MPI_Wtime(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#endif
