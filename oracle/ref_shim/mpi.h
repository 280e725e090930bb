/*
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * Single-rank stand-in for the MPI calls the reference's groundwater sources make
 * (src/core/MpiComm.cpp, src/re/ReSolver.cpp:916-920, src/perf/PerfRecorder.cpp), so they
 * compile here unchanged into oracle/_ref.  MPICH is not installed in this image.  One rank:
 * rank 0 of size 1, every neighbour is MPI_PROC_NULL (messages to it are dropped, as MPI
 * specifies), and a reduction over one rank copies its input.
 */
#ifndef FREHG_REF_SHIM_MPI_H
#define FREHG_REF_SHIM_MPI_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct MPI_Status {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_INT64_T 3
#define MPI_LONG_LONG 3
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3

static inline size_t frehg_ref_mpi_size_of(MPI_Datatype t) {
  return t == MPI_DOUBLE ? sizeof(double) : t == MPI_INT ? sizeof(int) : sizeof(int64_t);
}

static inline int MPI_Comm_rank(MPI_Comm, int* r) {
  *r = 0;
  return MPI_SUCCESS;
}
static inline int MPI_Comm_size(MPI_Comm, int* s) {
  *s = 1;
  return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void* in, void* out, int count, MPI_Datatype t, MPI_Op,
                                MPI_Comm) {
  if (in != out) memmove(out, in, (size_t)count * frehg_ref_mpi_size_of(t));
  return MPI_SUCCESS;
}
static inline int MPI_Sendrecv(const void*, int, MPI_Datatype, int dest, int, void*, int,
                               MPI_Datatype, int source, int, MPI_Comm, MPI_Status*) {
  /* one rank: both partners are MPI_PROC_NULL */
  if (dest != MPI_PROC_NULL || source != MPI_PROC_NULL) abort();
  return MPI_SUCCESS;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int dest, int, MPI_Comm) {
  if (dest != MPI_PROC_NULL) abort();
  return MPI_SUCCESS;
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int source, int, MPI_Comm, MPI_Status*) {
  if (source != MPI_PROC_NULL) abort();
  return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

#endif /* FREHG_REF_SHIM_MPI_H */
