/*
 * Single-rank stand-in for <mpi.h> — TEST INFRASTRUCTURE ONLY.
 *
 * MPI is not installed in this image. The reference's hot-path sources
 * (src/*.cpp and deps/2Decomp_C/{C2Decomp,MemSplitMerge,Transpose*}.cpp of
 * FattiMei/mpi-incompressible-fluid) are compiled against this header to build
 * the oracle library under oracle/_ref/. It restates the MPI standard's
 * semantics for a communicator of exactly one process:
 *   - MPI_Alltoallv with one peer is a copy of sendcounts[0] elements from
 *     sdispls[0] to rdispls[0] (deps/2Decomp_C/TransposeX2Y.cpp:38 and the
 *     three other transposes rely on it);
 *   - Cartesian topology calls return the parent communicator and coordinate 0;
 *   - point-to-point calls are never reached with one rank (the reference
 *     guards them with prev/next_proc != -1, src/Constants.cpp:98-101), so
 *     they abort loudly if called;
 *   - gathers copy the single contribution, MPI-IO writes go to a POSIX file
 *     (src/VTKDatExport.cpp's writers).
 * A datatype handle encodes its extent in bytes, which is all a single rank
 * needs (MPI_Type_size, MPI_Type_contiguous).
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef long MPI_Datatype; /* extent in bytes */
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_File;
typedef long long MPI_Offset;
typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_COMM_NULL (-1)
#define MPI_PROC_NULL (-2)
#define MPI_SUM 1
#define MPI_REQUEST_NULL 0
#define MPI_INFO_NULL 0
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1

static inline void oracle_mpi_unreachable(const char *what) {
  fprintf(stderr, "oracle mpi shim: %s is not available with a single rank\n", what);
  abort();
}

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Abort(MPI_Comm, int code) { fprintf(stderr, "MPI_Abort(%d)\n", code); abort(); }
static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

static inline int MPI_Type_size(MPI_Datatype t, int *size) { *size = (int)t; return MPI_SUCCESS; }
static inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out) {
  *out = (MPI_Datatype)count * old;
  return MPI_SUCCESS;
}
static inline int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }

static inline int MPI_Cart_create(MPI_Comm comm, int, const int *, const int *, int, MPI_Comm *out) {
  *out = comm;
  return MPI_SUCCESS;
}
static inline int MPI_Cart_coords(MPI_Comm, int, int ndims, int *coords) {
  for (int d = 0; d < ndims; ++d) coords[d] = 0;
  return MPI_SUCCESS;
}
static inline int MPI_Cart_sub(MPI_Comm comm, const int *, MPI_Comm *out) {
  *out = comm;
  return MPI_SUCCESS;
}
static inline int MPI_Cart_shift(MPI_Comm, int, int, int *src, int *dst) {
  *src = MPI_PROC_NULL;
  *dst = MPI_PROC_NULL;
  return MPI_SUCCESS;
}

/* One peer: element block [sdispls[0], +sendcounts[0]) goes to rdispls[0]. */
static inline int MPI_Alltoallv(const void *sendbuf, const int *sendcounts, const int *sdispls,
                                MPI_Datatype sendtype, void *recvbuf, const int *recvcounts,
                                const int *rdispls, MPI_Datatype recvtype, MPI_Comm) {
  if ((long)sendcounts[0] * sendtype != (long)recvcounts[0] * recvtype)
    oracle_mpi_unreachable("MPI_Alltoallv with mismatched byte counts");
  memmove((char *)recvbuf + (long)rdispls[0] * recvtype,
          (const char *)sendbuf + (long)sdispls[0] * sendtype, (size_t)sendcounts[0] * sendtype);
  return MPI_SUCCESS;
}
static inline int MPI_Ialltoallv(const void *sendbuf, const int *sendcounts, const int *sdispls,
                                 MPI_Datatype sendtype, void *recvbuf, const int *recvcounts,
                                 const int *rdispls, MPI_Datatype recvtype, MPI_Comm comm,
                                 MPI_Request *req) {
  *req = MPI_REQUEST_NULL;
  return MPI_Alltoallv(sendbuf, sendcounts, sdispls, sendtype, recvbuf, recvcounts, rdispls,
                       recvtype, comm);
}
static inline int MPI_Wait(MPI_Request *req, MPI_Status *) {
  if (*req != MPI_REQUEST_NULL) oracle_mpi_unreachable("MPI_Wait on a live request");
  return MPI_SUCCESS;
}
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
  oracle_mpi_unreachable("MPI_Isend");
  return 1;
}
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
  oracle_mpi_unreachable("MPI_Send");
  return 1;
}
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  oracle_mpi_unreachable("MPI_Recv");
  return 1;
}
/* One rank: the reduction of a single contribution is the contribution. */
static inline int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype t, int,
                                MPI_Comm) {
  memmove(recvbuf, sendbuf, (size_t)count * (size_t)t);
  return MPI_SUCCESS;
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

/* Gathers: the single contribution is the whole result. */
static inline int MPI_Allgather(const void *sendbuf, int scount, MPI_Datatype stype, void *recvbuf, int,
                                MPI_Datatype, MPI_Comm) {
  memmove(recvbuf, sendbuf, (size_t)scount * (size_t)stype);
  return MPI_SUCCESS;
}
static inline int MPI_Gather(const void *sendbuf, int scount, MPI_Datatype stype, void *recvbuf, int,
                             MPI_Datatype, int, MPI_Comm) {
  memmove(recvbuf, sendbuf, (size_t)scount * (size_t)stype);
  return MPI_SUCCESS;
}
/* The one contribution lands at the start of recvbuf. (writeDat computes its
 * displacement array from element -1, src/VTKDatExport.cpp:529-531; with one
 * rank the intended displacement is 0.) */
static inline int MPI_Gatherv(const void *sendbuf, int scount, MPI_Datatype stype, void *recvbuf, const int *,
                              const int *, MPI_Datatype, int, MPI_Comm) {
  memmove(recvbuf, sendbuf, (size_t)scount * (size_t)stype);
  return MPI_SUCCESS;
}

/* MPI-IO for one process: positioned writes on a POSIX file descriptor. An
 * existing file is not truncated (the MPI standard's MPI_File_open). */
#include <fcntl.h>
#include <unistd.h>
static inline int MPI_File_open(MPI_Comm, const char *filename, int amode, MPI_Info, MPI_File *fh) {
  const int flags = ((amode & MPI_MODE_CREATE) ? O_CREAT : 0) | ((amode & MPI_MODE_WRONLY) ? O_WRONLY : O_RDONLY);
  const int fd = open(filename, flags, 0644);
  if (fd < 0) return 1;
  *fh = fd;
  return MPI_SUCCESS;
}
static inline int MPI_File_write_at(MPI_File fh, MPI_Offset offset, const void *buf, int count, MPI_Datatype t,
                                    MPI_Status *) {
  const size_t n = (size_t)count * (size_t)t;
  return pwrite(fh, buf, n, (off_t)offset) == (ssize_t)n ? MPI_SUCCESS : 1;
}
static inline int MPI_File_close(MPI_File *fh) {
  close(*fh);
  *fh = -1;
  return MPI_SUCCESS;
}

#endif /* ORACLE_SHIM_MPI_H */
