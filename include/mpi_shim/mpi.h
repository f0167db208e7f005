/*
 * mpi.h - single-process stand-in for the MPI subset used by AccFFT programs.
 *
 * The GB300 path runs on one rank; builds without an MPI installation put
 * this directory on the include path.  Every communicator has one rank
 * (rank 0); Cartesian communicators must be 1 x 1; reductions copy their
 * input.  Programs that need more than one rank need a real MPI and are
 * outside this path.
 */
#ifndef ACCFFT_MPI_SHIM_H
#define ACCFFT_MPI_SHIM_H

#include <stddef.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef long long MPI_Offset;

#define MPI_COMM_WORLD 0x44000000
#define MPI_COMM_SELF 0x44000001
#define MPI_COMM_NULL 0x04000000
#define MPI_SUCCESS 0
#define MPI_ERR_DIMS 11

#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_LONG 8
#define MPI_LONG_LONG 9
#define MPI_FLOAT 14
#define MPI_DOUBLE 18
#define MPI_UNSIGNED 20

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline int accfft_mpi_shim_type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: case MPI_FLOAT: case MPI_UNSIGNED: return 4;
    case MPI_LONG: case MPI_LONG_LONG: case MPI_DOUBLE: return 8;
    default: return 0;
  }
}

static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Initialized(int* flag) { *flag = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return MPI_SUCCESS; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out) {
  (void)color; (void)key; *out = c; return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return MPI_SUCCESS; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; return code; }
static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Dims_create(int nnodes, int ndims, int* dims) {
  if (nnodes != 1) return MPI_ERR_DIMS;
  for (int i = 0; i < ndims; ++i) dims[i] = 1;
  return MPI_SUCCESS;
}
static inline int MPI_Cart_create(MPI_Comm c, int ndims, const int* dims, const int* periods, int reorder,
                                  MPI_Comm* out) {
  (void)periods; (void)reorder;
  for (int i = 0; i < ndims; ++i)
    if (dims[i] != 1) return MPI_ERR_DIMS;
  *out = c;
  return MPI_SUCCESS;
}
static inline int MPI_Cart_get(MPI_Comm c, int maxdims, int* dims, int* periods, int* coords) {
  (void)c;
  for (int i = 0; i < maxdims; ++i) { dims[i] = 1; periods[i] = 0; coords[i] = 0; }
  return MPI_SUCCESS;
}
static inline int MPI_Cart_coords(MPI_Comm c, int rank, int maxdims, int* coords) {
  (void)c; (void)rank;
  for (int i = 0; i < maxdims; ++i) coords[i] = 0;
  return MPI_SUCCESS;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
  (void)op; (void)root; (void)c;
  if (s != r) memcpy(r, s, (size_t)n * accfft_mpi_shim_type_size(t));
  return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  return MPI_Reduce(s, r, n, t, op, 0, c);
}
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)root; (void)c;
  return MPI_SUCCESS;
}

#endif /* ACCFFT_MPI_SHIM_H */
