/*
 * mpi.h - one-rank MPI for compiling AccFFT's CPU host code (src/accfft.cpp,
 * src/accfft_common.cpp, src/operators.cpp, src/transpose.cpp) as the
 * parity reference.  TEST INFRASTRUCTURE ONLY: nothing in the product links
 * it; oracle/build_ref.py compiles the reference against it into oracle/_ref.
 *
 * Every communicator has exactly one rank.  Collectives and self-sends copy
 * the caller's buffers (Alltoall(v/w), Sendrecv, Isend/Irecv matched by tag);
 * derived datatypes carry their data size and whether they are contiguous,
 * and a data movement with a non-contiguous one aborts with a message (at one
 * rank the reference's transposes return before any such call:
 * src/transpose.cpp:824-830).  Implemented in ref_shim.c.
 */
#ifndef ORACLE_REF_MPI_SHIM_H
#define ORACLE_REF_MPI_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef ptrdiff_t MPI_Aint;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
  long long count_bytes;
} MPI_Status;
typedef void MPI_User_function(void* invec, void* inoutvec, int* len, MPI_Datatype* datatype);

#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_REQUEST_NULL 0
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_PROC_NULL (-2)

/* predefined datatypes (handles 1..63); derived types get handles from 64 */
#define MPI_CHAR 1
#define MPI_BYTE 2
#define MPI_SHORT 3
#define MPI_INT 4
#define MPI_LONG 5
#define MPI_LONG_LONG_INT 6
#define MPI_LONG_LONG 6
#define MPI_UNSIGNED_CHAR 7
#define MPI_UNSIGNED_SHORT 8
#define MPI_UNSIGNED 9
#define MPI_UNSIGNED_LONG 10
#define MPI_FLOAT 11
#define MPI_DOUBLE 12
#define MPI_LONG_DOUBLE 13
#define MPI_FLOAT_INT 14
#define MPI_DOUBLE_INT 15
#define MPI_LONG_INT 16
#define MPI_SHORT_INT 17
#define MPI_LONG_DOUBLE_INT 18
#define MPI_2INT 19
#define MPI_UNSIGNED_LONG_LONG 20

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROD 4
#define MPI_LAND 5
#define MPI_LOR 6

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Initialized(int* flag);
double MPI_Wtime(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Barrier(MPI_Comm comm);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* out);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Dims_create(int nnodes, int ndims, int* dims);
int MPI_Cart_create(MPI_Comm comm, int ndims, const int* dims, const int* periods, int reorder, MPI_Comm* out);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int* coords);

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out);
int MPI_Type_vector(int count, int blocklen, int stride, MPI_Datatype old, MPI_Datatype* out);
int MPI_Type_hvector(int count, int blocklen, MPI_Aint stride, MPI_Datatype old, MPI_Datatype* out);
int MPI_Type_create_struct(int count, const int* blocklens, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* out);
int MPI_Type_commit(MPI_Datatype* t);
int MPI_Type_free(MPI_Datatype* t);
int MPI_Type_size(MPI_Datatype t, int* size);
int MPI_Op_create(MPI_User_function* fn, int commute, MPI_Op* op);
int MPI_Op_free(MPI_Op* op);

int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Alltoall(const void* s, int scount, MPI_Datatype st, void* r, int rcount, MPI_Datatype rt, MPI_Comm comm);
int MPI_Alltoallv(const void* s, const int* scounts, const int* sdispls, MPI_Datatype st, void* r, const int* rcounts,
                  const int* rdispls, MPI_Datatype rt, MPI_Comm comm);
int MPI_Alltoallw(const void* s, const int* scounts, const int* sdispls, const MPI_Datatype* sts, void* r,
                  const int* rcounts, const int* rdispls, const MPI_Datatype* rts, MPI_Comm comm);
int MPI_Sendrecv(const void* s, int scount, MPI_Datatype st, int dest, int stag, void* r, int rcount,
                 MPI_Datatype rt, int source, int rtag, MPI_Comm comm, MPI_Status* status);
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Issend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Wait(MPI_Request* req, MPI_Status* status);
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses);

#ifdef __cplusplus
}
#endif

#endif /* ORACLE_REF_MPI_SHIM_H */
