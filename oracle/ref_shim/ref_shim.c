/*
 * ref_shim.c - implementation of the one-rank MPI (mpi.h) and the FFTW3
 * subset (fftw3.h) that AccFFT's CPU host code is compiled against to serve
 * as the parity reference.  TEST INFRASTRUCTURE ONLY (see mpi.h, fftw3.h).
 *
 * The DFT itself is the oracle's long-double recursive mixed-radix transform
 * (oracle_core.h through fft_oracle.c), so the reference's own plan
 * geometry, pass order, index maps, transposes and wave-number loops run
 * unchanged around an independent restatement of FFTW's arithmetic.
 */
#include "../fft_oracle.c"

#include <stdint.h>
#include <stdio.h>
#include <time.h>

#include "fftw3.h"
#include "mpi.h"

static void shim_fail(const char* what) {
  fprintf(stderr, "oracle reference shim: %s\n", what);
  fflush(stderr);
  abort();
}

/* ================================================================== MPI */

#define SHIM_MAX_TYPES 8192
typedef struct {
  long long size; /* bytes of data in one element of this type */
  int contig;     /* 1 if those bytes are contiguous in memory */
  int live;
} shim_type;
static shim_type g_types[SHIM_MAX_TYPES];
static int g_next_type = 64;

static long long predefined_size(int t) {
  switch (t) {
    case MPI_CHAR: case MPI_BYTE: case MPI_UNSIGNED_CHAR: return 1;
    case MPI_SHORT: case MPI_UNSIGNED_SHORT: return 2;
    case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
    case MPI_LONG: case MPI_UNSIGNED_LONG: return (long long)sizeof(long);
    case MPI_LONG_LONG_INT: case MPI_UNSIGNED_LONG_LONG: case MPI_DOUBLE: return 8;
    case MPI_LONG_DOUBLE: return (long long)sizeof(long double);
    case MPI_FLOAT_INT: { struct { float a; int b; } s; return (long long)sizeof s; }
    case MPI_DOUBLE_INT: { struct { double a; int b; } s; return (long long)sizeof s; }
    case MPI_LONG_INT: { struct { long a; int b; } s; return (long long)sizeof s; }
    case MPI_SHORT_INT: { struct { short a; int b; } s; return (long long)sizeof s; }
    case MPI_LONG_DOUBLE_INT: { struct { long double a; int b; } s; return (long long)sizeof s; }
    case MPI_2INT: return 8;
    default: return -1;
  }
}

static shim_type type_of(MPI_Datatype t) {
  shim_type r = {0, 1, 1};
  long long p = predefined_size(t);
  if (p > 0) { r.size = p; return r; }
  if (t < 64 || t >= SHIM_MAX_TYPES || !g_types[t].live) shim_fail("unknown MPI datatype");
  return g_types[t];
}

static MPI_Datatype new_type(long long size, int contig) {
  if (g_next_type >= SHIM_MAX_TYPES) shim_fail("too many MPI datatypes");
  int h = g_next_type++;
  g_types[h].size = size;
  g_types[h].contig = contig;
  g_types[h].live = 1;
  return h;
}

static long long contig_bytes(MPI_Datatype t, long long count) {
  shim_type s = type_of(t);
  if (!s.contig && count > 0) shim_fail("data movement with a non-contiguous datatype (unreachable at one rank)");
  return s.size * count;
}

int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Initialized(int* flag) { *flag = 1; return MPI_SUCCESS; }
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Abort(MPI_Comm comm, int code) {
  (void)comm;
  fprintf(stderr, "oracle reference shim: MPI_Abort(%d)\n", code);
  exit(code ? code : 1);
}
int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int* rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm comm, int* size) { (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* out) {
  (void)color; (void)key;
  *out = comm;
  return MPI_SUCCESS;
}
int MPI_Comm_free(MPI_Comm* comm) { *comm = MPI_COMM_NULL; return MPI_SUCCESS; }
int MPI_Dims_create(int nnodes, int ndims, int* dims) {
  if (nnodes != 1) return MPI_ERR_OTHER;
  for (int i = 0; i < ndims; ++i) dims[i] = 1;
  return MPI_SUCCESS;
}
int MPI_Cart_create(MPI_Comm comm, int ndims, const int* dims, const int* periods, int reorder, MPI_Comm* out) {
  (void)periods; (void)reorder;
  for (int i = 0; i < ndims; ++i)
    if (dims[i] != 1) shim_fail("Cartesian grid other than 1 x 1 on one rank");
  *out = comm;
  return MPI_SUCCESS;
}
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords) {
  (void)comm;
  for (int i = 0; i < maxdims; ++i) { dims[i] = 1; periods[i] = 0; coords[i] = 0; }
  return MPI_SUCCESS;
}
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int* coords) {
  (void)comm; (void)rank;
  for (int i = 0; i < maxdims; ++i) coords[i] = 0;
  return MPI_SUCCESS;
}

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) {
  shim_type o = type_of(old);
  *out = new_type(o.size * count, o.contig);
  return MPI_SUCCESS;
}
int MPI_Type_vector(int count, int blocklen, int stride, MPI_Datatype old, MPI_Datatype* out) {
  shim_type o = type_of(old);
  *out = new_type(o.size * (long long)count * blocklen, o.contig && (count <= 1 || stride == blocklen));
  return MPI_SUCCESS;
}
int MPI_Type_hvector(int count, int blocklen, MPI_Aint stride, MPI_Datatype old, MPI_Datatype* out) {
  shim_type o = type_of(old);
  *out = new_type(o.size * (long long)count * blocklen,
                  o.contig && (count <= 1 || stride == (MPI_Aint)(o.size * blocklen)));
  return MPI_SUCCESS;
}
int MPI_Type_create_struct(int count, const int* blocklens, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* out) {
  long long size = 0;
  int contig = 1;
  for (int i = 0; i < count; ++i) {
    shim_type t = type_of(types[i]);
    if (displs[i] != (MPI_Aint)size || !t.contig) contig = 0;
    size += t.size * blocklens[i];
  }
  *out = new_type(size, contig);
  return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype* t) { (void)type_of(*t); return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype* t) {
  if (*t >= 64 && *t < SHIM_MAX_TYPES) g_types[*t].live = 0;
  *t = 0;
  return MPI_SUCCESS;
}
int MPI_Type_size(MPI_Datatype t, int* size) { *size = (int)type_of(t).size; return MPI_SUCCESS; }
int MPI_Op_create(MPI_User_function* fn, int commute, MPI_Op* op) {
  (void)fn; (void)commute;
  static int next = 100;
  *op = next++;
  return MPI_SUCCESS;
}
int MPI_Op_free(MPI_Op* op) { *op = 0; return MPI_SUCCESS; }

int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)t; (void)root; (void)comm;
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm) {
  (void)op; (void)root; (void)comm;
  if (s != r) memmove(r, s, (size_t)contig_bytes(t, count));
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm) {
  return MPI_Reduce(s, r, count, t, op, 0, comm);
}
int MPI_Alltoall(const void* s, int scount, MPI_Datatype st, void* r, int rcount, MPI_Datatype rt, MPI_Comm comm) {
  (void)comm;
  long long sb = contig_bytes(st, scount), rb = contig_bytes(rt, rcount);
  if (sb != rb) shim_fail("Alltoall with different send and receive sizes");
  if (s != r) memmove(r, s, (size_t)sb);
  return MPI_SUCCESS;
}
int MPI_Alltoallv(const void* s, const int* scounts, const int* sdispls, MPI_Datatype st, void* r, const int* rcounts,
                  const int* rdispls, MPI_Datatype rt, MPI_Comm comm) {
  (void)comm;
  long long sb = contig_bytes(st, scounts[0]), rb = contig_bytes(rt, rcounts[0]);
  if (sb != rb) shim_fail("Alltoallv with different send and receive sizes");
  memmove((char*)r + type_of(rt).size * rdispls[0], (const char*)s + type_of(st).size * sdispls[0], (size_t)sb);
  return MPI_SUCCESS;
}
int MPI_Alltoallw(const void* s, const int* scounts, const int* sdispls, const MPI_Datatype* sts, void* r,
                  const int* rcounts, const int* rdispls, const MPI_Datatype* rts, MPI_Comm comm) {
  (void)comm;
  long long sb = contig_bytes(sts[0], scounts[0]), rb = contig_bytes(rts[0], rcounts[0]);
  if (sb != rb) shim_fail("Alltoallw with different send and receive sizes");
  memmove((char*)r + rdispls[0], (const char*)s + sdispls[0], (size_t)sb);
  return MPI_SUCCESS;
}
int MPI_Sendrecv(const void* s, int scount, MPI_Datatype st, int dest, int stag, void* r, int rcount,
                 MPI_Datatype rt, int source, int rtag, MPI_Comm comm, MPI_Status* status) {
  (void)dest; (void)stag; (void)source; (void)rtag; (void)comm;
  long long sb = contig_bytes(st, scount), rb = contig_bytes(rt, rcount);
  if (sb > rb) shim_fail("Sendrecv message longer than the receive buffer");
  memmove(r, s, (size_t)sb);
  if (status) { status->MPI_SOURCE = 0; status->MPI_TAG = rtag; status->MPI_ERROR = 0; status->count_bytes = sb; }
  return MPI_SUCCESS;
}

/* self-messages: a send and a receive with the same tag are matched in the
 * order they were posted; the copy happens when the second one is posted */
#define SHIM_MAX_REQ 65536
typedef struct {
  int live, is_send, tag, done;
  const void* sbuf;
  void* rbuf;
  long long bytes;
} shim_req;
static shim_req g_req[SHIM_MAX_REQ];
static int g_next_req = 1;

static int post(int is_send, const void* sbuf, void* rbuf, long long bytes, int tag, MPI_Request* req) {
  for (int i = 1; i < g_next_req; ++i) {
    shim_req* q = &g_req[i];
    if (q->live && !q->done && q->is_send != is_send && (q->tag == tag || tag == MPI_ANY_TAG || q->tag == MPI_ANY_TAG)) {
      const void* src = is_send ? sbuf : q->sbuf;
      void* dst = is_send ? q->rbuf : rbuf;
      long long sb = is_send ? bytes : q->bytes, rb = is_send ? q->bytes : bytes;
      if (sb > rb) shim_fail("self-message longer than the receive buffer");
      memmove(dst, src, (size_t)sb);
      q->done = 1;
      *req = MPI_REQUEST_NULL;
      return MPI_SUCCESS;
    }
  }
  if (g_next_req >= SHIM_MAX_REQ) {
    /* recycle: every request below is complete once all are waited on */
    int busy = 0;
    for (int i = 1; i < g_next_req; ++i) busy |= g_req[i].live;
    if (busy) shim_fail("too many outstanding self-messages");
    g_next_req = 1;
  }
  int h = g_next_req++;
  shim_req q = {1, is_send, tag, 0, sbuf, rbuf, bytes};
  g_req[h] = q;
  *req = h;
  return MPI_SUCCESS;
}

int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request* req) {
  (void)comm;
  if (dest != 0) shim_fail("send to a rank other than 0");
  return post(1, buf, NULL, contig_bytes(t, count), tag, req);
}
int MPI_Issend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request* req) {
  return MPI_Isend(buf, count, t, dest, tag, comm, req);
}
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm, MPI_Request* req) {
  (void)comm;
  if (source != 0 && source != MPI_ANY_SOURCE) shim_fail("receive from a rank other than 0");
  return post(0, NULL, buf, contig_bytes(t, count), tag, req);
}
int MPI_Wait(MPI_Request* req, MPI_Status* status) {
  if (*req != MPI_REQUEST_NULL) {
    shim_req* q = &g_req[*req];
    if (!q->live || !q->done) shim_fail("wait on a self-message that nothing matched (would deadlock)");
    q->live = 0;
    *req = MPI_REQUEST_NULL;
  }
  if (status) { status->MPI_SOURCE = 0; status->MPI_TAG = 0; status->MPI_ERROR = 0; status->count_bytes = 0; }
  return MPI_SUCCESS;
}
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses) {
  for (int i = 0; i < count; ++i) MPI_Wait(&reqs[i], statuses ? &statuses[i] : MPI_STATUS_IGNORE);
  return MPI_SUCCESS;
}

/* ================================================================= FFTW */

enum { KIND_C2C = 0, KIND_R2C = 1, KIND_C2R = 2 };
#define SHIM_MAX_HM 4

struct oracle_fftw_plan_s {
  int kind, n, sign, hr;
  long long is, os;
  long long hn[SHIM_MAX_HM], his[SHIM_MAX_HM], hos[SHIM_MAX_HM];
  long long nlines;
  void* in;
  void* out;
  plan1d_l pl;
};

static int g_fftw_threads = 1;

static fftw_plan make(int kind, int rank, int n, long long is, long long os, int hr, const long long* hn,
                      const long long* his, const long long* hos, void* in, void* out, int sign) {
  if (rank != 1) shim_fail("FFTW plan of rank other than 1");
  if (hr < 0 || hr > SHIM_MAX_HM) shim_fail("FFTW howmany rank above 4");
  fftw_plan p = (fftw_plan)calloc(1, sizeof *p);
  p->kind = kind;
  p->n = n;
  p->sign = sign;
  p->is = is;
  p->os = os;
  p->hr = hr;
  p->nlines = 1;
  for (int i = 0; i < hr; ++i) {
    p->hn[i] = hn[i];
    p->his[i] = his[i];
    p->hos[i] = hos[i];
    p->nlines *= hn[i];
  }
  p->in = in;
  p->out = out;
  if (n < 1 || plan_init_l(&p->pl, n)) shim_fail("FFTW plan of an unsupported length");
  return p;
}

typedef struct {
  fftw_plan p;
  const void* in;
  void* out;
} shim_exec;

static void line_offsets(const struct oracle_fftw_plan_s* p, long long li, long long* io, long long* oo) {
  long long i = 0, o = 0;
  for (int d = p->hr - 1; d >= 0; --d) {
    long long c = li % p->hn[d];
    li /= p->hn[d];
    i += c * p->his[d];
    o += c * p->hos[d];
  }
  *io = i;
  *oo = o;
}

static void exec_worker(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  shim_exec* E = (shim_exec*)ctx;
  const struct oracle_fftw_plan_s* p = E->p;
  const int n = p->n, h = n / 2 + 1;
  cpx_l* buf = (cpx_l*)malloc(sizeof(cpx_l) * (3 * (size_t)n + 8));
  for (long long li = b0; li < b1; ++li) {
    long long io, oo;
    line_offsets(p, li, &io, &oo);
    if (p->kind == KIND_C2C) {
      const double* s = (const double*)E->in;
      for (int j = 0; j < n; ++j) {
        buf[j].re = s[2 * (io + j * p->is)];
        buf[j].im = s[2 * (io + j * p->is) + 1];
      }
      fft_line_l(&p->pl, buf, buf + n, p->sign, buf + 2 * n);
      double* d = (double*)E->out;
      for (int k = 0; k < n; ++k) {
        d[2 * (oo + k * p->os)] = (double)buf[n + k].re;
        d[2 * (oo + k * p->os) + 1] = (double)buf[n + k].im;
      }
    } else if (p->kind == KIND_R2C) {
      const double* s = (const double*)E->in;
      for (int j = 0; j < n; ++j) {
        buf[j].re = s[io + j * p->is];
        buf[j].im = 0;
      }
      fft_line_l(&p->pl, buf, buf + n, -1, buf + 2 * n);
      double* d = (double*)E->out;
      for (int k = 0; k < h; ++k) {
        d[2 * (oo + k * p->os)] = (double)buf[n + k].re;
        d[2 * (oo + k * p->os) + 1] = (double)buf[n + k].im;
      }
    } else {
      const double* s = (const double*)E->in;
      for (int k = 0; k < h; ++k) {
        buf[k].re = s[2 * (io + k * p->is)];
        buf[k].im = s[2 * (io + k * p->is) + 1];
      }
      buf[0].im = 0;
      if (n % 2 == 0) buf[n / 2].im = 0;
      for (int k = h; k < n; ++k) {
        buf[k].re = buf[n - k].re;
        buf[k].im = -buf[n - k].im;
      }
      fft_line_l(&p->pl, buf, buf + n, +1, buf + 2 * n);
      double* d = (double*)E->out;
      for (int j = 0; j < n; ++j) d[oo + j * p->os] = (double)buf[n + j].re;
    }
  }
  free(buf);
}

/* Lines are read completely before they are written, but an in-place plan
 * whose lines overlap one another (never in AccFFT's plans) would need the
 * whole input first: run those on one thread, line by line, in order. */
static void run(fftw_plan p, const void* in, void* out) {
  if (!p) shim_fail("execute of a NULL FFTW plan");
  shim_exec E = {p, in, out};
  orc_parallel(exec_worker, &E, p->nlines, in == out ? 1 : g_fftw_threads);
}

fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed, int istride,
                             int idist, fftw_complex* out, const int* onembed, int ostride, int odist, int sign,
                             unsigned flags) {
  (void)inembed; (void)onembed; (void)flags;
  long long hn = howmany, his = idist, hos = odist;
  return make(KIND_C2C, rank, n[0], istride, ostride, 1, &hn, &his, &hos, in, out, sign);
}
fftw_plan fftw_plan_many_dft_r2c(int rank, const int* n, int howmany, double* in, const int* inembed, int istride,
                                 int idist, fftw_complex* out, const int* onembed, int ostride, int odist,
                                 unsigned flags) {
  (void)inembed; (void)onembed; (void)flags;
  long long hn = howmany, his = idist, hos = odist;
  return make(KIND_R2C, rank, n[0], istride, ostride, 1, &hn, &his, &hos, in, out, -1);
}
fftw_plan fftw_plan_many_dft_c2r(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed,
                                 int istride, int idist, double* out, const int* onembed, int ostride, int odist,
                                 unsigned flags) {
  (void)inembed; (void)onembed; (void)flags;
  long long hn = howmany, his = idist, hos = odist;
  return make(KIND_C2R, rank, n[0], istride, ostride, 1, &hn, &his, &hos, in, out, +1);
}

static fftw_plan guru(int kind, int rank, const fftw_iodim* dims, int hr, const fftw_iodim* hd, void* in, void* out,
                      int sign) {
  long long hn[SHIM_MAX_HM], his[SHIM_MAX_HM], hos[SHIM_MAX_HM];
  if (hr > SHIM_MAX_HM) shim_fail("FFTW howmany rank above 4");
  for (int i = 0; i < hr; ++i) {
    hn[i] = hd[i].n;
    his[i] = hd[i].is;
    hos[i] = hd[i].os;
  }
  return make(kind, rank, dims[0].n, dims[0].is, dims[0].os, hr, hn, his, hos, in, out, sign);
}
fftw_plan fftw_plan_guru_dft(int rank, const fftw_iodim* dims, int howmany_rank, const fftw_iodim* howmany_dims,
                             fftw_complex* in, fftw_complex* out, int sign, unsigned flags) {
  (void)flags;
  return guru(KIND_C2C, rank, dims, howmany_rank, howmany_dims, in, out, sign);
}
fftw_plan fftw_plan_guru_dft_r2c(int rank, const fftw_iodim* dims, int howmany_rank,
                                 const fftw_iodim* howmany_dims, double* in, fftw_complex* out, unsigned flags) {
  (void)flags;
  return guru(KIND_R2C, rank, dims, howmany_rank, howmany_dims, in, out, -1);
}
fftw_plan fftw_plan_guru_dft_c2r(int rank, const fftw_iodim* dims, int howmany_rank,
                                 const fftw_iodim* howmany_dims, fftw_complex* in, double* out, unsigned flags) {
  (void)flags;
  return guru(KIND_C2R, rank, dims, howmany_rank, howmany_dims, in, out, +1);
}

void fftw_execute(const fftw_plan p) { run(p, p->in, p->out); }
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) {
  if (p->kind != KIND_C2C) shim_fail("fftw_execute_dft on a real plan");
  run(p, in, out);
}
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out) {
  if (p->kind != KIND_R2C) shim_fail("fftw_execute_dft_r2c on another kind of plan");
  run(p, in, out);
}
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out) {
  if (p->kind != KIND_C2R) shim_fail("fftw_execute_dft_c2r on another kind of plan");
  run(p, in, out);
}
void fftw_destroy_plan(fftw_plan p) {
  if (!p) return;
  plan_free_l(&p->pl);
  free(p);
}
void* fftw_malloc(size_t n) {
  void* p = NULL;
  if (posix_memalign(&p, 64, n ? n : 64)) return NULL;
  return p;
}
void fftw_free(void* p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { g_fftw_threads = nthreads < 1 ? 1 : nthreads; }
void fftw_cleanup_threads(void) {}
void fftw_cleanup(void) {}
