/*
 * fft_oracle.c - CPU restatement of AccFFT's single-rank 3-D FFT path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this file; tests/, the smoke check and bench.py's CPU baseline use it as
 * the checker.
 *
 * The reference's arithmetic lives in FFTW3 (CPU path, src/accfft.cpp) and
 * cuFFT (GPU path, src/accfft_gpu.cpp), neither of which is vendored in the
 * reference tree (FFTW version unpinned: cmake/FindFFTW.cmake; cuFFT from the
 * CUDA toolkit).  What this file restates is the published algorithm those
 * libraries implement - the unnormalised DFT
 *     X[k] = sum_n x[n] exp(sign * 2*pi*i*n*k/N),  sign = -1 forward, +1 backward,
 * with the half-spectrum real transforms (r2c keeps k = 0..N/2, c2r reads
 * k = 0..N/2 and ignores the imaginary parts of k = 0 and k = N/2) - together
 * with the reference's own pass structure and layouts:
 *   - z pass: batched real transform along the contiguous axis
 *     (src/accfft_gpu.cpp:170-206, CPU src/accfft.cpp:176-215)
 *   - y and x passes: complex transforms along the strided axes
 *     (src/accfft_gpu.cpp:207-253, CPU src/accfft.cpp:1352-1552)
 *   - single-axis real transforms for the x and y derivatives
 *     (src/accfft_gpu.cpp:254-323, 1319-1604)
 *
 * Transforms: mixed-radix Stockham stages (any factorisation; radix 2 and 4
 * butterflies, other prime factors by direct DFT), twiddles from an exactly
 * reduced angle.  Each
 * entry point computes in double (prec == 0) or long double (prec == 1);
 * arrays are always double (complex = interleaved re, im).
 * Lines are processed by `nthreads` POSIX threads.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAX_FACTORS 40

static void orc_parallel(void (*fn)(void*, long long, long long, int), void* ctx, long long total, int nthreads);

/* ------------------------------------------------------------- generic core
 * The transform code is written once in oracle_core.h and instantiated for
 * double (suffix _d) and long double (suffix _l). */
#define REAL double
#define SFX(name) name##_d
#define TRIG_COS cos
#define TRIG_SIN sin
#define REAL_PI_4 0.785398163397448309615660845819875721
#include "oracle_core.h"
#undef REAL
#undef SFX
#undef TRIG_COS
#undef TRIG_SIN
#undef REAL_PI_4

#define REAL long double
#define SFX(name) name##_l
#define TRIG_COS cosl
#define TRIG_SIN sinl
#define REAL_PI_4 0.785398163397448309615660845819875721L
#include "oracle_core.h"
#undef REAL
#undef SFX
#undef TRIG_COS
#undef TRIG_SIN
#undef REAL_PI_4

/* ------------------------------------------------------------ thread pool */
typedef struct {
  void (*fn)(void* ctx, long long begin, long long end, int tid);
  void* ctx;
  long long total;
  int nthreads;
  int tid;
} orc_job;

static void* orc_worker(void* arg) {
  orc_job* j = (orc_job*)arg;
  long long chunk = (j->total + j->nthreads - 1) / j->nthreads;
  long long b = (long long)j->tid * chunk;
  long long e = b + chunk;
  if (e > j->total) e = j->total;
  if (b < e) j->fn(j->ctx, b, e, j->tid);
  return NULL;
}

static void orc_parallel(void (*fn)(void*, long long, long long, int), void* ctx, long long total, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (total < nthreads) nthreads = total > 0 ? (int)total : 1;
  if (nthreads == 1) {
    fn(ctx, 0, total, 0);
    return;
  }
  pthread_t th[256];
  orc_job jobs[256];
  for (int t = 0; t < nthreads; ++t) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].total = total;
    jobs[t].nthreads = nthreads;
    jobs[t].tid = t;
    pthread_create(&th[t], NULL, orc_worker, &jobs[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* --------------------------------------------------------------- dispatch */
#define ORC_DISPATCH(prec, call_d, call_l) ((prec) ? (call_l) : (call_d))

int orc_fft1d(int n, const double* in, double* out, int sign, int prec) {
  return ORC_DISPATCH(prec, fft1d_d(n, in, out, sign), fft1d_l(n, in, out, sign));
}

/* complex transform along one axis of a complex [n0][n1][w] array, in place
 * (axis 0 = x, 1 = y, 2 = z; the z axis has length w) */
int orc_c2c_axis(int n0, int n1, int w, int axis, double* data, int sign, int prec, int nthreads) {
  return ORC_DISPATCH(prec, c2c_axis_d(n0, n1, w, axis, data, sign, nthreads),
                      c2c_axis_l(n0, n1, w, axis, data, sign, nthreads));
}

/* real transform along z: rows of n2 reals (row stride in_row) ->
 * rows of n2/2+1 complex (row stride out_row complex) */
int orc_r2c_z(long long rows, int n2, const double* in, long long in_row, double* out, long long out_row, int prec,
              int nthreads) {
  return ORC_DISPATCH(prec, r2c_z_d(rows, n2, in, in_row, out, out_row, nthreads),
                      r2c_z_l(rows, n2, in, in_row, out, out_row, nthreads));
}
int orc_c2r_z(long long rows, int n2, const double* in, long long in_row, double* out, long long out_row, int prec,
              int nthreads) {
  return ORC_DISPATCH(prec, c2r_z_d(rows, n2, in, in_row, out, out_row, nthreads),
                      c2r_z_l(rows, n2, in, in_row, out, out_row, nthreads));
}

/* real transform along a strided axis of a real [a][L][b] array (line
 * stride b): out is complex [a][L/2+1][b]; the inverse maps back */
int orc_r2c_strided(long long a, int L, long long b, const double* in, double* out, int prec, int nthreads) {
  return ORC_DISPATCH(prec, r2c_strided_d(a, L, b, in, out, nthreads), r2c_strided_l(a, L, b, in, out, nthreads));
}
int orc_c2r_strided(long long a, int L, long long b, const double* in, double* out, int prec, int nthreads) {
  return ORC_DISPATCH(prec, c2r_strided_d(a, L, b, in, out, nthreads), c2r_strided_l(a, L, b, in, out, nthreads));
}
