/*
 * fftw3.h - the subset of FFTW3's API that AccFFT's CPU host code calls,
 * backed by the oracle's own DFT (oracle_core.h, computed in long double).
 * TEST INFRASTRUCTURE ONLY: oracle/build_ref.py compiles the reference's
 * src/accfft.cpp, src/accfft_common.cpp, src/operators.cpp and
 * src/transpose.cpp against it into oracle/_ref.
 *
 * Semantics follow FFTW's published interface (advanced "many" and guru
 * interfaces, rank-1 transforms): unnormalised DFT with the given sign; r2c
 * keeps k = 0..n/2; c2r reads k = 0..n/2 and ignores the imaginary parts of
 * k = 0 and, for even n, k = n/2; strides and distances count elements of the
 * array's own type.  Plans keep their geometry; the new-array execute calls
 * apply it to other arrays.  Input arrays are never modified, in-place plans
 * are supported (each line is gathered before it is written).
 */
#ifndef ORACLE_REF_FFTW3_SHIM_H
#define ORACLE_REF_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct oracle_fftw_plan_s* fftw_plan;
typedef struct oracle_fftw_plan_s* fftwf_plan;
typedef struct {
  int n, is, os;
} fftw_iodim;
typedef fftw_iodim fftwf_iodim;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed, int istride,
                             int idist, fftw_complex* out, const int* onembed, int ostride, int odist, int sign,
                             unsigned flags);
fftw_plan fftw_plan_many_dft_r2c(int rank, const int* n, int howmany, double* in, const int* inembed, int istride,
                                 int idist, fftw_complex* out, const int* onembed, int ostride, int odist,
                                 unsigned flags);
fftw_plan fftw_plan_many_dft_c2r(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed,
                                 int istride, int idist, double* out, const int* onembed, int ostride, int odist,
                                 unsigned flags);
fftw_plan fftw_plan_guru_dft(int rank, const fftw_iodim* dims, int howmany_rank, const fftw_iodim* howmany_dims,
                             fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_guru_dft_r2c(int rank, const fftw_iodim* dims, int howmany_rank,
                                 const fftw_iodim* howmany_dims, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_guru_dft_c2r(int rank, const fftw_iodim* dims, int howmany_rank,
                                 const fftw_iodim* howmany_dims, fftw_complex* in, double* out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out);
void fftw_destroy_plan(fftw_plan p);
void* fftw_malloc(size_t n);
void fftw_free(void* p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
void fftw_cleanup(void);

#ifdef __cplusplus
}
#endif

#endif /* ORACLE_REF_FFTW3_SHIM_H */
