/*
 * accfft_common.h - declarations shared by AccFFT's GPU interface, for the
 * GB300 single-GPU path.  Same names and signatures as AccFFT's
 * include/accfft_common.h so existing programs compile unchanged; without an
 * MPI installation put include/mpi_shim on the include path.
 */
#ifndef ACCFFT_COMMON_H
#define ACCFFT_COMMON_H

#include <mpi.h>

#include <cstddef>
#include <cstdint>
#include <iostream>

#define PCOUT if (procid == 0) std::cout
typedef double Complex[2];
typedef float Complexf[2];

#define ACCFFT_FORWARD -1
#define ACCFFT_BACKWARD +1
#define ACCFFT_INVERSE +1
#define ACCFFT_ESTIMATE 1
#define ACCFFT_MEASURE 2
#define ACCFFT_PATIENT 4
/* Extension (no counterpart in the reference): OR into the flags of a
 * double plan to compute its transforms in double-float on the FP32 pipes
 * (FP64-class accuracy, 2.5x faster on GB300); the operators need a plain
 * double plan.  Same value as ACCFFT_C_F64_DF in accfft_gb300.h. */
#define ACCFFT_F64_DF 0x400u

/* Cartesian communicator (AccFFT src/accfft_common.cpp:275-305); the GB300
 * path needs a 1 x 1 grid and corrects c_dims to it like the reference. */
void accfft_create_comm(MPI_Comm in_comm, int* c_dims, MPI_Comm* c_comm);
int accfft_init();
int accfft_init(int nthreads);
void accfft_cleanup();
/* host allocation with 64-byte alignment (the reference uses fftw_malloc) */
void* accfft_alloc(ptrdiff_t size);
void accfft_free(void* ptr);

/* Local sizes at P = 1 (src/accfft_common.cpp:49-256).  They return the
 * reference's byte counts as int, or -1 with a message when the count does
 * not fit an int (accfft_c_local_size_* in accfft_gb300.h return 64 bits). */
template <typename T>
int dfft_get_local_size_t(int N0, int N1, int N2, int* isize, int* istart, MPI_Comm c_comm);
template <typename T>
int accfft_local_size_dft_r2c_t(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c_comm);
template <typename T>
int accfft_local_size_dft_c2c_t(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c_comm);

#endif
