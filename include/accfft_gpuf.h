/*
 * accfft_gpuf.h - AccFFT's single-precision GPU interface (include/accfft_gpuf.h
 * of the reference) served by the GB300 single-GPU path.  Signatures,
 * default arguments and the public plan fields are the reference's; the
 * plan's cuFFT handles and transpose engines are replaced by `impl`, an
 * opaque plan of the C ABI (accfft_gb300.h).
 */
#ifndef ACCFFT_GPUF_H
#define ACCFFT_GPUF_H

#include <bitset>
#include <cstddef>

#include "accfft_common.h"
#include "accfft_gb300.h"

struct accfft_plan_gpuf {
  int N[3];
  int alloc_max;
  int coord[2], np[2], periods[2];
  MPI_Comm c_comm, row_comm, col_comm;

  int osize_0[3], ostart_0[3];
  int osize_1[3], ostart_1[3];
  int osize_2[3], ostart_2[3];
  int osize_1i[3], ostart_1i[3];
  int osize_2i[3], ostart_2i[3];
  int isize[3], istart[3];
  int osize[3], ostart[3];
  int osize_y[3], osize_yi[3], ostart_y[3];
  int osize_x[3], osize_xi[3], ostart_x[3];

  float* data;
  float* data_out;
  Complexf* data_c;
  Complexf* data_out_c;
  int procid;
  bool inplace;
  bool oneD;
  bool r2c_plan_baked;
  bool c2c_plan_baked;
  accfft_c_plan* impl;

  accfft_plan_gpuf()
      : data(NULL), data_out(NULL), data_c(NULL), data_out_c(NULL), procid(0), inplace(false), oneD(true),
        r2c_plan_baked(false), c2c_plan_baked(false), impl(NULL) {}
};

int dfft_get_local_size_gpuf(int N0, int N1, int N2, int* isize, int* istart, MPI_Comm c_comm);

void accfft_cleanup_gpuf();

void accfft_destroy_plan(accfft_plan_gpuf* plan);
void accfft_destroy_plan_gpu(accfft_plan_gpuf* plan);

void accfft_execute_r2c_gpuf(accfft_plan_gpuf* plan, float* data = NULL, Complexf* data_out = NULL,
                             double* timer = NULL, std::bitset<3> xyz = 111);
void accfft_execute_c2r_gpuf(accfft_plan_gpuf* plan, Complexf* data = NULL, float* data_out = NULL,
                             double* timer = NULL, std::bitset<3> xyz = 111);
void accfft_execute_gpuf(accfft_plan_gpuf* plan, int direction, float* data_d = NULL, float* data_out_d = NULL,
                         double* timer = NULL, std::bitset<3> xyz = 111);
void accfft_execute_c2c_gpuf(accfft_plan_gpuf* plan, int direction, Complexf* data_d = NULL,
                             Complexf* data_out_d = NULL, double* timer = NULL, std::bitset<3> xyz = 111);
accfft_plan_gpuf* accfft_plan_dft_3d_c2c_gpuf(int* n, Complexf* data_d, Complexf* data_out_d, MPI_Comm c_comm,
                                              unsigned flags = ACCFFT_MEASURE);
int accfft_local_size_dft_c2c_gpuf(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c_comm);
accfft_plan_gpuf* accfft_plan_dft_3d_r2c_gpuf(int* n, float* data_d, float* data_out_d, MPI_Comm c_comm,
                                              unsigned flags = ACCFFT_MEASURE);
int accfft_local_size_dft_r2c_gpuf(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c_comm);

template <typename T, typename Tc>
void accfft_execute_r2c_gpu_t(accfft_plan_gpuf* plan, T* data, Tc* data_out, double* timer = NULL,
                              std::bitset<3> XYZ = 111);
template <typename Tc, typename T>
void accfft_execute_c2r_gpu_t(accfft_plan_gpuf* plan, Tc* data, T* data_out, double* timer = NULL,
                              std::bitset<3> XYZ = 111);

template <typename T>
int accfft_local_size_dft_r2c_gpu_t(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c_comm);

// single-axis transforms: z -> [N0][N1][N2/2+1], y -> [N0][N1/2+1][N2], x -> [N0/2+1][N1][N2]
template <typename T, typename Tc>
void accfft_execute_r2c_z_gpu_t(accfft_plan_gpuf* plan, T* data, Tc* data_out, double* timer = NULL);
template <typename Tc, typename T>
void accfft_execute_c2r_z_gpu_t(accfft_plan_gpuf* plan, Tc* data, T* data_out, double* timer = NULL);
template <typename T, typename Tc>
void accfft_execute_r2c_y_gpu_t(accfft_plan_gpuf* plan, T* data, Tc* data_out, double* timer = NULL);
template <typename Tc, typename T>
void accfft_execute_c2r_y_gpu_t(accfft_plan_gpuf* plan, Tc* data, T* data_out, double* timer = NULL);
template <typename T, typename Tc>
void accfft_execute_r2c_x_gpu_t(accfft_plan_gpuf* plan, T* data, Tc* data_out, double* timer = NULL);
template <typename Tc, typename T>
void accfft_execute_c2r_x_gpu_t(accfft_plan_gpuf* plan, Tc* data, T* data_out, double* timer = NULL);

#endif
