/*
 * accfft_operators_gpu.h - AccFFT's GPU spectral operators
 * (include/accfft_operators_gpu.h of the reference) on the GB300 path, plus
 * inv_laplace / inv_biharmonic, which the reference offers on the CPU only
 * (src/operators.txx:276-388).  All arrays live on the device and use the
 * plan's real layout.
 */
#ifndef ACCFFT_OPERATORS_GPU_H
#define ACCFFT_OPERATORS_GPU_H

#include <bitset>

#include "accfft_gpu.h"
#include "accfft_gpuf.h"

template <typename T, typename Tp>
void accfft_grad_gpu_slow_t(T* A_x, T* A_y, T* A_z, T* A, Tp* plan, std::bitset<3>* pXYZ = NULL,
                            double* timer = NULL);
template <typename T, typename Tp>
void accfft_grad_gpu_t(T* A_x, T* A_y, T* A_z, T* A, Tp* plan, std::bitset<3>* pXYZ = NULL, double* timer = NULL);
template <typename T, typename Tp>
void accfft_laplace_gpu_t(T* LA, T* A, Tp* plan, double* timer = NULL);
template <typename T, typename Tp>
void accfft_divergence_gpu_t(T* divA, T* A_x, T* A_y, T* A_z, Tp* plan, double* timer = NULL);
template <typename T, typename Tp>
void accfft_divergence_gpu_slow_t(T* divA, T* A_x, T* A_y, T* A_z, Tp* plan, double* timer = NULL);
template <typename T, typename Tp>
void accfft_biharmonic_gpu_t(T* LA, T* A, Tp* plan, double* timer = NULL);
template <typename T, typename Tp>
void accfft_inv_laplace_gpu_t(T* invLA, T* A, Tp* plan, double* timer = NULL);
template <typename T, typename Tp>
void accfft_inv_biharmonic_gpu_t(T* invBA, T* A, Tp* plan, double* timer = NULL);

void accfft_grad_gpu(double* A_x, double* A_y, double* A_z, double* A, accfft_plan_gpu* plan,
                     std::bitset<3>* pXYZ = NULL, double* timer = NULL);
void accfft_laplace_gpu(double* LA, double* A, accfft_plan_gpu* plan, double* timer = NULL);
void accfft_divergence_gpu(double* divA, double* A_x, double* A_y, double* A_z, accfft_plan_gpu* plan,
                           double* timer = NULL);
void accfft_divergence_slow_gpu(double* divA, double* A_x, double* A_y, double* A_z, accfft_plan_gpu* plan,
                                double* timer = NULL);
void accfft_biharmonic_gpu(double* LA, double* A, accfft_plan_gpu* plan, double* timer = NULL);
void accfft_inv_laplace_gpu(double* invLA, double* A, accfft_plan_gpu* plan, double* timer = NULL);
void accfft_inv_biharmonic_gpu(double* invBA, double* A, accfft_plan_gpu* plan, double* timer = NULL);

void accfft_grad_gpuf(float* A_x, float* A_y, float* A_z, float* A, accfft_plan_gpuf* plan,
                      std::bitset<3>* pXYZ = NULL, double* timer = NULL);
void accfft_laplace_gpuf(float* LA, float* A, accfft_plan_gpuf* plan, double* timer = NULL);
void accfft_divergence_slow_gpuf(float* divA, float* A_x, float* A_y, float* A_z, accfft_plan_gpuf* plan,
                                 double* timer = NULL);
void accfft_divergence_gpuf(float* divA, float* A_x, float* A_y, float* A_z, accfft_plan_gpuf* plan,
                            double* timer = NULL);
void accfft_biharmonic_gpuf(float* LA, float* A, accfft_plan_gpuf* plan, double* timer = NULL);
void accfft_inv_laplace_gpuf(float* invLA, float* A, accfft_plan_gpuf* plan, double* timer = NULL);
void accfft_inv_biharmonic_gpuf(float* invBA, float* A, accfft_plan_gpuf* plan, double* timer = NULL);

#endif
