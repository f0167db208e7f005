// AccFFT's C++ GPU interface (accfft_common.h, accfft_gpu.h, accfft_gpuf.h,
// accfft_operators_gpu.h) implemented on the C ABI of accfft_gb300.h.
//
// Behaviour follows the reference's single-rank code: plans return NULL on
// failure with a message on stderr (src/accfft_gpu.cpp:187-191), execute on a
// plan of the wrong kind prints and returns (:642-646), every call blocks
// until the GPU work is done, and the timer's slot 4 accumulates device time.
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "accfft_common.h"
#include "accfft_gb300.h"
#include "accfft_gpu.h"
#include "accfft_gpuf.h"
#include "accfft_operators_gpu.h"

namespace {

int to_int_bytes(long long v, const char* what) {
  if (v > INT_MAX || v < 0) {
    std::cerr << "! " << what << ": " << v << " bytes do not fit the int interface; "
              << "use accfft_c_local_size_* for 64-bit sizes\n";
    return -1;
  }
  return (int)v;
}

void report(int rc, const char* what) {
  if (rc != ACCFFT_C_OK) std::cout << "Error in " << what << ": " << accfft_c_last_error() << std::endl;
}

unsigned bits(std::bitset<3> b) { return (unsigned)b.to_ulong(); }

int comm_size(MPI_Comm c) {
  int n = 1;
  MPI_Comm_size(c, &n);
  return n;
}

void set3(int* d, int a, int b, int c) {
  d[0] = a;
  d[1] = b;
  d[2] = c;
}

// plan fields at P = 1 (src/accfft_gpu.cpp:105-167; every pencil layout is
// the natural one)
template <typename Plan>
void fill_r2c_fields(Plan* p, const int* n) {
  const int h = n[2] / 2 + 1;
  for (int i = 0; i < 3; ++i) p->N[i] = n[i];
  for (int* o : {p->osize_0, p->osize_1, p->osize_2, p->osize_1i, p->osize_2i, p->osize}) set3(o, n[0], n[1], h);
  for (int* o : {p->ostart_0, p->ostart_1, p->ostart_2, p->ostart_1i, p->ostart_2i, p->ostart, p->istart,
                 p->ostart_y})
    set3(o, 0, 0, 0);
  set3(p->isize, n[0], n[1], n[2]);
  set3(p->osize_y, n[0], n[1], n[2]);
  set3(p->osize_yi, n[0], n[1] / 2 + 1, n[2]);
  set3(p->osize_x, n[0], n[1] * n[2], 1);
  set3(p->osize_xi, n[0] / 2 + 1, n[1] * n[2], 1);
  set3(p->ostart_x, 0, -(1 << 8), -(1 << 8));
}

template <typename Plan>
void fill_c2c_fields(Plan* p, const int* n) {
  fill_r2c_fields(p, n);
  for (int* o : {p->osize_0, p->osize_1, p->osize_2, p->osize_1i, p->osize_2i, p->osize}) set3(o, n[0], n[1], n[2]);
}

template <typename Plan>
void fill_common(Plan* p, MPI_Comm c_comm, void* data, void* data_out) {
  p->procid = 0;
  MPI_Comm_rank(c_comm, &p->procid);
  MPI_Cart_get(c_comm, 2, p->np, p->periods, p->coord);
  p->c_comm = c_comm;
  MPI_Comm_split(c_comm, p->coord[0], p->coord[1], &p->row_comm);
  MPI_Comm_split(c_comm, p->coord[1], p->coord[0], &p->col_comm);
  p->oneD = true;
  p->inplace = data == data_out;
}

template <typename Plan, typename Make, typename Real>
Plan* make_r2c(int* n, Real* data, Real* data_out, MPI_Comm c_comm, unsigned flags, Make make) {
  if (comm_size(c_comm) != 1) {
    std::cerr << "accfft_plan_dft_3d_r2c_gpu: the GB300 path runs on one rank\n";
    return NULL;
  }
  accfft_c_plan* impl = make(n, data, data_out, flags);
  if (!impl) {
    std::cerr << "accfft_plan_dft_3d_r2c_gpu: " << accfft_c_last_error() << "\n";
    return NULL;
  }
  Plan* p = new Plan;
  p->impl = impl;
  fill_common(p, c_comm, data, data_out);
  fill_r2c_fields(p, n);
  p->data = data;
  p->data_out = data_out;
  int is[3], ist[3], os[3], ost[3];
  p->alloc_max = to_int_bytes(accfft_c_local_size_dft_r2c(n, is, ist, os, ost, (int)sizeof(Real)), "alloc_max");
  p->r2c_plan_baked = true;
  return p;
}

template <typename Plan, typename Make, typename Cplx, typename Real>
Plan* make_c2c(int* n, Cplx* data, Cplx* data_out, MPI_Comm c_comm, unsigned flags, Make make) {
  if (comm_size(c_comm) != 1) {
    std::cerr << "accfft_plan_dft_3d_c2c_gpu: the GB300 path runs on one rank\n";
    return NULL;
  }
  accfft_c_plan* impl = make(n, (Real*)data, (Real*)data_out, flags);
  if (!impl) {
    std::cerr << "accfft_plan_dft_3d_c2c_gpu: " << accfft_c_last_error() << "\n";
    return NULL;
  }
  Plan* p = new Plan;
  p->impl = impl;
  fill_common(p, c_comm, data, data_out);
  fill_c2c_fields(p, n);
  p->data_c = data;
  p->data_out_c = data_out;
  int is[3], ist[3], os[3], ost[3];
  p->alloc_max = to_int_bytes(accfft_c_local_size_dft_c2c(n, is, ist, os, ost, (int)sizeof(Real)), "alloc_max");
  p->c2c_plan_baked = true;
  return p;
}

template <typename Plan>
bool baked_r2c(Plan* p) {
  if (p && p->r2c_plan_baked && p->impl) return true;
  std::cout << "Error. r2c plan has not been made correctly. Please first create the plan before calling "
               "execute functions."
            << std::endl;
  return false;
}

template <typename Plan>
bool baked_c2c(Plan* p) {
  if (p && p->c2c_plan_baked && p->impl) return true;
  std::cout << "Error. c2c plan has not been made correctly. Please first create the plan before calling "
               "execute functions."
            << std::endl;
  return false;
}

template <typename Plan>
void destroy(Plan* p) {
  if (!p) return;
  accfft_c_destroy_plan(p->impl);
  p->impl = NULL;
  p->r2c_plan_baked = p->c2c_plan_baked = false;
  MPI_Comm_free(&p->row_comm);
  MPI_Comm_free(&p->col_comm);
}

}  // namespace

// ------------------------------------------------------------ common
void accfft_create_comm(MPI_Comm in_comm, int* c_dims, MPI_Comm* c_comm) {
  int nprocs = 1, procid = 0;
  MPI_Comm_rank(in_comm, &procid);
  MPI_Comm_size(in_comm, &nprocs);
  if (c_dims[0] * c_dims[1] != nprocs) {
    c_dims[0] = 0;
    c_dims[1] = 0;
    MPI_Dims_create(nprocs, 2, c_dims);
    PCOUT << "Input c_dim[0] * c_dims[1] != nprocs. Automatically switching to c_dims[0] = " << c_dims[0]
          << " , c_dims_1 = " << c_dims[1] << std::endl;
  }
  int period[2] = {0, 0};
  MPI_Cart_create(in_comm, 2, c_dims, period, 1, c_comm);
}

int accfft_init() { return 0; }
int accfft_init(int) { return 0; }
void accfft_cleanup() {}
void accfft_cleanup_gpu() {}
void accfft_cleanup_gpuf() {}

void* accfft_alloc(ptrdiff_t size) {
  void* p = NULL;
  if (size <= 0 || posix_memalign(&p, 64, (size_t)size)) return NULL;
  return p;
}
void accfft_free(void* ptr) { free(ptr); }

template <typename T>
int dfft_get_local_size_t(int N0, int N1, int N2, int* isize, int* istart, MPI_Comm) {
  return to_int_bytes(accfft_c_dfft_get_local_size(N0, N1, N2, isize, istart, (int)sizeof(T)), "local size");
}
template <typename T>
int accfft_local_size_dft_r2c_t(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm) {
  return to_int_bytes(accfft_c_local_size_dft_r2c(n, isize, istart, osize, ostart, (int)sizeof(T)), "r2c local size");
}
template <typename T>
int accfft_local_size_dft_c2c_t(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm) {
  return to_int_bytes(accfft_c_local_size_dft_c2c(n, isize, istart, osize, ostart, (int)sizeof(T)), "c2c local size");
}
template <typename T>
int accfft_local_size_dft_r2c_gpu_t(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c) {
  return accfft_local_size_dft_r2c_t<T>(n, isize, istart, osize, ostart, c);
}

#define AFG_INST_SIZES(T)                                                                          \
  template int dfft_get_local_size_t<T>(int, int, int, int*, int*, MPI_Comm);                      \
  template int accfft_local_size_dft_r2c_t<T>(int*, int*, int*, int*, int*, MPI_Comm);             \
  template int accfft_local_size_dft_c2c_t<T>(int*, int*, int*, int*, int*, MPI_Comm);             \
  template int accfft_local_size_dft_r2c_gpu_t<T>(int*, int*, int*, int*, int*, MPI_Comm);
AFG_INST_SIZES(double)
AFG_INST_SIZES(float)
AFG_INST_SIZES(Complex)
AFG_INST_SIZES(Complexf)
#undef AFG_INST_SIZES

int dfft_get_local_size_gpu(int N0, int N1, int N2, int* isize, int* istart, MPI_Comm c) {
  return dfft_get_local_size_t<double>(N0, N1, N2, isize, istart, c);
}
int dfft_get_local_size_gpuf(int N0, int N1, int N2, int* isize, int* istart, MPI_Comm c) {
  return dfft_get_local_size_t<float>(N0, N1, N2, isize, istart, c);
}
int accfft_local_size_dft_r2c_gpu(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c) {
  return accfft_local_size_dft_r2c_t<double>(n, isize, istart, osize, ostart, c);
}
int accfft_local_size_dft_r2c_gpuf(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c) {
  return accfft_local_size_dft_r2c_t<float>(n, isize, istart, osize, ostart, c);
}
int accfft_local_size_dft_c2c_gpu(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c) {
  return accfft_local_size_dft_c2c_t<double>(n, isize, istart, osize, ostart, c);
}
int accfft_local_size_dft_c2c_gpuf(int* n, int* isize, int* istart, int* osize, int* ostart, MPI_Comm c) {
  return accfft_local_size_dft_c2c_t<float>(n, isize, istart, osize, ostart, c);
}

// ------------------------------------------------------------- plans
accfft_plan_gpu* accfft_plan_dft_3d_r2c_gpu(int* n, double* data_d, double* data_out_d, MPI_Comm c_comm,
                                            unsigned flags) {
  return make_r2c<accfft_plan_gpu>(n, data_d, data_out_d, c_comm, flags, accfft_c_plan_dft_3d_r2c_gpu);
}
accfft_plan_gpuf* accfft_plan_dft_3d_r2c_gpuf(int* n, float* data_d, float* data_out_d, MPI_Comm c_comm,
                                              unsigned flags) {
  return make_r2c<accfft_plan_gpuf>(n, data_d, data_out_d, c_comm, flags, accfft_c_plan_dft_3d_r2c_gpuf);
}
accfft_plan_gpu* accfft_plan_dft_3d_c2c_gpu(int* n, Complex* data_d, Complex* data_out_d, MPI_Comm c_comm,
                                            unsigned flags) {
  return make_c2c<accfft_plan_gpu, decltype(&accfft_c_plan_dft_3d_c2c_gpu), Complex, double>(
      n, data_d, data_out_d, c_comm, flags, accfft_c_plan_dft_3d_c2c_gpu);
}
accfft_plan_gpuf* accfft_plan_dft_3d_c2c_gpuf(int* n, Complexf* data_d, Complexf* data_out_d, MPI_Comm c_comm,
                                              unsigned flags) {
  return make_c2c<accfft_plan_gpuf, decltype(&accfft_c_plan_dft_3d_c2c_gpuf), Complexf, float>(
      n, data_d, data_out_d, c_comm, flags, accfft_c_plan_dft_3d_c2c_gpuf);
}

// The plan struct itself stays valid after destruction (as in the reference,
// which never deletes it); its device resources are released.
void accfft_destroy_plan(accfft_plan_gpu* plan) { destroy(plan); }
void accfft_destroy_plan_gpu(accfft_plan_gpu* plan) { destroy(plan); }
void accfft_destroy_plan(accfft_plan_gpuf* plan) { destroy(plan); }
void accfft_destroy_plan_gpu(accfft_plan_gpuf* plan) { destroy(plan); }

// ----------------------------------------------------------- execute
void accfft_execute_gpu(accfft_plan_gpu* plan, int direction, double* data_d, double* data_out_d, double* timer,
                        std::bitset<3> xyz) {
  if (!baked_r2c(plan)) return;
  report(accfft_c_execute_gpu(plan->impl, direction, data_d, data_out_d, timer, bits(xyz)), "accfft_execute_gpu");
}
void accfft_execute_gpuf(accfft_plan_gpuf* plan, int direction, float* data_d, float* data_out_d, double* timer,
                         std::bitset<3> xyz) {
  if (!baked_r2c(plan)) return;
  report(accfft_c_execute_gpuf(plan->impl, direction, data_d, data_out_d, timer, bits(xyz)), "accfft_execute_gpuf");
}
void accfft_execute_r2c_gpu(accfft_plan_gpu* plan, double* data, Complex* data_out, double* timer,
                            std::bitset<3> xyz) {
  if (!baked_r2c(plan)) return;
  report(accfft_c_execute_r2c_gpu(plan->impl, data, (double*)data_out, timer, bits(xyz)), "accfft_execute_r2c_gpu");
}
void accfft_execute_c2r_gpu(accfft_plan_gpu* plan, Complex* data, double* data_out, double* timer,
                            std::bitset<3> xyz) {
  if (!baked_r2c(plan)) return;
  report(accfft_c_execute_c2r_gpu(plan->impl, (double*)data, data_out, timer, bits(xyz)), "accfft_execute_c2r_gpu");
}
void accfft_execute_r2c_gpuf(accfft_plan_gpuf* plan, float* data, Complexf* data_out, double* timer,
                             std::bitset<3> xyz) {
  if (!baked_r2c(plan)) return;
  report(accfft_c_execute_r2c_gpuf(plan->impl, data, (float*)data_out, timer, bits(xyz)), "accfft_execute_r2c_gpuf");
}
void accfft_execute_c2r_gpuf(accfft_plan_gpuf* plan, Complexf* data, float* data_out, double* timer,
                             std::bitset<3> xyz) {
  if (!baked_r2c(plan)) return;
  report(accfft_c_execute_c2r_gpuf(plan->impl, (float*)data, data_out, timer, bits(xyz)), "accfft_execute_c2r_gpuf");
}
void accfft_execute_c2c_gpu(accfft_plan_gpu* plan, int direction, Complex* data_d, Complex* data_out_d,
                            double* timer, std::bitset<3> xyz) {
  if (!baked_c2c(plan)) return;
  report(accfft_c_execute_c2c_gpu(plan->impl, direction, (double*)data_d, (double*)data_out_d, timer, bits(xyz)),
         "accfft_execute_c2c_gpu");
}
void accfft_execute_c2c_gpuf(accfft_plan_gpuf* plan, int direction, Complexf* data_d, Complexf* data_out_d,
                             double* timer, std::bitset<3> xyz) {
  if (!baked_c2c(plan)) return;
  report(accfft_c_execute_c2c_gpuf(plan->impl, direction, (float*)data_d, (float*)data_out_d, timer, bits(xyz)),
         "accfft_execute_c2c_gpuf");
}

template <typename T, typename Tc>
void accfft_execute_r2c_gpu_t(accfft_plan_gpu* plan, T* data, Tc* data_out, double* timer, std::bitset<3> XYZ) {
  accfft_execute_r2c_gpu(plan, data, data_out, timer, XYZ);
}
template <typename Tc, typename T>
void accfft_execute_c2r_gpu_t(accfft_plan_gpu* plan, Tc* data, T* data_out, double* timer, std::bitset<3> XYZ) {
  accfft_execute_c2r_gpu(plan, data, data_out, timer, XYZ);
}
template <typename T, typename Tc>
void accfft_execute_r2c_gpu_t(accfft_plan_gpuf* plan, T* data, Tc* data_out, double* timer, std::bitset<3> XYZ) {
  accfft_execute_r2c_gpuf(plan, data, data_out, timer, XYZ);
}
template <typename Tc, typename T>
void accfft_execute_c2r_gpu_t(accfft_plan_gpuf* plan, Tc* data, T* data_out, double* timer, std::bitset<3> XYZ) {
  accfft_execute_c2r_gpuf(plan, data, data_out, timer, XYZ);
}
template void accfft_execute_r2c_gpu_t<double, Complex>(accfft_plan_gpu*, double*, Complex*, double*, std::bitset<3>);
template void accfft_execute_c2r_gpu_t<Complex, double>(accfft_plan_gpu*, Complex*, double*, double*, std::bitset<3>);
template void accfft_execute_r2c_gpu_t<float, Complexf>(accfft_plan_gpuf*, float*, Complexf*, double*, std::bitset<3>);
template void accfft_execute_c2r_gpu_t<Complexf, float>(accfft_plan_gpuf*, Complexf*, float*, double*, std::bitset<3>);

// single-axis transforms (src/accfft_gpu.cpp:1212-1604)
#define AFG_AXIS(NAME, PLAN, AXIS, DIR)                                                             \
  template <typename A, typename B>                                                                 \
  void NAME(PLAN* plan, A* data, B* data_out, double* timer) {                                      \
    if (!baked_r2c(plan)) return;                                                                   \
    report(DIR ? accfft_c_execute_c2r_axis(plan->impl, AXIS, data, data_out, timer)                 \
               : accfft_c_execute_r2c_axis(plan->impl, AXIS, data, data_out, timer),                \
           #NAME);                                                                                  \
  }
AFG_AXIS(accfft_execute_r2c_z_gpu_t, accfft_plan_gpu, 2, 0)
AFG_AXIS(accfft_execute_c2r_z_gpu_t, accfft_plan_gpu, 2, 1)
AFG_AXIS(accfft_execute_r2c_y_gpu_t, accfft_plan_gpu, 1, 0)
AFG_AXIS(accfft_execute_c2r_y_gpu_t, accfft_plan_gpu, 1, 1)
AFG_AXIS(accfft_execute_r2c_x_gpu_t, accfft_plan_gpu, 0, 0)
AFG_AXIS(accfft_execute_c2r_x_gpu_t, accfft_plan_gpu, 0, 1)
AFG_AXIS(accfft_execute_r2c_z_gpu_t, accfft_plan_gpuf, 2, 0)
AFG_AXIS(accfft_execute_c2r_z_gpu_t, accfft_plan_gpuf, 2, 1)
AFG_AXIS(accfft_execute_r2c_y_gpu_t, accfft_plan_gpuf, 1, 0)
AFG_AXIS(accfft_execute_c2r_y_gpu_t, accfft_plan_gpuf, 1, 1)
AFG_AXIS(accfft_execute_r2c_x_gpu_t, accfft_plan_gpuf, 0, 0)
AFG_AXIS(accfft_execute_c2r_x_gpu_t, accfft_plan_gpuf, 0, 1)
#undef AFG_AXIS
#define AFG_AXIS_INST(T, C, PLAN)                                                                   \
  template void accfft_execute_r2c_z_gpu_t<T, C>(PLAN*, T*, C*, double*);                           \
  template void accfft_execute_c2r_z_gpu_t<C, T>(PLAN*, C*, T*, double*);                           \
  template void accfft_execute_r2c_y_gpu_t<T, C>(PLAN*, T*, C*, double*);                           \
  template void accfft_execute_c2r_y_gpu_t<C, T>(PLAN*, C*, T*, double*);                           \
  template void accfft_execute_r2c_x_gpu_t<T, C>(PLAN*, T*, C*, double*);                           \
  template void accfft_execute_c2r_x_gpu_t<C, T>(PLAN*, C*, T*, double*);
AFG_AXIS_INST(double, Complex, accfft_plan_gpu)
AFG_AXIS_INST(float, Complexf, accfft_plan_gpuf)
#undef AFG_AXIS_INST

// --------------------------------------------------------- operators
namespace {
template <typename Tp>
bool op_plan(Tp* plan, const char* what) {
  if (plan && plan->r2c_plan_baked && plan->impl) return true;
  std::cout << "Error in " << what << "! plan is not correctly made." << std::endl;
  return false;
}
}  // namespace

template <typename T, typename Tp>
void accfft_grad_gpu_t(T* A_x, T* A_y, T* A_z, T* A, Tp* plan, std::bitset<3>* pXYZ, double* timer) {
  if (!op_plan(plan, "accfft_grad")) return;
  unsigned xyz = pXYZ ? bits(*pXYZ) : 7u;
  report(accfft_c_grad(plan->impl, A_x, A_y, A_z, A, xyz, timer), "accfft_grad");
}
template <typename T, typename Tp>
void accfft_grad_gpu_slow_t(T* A_x, T* A_y, T* A_z, T* A, Tp* plan, std::bitset<3>* pXYZ, double* timer) {
  if (!op_plan(plan, "accfft_grad")) return;
  unsigned xyz = pXYZ ? bits(*pXYZ) : 7u;
  report(accfft_c_grad_slow(plan->impl, A_x, A_y, A_z, A, xyz, timer), "accfft_grad");
}
template <typename T, typename Tp>
void accfft_laplace_gpu_t(T* LA, T* A, Tp* plan, double* timer) {
  if (!op_plan(plan, "accfft_laplace")) return;
  report(accfft_c_laplace(plan->impl, LA, A, timer), "accfft_laplace");
}
template <typename T, typename Tp>
void accfft_divergence_gpu_t(T* divA, T* A_x, T* A_y, T* A_z, Tp* plan, double* timer) {
  if (!op_plan(plan, "accfft_divergence")) return;
  report(accfft_c_divergence(plan->impl, divA, A_x, A_y, A_z, timer), "accfft_divergence");
}
template <typename T, typename Tp>
void accfft_divergence_gpu_slow_t(T* divA, T* A_x, T* A_y, T* A_z, Tp* plan, double* timer) {
  if (!op_plan(plan, "accfft_divergence")) return;
  report(accfft_c_divergence_slow(plan->impl, divA, A_x, A_y, A_z, timer), "accfft_divergence");
}
template <typename T, typename Tp>
void accfft_biharmonic_gpu_t(T* LA, T* A, Tp* plan, double* timer) {
  if (!op_plan(plan, "accfft_biharmonic")) return;
  report(accfft_c_biharmonic(plan->impl, LA, A, timer), "accfft_biharmonic");
}
template <typename T, typename Tp>
void accfft_inv_laplace_gpu_t(T* invLA, T* A, Tp* plan, double* timer) {
  if (!op_plan(plan, "accfft_inv_laplace")) return;
  report(accfft_c_inv_laplace(plan->impl, invLA, A, timer), "accfft_inv_laplace");
}
template <typename T, typename Tp>
void accfft_inv_biharmonic_gpu_t(T* invBA, T* A, Tp* plan, double* timer) {
  if (!op_plan(plan, "accfft_inv_biharmonic")) return;
  report(accfft_c_inv_biharmonic(plan->impl, invBA, A, timer), "accfft_inv_biharmonic");
}

#define AFG_OP_INST(T, PLAN)                                                                           \
  template void accfft_grad_gpu_t<T, PLAN>(T*, T*, T*, T*, PLAN*, std::bitset<3>*, double*);           \
  template void accfft_grad_gpu_slow_t<T, PLAN>(T*, T*, T*, T*, PLAN*, std::bitset<3>*, double*);      \
  template void accfft_laplace_gpu_t<T, PLAN>(T*, T*, PLAN*, double*);                                 \
  template void accfft_divergence_gpu_t<T, PLAN>(T*, T*, T*, T*, PLAN*, double*);                      \
  template void accfft_divergence_gpu_slow_t<T, PLAN>(T*, T*, T*, T*, PLAN*, double*);                 \
  template void accfft_biharmonic_gpu_t<T, PLAN>(T*, T*, PLAN*, double*);                              \
  template void accfft_inv_laplace_gpu_t<T, PLAN>(T*, T*, PLAN*, double*);                             \
  template void accfft_inv_biharmonic_gpu_t<T, PLAN>(T*, T*, PLAN*, double*);
AFG_OP_INST(double, accfft_plan_gpu)
AFG_OP_INST(float, accfft_plan_gpuf)
#undef AFG_OP_INST

void accfft_grad_gpu(double* A_x, double* A_y, double* A_z, double* A, accfft_plan_gpu* plan, std::bitset<3>* pXYZ,
                     double* timer) {
  accfft_grad_gpu_t<double, accfft_plan_gpu>(A_x, A_y, A_z, A, plan, pXYZ, timer);
}
void accfft_laplace_gpu(double* LA, double* A, accfft_plan_gpu* plan, double* timer) {
  accfft_laplace_gpu_t<double, accfft_plan_gpu>(LA, A, plan, timer);
}
void accfft_divergence_gpu(double* divA, double* A_x, double* A_y, double* A_z, accfft_plan_gpu* plan,
                           double* timer) {
  accfft_divergence_gpu_t<double, accfft_plan_gpu>(divA, A_x, A_y, A_z, plan, timer);
}
void accfft_divergence_slow_gpu(double* divA, double* A_x, double* A_y, double* A_z, accfft_plan_gpu* plan,
                                double* timer) {
  accfft_divergence_gpu_slow_t<double, accfft_plan_gpu>(divA, A_x, A_y, A_z, plan, timer);
}
void accfft_biharmonic_gpu(double* LA, double* A, accfft_plan_gpu* plan, double* timer) {
  accfft_biharmonic_gpu_t<double, accfft_plan_gpu>(LA, A, plan, timer);
}
void accfft_inv_laplace_gpu(double* invLA, double* A, accfft_plan_gpu* plan, double* timer) {
  accfft_inv_laplace_gpu_t<double, accfft_plan_gpu>(invLA, A, plan, timer);
}
void accfft_inv_biharmonic_gpu(double* invBA, double* A, accfft_plan_gpu* plan, double* timer) {
  accfft_inv_biharmonic_gpu_t<double, accfft_plan_gpu>(invBA, A, plan, timer);
}
void accfft_grad_gpuf(float* A_x, float* A_y, float* A_z, float* A, accfft_plan_gpuf* plan, std::bitset<3>* pXYZ,
                      double* timer) {
  accfft_grad_gpu_t<float, accfft_plan_gpuf>(A_x, A_y, A_z, A, plan, pXYZ, timer);
}
void accfft_laplace_gpuf(float* LA, float* A, accfft_plan_gpuf* plan, double* timer) {
  accfft_laplace_gpu_t<float, accfft_plan_gpuf>(LA, A, plan, timer);
}
void accfft_divergence_slow_gpuf(float* divA, float* A_x, float* A_y, float* A_z, accfft_plan_gpuf* plan,
                                 double* timer) {
  accfft_divergence_gpu_slow_t<float, accfft_plan_gpuf>(divA, A_x, A_y, A_z, plan, timer);
}
void accfft_divergence_gpuf(float* divA, float* A_x, float* A_y, float* A_z, accfft_plan_gpuf* plan, double* timer) {
  accfft_divergence_gpu_t<float, accfft_plan_gpuf>(divA, A_x, A_y, A_z, plan, timer);
}
void accfft_biharmonic_gpuf(float* LA, float* A, accfft_plan_gpuf* plan, double* timer) {
  accfft_biharmonic_gpu_t<float, accfft_plan_gpuf>(LA, A, plan, timer);
}
void accfft_inv_laplace_gpuf(float* invLA, float* A, accfft_plan_gpuf* plan, double* timer) {
  accfft_inv_laplace_gpu_t<float, accfft_plan_gpuf>(invLA, A, plan, timer);
}
void accfft_inv_biharmonic_gpuf(float* invBA, float* A, accfft_plan_gpuf* plan, double* timer) {
  accfft_inv_biharmonic_gpu_t<float, accfft_plan_gpuf>(invBA, A, plan, timer);
}
