/*
 * ref_driver.cpp - extern "C" entry points over AccFFT's own CPU API, for
 * generating reference-produced fixtures.  TEST INFRASTRUCTURE ONLY:
 * oracle/build_ref.py compiles this file together with the reference's
 * unmodified src/accfft.cpp, src/accfft_common.cpp, src/operators.cpp and
 * src/transpose.cpp (against the one-rank MPI and FFTW shims in ref_shim/)
 * into oracle/_ref/libaccfft_ref.so; tests/golden/gen_ref_cases.py calls it.
 *
 * Every call builds a plan on one rank exactly as the reference's step
 * programs do (accfft_create_comm with a 1 x 1 grid, accfft_local_size_*,
 * accfft_alloc of alloc_max bytes, accfft_plan_dft_3d_*), runs the reference
 * function named, copies the result out and destroys the plan.  Arrays are
 * double; complex arrays interleave (re, im).  Returns 0, or -1 on a plan
 * the reference failed to make.
 */
#include <string.h>

#include <bitset>

#include "accfft.h"
#include "accfft_operators.h"

namespace {

MPI_Comm one_rank_comm() {
  int c_dims[2] = {1, 1};
  MPI_Comm c_comm;
  accfft_create_comm(MPI_COMM_WORLD, c_dims, &c_comm);
  return c_comm;
}

long long real_count(const int* n) { return (long long)n[0] * n[1] * n[2]; }

struct R2C {
  int n[3], isize[3], istart[3], osize[3], ostart[3];
  long long alloc_max;
  double* data = nullptr;
  Complex* data_hat = nullptr;
  accfft_plan* plan = nullptr;
  explicit R2C(const int* nn, bool inplace = false) {
    memcpy(n, nn, sizeof n);
    MPI_Comm c = one_rank_comm();
    alloc_max = accfft_local_size_dft_r2c(n, isize, istart, osize, ostart, c);
    data_hat = (Complex*)accfft_alloc(alloc_max);
    data = inplace ? (double*)data_hat : (double*)accfft_alloc(alloc_max);
    memset(data_hat, 0, alloc_max);
    if (!inplace) memset(data, 0, alloc_max);
    plan = accfft_plan_dft_3d_r2c(n, data, (double*)data_hat, c, ACCFFT_MEASURE);
  }
  ~R2C() {
    if (plan) accfft_destroy_plan(plan);
    if ((void*)data != (void*)data_hat) accfft_free(data);
    accfft_free(data_hat);
  }
};

}  // namespace

extern "C" {

int ref_init(int nthreads) { return accfft_init(nthreads); }

/* src/accfft_common.cpp:98-192: alloc_max of an r2c plan (bytes) */
long long ref_alloc_max_r2c(const int* n) {
  int n3[3] = {n[0], n[1], n[2]}, isize[3], istart[3], osize[3], ostart[3];
  return accfft_local_size_dft_r2c(n3, isize, istart, osize, ostart, one_rank_comm());
}
/* src/accfft_common.cpp:203-256 */
long long ref_alloc_max_c2c(const int* n) {
  int n3[3] = {n[0], n[1], n[2]}, isize[3], istart[3], osize[3], ostart[3];
  return accfft_local_size_dft_c2c(n3, isize, istart, osize, ostart, one_rank_comm());
}

/* src/accfft.cpp:766 accfft_execute_r2c (pass sequence src/accfft.cpp:1352-1460).
 * xyz bit 0 = x, 1 = y, 2 = z.  With z set: in real [n0][n1][n2], out complex
 * [n0][n1][n2/2+1].  With z cleared the reference runs the remaining passes
 * in place on the input array ("data_out = data"): in and out are then both
 * complex [n0][n1][n2/2+1], and the result is read back from that array. */
int ref_r2c(const int* n, int xyz, const double* in, double* out) {
  R2C p(n);
  if (!p.plan) return -1;
  const long long H2 = 2LL * n[0] * n[1] * (n[2] / 2 + 1);
  memcpy(p.data, in, sizeof(double) * ((xyz & 4) ? real_count(n) : H2));
  accfft_execute_r2c(p.plan, p.data, p.data_hat, NULL, std::bitset<3>(xyz));
  memcpy(out, (xyz & 4) ? (double*)p.data_hat : p.data, sizeof(double) * H2);
  return 0;
}

/* src/accfft.cpp:789 accfft_execute_c2r (x, y backward in place on the input
 * spectrum, then z c2r: src/accfft.cpp:1462-1552).  With z cleared the result
 * is the input array itself, complex [n0][n1][n2/2+1]. */
int ref_c2r(const int* n, int xyz, const double* in, double* out) {
  R2C p(n);
  if (!p.plan) return -1;
  const long long H2 = 2LL * n[0] * n[1] * (n[2] / 2 + 1);
  memcpy(p.data_hat, in, sizeof(double) * H2);
  accfft_execute_c2r(p.plan, p.data_hat, p.data, NULL, std::bitset<3>(xyz));
  if (xyz & 4) memcpy(out, p.data, sizeof(double) * real_count(n));
  else memcpy(out, p.data_hat, sizeof(double) * H2);
  return 0;
}

/* In-place r2c / c2r (steps/step2): the real array's z rows are padded to
 * 2*(n2/2+1) doubles.  in / out here are unpadded [n0][n1][n2] (r2c input,
 * c2r output) and [n0][n1][n2/2+1] complex (r2c output, c2r input). */
int ref_r2c_inplace(const int* n, const double* in, double* out) {
  R2C p(n, true);
  if (!p.plan) return -1;
  const int pad = 2 * (n[2] / 2 + 1);
  for (long long r = 0; r < (long long)n[0] * n[1]; ++r) memcpy(p.data + r * pad, in + r * n[2], sizeof(double) * n[2]);
  accfft_execute_r2c(p.plan, p.data, p.data_hat);
  memcpy(out, p.data_hat, sizeof(double) * 2 * (long long)n[0] * n[1] * (n[2] / 2 + 1));
  return 0;
}
int ref_c2r_inplace(const int* n, const double* in, double* out) {
  R2C p(n, true);
  if (!p.plan) return -1;
  const int pad = 2 * (n[2] / 2 + 1);
  memcpy(p.data_hat, in, sizeof(double) * 2 * (long long)n[0] * n[1] * (n[2] / 2 + 1));
  accfft_execute_c2r(p.plan, p.data_hat, p.data);
  for (long long r = 0; r < (long long)n[0] * n[1]; ++r) memcpy(out + r * n[2], p.data + r * pad, sizeof(double) * n[2]);
  return 0;
}

/* src/accfft.cpp:812 accfft_execute_c2c: complex [n0][n1][n2] both ways;
 * with z cleared the result is left in the input array */
int ref_c2c(const int* n, int dir, int xyz, const double* in, double* out) {
  int n3[3] = {n[0], n[1], n[2]}, isize[3], istart[3], osize[3], ostart[3];
  MPI_Comm c = one_rank_comm();
  long long alloc_max = accfft_local_size_dft_c2c(n3, isize, istart, osize, ostart, c);
  Complex* a = (Complex*)accfft_alloc(alloc_max);
  Complex* b = (Complex*)accfft_alloc(alloc_max);
  accfft_plan* plan = accfft_plan_dft_3d_c2c(n3, a, b, c, ACCFFT_MEASURE);
  if (!plan) return -1;
  memcpy(a, in, sizeof(double) * 2 * real_count(n));
  accfft_execute_c2c(plan, dir, a, b, NULL, std::bitset<3>(xyz));
  memcpy(out, (xyz & 4) ? b : a, sizeof(double) * 2 * real_count(n));
  accfft_destroy_plan(plan);
  accfft_free(a);
  accfft_free(b);
  return 0;
}

/* Single-axis real transforms of the CPU path (src/accfft.cpp:1051-1331,
 * accfft_execute_{r2c,c2r}_{x,y,z}_t).  dir -1: in real [n0][n1][n2] -> out
 * as the reference stores it; dir +1: that layout back to real.  The CPU
 * path's layouts at one rank: z [n0][n1][n2/2+1]; y [n0][n2][n1/2+1] (each
 * x-slab transposed by T_plan_y); x [n1][n2][n0/2+1] (T_plan_x).  out_len is
 * the caller's capacity in doubles; the spectrum has 2*prod(layout) doubles. */
int ref_axis(const int* n, int axis, int dir, const double* in, double* out, long long out_len) {
  R2C p(n);
  if (!p.plan) return -1;
  long long spec = 2LL * (axis == 2 ? (long long)n[0] * n[1] * (n[2] / 2 + 1)
                        : axis == 1 ? (long long)n[0] * n[2] * (n[1] / 2 + 1)
                                    : (long long)n[1] * n[2] * (n[0] / 2 + 1));
  long long need = dir < 0 ? spec : real_count(n);
  if (out_len < need) return -2;
  if (dir < 0) {
    memcpy(p.data, in, sizeof(double) * real_count(n));
    if (axis == 2) accfft_execute_r2c_z_t<double, Complex, accfft_plan>(p.plan, p.data, p.data_hat, NULL);
    else if (axis == 1) accfft_execute_r2c_y_t<double, Complex, accfft_plan>(p.plan, p.data, p.data_hat, NULL);
    else accfft_execute_r2c_x_t<double, Complex, accfft_plan>(p.plan, p.data, p.data_hat, NULL);
    memcpy(out, p.data_hat, sizeof(double) * spec);
  } else {
    memcpy(p.data_hat, in, sizeof(double) * spec);
    if (axis == 2) accfft_execute_c2r_z_t<Complex, double, accfft_plan>(p.plan, p.data_hat, p.data, NULL);
    else if (axis == 1) accfft_execute_c2r_y_t<Complex, double, accfft_plan>(p.plan, p.data_hat, p.data, NULL);
    else accfft_execute_c2r_x_t<Complex, double, accfft_plan>(p.plan, p.data_hat, p.data, NULL);
    memcpy(out, p.data, sizeof(double) * real_count(n));
  }
  return 0;
}

/* Spectral operators (src/operators.txx:794-1378, the CPU drivers):
 *   kind 0 grad, 1 grad_slow (in: 1 field, out: 3 fields x, y, z; pxyz
 *   selects components, unselected outputs are left untouched);
 *   2 laplace, 5 biharmonic, 6 inv_laplace, 7 inv_biharmonic (1 -> 1);
 *   3 divergence, 4 divergence_slow (3 fields -> 1).
 * Fields are real [n0][n1][n2], stored one after another. */
int ref_op(const int* n, int kind, int pxyz, const double* in, double* out) {
  R2C p(n);
  if (!p.plan) return -1;
  const long long N = real_count(n);
  const size_t bytes = (size_t)p.alloc_max > sizeof(double) * N ? (size_t)p.alloc_max : sizeof(double) * N;
  double* f[4];
  for (int i = 0; i < 4; ++i) {
    f[i] = (double*)accfft_alloc(bytes);
    memset(f[i], 0, bytes);
  }
  std::bitset<3> XYZ(pxyz);
  int rc = 0;
  switch (kind) {
    case 0:
    case 1:
      memcpy(f[0], in, sizeof(double) * N);
      for (int i = 1; i < 4; ++i) memcpy(f[i], out + (i - 1) * N, sizeof(double) * N);
      if (kind == 0) accfft_grad(f[1], f[2], f[3], f[0], p.plan, &XYZ, NULL);
      else accfft_grad_slow_t<double, accfft_plan>(f[1], f[2], f[3], f[0], p.plan, &XYZ, NULL);
      for (int i = 1; i < 4; ++i) memcpy(out + (i - 1) * N, f[i], sizeof(double) * N);
      break;
    case 3:
    case 4:
      for (int i = 0; i < 3; ++i) memcpy(f[i], in + i * N, sizeof(double) * N);
      if (kind == 3) accfft_divergence(f[3], f[0], f[1], f[2], p.plan, NULL);
      else accfft_divergence_slow_t<double, accfft_plan>(f[3], f[0], f[1], f[2], p.plan, NULL);
      memcpy(out, f[3], sizeof(double) * N);
      break;
    case 2:
    case 5:
    case 6:
    case 7:
      memcpy(f[0], in, sizeof(double) * N);
      if (kind == 2) accfft_laplace(f[1], f[0], p.plan, NULL);
      else if (kind == 5) accfft_biharmonic(f[1], f[0], p.plan, NULL);
      else if (kind == 6) accfft_inv_laplace(f[1], f[0], p.plan, NULL);
      else accfft_inv_biharmonic(f[1], f[0], p.plan, NULL);
      memcpy(out, f[1], sizeof(double) * N);
      break;
    default:
      rc = -3;
  }
  for (int i = 0; i < 4; ++i) accfft_free(f[i]);
  return rc;
}

}  // extern "C"
