// C++ API check: builds against include/accfft_gpu.h, accfft_gpuf.h and
// accfft_operators_gpu.h the way an AccFFT program does, and checks
//   - r2c -> c2r round trips, double and float, out of place (as steps/step1)
//   - the in-place r2c with padded rows (as steps/step2)
//   - c2c forward -> backward, double and float (as steps/step3)
//   - grad, laplace, biharmonic, divergence(grad) against closed forms (as steps/step5)
// Prints one line per check and exits with the number of failures.
#include <mpi.h>
#include <cuda_runtime_api.h>

#include <accfft_gpu.h>
#include <accfft_gpuf.h>
#include <accfft_operators_gpu.h>

#include <cmath>
#include <cstdio>
#include <vector>

static int failures = 0;

static void report(const char* name, double err, double tol) {
  bool ok = err < tol;
  printf("%-36s rel_err %.3e (tol %.0e) %s\n", name, err, tol, ok ? "CORRECT" : "NOT CORRECT");
  if (!ok) ++failures;
}

template <typename T>
static T* dev(size_t n) {
  T* p = nullptr;
  if (cudaMalloc((void**)&p, n * sizeof(T)) != cudaSuccess) { printf("cudaMalloc failed\n"); exit(99); }
  return p;
}

static double gauss(double x, double y, double z) {
  const double pi = M_PI;
  return std::exp(-4.0 * ((x - pi) * (x - pi) + (y - pi) * (y - pi) + (z - pi) * (z - pi)));
}

template <typename T>
static std::vector<T> field(const int* n, size_t row) {
  std::vector<T> u((size_t)n[0] * n[1] * row, T(0));
  for (int i = 0; i < n[0]; ++i)
    for (int j = 0; j < n[1]; ++j)
      for (int k = 0; k < n[2]; ++k)
        u[((size_t)i * n[1] + j) * row + k] =
            T(gauss(2 * M_PI * i / n[0], 2 * M_PI * j / n[1], 2 * M_PI * k / n[2]));
  return u;
}

template <typename T>
static double rel_l1(const std::vector<T>& a, const std::vector<T>& b, const int* n, size_t row, double scale) {
  double e = 0, s = 0;
  for (int i = 0; i < n[0]; ++i)
    for (int j = 0; j < n[1]; ++j)
      for (int k = 0; k < n[2]; ++k) {
        size_t q = ((size_t)i * n[1] + j) * row + k;
        e += std::fabs(a[q] / scale - b[q]);
        s += std::fabs(b[q]);
      }
  return e / s;
}

// out-of-place round trip through the typed API of each precision (for
// double also with the double-float flag, an extension of the flags word)
static void step1_double(int* n, MPI_Comm c_comm, unsigned flags = ACCFFT_MEASURE,
                         const char* name = "step1 r2c/c2r double") {
  int isize[3], osize[3], istart[3], ostart[3];
  int alloc_max = accfft_local_size_dft_r2c_gpu(n, isize, istart, osize, ostart, c_comm);
  size_t N = (size_t)n[0] * n[1] * n[2];
  double* u = dev<double>(N);
  double* u2 = dev<double>(N);
  Complex* uh = (Complex*)dev<char>(alloc_max);
  accfft_plan_gpu* plan = accfft_plan_dft_3d_r2c_gpu(n, u, (double*)uh, c_comm, flags);
  std::vector<double> h = field<double>(n, n[2]), back(N);
  cudaMemcpy(u, h.data(), N * sizeof(double), cudaMemcpyHostToDevice);
  double timer[5] = {0, 0, 0, 0, 0};
  accfft_execute_r2c_gpu(plan, u, uh, timer);
  accfft_execute_c2r_gpu(plan, uh, u2, timer);
  cudaMemcpy(back.data(), u2, N * sizeof(double), cudaMemcpyDeviceToHost);
  report(name, rel_l1(back, h, n, n[2], (double)N), 1e-10);
  if (!(timer[4] > 0)) { printf("timer slot 4 not filled\n"); ++failures; }
  accfft_destroy_plan(plan);
  cudaFree(u); cudaFree(u2); cudaFree(uh);
}

static void step1_float(int* n, MPI_Comm c_comm) {
  int isize[3], osize[3], istart[3], ostart[3];
  int alloc_max = accfft_local_size_dft_r2c_gpuf(n, isize, istart, osize, ostart, c_comm);
  size_t N = (size_t)n[0] * n[1] * n[2];
  float* u = dev<float>(N);
  float* u2 = dev<float>(N);
  Complexf* uh = (Complexf*)dev<char>(alloc_max);
  accfft_plan_gpuf* plan = accfft_plan_dft_3d_r2c_gpuf(n, u, (float*)uh, c_comm, ACCFFT_MEASURE);
  std::vector<float> h = field<float>(n, n[2]), back(N);
  cudaMemcpy(u, h.data(), N * sizeof(float), cudaMemcpyHostToDevice);
  accfft_execute_r2c_gpuf(plan, u, uh);
  accfft_execute_c2r_gpuf(plan, uh, u2);
  cudaMemcpy(back.data(), u2, N * sizeof(float), cudaMemcpyDeviceToHost);
  report("step1 r2c/c2r float", rel_l1(back, h, n, n[2], (double)N), 1e-5);
  accfft_destroy_plan_gpu(plan);
  cudaFree(u); cudaFree(u2); cudaFree(uh);
}

// in-place: rows padded to 2*(N2/2+1)
static void step2_inplace(int* n, MPI_Comm c_comm) {
  int isize[3], osize[3], istart[3], ostart[3];
  int alloc_max = accfft_local_size_dft_r2c_gpu(n, isize, istart, osize, ostart, c_comm);
  size_t row = 2 * (n[2] / 2 + 1);
  size_t N = (size_t)n[0] * n[1] * n[2];
  double* d = (double*)dev<char>(alloc_max);
  accfft_plan_gpu* plan = accfft_plan_dft_3d_r2c_gpu(n, d, d, c_comm, ACCFFT_MEASURE);
  if (!plan->inplace) { printf("in-place plan not detected\n"); ++failures; }
  std::vector<double> h = field<double>(n, row), back(h.size());
  cudaMemcpy(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  accfft_execute_r2c_gpu(plan, d, (Complex*)d);
  accfft_execute_c2r_gpu(plan, (Complex*)d, d);
  cudaMemcpy(back.data(), d, h.size() * sizeof(double), cudaMemcpyDeviceToHost);
  report("step2 in-place r2c/c2r double", rel_l1(back, h, n, row, (double)N), 1e-10);
  accfft_destroy_plan(plan);
  cudaFree(d);
}

template <typename Cx, typename Plan, typename Real>
static void step3_c2c(int* n, MPI_Comm c_comm, const char* name, double tol) {
  size_t N = (size_t)n[0] * n[1] * n[2];
  Cx* a = (Cx*)dev<char>(N * sizeof(Cx));
  Cx* b = (Cx*)dev<char>(N * sizeof(Cx));
  Plan* plan;
  if constexpr (sizeof(Real) == 8) plan = accfft_plan_dft_3d_c2c_gpu(n, a, b, c_comm, ACCFFT_MEASURE);
  else plan = accfft_plan_dft_3d_c2c_gpuf(n, a, b, c_comm, ACCFFT_MEASURE);
  std::vector<Real> h(2 * N), back(2 * N);
  std::vector<Real> g = field<Real>(n, n[2]);
  for (size_t q = 0; q < N; ++q) h[2 * q] = h[2 * q + 1] = g[q];
  cudaMemcpy(a, h.data(), 2 * N * sizeof(Real), cudaMemcpyHostToDevice);
  if constexpr (sizeof(Real) == 8) {
    accfft_execute_c2c_gpu(plan, ACCFFT_FORWARD, a, b);
    accfft_execute_c2c_gpu(plan, ACCFFT_BACKWARD, b, a);
  } else {
    accfft_execute_c2c_gpuf(plan, ACCFFT_FORWARD, a, b);
    accfft_execute_c2c_gpuf(plan, ACCFFT_BACKWARD, b, a);
  }
  cudaMemcpy(back.data(), a, 2 * N * sizeof(Real), cudaMemcpyDeviceToHost);
  double e = 0, s = 0;
  for (size_t q = 0; q < 2 * N; ++q) { e += std::fabs(back[q] / N - h[q]); s += std::fabs(h[q]); }
  report(name, e / s, tol);
  accfft_destroy_plan(plan);
  cudaFree(a); cudaFree(b);
}

// step5 field and closed forms
static const double SIG = 32.0;
static double f5(double x, double y, double z) {
  const double pi = M_PI;
  return std::sin(x) * std::sin(y) * std::sin(z) +
         std::exp(-SIG * ((x - pi) * (x - pi) + (y - pi) * (y - pi) + (z - pi) * (z - pi)));
}
static double g5(double x, double y, double z, int d) {
  const double pi = M_PI;
  double e = std::exp(-SIG * ((x - pi) * (x - pi) + (y - pi) * (y - pi) + (z - pi) * (z - pi)));
  if (d == 0) return std::cos(x) * std::sin(y) * std::sin(z) - 2 * SIG * (x - pi) * e;
  if (d == 1) return std::sin(x) * std::cos(y) * std::sin(z) - 2 * SIG * (y - pi) * e;
  return std::sin(x) * std::sin(y) * std::cos(z) - 2 * SIG * (z - pi) * e;
}
static double l5(double x, double y, double z) {
  const double pi = M_PI;
  double r2 = (x - pi) * (x - pi) + (y - pi) * (y - pi) + (z - pi) * (z - pi);
  return -3 * std::sin(x) * std::sin(y) * std::sin(z) + (4 * SIG * SIG * r2 - 6 * SIG) * std::exp(-SIG * r2);
}

static void step5_ops(int* n, MPI_Comm c_comm) {
  size_t N = (size_t)n[0] * n[1] * n[2];
  std::vector<double> a(N), gx(N), gy(N), gz(N), la(N);
  for (int i = 0; i < n[0]; ++i)
    for (int j = 0; j < n[1]; ++j)
      for (int k = 0; k < n[2]; ++k) {
        double x = 2 * M_PI * i / n[0], y = 2 * M_PI * j / n[1], z = 2 * M_PI * k / n[2];
        size_t q = ((size_t)i * n[1] + j) * n[2] + k;
        a[q] = f5(x, y, z);
        gx[q] = g5(x, y, z, 0); gy[q] = g5(x, y, z, 1); gz[q] = g5(x, y, z, 2);
        la[q] = l5(x, y, z);
      }
  int isize[3], osize[3], istart[3], ostart[3];
  int alloc_max = accfft_local_size_dft_r2c_gpu(n, isize, istart, osize, ostart, c_comm);
  double* A = dev<double>(N);
  double* G[3] = {dev<double>(N), dev<double>(N), dev<double>(N)};
  double* L = dev<double>(N);
  Complex* scratch = (Complex*)dev<char>(alloc_max);
  accfft_plan_gpu* plan = accfft_plan_dft_3d_r2c_gpu(n, A, (double*)scratch, c_comm, ACCFFT_MEASURE);
  cudaMemcpy(A, a.data(), N * sizeof(double), cudaMemcpyHostToDevice);
  std::bitset<3> xyz(7);
  accfft_grad_gpu(G[0], G[1], G[2], A, plan, &xyz);
  std::vector<double> back(N);
  const std::vector<double>* ref[3] = {&gx, &gy, &gz};
  const char* gn[3] = {"step5 grad x double", "step5 grad y double", "step5 grad z double"};
  for (int d = 0; d < 3; ++d) {
    cudaMemcpy(back.data(), G[d], N * sizeof(double), cudaMemcpyDeviceToHost);
    report(gn[d], rel_l1(back, *ref[d], n, n[2], 1.0), 1e-10);
  }
  accfft_laplace_gpu(L, A, plan);
  cudaMemcpy(back.data(), L, N * sizeof(double), cudaMemcpyDeviceToHost);
  report("step5 laplace double", rel_l1(back, la, n, n[2], 1.0), 1e-10);
  accfft_divergence_gpu(L, G[0], G[1], G[2], plan);
  cudaMemcpy(back.data(), L, N * sizeof(double), cudaMemcpyDeviceToHost);
  report("step5 div(grad) double", rel_l1(back, la, n, n[2], 1.0), 1e-10);
  // inv_laplace(laplace(u)) returns u minus its mean (no Nyquist content at this resolution)
  accfft_laplace_gpu(L, A, plan);
  accfft_inv_laplace_gpu(G[0], L, plan);
  cudaMemcpy(back.data(), G[0], N * sizeof(double), cudaMemcpyDeviceToHost);
  double mean = 0;
  for (double v : a) mean += v;
  mean /= N;
  std::vector<double> am(N);
  for (size_t q = 0; q < N; ++q) am[q] = a[q] - mean;
  report("inv_laplace(laplace) double", rel_l1(back, am, n, n[2], 1.0), 1e-9);
  accfft_destroy_plan(plan);
  cudaFree(A); cudaFree(L); cudaFree(scratch);
  for (double* g : G) cudaFree(g);
}

static void unbaked_plan_is_reported() {
  accfft_plan_gpu plan;   // never baked: the call must print and return
  accfft_execute_r2c_gpu(&plan, nullptr, nullptr);
}

int main(int argc, char** argv) {
  MPI_Init(&argc, &argv);
  int n[3] = {64, 64, 64};
  if (argc > 3) { n[0] = atoi(argv[1]); n[1] = atoi(argv[2]); n[2] = atoi(argv[3]); }
  int c_dims[2] = {0, 0};
  MPI_Comm c_comm;
  accfft_create_comm(MPI_COMM_WORLD, c_dims, &c_comm);
  step1_double(n, c_comm);
  step1_double(n, c_comm, ACCFFT_MEASURE | ACCFFT_F64_DF, "step1 r2c/c2r double, double-float plan");
  step1_float(n, c_comm);
  step2_inplace(n, c_comm);
  step3_c2c<Complex, accfft_plan_gpu, double>(n, c_comm, "step3 c2c double", 1e-10);
  step3_c2c<Complexf, accfft_plan_gpuf, float>(n, c_comm, "step3 c2c float", 1e-5);
  int m[3] = {128, 128, 128};
  step5_ops(m, c_comm);
  unbaked_plan_is_reported();
  accfft_cleanup_gpu();
  MPI_Finalize();
  printf("%d failure(s)\n", failures);
  return failures;
}
