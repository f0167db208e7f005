// The symbol multiply of the 3-D operators that run as r2c, a pass over the
// spectrum and c2r (plan.cpp, op3d): double-float plans, and plans with an
// axis length that has no compiled kernels.  The spectrum [n0][n1][h2] (the
// plan's scratch, in the plan's array type) is multiplied by the operator's
// symbol at (kx, ky, kz), in the array's precision, with the same symbol
// code as the fused passes.
#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace afg {

namespace {

constexpr int kSymThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kSymThreads) k_sym_spectrum(typename CT<T>::V* __restrict__ spec, long long n0,
                                                              long long cols, const SymArgs s, int early) {
  PassScope scope(early);
  const long long total = n0 * cols;
  with_symbol<T>(s, [&](auto sf) {
    for (long long e = (long long)blockIdx.x * kSymThreads + threadIdx.x; e < total;
         e += (long long)gridDim.x * kSymThreads) {
      const long long x = e / cols;
      const SymCol c = sym_column(s, e - x * cols);   // column (y, kz), frequency kx = x
      spec[e] = sf(c, int(x), spec[e]);
    }
  });
}

template <typename T>
bool run_sym(void* spec, long long n0, long long cols, const SymArgs& s, cudaStream_t st) {
  static PerDevice occupancy;
  auto k = k_sym_spectrum<T>;
  const long long tiles = (n0 * cols + kSymThreads - 1) / kSymThreads;
  const long long grid = persistent_grid(occupancy, k, kSymThreads, 0, tiles);
  if (grid <= 0) return false;
  return launch_pass(k, unsigned(grid), kSymThreads, 0, st, static_cast<typename CT<T>::V*>(spec), n0, cols, s,
                     int(pdl_mode() == 2)) == cudaSuccess;
}

}  // namespace

// float spectra for float plans; double spectra for double and double-float
// plans (whose arrays are IEEE double)
bool launch_sym_spectrum(bool dbl, void* spec, long long n0, long long cols, const SymArgs& s, cudaStream_t st) {
  return dbl ? run_sym<double>(spec, n0, cols, s, st) : run_sym<float>(spec, n0, cols, s, st);
}

}  // namespace afg
