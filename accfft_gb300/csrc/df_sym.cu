// The symbol multiply of the 3-D operators of double-float plans: the
// spectrum [n0][n1][h2] (IEEE double, the plan's scratch) times the operator's
// symbol at (kx, ky, kz), in double.  The operator runs as the plan's r2c,
// this pass and the plan's c2r (plan.cpp, op3d), so no fused double-float
// symbol kernel has to be compiled for every length.
#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace afg {

namespace {

constexpr int kSymThreads = 256;

__global__ void __launch_bounds__(kSymThreads) k_sym_spectrum(double2* __restrict__ spec, long long n0,
                                                              long long cols, const SymArgs s, int early) {
  PassScope scope(early);
  const long long total = n0 * cols;
  with_symbol<double>(s, [&](auto sf) {
    for (long long e = (long long)blockIdx.x * kSymThreads + threadIdx.x; e < total;
         e += (long long)gridDim.x * kSymThreads) {
      const long long x = e / cols;
      const SymCol c = sym_column(s, e - x * cols);   // column (y, kz), frequency kx = x
      spec[e] = sf(c, int(x), spec[e]);
    }
  });
}

}  // namespace

bool launch_sym_spectrum_f64(void* spec, long long n0, long long cols, const SymArgs& s, cudaStream_t st) {
  static PerDevice occupancy;
  const long long tiles = (n0 * cols + kSymThreads - 1) / kSymThreads;
  const long long grid = persistent_grid(occupancy, k_sym_spectrum, kSymThreads, 0, tiles);
  if (grid <= 0) return false;
  return launch_pass(k_sym_spectrum, unsigned(grid), kSymThreads, 0, st, static_cast<double2*>(spec), n0, cols, s,
                     int(pdl_mode() == 2)) == cudaSuccess;
}

}  // namespace afg
