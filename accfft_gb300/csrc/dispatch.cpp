// Length registry and dispatch over the per-translation-unit launchers.
#include <atomic>

#include "launch.h"

namespace afg {

namespace {
std::atomic<unsigned long long> g_launches{0};
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

bool length_supported(int L) {
  switch (L) {
#define AFG_CASE(n) case n:
    AFG_LENGTHS_G0(AFG_CASE)
    AFG_LENGTHS_G1(AFG_CASE)
#undef AFG_CASE
    return true;
    default:
      return false;
  }
}

bool launch_strided(bool dbl, int L, int mode, const StridedArgs& a, cudaStream_t s) {
  return dbl ? (launch_strided_f64_g0(L, mode, a, s) || launch_strided_f64_g1(L, mode, a, s))
             : (launch_strided_f32_g0(L, mode, a, s) || launch_strided_f32_g1(L, mode, a, s));
}
#define AFG_DISPATCH(K)                                                              \
  bool launch_##K(bool dbl, int L, const ContigArgs& a, cudaStream_t s) {           \
    return dbl ? (launch_##K##_f64_g0(L, a, s) || launch_##K##_f64_g1(L, a, s))     \
               : (launch_##K##_f32_g0(L, a, s) || launch_##K##_f32_g1(L, a, s));    \
  }
AFG_DISPATCH(zc2c)
AFG_DISPATCH(zr2c)
AFG_DISPATCH(zc2r)
AFG_DISPATCH(zsym)
#undef AFG_DISPATCH

}  // namespace afg
