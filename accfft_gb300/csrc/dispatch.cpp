// Length registry and dispatch over the per-translation-unit launchers.
#include <atomic>
#include <cstdlib>

#include "launch.h"

namespace afg {

namespace {
std::atomic<unsigned long long> g_launches{0};
// -1: not yet read from the environment
std::atomic<int> g_pdl{-1};
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

int pdl_mode() {
  int v = g_pdl.load(std::memory_order_relaxed);
  if (v < 0) {
    const char* e = getenv("ACCFFT_GB300_PDL");
    v = (e && e[0] >= '0' && e[0] <= '2' && e[1] == 0) ? e[0] - '0' : 1;
    g_pdl.store(v, std::memory_order_relaxed);
  }
  return v;
}
void set_pdl(int mode) { g_pdl.store(mode < 0 ? 0 : (mode > 2 ? 2 : mode), std::memory_order_relaxed); }

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

bool launch_strided(int prec, int L, int mode, const StridedArgs& a, cudaStream_t s) {
  if (prec == PREC_F32 && mode == 0 && a.variant > 0) {
    if (launch_strided_variant_f32(L, a.variant, a, s)) return true;
    if (a.variant == 2) return false;   // a.tw holds the alternative radix's twiddles
  }
  switch (prec) {
    case PREC_F32: return launch_strided_f32_g0(L, mode, a, s) || launch_strided_f32_g1(L, mode, a, s);
    case PREC_F64: return launch_strided_f64_g0(L, mode, a, s) || launch_strided_f64_g1(L, mode, a, s);
    case PREC_DF: return launch_strided_fdf_g0(L, mode, a, s) || launch_strided_fdf_g1(L, mode, a, s);
    default: return false;
  }
}
#define AFG_DISPATCH(NAME, K, DF)                                                            \
  bool NAME(int prec, int L, const ContigArgs& a, cudaStream_t s) {                         \
    switch (prec) {                                                                          \
      case PREC_F32: return launch_##K##_f32_g0(L, a, s) || launch_##K##_f32_g1(L, a, s);   \
      case PREC_F64: return launch_##K##_f64_g0(L, a, s) || launch_##K##_f64_g1(L, a, s);   \
      case PREC_DF: return DF;                                                               \
      default: return false;                                                                 \
    }                                                                                        \
  }
AFG_DISPATCH(launch_zc2c, zc2c, launch_zc2c_fdf_g0(L, a, s) || launch_zc2c_fdf_g1(L, a, s))
AFG_DISPATCH(launch_zr2c_default, zr2c, launch_zr2c_fdf_g0(L, a, s) || launch_zr2c_fdf_g1(L, a, s))
AFG_DISPATCH(launch_zc2r_default, zc2r, launch_zc2r_fdf_g0(L, a, s) || launch_zc2r_fdf_g1(L, a, s))
AFG_DISPATCH(launch_zsym, zsym, false)
#undef AFG_DISPATCH

bool launch_zr2c(int prec, int M, const ContigArgs& a, cudaStream_t s) {
  if (prec == PREC_F32 && a.variant > 0) {
    if (launch_contig_variant_f32(true, M, a.variant, a, s)) return true;
    if (a.variant == 2) return false;   // a.tw holds the alternative radix's twiddles
  }
  return launch_zr2c_default(prec, M, a, s);
}
bool launch_zc2r(int prec, int M, const ContigArgs& a, cudaStream_t s) {
  if (prec == PREC_F32 && a.variant > 0) {
    if (launch_contig_variant_f32(false, M, a.variant, a, s)) return true;
    if (a.variant == 2) return false;   // a.tw holds the alternative radix's twiddles
  }
  return launch_zc2r_default(prec, M, a, s);
}

long long grouped_tiles(int kind, int L, const void* args) {
  long long t = -1;
  if (kind == PK_STRIDED) {
    const auto& a = *static_cast<const StridedArgs*>(args);
    t = tiles_strided_f32_g0(L, a);
    if (t < 0) t = tiles_strided_f32_g1(L, a);
  } else if (kind == PK_ZR2C || kind == PK_ZC2R) {
    const auto& a = *static_cast<const ContigArgs*>(args);
    t = kind == PK_ZR2C ? tiles_zr2c_f32_g0(L, a) : tiles_zc2r_f32_g0(L, a);
    if (t < 0) t = kind == PK_ZR2C ? tiles_zr2c_f32_g1(L, a) : tiles_zc2r_f32_g1(L, a);
  }
  return t;
}

bool launch_grouped(int kind, int L, int mode, const void* tab, const long long* starts, int ntasks, long long grid,
                    cudaStream_t s) {
  if (kind == PK_STRIDED) {
    const auto* t = static_cast<const StridedArgs*>(tab);
    return launch_strided_grouped_f32_g0(L, mode, t, starts, ntasks, grid, s) ||
           launch_strided_grouped_f32_g1(L, mode, t, starts, ntasks, grid, s);
  }
  const auto* t = static_cast<const ContigArgs*>(tab);
  if (kind == PK_ZR2C)
    return launch_zr2c_grouped_f32_g0(L, t, starts, ntasks, grid, s) ||
           launch_zr2c_grouped_f32_g1(L, t, starts, ntasks, grid, s);
  if (kind == PK_ZC2R)
    return launch_zc2r_grouped_f32_g0(L, t, starts, ntasks, grid, s) ||
           launch_zc2r_grouped_f32_g1(L, t, starts, ntasks, grid, s);
  return false;
}

}  // namespace afg
