// One translation unit per (precision, kernel kind, length group): the build
// compiles this file with -DAFG_PREC=<0..2> -DAFG_KIND=<0..4> -DAFG_GROUP=<0|1>
// so the template instantiations spread over parallel nvcc processes.
//   AFG_PREC 0 = float, 1 = double, 2 = double-float arithmetic on double
//            arrays (plain transforms only: kinds 0..3, strided mode 0)
//   AFG_KIND 0 = strided (MODE 0..4), 1 = zc2c, 2 = zr2c, 3 = zc2r, 4 = zsym (with and without accumulate)
#include "passes.cuh"
#include "launch.h"
#include "per_device.h"

#if !defined(AFG_PREC) || !defined(AFG_KIND) || !defined(AFG_GROUP)
#error "AFG_PREC, AFG_KIND and AFG_GROUP must be defined"
#endif

#if AFG_PREC == 0
typedef float Real;
#define AFG_P f32
#elif AFG_PREC == 1
typedef double Real;
#define AFG_P f64
#else
typedef afg::df Real;
#define AFG_P fdf
#if AFG_KIND == 4
#error "double-float plans have no symbol kernels"
#endif
#endif
#if AFG_GROUP == 0
#define AFG_G g0
#define AFG_LIST AFG_LENGTHS_G0
#else
#define AFG_G g1
#define AFG_LIST AFG_LENGTHS_G1
#endif
#if AFG_KIND == 0
#define AFG_K launch_strided
#elif AFG_KIND == 1
#define AFG_K launch_zc2c
#elif AFG_KIND == 2
#define AFG_K launch_zr2c
#elif AFG_KIND == 3
#define AFG_K launch_zc2r
#else
#define AFG_K launch_zsym
#endif
#define AFG_CAT4_(a, b, c) a##_##b##_##c
#define AFG_CAT4(a, b, c) AFG_CAT4_(a, b, c)
#define AFG_NAME AFG_CAT4(AFG_K, AFG_P, AFG_G)

namespace afg {


#if AFG_KIND == 0
template <int L, int MODE>
static void run_strided(const StridedArgs& a, cudaStream_t s) {
  typedef StridedShape<Real, L> SH;
  auto k = k_strided<Real, L, MODE>;
  static PerDevice prepared;   // per instantiation, per device
  prepare_smem(prepared, k, SH::smem);
  unsigned grid = unsigned((a.ncols + SH::TC - 1) / SH::TC);
  StridedArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  launch_pass(k, grid, SH::threads, SH::smem, s, b);
}
bool AFG_NAME(int L, int mode, const StridedArgs& a, cudaStream_t s) {
#if AFG_PREC == 2
  if (mode != 0) return false;
  switch (L) {
#define AFG_CASE(n)             \
  case n:                       \
    run_strided<n, 0>(a, s);    \
    return true;
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
#else
  switch (L) {
#define AFG_CASE(n)                        \
  case n:                                  \
    switch (mode) {                        \
      case 0: run_strided<n, 0>(a, s); break; \
      case 1: run_strided<n, 1>(a, s); break; \
      case 2: run_strided<n, 2>(a, s); break; \
      case 3: run_strided<n, 3>(a, s); break; \
      default: run_strided<n, 4>(a, s); break; \
    }                                      \
    return true;
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
#endif
}
#else
// float z c2r tiles of 256-point (and longer) half lines hold half the
// default lines per CTA (more, smaller CTAs per SM: measured 5 % faster at
// N2/2 = 256; the r2c pass prefers the default)
template <int L>
constexpr int contig_tl() {
#if AFG_KIND == 3
  return sizeof(Real) == 4 && L >= 256 && ContigShape<Real, L>::TL >= 2 ? ContigShape<Real, L>::TL / 2 : 0;
#else
  return 0;
#endif
}

template <int L, bool ACC = false>
static void run_contig(const ContigArgs& a, cudaStream_t s) {
  typedef ContigShape<Real, L, 0, contig_tl<L>()> SH;
#if AFG_KIND == 1
  auto k = k_zc2c<Real, L>;
#elif AFG_KIND == 2
  auto k = k_zr2c<Real, L>;
#elif AFG_KIND == 3
  auto k = k_zc2r<Real, L, 0, contig_tl<L>()>;
#else
  auto k = k_zsym<Real, L, 0, 0, ACC>;
#endif
  static PerDevice prepared;   // per instantiation, per device
  prepare_smem(prepared, k, SH::smem);
  unsigned grid = unsigned((a.nlines + SH::TL - 1) / SH::TL);
  ContigArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  launch_pass(k, grid, SH::threads, SH::smem, s, b);
}
bool AFG_NAME(int L, const ContigArgs& a, cudaStream_t s) {
  switch (L) {
#if AFG_KIND == 4
#define AFG_CASE(n)                                   \
  case n:                                             \
    if (a.acc) run_contig<n, true>(a, s);             \
    else run_contig<n, false>(a, s);                  \
    return true;
#else
#define AFG_CASE(n) case n: run_contig<n>(a, s); return true;
#endif
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
}
#endif

}  // namespace afg
