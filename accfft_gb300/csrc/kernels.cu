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
#if AFG_PREC == 0
// grouped launches (float, lengths up to 256, modes 0 and 1): the batches'
// passes; tiles per task are ceil(ncols / TC)
template <int L>
static long long tiles_strided(const StridedArgs& a) {
  return (a.ncols + StridedShape<Real, L>::TC - 1) / StridedShape<Real, L>::TC;
}
template <int L, int MODE>
static bool run_strided_grouped(const StridedArgs* tab, const long long* starts, int ntasks, long long grid,
                                cudaStream_t s) {
  typedef StridedShape<Real, L> SH;
  auto k = k_strided_grouped<Real, L, MODE>;
  static PerDevice prepared, occupancy;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  const long long g = persistent_grid(occupancy, k, SH::threads, SH::smem, grid);
  return g > 0 && launch_pass(k, unsigned(g), SH::threads, SH::smem, s, tab, starts, ntasks, grid,
                              int(pdl_mode() == 2)) == cudaSuccess;
}
// lengths above 256 have no grouped kernel (kept out of the build)
template <int L>
static long long tiles_strided_if(const StridedArgs& a) {
  if constexpr (L <= 256) return tiles_strided<L>(a);
  else return -1;
}
template <int L>
static bool run_strided_grouped_if(int mode, const StridedArgs* tab, const long long* starts, int ntasks,
                                   long long grid, cudaStream_t s) {
  if constexpr (L <= 256) {
    if (mode == 0) return run_strided_grouped<L, 0>(tab, starts, ntasks, grid, s);
    if (mode == 1) return run_strided_grouped<L, 1>(tab, starts, ntasks, grid, s);
  }
  return false;
}
long long AFG_CAT4(tiles_strided, AFG_P, AFG_G)(int L, const StridedArgs& a) {
  switch (L) {
#define AFG_CASE(n) case n: return tiles_strided_if<n>(a);
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return -1;
  }
}
bool AFG_CAT4(launch_strided_grouped, AFG_P, AFG_G)(int L, int mode, const StridedArgs* tab, const long long* starts,
                                                    int ntasks, long long grid, cudaStream_t s) {
  switch (L) {
#define AFG_CASE(n) case n: return run_strided_grouped_if<n>(mode, tab, starts, ntasks, grid, s);
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
}
#endif
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
static bool run_contig(const ContigArgs& a, cudaStream_t s) {
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
  // pair mode (k_zr2c / k_zc2r): TL/2 mirror pairs per CTA
  const long long per = a.pair_n1 > 0 ? SH::TL / 2 : SH::TL;
  const long long units = a.pair_n1 > 0 ? a.nlines / 2 : a.nlines;
  if (per < 1) return false;
  unsigned grid = unsigned((units + per - 1) / per);
  ContigArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  launch_pass(k, grid, SH::threads, SH::smem, s, b);
  return true;
}
bool AFG_NAME(int L, const ContigArgs& a, cudaStream_t s) {
  switch (L) {
#if AFG_KIND == 4
#define AFG_CASE(n)                                   \
  case n:                                             \
    return a.acc ? run_contig<n, true>(a, s) : run_contig<n, false>(a, s);
#else
#define AFG_CASE(n) case n: return run_contig<n>(a, s);
#endif
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
}
#if AFG_PREC == 0 && (AFG_KIND == 2 || AFG_KIND == 3)
// grouped launches (float z r2c / c2r, half lengths up to 256): tiles per
// task are ceil(nlines / TL), or ceil(pairs / (TL / 2)) in pair mode
template <int L>
static long long tiles_contig(const ContigArgs& a) {
  constexpr int TL = ContigShape<Real, L, 0, contig_tl<L>()>::TL;
  const long long per = a.pair_n1 > 0 ? TL / 2 : TL;
  const long long units = a.pair_n1 > 0 ? a.nlines / 2 : a.nlines;
  return per < 1 ? -1 : (units + per - 1) / per;
}
template <int L>
static bool run_contig_grouped(const ContigArgs* tab, const long long* starts, int ntasks, long long grid,
                               cudaStream_t s) {
  typedef ContigShape<Real, L, 0, contig_tl<L>()> SH;
#if AFG_KIND == 2
  auto k = k_zr2c_grouped<Real, L>;
#else
  auto k = k_zc2r_grouped<Real, L, contig_tl<L>()>;
#endif
  static PerDevice prepared, occupancy;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  const long long g = persistent_grid(occupancy, k, SH::threads, SH::smem, grid);
  return g > 0 && launch_pass(k, unsigned(g), SH::threads, SH::smem, s, tab, starts, ntasks, grid,
                              int(pdl_mode() == 2)) == cudaSuccess;
}
template <int L>
static long long tiles_contig_if(const ContigArgs& a) {
  if constexpr (L <= 256) return tiles_contig<L>(a);
  else return -1;
}
template <int L>
static bool run_contig_grouped_if(const ContigArgs* tab, const long long* starts, int ntasks, long long grid,
                                  cudaStream_t s) {
  if constexpr (L <= 256) return run_contig_grouped<L>(tab, starts, ntasks, grid, s);
  else return false;
}
#if AFG_KIND == 2
#define AFG_GL launch_zr2c_grouped
#define AFG_GT tiles_zr2c
#else
#define AFG_GL launch_zc2r_grouped
#define AFG_GT tiles_zc2r
#endif
long long AFG_CAT4(AFG_GT, AFG_P, AFG_G)(int L, const ContigArgs& a) {
  switch (L) {
#define AFG_CASE(n) case n: return tiles_contig_if<n>(a);
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return -1;
  }
}
bool AFG_CAT4(AFG_GL, AFG_P, AFG_G)(int L, const ContigArgs* tab, const long long* starts, int ntasks, long long grid,
                                    cudaStream_t s) {
  switch (L) {
#define AFG_CASE(n) case n: return run_contig_grouped_if<n>(tab, starts, ntasks, grid, s);
    AFG_LIST(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
}
#endif
#endif

}  // namespace afg
