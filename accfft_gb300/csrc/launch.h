// Host-side entry points into the pass kernels.  Each launcher returns false
// when the line length has no compiled kernel; the plan layer checks every
// axis against afg_length_supported() before it accepts a size.
#pragma once
#include <cuda_runtime.h>
#include "args.h"

// Lengths with compiled line kernels (complex line length L for c2c axes,
// half length M = N2/2 for the real z axis), split in two groups so the
// instantiations compile in parallel translation units.
#define AFG_LENGTHS_G0(X) \
  X(1) X(2) X(3) X(4) X(5) X(6) X(8) X(9) X(10) X(12) X(16) X(20) X(24) X(25) X(32) X(40) X(48) \
  X(64) X(80) X(90) X(96) X(100) X(128)
#define AFG_LENGTHS_G1(X) X(160) X(180) X(192) X(200) X(256) X(384) X(512) X(768) X(1024)

namespace afg {

bool length_supported(int L);

// Per-translation-unit launchers, one per (kernel kind, precision, length
// group); the ungrouped launchers below dispatch over all of them.
#define AFG_DECL_LAUNCHERS(P, G) \
  bool launch_strided_##P##_##G(int L, int mode, const StridedArgs& a, cudaStream_t s); \
  bool launch_zc2c_##P##_##G(int L, const ContigArgs& a, cudaStream_t s); \
  bool launch_zr2c_##P##_##G(int M, const ContigArgs& a, cudaStream_t s); \
  bool launch_zc2r_##P##_##G(int M, const ContigArgs& a, cudaStream_t s); \
  bool launch_zsym_##P##_##G(int M, const ContigArgs& a, cudaStream_t s);
AFG_DECL_LAUNCHERS(f32, g0)
AFG_DECL_LAUNCHERS(f32, g1)
AFG_DECL_LAUNCHERS(f64, g0)
AFG_DECL_LAUNCHERS(f64, g1)
AFG_DECL_LAUNCHERS(fdf, g0)   // double-float: no zsym, strided mode 0 only
AFG_DECL_LAUNCHERS(fdf, g1)

// grouped launches (float; lengths up to 256): one grid over the tiles of
// ntasks independent tasks whose arguments are tab[0..ntasks) in device
// memory, task k owning CTAs [starts[k], starts[k+1]), grid CTAs in all.
// tiles_* give a task's CTA count (-1: no grouped kernel for the length).
long long tiles_strided_f32_g0(int L, const StridedArgs& a);
long long tiles_strided_f32_g1(int L, const StridedArgs& a);
long long tiles_zr2c_f32_g0(int M, const ContigArgs& a);
long long tiles_zr2c_f32_g1(int M, const ContigArgs& a);
long long tiles_zc2r_f32_g0(int M, const ContigArgs& a);
long long tiles_zc2r_f32_g1(int M, const ContigArgs& a);
bool launch_strided_grouped_f32_g0(int L, int mode, const StridedArgs* tab, const long long* starts, int ntasks,
                                   long long grid, cudaStream_t s);
bool launch_strided_grouped_f32_g1(int L, int mode, const StridedArgs* tab, const long long* starts, int ntasks,
                                   long long grid, cudaStream_t s);
bool launch_zr2c_grouped_f32_g0(int M, const ContigArgs* tab, const long long* starts, int ntasks, long long grid,
                                cudaStream_t s);
bool launch_zr2c_grouped_f32_g1(int M, const ContigArgs* tab, const long long* starts, int ntasks, long long grid,
                                cudaStream_t s);
bool launch_zc2r_grouped_f32_g0(int M, const ContigArgs* tab, const long long* starts, int ntasks, long long grid,
                                cudaStream_t s);
bool launch_zc2r_grouped_f32_g1(int M, const ContigArgs* tab, const long long* starts, int ntasks, long long grid,
                                cudaStream_t s);

// arithmetic of a plan's kernels (the arrays are float for PREC_F32, IEEE
// double for the other two)
enum Prec { PREC_F32 = 0, PREC_F64 = 1, PREC_DF = 2 };

bool launch_strided(int prec, int L, int mode, const StridedArgs& a, cudaStream_t s);
bool launch_zc2c(int prec, int L, const ContigArgs& a, cudaStream_t s);
bool launch_zr2c(int prec, int M, const ContigArgs& a, cudaStream_t s);
bool launch_zc2r(int prec, int M, const ContigArgs& a, cudaStream_t s);
bool launch_zsym(int prec, int M, const ContigArgs& a, cudaStream_t s);

// fused z+y slab passes (thread-block clusters); false when the grid has no
// slab kernel or its cluster cannot be scheduled on this device
bool slab_available(bool dbl, int N1, int N2);
bool launch_slab(bool dbl, int N1, int N2, bool forward, const SlabArgs& a, cudaStream_t s);

// tensor-core forms of the r2c/c2r passes (float; form 1 = 3xTF32, 2 = split
// BF16): lengths 128, 256, 512, 1024 (strided) and 128, 256, 512 (z half
// length); err is a device word set when a completion wait gave up (after
// a.wait_limit polls)
bool tc_length_supported(int len, bool contig);
bool launch_strided_tc(int form, int L, const StridedArgs& a, int* err, cudaStream_t s);
bool launch_z_tc(int form, bool r2c, int M, const ContigArgs& a, int* err, cudaStream_t s);

// persistent z+y kernels (zy_fused.cu): grids whose z rows and y columns
// run on the same tile shape; ctl holds 1 + n0 zeroed words; *err is set
// when a wait between items gave up (after z.wait_limit / y.wait_limit polls)
bool zy_persistent_available(bool dbl, int M, int L);
bool launch_zy_persistent(bool dbl, bool forward, int M, int L, const ContigArgs& z, const StridedArgs& y,
                          unsigned* ctl, int* err, int n0, int lead, cudaStream_t s);

// double-float plans: the largest biased exponent of `rows` rows of `len`
// doubles, `stride` apart, into *out (zeroed first), on stream s
bool launch_df_scan(const void* x, long long rows, long long len, long long stride, int* out, cudaStream_t s);

// out[r][c] += in[r][c], c < len, over `rows` rows with their own strides
// (reals of the plan's precision), on stream s
bool launch_add_rows(bool dbl, void* out, long long out_row, const void* in, long long in_row, long long rows,
                     int len, cudaStream_t s);

// tuned variants of the float passes (variants.cu): false when the variant
// does not exist for the length; variant_shape gives its first radix and
// tile width (columns or lines per CTA), 0 when it does not exist
bool launch_strided_variant_f32(int L, int v, const StridedArgs& a, cudaStream_t s);
bool launch_contig_variant_f32(bool r2c, int M, int v, const ContigArgs& a, cudaStream_t s);
void variant_shape(int kind, int L, int v, int* E, int* tile);
constexpr int kMaxVariant = 4;
// spec[n0][cols] (complex, float or double) *= the symbol of s at
// (x, column), for the operators that run as r2c, symbol, c2r
// (sym_spectrum.cu)
bool launch_sym_spectrum(bool dbl, void* spec, long long n0, long long cols, const SymArgs& s, cudaStream_t st);
// lines of lengths without compiled kernels (gen.cu): mode 0 strided c2c,
// 1 contiguous c2c, 2 r2c, 3 c2r; float and double plans
bool launch_gen(int prec, int mode, const GenArgs& g, cudaStream_t s);
int gen_lines_per_cta(int L, bool dbl);

// pass kinds of a recorded batch task (plan.cpp) and their grouped launch
enum PassKind { PK_STRIDED = 0, PK_ZR2C = 2, PK_ZC2R = 3 };
long long grouped_tiles(int kind, int L, const void* args);
bool launch_grouped(int kind, int L, int mode, const void* tab, const long long* starts, int ntasks, long long grid,
                    cudaStream_t s);

// number of kernel launches issued by this process through the launchers
unsigned long long launch_count();
void count_launch();

// Programmatic dependent launch of the pass kernels: 0 off, 1 the next pass
// is released at the end of each CTA, 2 at its start (PassScope).  Read from
// ACCFFT_GB300_PDL on first use; set_pdl overrides it for the process.
int pdl_mode();
void set_pdl(int mode);

// Launch a pass kernel (one that opens a PassScope) on stream s, with the
// programmatic-serialisation attribute when PDL is on, and count it.
template <typename... Params, typename... Args>
inline cudaError_t launch_pass(void (*kernel)(Params...), unsigned grid, unsigned threads, size_t smem,
                               cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_mode() > 0 ? 1 : 0;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
  count_launch();
  return e;
}

}  // namespace afg
