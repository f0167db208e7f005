// Kernel argument blocks passed by value from the host plan layer to the
// pass kernels.  Plain C++: shared by nvcc and host compilers.
#pragma once

namespace afg {

enum SymKind {
  SYM_NONE = 0,
  SYM_LAPLACE = 1,      // -(wx^2+wy^2+wz^2) * scale
  SYM_BIHARM = 2,       // (wx^2+wy^2+wz^2)^2 * scale
  SYM_INVLAP = 3,       // scale / -(wx^2+wy^2+wz^2), 0 where the sum is 0
  SYM_INVBIHARM = 4,    // scale / (kx^2+ky^2+kz^2)^2 without Nyquist folding, 1 where 0
  SYM_GRADX = 5,        // i * wx * scale   (3-D spectrum)
  SYM_GRADY = 6,
  SYM_GRADZ = 7,
  SYM_DERIV1 = 8,       // i * w(p) * scale (1-D symbol along the pass axis)
  SYM_DERIV2 = 9,       // -w(p)^2 * scale
  SYM_HEAT = 10,        // exp(-(wx^2+wy^2+wz^2) * param) * scale
  SYM_HELMHOLTZ = 11,   // scale / (param + wx^2+wy^2+wz^2), 0 where that is 0
  SYM_POISSON_FD = 12,  // scale / (Dx + Dy + Dz), D_i = 2 (cos(2 pi k_i/N_i) - 1) N_i^2 (unit cube,
                        // finite-difference Laplacian); 0 at k = 0
  SYM_POISSON_SPEC = 13 // scale / (-4 pi^2 (kx^2+ky^2+kz^2)), k folded above N/2 without the
                        // Nyquist filter; 0 at k = 0
};

struct SymArgs {
  int kind;
  int n0, n1, n2;   // grid sizes used to fold indices into wave numbers
  int h2;           // spectrum columns per y row (N2/2+1 for r2c spectra)
  int axis_len;     // line length for the 1-D symbols
  double scale;
  double param;     // time (SYM_HEAT) or shift (SYM_HELMHOLTZ)
  // SYM_POISSON_FD: tables D_i(|k|), |k| = 0..N_i/2, in the plan's precision,
  // for x at fd_tab, y at fd_tab + fd_y, z at fd_tab + fd_z
  const void* fd_tab;
  int fd_y, fd_z;
};

struct StridedArgs {
  const void* in;
  void* out;
  const void* acc;          // optional addend, laid out like out (MODE 1)
  const void* tw;           // stage twiddles of the line length
  long long ncols;          // columns over all slabs
  long long cps;            // columns per slab
  long long in_slab, in_line;
  long long out_slab, out_line;
  int inverse;              // MODE 0: conjugate on load and store
  SymArgs sym;              // MODE 1
  // split layout (aligned main part + Nyquist plane): when ncols_main > 0,
  // columns g >= ncols_main are Nyquist columns: column j = g - ncols_main
  // reads in_nyq + j*nyq_slab and writes out_nyq + j*nyq_slab, line stride
  // nyq_line; the main columns g < ncols_main use the fields above
  long long ncols_main;
  const void* in_nyq;
  void* out_nyq;
  long long nyq_slab, nyq_line;
  int early_trigger;        // set by the launcher: release the next pass at CTA start
  // double-float plans: the largest biased exponent of the transform's input
  // (the passes scale by an exact power of two around their arithmetic)
  const int* dfx;
  // polls a device-side wait makes before it gives up (tensor-core and
  // persistent kernels; accfft_c_set_wait_limit)
  unsigned wait_limit;
  // radix / tile variant of a float MODE 0 pass (variants.cu; 0 = default)
  int variant;
  // set to 1 when a bounded wait of the pass gave up (variant 4)
  int* wait_err;
};

struct ContigArgs {
  const void* in;
  void* out;
  const void* acc;          // optional addend (k_zsym), laid out like out
  const void* tw;           // stage twiddles of the line length
  const void* tw_post;      // r2c split twiddles w_{2M}^k, k = 0..M
  long long nlines;
  long long in_dist, out_dist;   // in elements of the array's own type
  int inverse;
  // adjoint weighting of the half spectrum (interior planes 0 < kz < N2/2):
  // 1 = k_zc2r reads them at weight 1/2, 2 = k_zr2c writes them at weight 2
  int weight;
  // separate Nyquist plane: k_zr2c writes X[M] of line l to nyq_out[l] (and
  // rows of M entries), k_zc2r reads it from nyq_in[l]
  void* nyq_out;
  const void* nyq_in;
  SymArgs sym;
  int early_trigger;        // set by the launcher: release the next pass at CTA start
  const int* dfx;           // as StridedArgs::dfx
  unsigned wait_limit;      // as StridedArgs::wait_limit
  // packed pass order (k_zr2c / k_zc2r only): when pair_n1 > 0 the lines are
  // the z lines of an [pair_n0][pair_n1] grid taken in mirror pairs
  // (x, y) / ((n0-x)%n0, (n1-y)%n1), both lines of a pair in one CTA; nlines
  // is twice the number of pairs (pair_lines() in passes.cuh)
  int pair_n0, pair_n1;
  int variant;              // as StridedArgs::variant (float z r2c / z c2r)
};

// Lines of a length without compiled kernels (gen.cu): a runtime radix plan
// (radix[s], stage twiddles at tw + off[s]: entry (r-1)*Ns + k is
// w_{Ns*R}^{r*k}), run over the lines of one pass.
constexpr int kGenMaxStages = 16;
struct GenPlan {
  int L;                    // line length (the full real length N2 for r2c / c2r)
  int nst;
  int radix[kGenMaxStages];
  int off[kGenMaxStages];   // complex entries into tw
  const void* tw;           // in the plan's precision
};
struct GenArgs {
  GenPlan g;
  const void* in;
  void* out;
  long long nlines;         // lines (columns of a strided pass)
  // strided lines (y and x passes): line c starts at slab * slab + cc, c =
  // slab * cps + cc, element p at p * line (complex elements)
  long long cps, in_slab, out_slab, in_line, out_line;
  // contiguous lines (z passes): line l starts at l * dist (elements of the
  // array's own type: reals for the real side of r2c / c2r)
  long long in_dist, out_dist;
  int inverse;
  int tc;                   // lines per CTA (a power of two up to 16)
  int early_trigger;
};

struct SlabArgs {
  const void* in;           // forward: real [N0][N1][row]; inverse: spectrum [N0][N1][N2/2+1]
  void* out;                // forward: spectrum; inverse: real
  const void* tw_y;         // stage twiddles of N1
  const void* tw_z;         // stage twiddles of N2/2
  const void* tw_post;      // r2c split twiddles
  long long n0;             // slabs
  long long real_row;       // reals per row of the real array
};

}  // namespace afg
