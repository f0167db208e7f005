// Pass kernels: each kernel moves one batch of lines HBM -> registers ->
// (shared-memory Stockham exchanges) -> HBM exactly once.
//
//   k_strided   lines along a strided axis (y or x of a row-major 3-D array).
//               A CTA owns TC adjacent "columns" (the contiguous index) and
//               the whole line of each, so loads/stores of one line position
//               are TC*sizeof(complex) contiguous bytes.  Columns are numbered
//               across slabs (g -> slab g/cps, column g%cps), so ragged column
//               counts (e.g. N2/2+1) never leave idle tiles.  MODE 1 fuses
//               forward FFT -> spectral symbol -> inverse FFT on the same line
//               (operators, single-axis derivatives); MODE 4 is MODE 1
//               plus an accumulate input of the output's layout.
//   k_zc2c      contiguous complex lines (the z axis of a c2c transform).
//   k_zr2c      contiguous real lines of length 2M: one M-point complex FFT
//               of the even/odd packed samples + split to M+1 outputs.
//   k_zc2r      the inverse of k_zr2c (imaginary parts of the DC and Nyquist
//               inputs are ignored, as a Hermitian-input real transform does).
//   k_zsym      r2c -> per-frequency symbol -> c2r on contiguous real lines
//               (z-direction derivatives) with an optional accumulate input.
#pragma once
#include "fft_core.cuh"
#include "args.h"

namespace afg {

// wave number of index i on an axis of length n: i, i-n above n/2, and 0 at
// i == n/2 (integer n/2, the Nyquist filter of the reference's kernels)
__device__ __forceinline__ int fold_wave(int i, int n) {
  int w = i;
  if (i > n / 2) w -= n;
  if (i == n / 2) w = 0;
  return w;
}
__device__ __forceinline__ int fold_wave_nofilter(int i, int n) { return i > n / 2 ? i - n : i; }
// 1-D line symbols zero the mirror of n/2 as well, so that the symbol stays
// Hermitian-consistent for odd n (a real-to-real operator on complex-packed
// real pairs); for even n the two indices coincide
__device__ __forceinline__ int fold_wave_line(int i, int n) {
  return (i == n - n / 2) ? 0 : fold_wave(i, n);
}

// per-column part of a 3-D symbol evaluated in the x pass (column g = y*h2 + kz)
struct SymCol {
  int wy, wz;       // folded wave numbers
  int wy_nf, wz_nf; // unfiltered (for SYM_INVBIHARM)
};
__device__ __forceinline__ SymCol sym_column(const SymArgs& s, long long g) {
  SymCol c{0, 0, 0, 0};
  if ((s.kind >= SYM_LAPLACE && s.kind <= SYM_GRADZ) || s.kind >= SYM_HEAT) {
    int y = int(g / s.h2), kz = int(g - (long long)y * s.h2);
    c.wy = fold_wave(y, s.n1); c.wz = fold_wave(kz, s.n2);
    c.wy_nf = fold_wave_nofilter(y, s.n1); c.wz_nf = fold_wave_nofilter(kz, s.n2);
  }
  return c;
}

// a column of the Nyquist plane of the split layout: y = j, kz = N2/2
__device__ __forceinline__ SymCol sym_column_nyq(const SymArgs& s, long long j) {
  SymCol c{0, 0, 0, 0};
  int y = int(j), kz = s.n2 / 2;
  c.wy = fold_wave(y, s.n1); c.wz = fold_wave(kz, s.n2);
  c.wy_nf = fold_wave_nofilter(y, s.n1); c.wz_nf = fold_wave_nofilter(kz, s.n2);
  return c;
}

// multiply x (frequency p along the pass axis, column part c) by the symbol
// of kind K (a compile-time kind: the element loops that call it are
// specialised per kind by with_symbol(), so no per-element dispatch remains)
template <typename T, int K, typename V>
__device__ __forceinline__ V sym_apply_k(const SymArgs& s, const SymCol& c, int p, V x) {
  const T sc = T(s.scale);
  if constexpr (K == SYM_LAPLACE) {
    int wx = fold_wave(p, s.n0);
    T w = T(-(wx * wx + c.wy * c.wy + c.wz * c.wz)) * sc;
    return c_scale(x, w);
  } else if constexpr (K == SYM_BIHARM) {
    int wx = fold_wave(p, s.n0);
    T w = T(wx * wx + c.wy * c.wy + c.wz * c.wz);
    return c_scale(x, w * w * sc);
  } else if constexpr (K == SYM_INVLAP) {
    int wx = fold_wave(p, s.n0);
    int w = -(wx * wx + c.wy * c.wy + c.wz * c.wz);
    T m = (w == 0) ? T(0) : sc / T(w);
    return c_scale(x, m);
  } else if constexpr (K == SYM_INVBIHARM) {
    int wx = fold_wave_nofilter(p, s.n0);
    T w = T(wx * wx + c.wy_nf * c.wy_nf + c.wz_nf * c.wz_nf);
    w = w * w;
    if (w == T(0)) w = T(1);
    return c_scale(x, sc / w);
  } else if constexpr (K == SYM_GRADX || K == SYM_GRADY || K == SYM_GRADZ) {
    int w = K == SYM_GRADX ? fold_wave(p, s.n0) : (K == SYM_GRADY ? c.wy : c.wz);
    T m = T(w) * sc;
    return c_make<V>(-m * x.y, m * x.x);
  } else if constexpr (K == SYM_DERIV1) {
    T m = T(fold_wave_line(p, s.axis_len)) * sc;
    return c_make<V>(-m * x.y, m * x.x);
  } else if constexpr (K == SYM_DERIV2) {
    int w = fold_wave_line(p, s.axis_len);
    return c_scale(x, -T(w * w) * sc);
  } else if constexpr (K == SYM_HEAT) {
    int wx = fold_wave(p, s.n0);
    T k2 = T(wx * wx + c.wy * c.wy + c.wz * c.wz);
    return c_scale(x, exp(-k2 * T(s.param)) * sc);
  } else if constexpr (K == SYM_HELMHOLTZ) {
    int wx = fold_wave(p, s.n0);
    T d = T(s.param) + T(wx * wx + c.wy * c.wy + c.wz * c.wz);
    return c_scale(x, d == T(0) ? T(0) : sc / d);
  } else if constexpr (K == SYM_POISSON_FD) {
    const int wx = fold_wave_nofilter(p, s.n0);
    if (wx == 0 && c.wy_nf == 0 && c.wz_nf == 0) return c_make<V>(T(0), T(0));
    const T* tab = static_cast<const T*>(s.fd_tab);
    const T d = __ldg(tab + abs(wx)) + __ldg(tab + s.fd_y + abs(c.wy_nf)) + __ldg(tab + s.fd_z + abs(c.wz_nf));
    return c_scale(x, sc / d);
  } else if constexpr (K == SYM_POISSON_SPEC) {
    const int wx = fold_wave_nofilter(p, s.n0);
    const int k2 = wx * wx + c.wy_nf * c.wy_nf + c.wz_nf * c.wz_nf;
    if (k2 == 0) return c_make<V>(T(0), T(0));
    return c_scale(x, sc / (T(-39.4784176043574344753379639995) * T(k2)));   // -4 pi^2 k^2
  } else {
    return x;
  }
}

template <typename T, int K> struct SymFn {
  const SymArgs& s;
  template <typename V>
  __device__ __forceinline__ V operator()(const SymCol& c, int p, V x) const {
    return sym_apply_k<T, K>(s, c, p, x);
  }
};

// call f(SymFn<T, kind>) once, with the launch's (uniform) symbol kind
template <typename T, class F>
__device__ __forceinline__ void with_symbol(const SymArgs& s, F&& f) {
  switch (s.kind) {
    case SYM_LAPLACE: f(SymFn<T, SYM_LAPLACE>{s}); break;
    case SYM_BIHARM: f(SymFn<T, SYM_BIHARM>{s}); break;
    case SYM_INVLAP: f(SymFn<T, SYM_INVLAP>{s}); break;
    case SYM_INVBIHARM: f(SymFn<T, SYM_INVBIHARM>{s}); break;
    case SYM_GRADX: f(SymFn<T, SYM_GRADX>{s}); break;
    case SYM_GRADY: f(SymFn<T, SYM_GRADY>{s}); break;
    case SYM_GRADZ: f(SymFn<T, SYM_GRADZ>{s}); break;
    case SYM_DERIV1: f(SymFn<T, SYM_DERIV1>{s}); break;
    case SYM_DERIV2: f(SymFn<T, SYM_DERIV2>{s}); break;
    case SYM_HEAT: f(SymFn<T, SYM_HEAT>{s}); break;
    case SYM_HELMHOLTZ: f(SymFn<T, SYM_HELMHOLTZ>{s}); break;
    case SYM_POISSON_FD: f(SymFn<T, SYM_POISSON_FD>{s}); break;
    case SYM_POISSON_SPEC: f(SymFn<T, SYM_POISSON_SPEC>{s}); break;
    default: f(SymFn<T, SYM_NONE>{s}); break;
  }
}

// ------------------------------------------------------------ tile shapes
// EF forces the first radix, TCF / TLF the columns / lines per CTA (tuning
// sweeps); 0 selects the defaults
template <typename T, int L, int EF = 0, int TCF = 0> struct StridedShape {
  static constexpr int P = LineFFT<T, L, EF>::P;
  static constexpr int tmin = sizeof(T) == 4 ? 16 : 8;      // 128-byte row segments
  static constexpr int want = (sizeof(T) == 4 ? 256 : 128) / P;
  static constexpr int TC = TCF ? TCF : (want > tmin ? (want > 64 ? 64 : want) : tmin);
  static constexpr int threads = P * TC;
  static constexpr size_t smem = size_t(L) * TC * sizeof(typename CT<T>::V);
};

template <typename T, int L, int EF = 0, int TLF = 0> struct ContigShape {
  static constexpr int E = LineFFT<T, L, EF>::E;
  static constexpr int P = LineFFT<T, L, EF>::P;
  static constexpr int want = (sizeof(T) == 4 ? 256 : 128) / P;
  static constexpr int TL = TLF ? TLF : (want > 1 ? want : 1);
  static constexpr int threads = P * TL;
  // Line-major shared memory.  Stage 0 writes position j*E + r (stride E
  // across threads), so one pad slot after every PW = max(E, bank row)
  // entries spreads those writes over all banks; consecutive positions stay
  // consecutive.
  static constexpr int slots = sizeof(T) == 4 ? 16 : 8;    // complex slots per 128-byte bank row
  static constexpr int PW = E > slots ? E : slots;
  __host__ __device__ static constexpr int pad(int p) { return p + p / PW; }
  // line pitch: room for L+1 entries (r2c spectra) after padding, rounded to a
  // bank row, plus a shift of P slots when several lines share a warp
  static constexpr int LP = ((pad(L) + 1 + slots - 1) / slots) * slots + (P < slots ? P : 0);
  static constexpr size_t smem = size_t(LP) * TL * sizeof(typename CT<T>::V);
};

// ------------------------------------------------------------------ kernels
// float tiles of 512-point (and longer) lines with up to 256 threads are
// compiled for two CTAs per SM: the 128-register budget this fixes measured
// faster than the compiler's own choice there (one CTA's loads in flight
// while the other computes).  Shorter lines keep the compiler's choice, which
// leaves room for more CTAs; larger or double tiles would spill.
// Double-float tiles with E <= 8 aim at 64 registers a thread (two 512-thread
// CTAs per SM for 512-point lines: measured 1.34 ms against 1.72 ms for the
// compiler's 92 registers and one CTA).
template <typename T, int L, int EF, int TCF>
constexpr int strided_min_blocks() {
  return std::is_same<T, df>::value
             ? ((LineFFT<T, L, EF>::E <= 8 && StridedShape<T, L, EF, TCF>::threads >= 64)
                    ? 1024 / StridedShape<T, L, EF, TCF>::threads
                    : 1)
             : ((sizeof(T) == 4 && L >= 512 && StridedShape<T, L, EF, TCF>::threads <= 256) ? 2 : 1);
}
// One column tile of the strided pass (the body of k_strided; also run by the
// persistent z+y kernels).  CG loads the input through L2 only.
template <typename T, int L, int MODE, int EF = 0, int TCF = 0, bool CG = false>
__device__ __forceinline__ void strided_tile(const StridedArgs& a, long long tile) {
  typedef LineFFT<T, L, EF> LN;
  typedef typename CT<T>::V V;
  typedef typename Mem<T>::C MC;   // array element (IEEE double for double-float)
  constexpr int TC = StridedShape<T, L, EF, TCF>::TC;
  const int sh = pass_shift<T>(a.dfx);
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  const int c = threadIdx.x % TC;
  const int t = threadIdx.x / TC;
  const long long g = tile * TC + c;
  const bool valid = g < a.ncols;
  const long long gs = valid ? g : 0;          // idle lanes read column 0, store nothing
  long long slab = gs / a.cps;
  long long cc = gs - slab * a.cps;
  const MC* in = static_cast<const MC*>(a.in) + slab * a.in_slab + cc;
  MC* out = static_cast<MC*>(a.out) + slab * a.out_slab + cc;
  long long il = a.in_line, ol = a.out_line;
  if (a.ncols_main > 0 && gs >= a.ncols_main) {   // a Nyquist column of the split layout
    const long long j = gs - a.ncols_main;
    in = static_cast<const MC*>(a.in_nyq) + j * a.nyq_slab;
    out = static_cast<MC*>(a.out_nyq) + j * a.nyq_slab;
    il = ol = a.nyq_line;
    slab = j;
    cc = -1;
  }
  const V* tw = static_cast<const V*>(a.tw);
  auto xw = [&](int p, V x) { sm[p * TC + c] = x; };
  auto xr = [&](int p) { return sm[p * TC + c]; };
  if constexpr (MODE == 0) {
    const T sg = a.inverse ? T(-1) : T(1);
    auto ld = [&](int p) {
      V x;
      if constexpr (CG) x = to_reg<T>(sh, __ldcg(in + p * il));
      else x = to_reg<T>(sh, in[p * il]);
      x.y *= sg;
      return x;
    };
    auto st = [&](int p, V x) { x.y *= sg; if (valid) out[p * ol] = to_mem<T>(sh, x); };
    LN::template run<false, false>(t, tw, ld, st, xw, xr);
  } else if constexpr (MODE == 2) {
    // real transform along the line of column pairs (2cc, 2cc+1) packed as
    // u = a + i*b: A[k] = (U[k] + conj U[L-k])/2, B[k] = (U[k] - conj U[L-k])/(2i),
    // written to the half spectrum at complex columns 2cc and 2cc+1
    MC* o2 = static_cast<MC*>(a.out) + slab * a.out_slab + 2 * cc;
    auto ld = [&](int p) { return to_reg<T>(sh, in[p * il]); };
    LN::template run<true, false>(t, tw, ld, xw, xw, xr);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < LN::E; ++r) {
      const int k = t + r * LN::P;
      if (2 * k <= L) {
        V uk = xr(k), um = xr(k == 0 ? 0 : L - k);
        V A = c_make<V>(T(0.5) * (uk.x + um.x), T(0.5) * (uk.y - um.y));
        V B = c_make<V>(T(0.5) * (uk.y + um.y), T(-0.5) * (uk.x - um.x));
        if (valid) {
          o2[k * ol] = to_mem<T>(sh, A);
          o2[k * ol + 1] = to_mem<T>(sh, B);
        }
      }
    }
  } else if constexpr (MODE == 3) {
    // inverse of MODE 2: U[k] = A[k] + i B[k], U[L-k] = conj A[k] + i conj B[k]
    // (imaginary parts of A, B at k = 0 and k = L/2 dropped), inverse complex
    // FFT, the real pair (a, b) stored at columns (2cc, 2cc+1)
    const MC* i2 = static_cast<const MC*>(a.in) + slab * a.in_slab + 2 * cc;
#pragma unroll
    for (int r = 0; r < LN::E; ++r) {
      const int k = t + r * LN::P;
      if (2 * k <= L) {
        V A = to_reg<T>(sh, i2[k * il]), B = to_reg<T>(sh, i2[k * il + 1]);
        if (k == 0 || 2 * k == L) { A.y = T(0); B.y = T(0); }
        // conjugated for the forward-engine inverse
        xw(k, c_make<V>(A.x - B.y, -(A.y + B.x)));
        if (k != 0 && 2 * k != L) xw(L - k, c_make<V>(A.x + B.y, A.y - B.x));
      }
    }
    __syncthreads();
    auto st = [&](int p, V x) { x.y = -x.y; if (valid) out[p * ol] = to_mem<T>(sh, x); };
    LN::template run<false, true>(t, tw, xr, st, xw, xr);
  } else {
    // the symbol sees the column as (y, kz); Nyquist column j of the split
    // layout is (j, N2/2)
    const SymCol scol = cc >= 0 ? sym_column(a.sym, gs) : sym_column_nyq(a.sym, slab);
    auto ld = [&](int p) { return to_reg<T>(sh, in[p * il]); };
    // forward transform; the symbol is applied in registers and the result
    // conjugated for the inverse run, which starts from the same registers
    // (LineFFT::to_load_order) instead of a shared-memory round trip
    V v[LN::E];
    LN::compute(t, tw, ld, xw, xr, [] {}, v);
    with_symbol<T>(a.sym, [&](auto sf) { LN::for_outputs(t, v, [&](int p, V& x) { x = c_conj(sf(scol, p, x)); }); });
    LN::to_load_order(v);
    // the inverse's first exchange waits until every thread has read the
    // forward's last one
    LN::stages(t, tw, xw, xr, [] { __syncthreads(); }, v);
    if constexpr (MODE == 1) {
      LN::emit(t, v, [&](int p, V x) {
        x.y = -x.y;
        if (valid) out[p * ol] = to_mem<T>(sh, x);
      });
    } else {
      // the accumulate input has the output's layout (main columns only);
      // the result is staged in shared memory so that all of this thread's
      // accumulate loads are in flight together
      const MC* acc = static_cast<const MC*>(a.acc) + (out - static_cast<MC*>(a.out));
      if constexpr (LN::NS >= 2) __syncthreads();   // last exchange read before the staging writes
      LN::emit(t, v, [&](int p, V x) { sm[p * TC + c] = c_conj(x); });
      __syncthreads();
      constexpr int CH = LN::E < 8 ? LN::E : 8;   // loads in flight per chunk (last chunk may be partial)
#pragma unroll
      for (int r0 = 0; r0 < LN::E; r0 += CH) {
        V av[CH];
#pragma unroll
        for (int j = 0; j < CH; ++j)
          if (r0 + j < LN::E) av[j] = to_reg<T>(sh, acc[(t + (r0 + j) * LN::P) * ol]);
#pragma unroll
        for (int j = 0; j < CH; ++j)
          if (valid && r0 + j < LN::E)
            out[(t + (r0 + j) * LN::P) * ol] = to_mem<T>(sh, c_add(sm[(t + (r0 + j) * LN::P) * TC + c], av[j]));
      }
    }
  }
}

// Programmatic dependent launch.  Every pass kernel opens a PassScope before
// its first global-memory access: griddepcontrol.wait returns once the grid
// ahead of it in the stream has finished and its writes are visible (at once
// when the kernel was launched without the programmatic-serialisation
// attribute).  launch_dependents releases the next pass's launch; it takes
// effect when every CTA of this grid has executed it or exited.  At the end
// of the CTA (the default) that hides only the next launch's latency; at CTA
// start (early) the next pass's CTAs are placed on the SMs this grid's last
// wave leaves idle and wait there.  Either way the next pass is launched only
// after every CTA of this grid is resident, so its waiting CTAs never take a
// slot one of ours still needs, and it reads nothing before the wait.
struct PassScope {
  __device__ __forceinline__ explicit PassScope(int early) {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (early) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  }
  __device__ __forceinline__ ~PassScope() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
};

template <typename T, int L, int MODE, int EF = 0, int TCF = 0>
__global__ void __launch_bounds__(StridedShape<T, L, EF, TCF>::threads, (strided_min_blocks<T, L, EF, TCF>()))
k_strided(const StridedArgs a) {
  PassScope scope(a.early_trigger);
  strided_tile<T, L, MODE, EF, TCF>(a, blockIdx.x);
}

// Contiguous-line kernels share this prologue: thread t of line li of the
// CTA, the line's padded shared-memory row and the validity of the line.
#define AFG_CONTIG_PROLOGUE(L_)                                                \
  typedef LineFFT<T, L_, EF> LN;                                               \
  typedef ContigShape<T, L_, EF, TLF> SH;                                      \
  typedef typename CT<T>::V V;                                                 \
  typedef typename Mem<T>::C MC;                                               \
  typedef typename Mem<T>::R MR;                                               \
  const int sh = pass_shift<T>(a.dfx);                                         \
  constexpr int P = LN::P, TL = SH::TL;                                        \
  extern __shared__ __align__(16) unsigned char smraw[];                       \
  V* sm = reinterpret_cast<V*>(smraw);                                         \
  const int t = threadIdx.x % P, li = threadIdx.x / P;                         \
  const long long line = tile * TL + li;                                       \
  const bool valid = line < a.nlines;                                          \
  const long long ls = valid ? line : 0;                                       \
  V* sl = sm + li * SH::LP;                                                    \
  auto xw = [&](int p, V x) { sl[SH::pad(p)] = x; };                          \
  auto xr = [&](int p) { return sl[SH::pad(p)]; };

template <typename T, int L, int EF = 0, int TLF = 0>
__global__ void __launch_bounds__(ContigShape<T, L, EF, TLF>::threads)
k_zc2c(const ContigArgs a) {
  PassScope scope(a.early_trigger);
  const long long tile = blockIdx.x;
  AFG_CONTIG_PROLOGUE(L)
  const MC* in = static_cast<const MC*>(a.in) + ls * a.in_dist;
  MC* out = static_cast<MC*>(a.out) + ls * a.out_dist;
  const T sg = a.inverse ? T(-1) : T(1);
  auto ld = [&](int p) { V x = to_reg<T>(sh, in[p]); x.y *= sg; return x; };
  auto st = [&](int p, V x) { x.y *= sg; if (valid) out[p] = to_mem<T>(sh, x); };
  LN::template run<false, false>(t, static_cast<const V*>(a.tw), ld, st, xw, xr);
}

// X[k] from the packed half-length spectrum: zk = Z[k mod M], zm = Z[(M-k) mod M], w = w_{2M}^k
template <typename V>
__device__ __forceinline__ V r2c_split(V zk, V zm, V w) {
  typedef decltype(V().x) T;
  V e = c_make<V>(T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y));
  V o = c_make<V>(T(0.5) * (zk.y + zm.y), T(-0.5) * (zk.x - zm.x));
  return c_add(e, c_mul(w, o));
}
// Z[k] of the packed inverse from X[k], X[M-k] and wc = conj(w_{2M}^k)
template <typename V>
__device__ __forceinline__ V c2r_merge(V xk, V xm, V wc) {
  V s = c_make<V>(xk.x + xm.x, xk.y - xm.y);
  V d = c_make<V>(xk.x - xm.x, xk.y + xm.y);
  V wd = c_mul(wc, d);
  return c_make<V>(s.x - wd.y, s.y + wd.x);
}

// Mirror pairs of the packed pass order.  Pair q of the z lines of an
// [n0][n1] grid: for q < xc*n1 (xc = (n0-1)/2) line (x, y) = (1 + q/n1, q%n1)
// with its mirror (n0-x, (n1-y)%n1) in another x-slab; the rest pair lines
// within slab 0 and, for even n0, slab n0/2: (x, y) with (x, (n1-y)%n1) for
// y = 0..n1/2 (y = 0, and y = n1/2 for even n1, are their own mirror).
// Pairs in all: xc*n1 + (1 + (n0 even)) * (n1/2 + 1).
__device__ __forceinline__ void pair_lines(long long q, int n0, int n1, long long& i, long long& j) {
  const long long xc = (n0 - 1) / 2;
  long long x, y, xm;
  if (q < xc * n1) {
    x = 1 + q / n1;
    y = q % n1;
    xm = n0 - x;
  } else {
    const long long r = q - xc * n1, per = n1 / 2 + 1;
    x = (r / per) * (n0 / 2);
    y = r % per;
    xm = x;
  }
  i = x * n1 + y;
  j = xm * n1 + (n1 - y) % n1;
}

// Line of a contiguous-pass slot: the plain mapping (slot li of tile ->
// line tile*TL + li) or, in pair mode, the slots (2m, 2m+1) of a CTA hold
// pair tile*(TL/2) + m, first line and mirror (an odd TL leaves its last
// slot idle).  wr: this slot stores (a self-mirror pair stores once).
template <int TL>
struct ContigSlot {
  long long row;
  bool valid, wr;
  int partner;   // slot holding the mirror line (the slot itself in plain mode)
  __device__ __forceinline__ ContigSlot(const ContigArgs& a, long long tile, int li) {
    if (a.pair_n1 > 0) {
      constexpr int PP = TL / 2;
      const long long q = tile * PP + (li >> 1);
      valid = li < 2 * PP && q < a.nlines / 2;
      long long i = 0, j = 0;
      pair_lines(valid ? q : 0, a.pair_n0, a.pair_n1, i, j);
      row = (li & 1) ? j : i;
      wr = valid && !((li & 1) && i == j);
      // the idle last slot of an odd TL has no partner slot in the CTA
      partner = li < 2 * PP ? (li ^ 1) : li;
    } else {
      const long long line = tile * TL + li;
      valid = wr = line < a.nlines;
      row = valid ? line : 0;
      partner = li;
    }
  }
};

template <typename T, int M, int EF = 0, int TLF = 0>
__device__ __forceinline__ void zr2c_tile(const ContigArgs& a, long long tile) {
  AFG_CONTIG_PROLOGUE(M)
  const ContigSlot<TL> slot(a, tile, li);
  const V* sp = sm + slot.partner * SH::LP;   // the mirror line's spectrum (pair mode), else this line's
  const MC* in = reinterpret_cast<const MC*>(static_cast<const MR*>(a.in) + slot.row * a.in_dist);
  MC* out = static_cast<MC*>(a.out) + slot.row * a.out_dist;
  auto ld = [&](int p) { return to_reg<T>(sh, in[p]); };
  const V* twp = static_cast<const V*>(a.tw_post);
  const T wint = a.weight == 2 ? T(2) : T(1);
  if constexpr (std::is_same<T, float>::value && LN::E <= 16 && P <= 16 && 32 % (2 * P) == 0 && TL % 2 == 0) {
    if (a.pair_n1 > 0) {
      // Mirror pairs whose two lines share a warp: after the transform
      // (registers back in stage-0 order, LineFFT::to_load_order) thread t
      // holds Z[t + r*P], and Z[M-k] of the mirror line is the mirror
      // thread's entry r' = E-1-r (t != 0) or (E-r) mod E (t = 0), taken by
      // warp shuffle as in zc2r_tile; the split needs no shared-memory round
      // trip.  The same split arithmetic as the staged path below.
      constexpr int E = LN::E;
      V v[E];
      LN::compute(t, static_cast<const V*>(a.tw), ld, xw, xr, [] {}, v);
      LN::to_load_order(v);
      const int lane = threadIdx.x & 31;
      const int src = ((lane ^ P) & ~(P - 1)) | ((P - t) & (P - 1));
      V zp0 = v[0];
#pragma unroll
      for (int r = 0; r < E; ++r) {
        const V y = t == 0 ? v[(E - r) % E] : v[E - 1 - r];
        const V zm = c_make<V>(__shfl_sync(0xffffffffu, y.x, src), __shfl_sync(0xffffffffu, y.y, src));
        if (r == 0) zp0 = zm;   // Z[0] of the mirror line on thread 0
        const int k = t + r * P;
        V x = r2c_split(v[r], zm, ld_tw(twp + k));
        if (k != 0) x = c_scale(x, wint);
        if (slot.wr) out[k] = to_mem<T>(sh, x);
      }
      if (t == 0 && slot.wr) {
        const V z0 = v[0], zp = zp0;
        const V xn = c_make<V>(T(0.5) * ((z0.x + zp.x) - (z0.y + zp.y)), T(0.5) * ((z0.y - zp.y) + (z0.x - zp.x)));
        if (a.nyq_out) static_cast<MC*>(a.nyq_out)[slot.row] = to_mem<T>(sh, xn);
        else out[M] = to_mem<T>(sh, xn);
      }
      return;
    }
  }
  LN::template run<true, false>(t, static_cast<const V*>(a.tw), ld, xw, xw, xr);
  __syncthreads();
  // outputs k = t + r*P (r < E) cover 0..M-1; thread 0 also writes k = M
#pragma unroll
  for (int r = 0; r < LN::E; ++r) {
    const int k = t + r * P;
    V x = r2c_split(xr(k), sp[SH::pad(k == 0 ? 0 : M - k)], ld_tw(twp + k));
    if (k != 0) x = c_scale(x, wint);
    if (slot.wr) out[k] = to_mem<T>(sh, x);
  }
  if (t == 0) {
    // X[M] = r2c_split(Z[0], Zmirror[0], -1)
    const V z0 = xr(0), zp = sp[SH::pad(0)];
    const V xn = a.pair_n1 > 0
                     ? c_make<V>(T(0.5) * ((z0.x + zp.x) - (z0.y + zp.y)), T(0.5) * ((z0.y - zp.y) + (z0.x - zp.x)))
                     : c_make<V>(z0.x - z0.y, T(0));
    if (slot.wr) {
      if (a.nyq_out) static_cast<MC*>(a.nyq_out)[slot.row] = to_mem<T>(sh, xn);
      else out[M] = to_mem<T>(sh, xn);
    }
  }
}

template <typename T, int M, int EF = 0, int TLF = 0>
__global__ void __launch_bounds__(ContigShape<T, M, EF, TLF>::threads)
k_zr2c(const ContigArgs a) {
  PassScope scope(a.early_trigger);
  zr2c_tile<T, M, EF, TLF>(a, blockIdx.x);
}

// the body of k_zc2r for one tile of TL lines
template <typename T, int M, int EF = 0, int TLF = 0, bool CG = false>
__device__ __forceinline__ void zc2r_tile(const ContigArgs& a, long long tile) {
  AFG_CONTIG_PROLOGUE(M)
  const ContigSlot<TL> slot(a, tile, li);
  const long long ls2 = slot.row;
  const V* sp = sm + slot.partner * SH::LP;   // the mirror line's entries (pair mode), else this line's
  const MC* in = static_cast<const MC*>(a.in) + ls2 * a.in_dist;
  MC* out = reinterpret_cast<MC*>(static_cast<MR*>(a.out) + ls2 * a.out_dist);
  const V* twp = static_cast<const V*>(a.tw_post);
  const T wint = a.weight == 1 ? T(0.5) : T(1);
  auto st = [&](int p, V x) { x.y = -x.y; if (slot.wr) out[p] = to_mem<T>(sh, x); };
  if constexpr (!CG && std::is_same<T, float>::value && LN::E <= 16 && P <= 16 && 32 % (2 * P) == 0 && TL % 2 == 0) {
    if (a.pair_n1 > 0) {
      // Mirror pairs whose two lines share a warp (slot 2m on the lanes below
      // slot 2m+1's).  X[M-p] of the mirror line, p = t + r*P, is the stage-0
      // entry r' = E-1-r of the mirror line's thread t' = P-t (t != 0), or
      // entry (E-r) mod E of its thread 0 (t = 0; r = 0 gives its X[0]), so
      // each thread loads only its own entries and takes the mirror line's
      // from a warp shuffle instead of staging both lines in shared memory.
      // The same merge arithmetic as the staged path below.
      constexpr int E = LN::E;
      V x[E];
#pragma unroll
      for (int r = 0; r < E; ++r) x[r] = to_reg<T>(sh, in[t + r * P]);
      const V xn = to_reg<T>(sh, in[M]);   // X[M] of this line (one address per line)
      const int lane = threadIdx.x & 31;
      const int src = ((lane ^ P) & ~(P - 1)) | ((P - t) & (P - 1));
      auto shfl = [&](V y) { return c_make<V>(__shfl_sync(0xffffffffu, y.x, src), __shfl_sync(0xffffffffu, y.y, src)); };
      const V pn = shfl(xn);               // X[M] of the mirror line
      V v[E];
#pragma unroll
      for (int r = 0; r < E; ++r) {
        const V xm = shfl(t == 0 ? x[(E - r) % E] : x[E - 1 - r]);
        V xk = x[r], xq = xm;
        if (r == 0 && t == 0) {
          xk = c_make<V>(T(0.5) * (xk.x + xm.x), T(0.5) * (xk.y - xm.y));
          xq = c_make<V>(T(0.5) * (xn.x + pn.x), T(0.5) * (pn.y - xn.y));
        } else {
          xk = c_scale(xk, wint);
          xq = c_scale(xq, wint);
        }
        v[r] = c_conj(c2r_merge(xk, xq, c_conj(ld_tw(twp + t + r * P))));
      }
      LN::stages(t, static_cast<const V*>(a.tw), xw, xr, [] {}, v);
      LN::emit(t, v, st);
      return;
    }
  }
  {
    // stage the M+1 input entries: E independent loads per thread, then the
    // Nyquist entry by thread 0
    V v[LN::E];
    V nyq;
    if constexpr (CG) {
#pragma unroll
      for (int r = 0; r < LN::E; ++r) v[r] = to_reg<T>(sh, __ldcg(in + t + r * P));
      nyq = to_reg<T>(sh, __ldcg(in + (t == 0 ? M : 0)));
    } else {
#pragma unroll
      for (int r = 0; r < LN::E; ++r) v[r] = to_reg<T>(sh, in[t + r * P]);
      nyq = to_reg<T>(sh, a.nyq_in ? static_cast<const MC*>(a.nyq_in)[ls2] : in[t == 0 ? M : 0]);
    }
#pragma unroll
    for (int r = 0; r < LN::E; ++r) xw(t + r * P, v[r]);
    if (t == 0) xw(M, nyq);
  }
  __syncthreads();
  // X[k] of this line with X[M-k] of the mirror line (this line in plain
  // mode).  k = 0 and k = M enter as the Hermitian parts over the pair,
  // H[k] = (X[k] + conj Xmirror[k]) / 2 (the merge takes conj H[M] as its
  // second argument): the real part of a line that is its own mirror, which
  // is what the reference's c2r reads there (x and y inverse passes first,
  // then the imaginary parts of kz = 0 and N2/2 dropped).
  auto ld = [&](int p) {
    V xk = xr(p), xm = sp[SH::pad(M - p)];
    if (p == 0) {
      const V xp = sp[SH::pad(0)], xn = xr(M);
      xk = c_make<V>(T(0.5) * (xk.x + xp.x), T(0.5) * (xk.y - xp.y));
      xm = c_make<V>(T(0.5) * (xn.x + xm.x), T(0.5) * (xm.y - xn.y));
    } else {
      xk = c_scale(xk, wint);
      xm = c_scale(xm, wint);
    }
    return c_conj(c2r_merge(xk, xm, c_conj(ld_tw(twp + p))));
  };
  LN::template run<false, true>(t, static_cast<const V*>(a.tw), ld, st, xw, xr);
}

template <typename T, int M, int EF = 0, int TLF = 0>
__global__ void __launch_bounds__(ContigShape<T, M, EF, TLF>::threads)
k_zc2r(const ContigArgs a) {
  PassScope scope(a.early_trigger);
  zc2r_tile<T, M, EF, TLF>(a, blockIdx.x);
}

// ------------------------------------------------------- grouped launches
// One persistent grid over the tiles of several independent tasks of one
// line length (the same pass of many transforms of a batch): task k owns the
// tiles [starts[k], starts[k+1]) of the `total` tiles and reads its
// arguments from tab[k] in global memory; CTA b runs tiles b, b + gridDim.x,
// ... (a work list walked in order, at most as many CTAs as fit the GPU at
// once).  The tile bodies are the single-task kernels'.
__device__ __forceinline__ int group_task(const long long* __restrict__ starts, int ntasks, long long b) {
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(starts + mid) <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <typename T, int L, int MODE>
__global__ void __launch_bounds__(StridedShape<T, L>::threads, (strided_min_blocks<T, L, 0, 0>()))
k_strided_grouped(const StridedArgs* __restrict__ tab, const long long* __restrict__ starts, int ntasks, long long total,
                  int early) {
  PassScope scope(early);
  for (long long b = blockIdx.x; b < total; b += gridDim.x) {
    if (b != blockIdx.x) __syncthreads();   // the last tile's shared-memory reads are done
    const int k = group_task(starts, ntasks, b);
    strided_tile<T, L, MODE>(tab[k], b - __ldg(starts + k));
  }
}

template <typename T, int M>
__global__ void __launch_bounds__(ContigShape<T, M>::threads)
k_zr2c_grouped(const ContigArgs* __restrict__ tab, const long long* __restrict__ starts, int ntasks, long long total,
               int early) {
  PassScope scope(early);
  for (long long b = blockIdx.x; b < total; b += gridDim.x) {
    if (b != blockIdx.x) __syncthreads();   // the last tile's shared-memory reads are done
    const int k = group_task(starts, ntasks, b);
    zr2c_tile<T, M>(tab[k], b - __ldg(starts + k));
  }
}

template <typename T, int M, int TLF = 0>
__global__ void __launch_bounds__(ContigShape<T, M, 0, TLF>::threads)
k_zc2r_grouped(const ContigArgs* __restrict__ tab, const long long* __restrict__ starts, int ntasks, long long total,
               int early) {
  PassScope scope(early);
  for (long long b = blockIdx.x; b < total; b += gridDim.x) {
    if (b != blockIdx.x) __syncthreads();   // the last tile's shared-memory reads are done
    const int k = group_task(starts, ntasks, b);
    zc2r_tile<T, M, 0, TLF>(tab[k], b - __ldg(starts + k));
  }
}

// real line r2c -> i k / N -> c2r, one pass (z-direction derivative: the
// kernel applies SYM_DERIV1 whatever a.sym.kind says); ACC adds the
// accumulate input a.acc
template <typename T, int M, int EF = 0, int TLF = 0, bool ACC = false>
__global__ void __launch_bounds__(ContigShape<T, M, EF, TLF>::threads)
k_zsym(const ContigArgs a) {
  PassScope scope(a.early_trigger);
  const long long tile = blockIdx.x;
  AFG_CONTIG_PROLOGUE(M)
  const MC* in = reinterpret_cast<const MC*>(static_cast<const MR*>(a.in) + ls * a.in_dist);
  MC* out = reinterpret_cast<MC*>(static_cast<MR*>(a.out) + ls * a.out_dist);
  const MC* acc = ACC ? reinterpret_cast<const MC*>(static_cast<const MR*>(a.acc) + ls * a.out_dist) : nullptr;
  const V* tw = static_cast<const V*>(a.tw);
  auto ld = [&](int p) { return to_reg<T>(sh, in[p]); };
  LN::template run<true, false>(t, tw, ld, xw, xw, xr);
  __syncthreads();
  const V* twp = static_cast<const V*>(a.tw_post);
  const SymCol none{0, 0, 0, 0};
#pragma unroll
  for (int r = 0; r <= LN::E / 2; ++r) {
    const int k = t + r * P;
    if (2 * k > M) continue;
    if (k == 0) {
      V z0 = xr(0);
      V x0 = sym_apply_k<T, SYM_DERIV1>(a.sym, none, 0, c_make<V>(z0.x + z0.y, T(0)));
      V xn = sym_apply_k<T, SYM_DERIV1>(a.sym, none, M, c_make<V>(z0.x - z0.y, T(0)));
      // imaginary parts of DC and Nyquist are dropped by the real inverse
      xw(0, c_make<V>(x0.x + xn.x, -(x0.x - xn.x)));   // conj(Z'[0])
    } else {
      V zk = xr(k), zm = xr(M - k);
      V wk = ld_tw(twp + k), wm = ld_tw(twp + (M - k));
      V xk = sym_apply_k<T, SYM_DERIV1>(a.sym, none, k, r2c_split(zk, zm, wk));
      if (2 * k == M) {
        xw(k, c_conj(c2r_merge(xk, xk, c_conj(wk))));
      } else {
        V xm = sym_apply_k<T, SYM_DERIV1>(a.sym, none, M - k, r2c_split(zm, zk, wm));
        xw(k, c_conj(c2r_merge(xk, xm, c_conj(wk))));
        xw(M - k, c_conj(c2r_merge(xm, xk, c_conj(wm))));
      }
    }
  }
  __syncthreads();
  if constexpr (!ACC) {
    auto gst = [&](int p, V x) {
      x.y = -x.y;
      if (valid) out[p] = to_mem<T>(sh, x);
    };
    LN::template run<false, true>(t, tw, xr, gst, xw, xr);
    return;
  }
  // accumulate: stage the result in shared memory, then read all of this
  // thread's accumulate entries at once (one memory latency, not one per
  // element) and store result + accumulate
  auto sst = [&](int p, V x) { xw(p, c_conj(x)); };
  LN::template run<true, true>(t, tw, xr, sst, xw, xr);
  __syncthreads();
  constexpr int CH = LN::E < 8 ? LN::E : 8;   // loads in flight per chunk (last chunk may be partial)
#pragma unroll
  for (int r0 = 0; r0 < LN::E; r0 += CH) {
    V av[CH];
#pragma unroll
    for (int j = 0; j < CH; ++j)
      if (r0 + j < LN::E) av[j] = to_reg<T>(sh, acc[t + (r0 + j) * P]);
#pragma unroll
    for (int j = 0; j < CH; ++j)
      if (valid && r0 + j < LN::E) out[t + (r0 + j) * P] = to_mem<T>(sh, c_add(xr(t + (r0 + j) * P), av[j]));
  }
}

#undef AFG_CONTIG_PROLOGUE

}  // namespace afg
