// Tensor-core forms of the three r2c/c2r pass kernels (float): the strided
// y/x pass, the z r2c pass and the z c2r pass, with every radix-16 stage on
// the tensor cores (tc_engine.cuh).  They mirror k_strided<MODE 0>, k_zr2c
// and k_zc2r of passes.cuh; plans made with ACCFFT_C_TC_TF32 or
// ACCFFT_C_TC_BF16 run them for full r2c/c2r transforms.
#include <cuda_bf16.h>

#include "launch.h"
#include "passes.cuh"
#include "per_device.h"
#include "tc_engine.cuh"

namespace afg {

// Shared memory of a tensor-core CTA: the exchange buffer of the line engine
// plus the engine's B operands; at least tc_smem_floor() so that no more CTAs
// share an SM than its 512 tensor-memory columns hold (each 128-row block
// takes 128 columns: four 128-thread CTAs, two 256-thread CTAs, one
// 512-thread CTA; 228 KB of shared memory per SM)
template <int THREADS>
constexpr size_t tc_smem_floor() {
  return THREADS <= 128 ? size_t(52) * 1024 : THREADS <= 256 ? size_t(80) * 1024 : size_t(120) * 1024;
}

// CTAs per SM the register budget aims at (as many as tensor memory holds)
template <int THREADS>
constexpr int tc_min_blocks() {
  return THREADS <= 128 ? 4 : THREADS <= 256 ? 2 : 1;
}

// Two CTA widths W: 256 threads (two CTAs per SM, each issuing the products
// of two 128-row blocks at once) and 128 threads (four CTAs per SM, one block
// each: twice the independent round trips per SM to hide the latency of a
// stage's store - product - load).  Lines of 1024 keep 512 threads.
// strided tiles: TC columns x L
template <int L, TcForm F, int W = 256> struct TcStridedShape {
  static constexpr int P = L / 16;
  static constexpr int TC = L >= 1024 ? 8 : W == 256 ? (P >= 32 ? 8 : 16) : W / P;
  static constexpr int threads = P * TC;
  static_assert(threads % 128 == 0, "tensor-core CTAs hold whole 128-row blocks");
  static constexpr size_t exch = size_t(L) * TC * sizeof(float2);
  static constexpr size_t need = exch + tc_extra_smem<F>(threads);
  static constexpr size_t smem = need > tc_smem_floor<threads>() ? need : tc_smem_floor<threads>();
};

template <int M, TcForm F, int W = 256> struct TcContigShape {
  typedef ContigShape<float, M, 16, W / LineFFT<float, M, 16>::P> CS;
  static constexpr int threads = CS::threads;
  static_assert(threads == W, "one 16-point butterfly per thread per line position");
  static constexpr size_t exch = (CS::smem + 15) / 16 * 16;
  static constexpr size_t need = exch + tc_extra_smem<F>(threads);
  static constexpr size_t smem = need > tc_smem_floor<threads>() ? need : tc_smem_floor<threads>();
};

template <int L, TcForm F, int W>
__global__ void __launch_bounds__(TcStridedShape<L, F, W>::threads, tc_min_blocks<TcStridedShape<L, F, W>::threads>())
k_strided_tc(const StridedArgs a, int* err) {
  typedef TcStridedShape<L, F, W> SH;
  typedef LineFFTTC<L, F, SH::threads> LN;
  typedef float2 V;
  constexpr int TC = SH::TC;
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  TcCtx ctx;
  tc_begin<F, SH::threads>(ctx, smraw + SH::exch, err, a.wait_limit);
  const int c = threadIdx.x % TC;
  const int t = threadIdx.x / TC;
  const long long g = (long long)blockIdx.x * TC + c;
  const bool valid = g < a.ncols;
  const long long gs = valid ? g : 0;          // idle lanes read column 0, store nothing
  const long long slab = gs / a.cps;
  const long long cc = gs - slab * a.cps;
  const V* in = static_cast<const V*>(a.in) + slab * a.in_slab + cc;
  V* out = static_cast<V*>(a.out) + slab * a.out_slab + cc;
  const long long il = a.in_line, ol = a.out_line;
  const float sg = a.inverse ? -1.f : 1.f;
  auto xw = [&](int p, V x) { sm[p * TC + c] = x; };
  auto xr = [&](int p) { return sm[p * TC + c]; };
  auto ld = [&](int p) { V x = in[p * il]; x.y *= sg; return x; };
  V v[16];
  LN::compute(ctx, t, static_cast<const V*>(a.tw), ld, xw, xr, [] {}, v);
  LN::emit(t, v, [&](int p, V x) {
    x.y *= sg;
    if (valid) out[p * ol] = x;
  });
  tc_end<SH::threads>(ctx);
}

template <int M, TcForm F, int W>
__global__ void __launch_bounds__(TcContigShape<M, F, W>::threads, tc_min_blocks<TcContigShape<M, F, W>::threads>())
k_zr2c_tc(const ContigArgs a, int* err) {
  typedef TcContigShape<M, F, W> TS;
  typedef LineFFTTC<M, F, TS::threads> LN;
  typedef typename TS::CS SH;
  typedef float2 V;
  constexpr int P = LN::P, TL = SH::TL;
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  TcCtx ctx;
  tc_begin<F, TS::threads>(ctx, smraw + TS::exch, err, a.wait_limit);
  const int t = threadIdx.x % P, li = threadIdx.x / P;
  const long long line = (long long)blockIdx.x * TL + li;
  const bool valid = line < a.nlines;
  const long long ls = valid ? line : 0;
  V* sl = sm + li * SH::LP;
  auto xw = [&](int p, V x) { sl[SH::pad(p)] = x; };
  auto xr = [&](int p) { return sl[SH::pad(p)]; };
  const V* in = reinterpret_cast<const V*>(static_cast<const float*>(a.in) + ls * a.in_dist);
  V* out = static_cast<V*>(a.out) + ls * a.out_dist;
  V v[16];
  LN::compute(ctx, t, static_cast<const V*>(a.tw), [&](int p) { return in[p]; }, xw, xr, [] {}, v);
  __syncthreads();   // the last stage's exchange reads (or MMA reads) end before the spectrum lands
  LN::emit(t, v, xw);
  __syncthreads();
  const V* twp = static_cast<const V*>(a.tw_post);
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    const int k = t + r * P;
    const V x = r2c_split(xr(k), xr(k == 0 ? 0 : M - k), __ldg(twp + k));
    if (valid) out[k] = x;
  }
  if (t == 0 && valid) {
    const V z0 = xr(0);
    out[M] = make_float2(z0.x - z0.y, 0.f);
  }
  tc_end<TS::threads>(ctx);
}

template <int M, TcForm F, int W>
__global__ void __launch_bounds__(TcContigShape<M, F, W>::threads, tc_min_blocks<TcContigShape<M, F, W>::threads>())
k_zc2r_tc(const ContigArgs a, int* err) {
  typedef TcContigShape<M, F, W> TS;
  typedef LineFFTTC<M, F, TS::threads> LN;
  typedef typename TS::CS SH;
  typedef float2 V;
  constexpr int P = LN::P, TL = SH::TL;
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  TcCtx ctx;
  tc_begin<F, TS::threads>(ctx, smraw + TS::exch, err, a.wait_limit);
  const int t = threadIdx.x % P, li = threadIdx.x / P;
  const long long line = (long long)blockIdx.x * TL + li;
  const bool valid = line < a.nlines;
  const long long ls = valid ? line : 0;
  V* sl = sm + li * SH::LP;
  auto xw = [&](int p, V x) { sl[SH::pad(p)] = x; };
  auto xr = [&](int p) { return sl[SH::pad(p)]; };
  const V* in = static_cast<const V*>(a.in) + ls * a.in_dist;
  V* out = reinterpret_cast<V*>(static_cast<float*>(a.out) + ls * a.out_dist);
  {
    V s[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) s[r] = in[t + r * P];
    const V nyq = in[t == 0 ? M : 0];
#pragma unroll
    for (int r = 0; r < 16; ++r) xw(t + r * P, s[r]);
    if (t == 0) xw(M, nyq);
  }
  __syncthreads();
  const V* twp = static_cast<const V*>(a.tw_post);
  auto ld = [&](int p) {
    V xk = xr(p), xm = xr(M - p);
    if (p == 0) {
      xk.y = 0.f;
      xm.y = 0.f;
    }
    return c_conj(c2r_merge(xk, xm, c_conj(__ldg(twp + p))));
  };
  V v[16];
  LN::compute(ctx, t, static_cast<const V*>(a.tw), ld, xw, xr, [] {}, v);
  LN::emit(t, v, [&](int p, V x) {
    x.y = -x.y;
    if (valid) out[p] = x;
  });
  tc_end<TS::threads>(ctx);
}

// ------------------------------------------------------------------ launches

template <int L, TcForm F, int W>
static bool run_strided_tc(const StridedArgs& a, int* err, cudaStream_t s) {
  typedef TcStridedShape<L, F, W> SH;
  auto k = k_strided_tc<L, F, W>;
  static PerDevice prepared;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  k<<<unsigned((a.ncols + SH::TC - 1) / SH::TC), SH::threads, SH::smem, s>>>(a, err);
  count_launch();
  return true;
}

template <int M, TcForm F, bool R2C, int W>
static bool run_contig_tc(const ContigArgs& a, int* err, cudaStream_t s) {
  typedef TcContigShape<M, F, W> SH;
  auto k = R2C ? k_zr2c_tc<M, F, W> : k_zc2r_tc<M, F, W>;
  static PerDevice prepared;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  k<<<unsigned((a.nlines + SH::CS::TL - 1) / SH::CS::TL), SH::threads, SH::smem, s>>>(a, err);
  count_launch();
  return true;
}

template <int L, int W>
static bool strided_tc_form(int form, const StridedArgs& a, int* err, cudaStream_t s) {
  return (form & 3) == 1 ? run_strided_tc<L, TcForm::TF32x3, W>(a, err, s)
                         : run_strided_tc<L, TcForm::BF16x6, W>(a, err, s);
}
template <int M, int W>
static bool z_tc_form(int form, bool r2c, const ContigArgs& a, int* err, cudaStream_t s) {
  if ((form & 3) == 1)
    return r2c ? run_contig_tc<M, TcForm::TF32x3, true, W>(a, err, s) : run_contig_tc<M, TcForm::TF32x3, false, W>(a, err, s);
  return r2c ? run_contig_tc<M, TcForm::BF16x6, true, W>(a, err, s) : run_contig_tc<M, TcForm::BF16x6, false, W>(a, err, s);
}

bool tc_length_supported(int len, bool contig) {
  return len == 128 || len == 256 || len == 512 || (!contig && len == 1024);
}

// form: 1 3xTF32, 2 split BF16; plus kTcNarrow for 128-thread CTAs
bool launch_strided_tc(int form, int L, const StridedArgs& a, int* err, cudaStream_t s) {
  const bool narrow = (form & kTcNarrow) != 0;
  switch (L) {
    case 128: return narrow ? strided_tc_form<128, 128>(form, a, err, s) : strided_tc_form<128, 256>(form, a, err, s);
    case 256: return narrow ? strided_tc_form<256, 128>(form, a, err, s) : strided_tc_form<256, 256>(form, a, err, s);
    case 512: return narrow ? strided_tc_form<512, 128>(form, a, err, s) : strided_tc_form<512, 256>(form, a, err, s);
    case 1024: return strided_tc_form<1024, 256>(form, a, err, s);
    default: return false;
  }
}

bool launch_z_tc(int form, bool r2c, int M, const ContigArgs& a, int* err, cudaStream_t s) {
  const bool narrow = (form & kTcNarrow) != 0;
  switch (M) {
    case 128: return narrow ? z_tc_form<128, 128>(form, r2c, a, err, s) : z_tc_form<128, 256>(form, r2c, a, err, s);
    case 256: return narrow ? z_tc_form<256, 128>(form, r2c, a, err, s) : z_tc_form<256, 256>(form, r2c, a, err, s);
    case 512: return narrow ? z_tc_form<512, 128>(form, r2c, a, err, s) : z_tc_form<512, 256>(form, r2c, a, err, s);
    default: return false;
  }
}

}  // namespace afg
