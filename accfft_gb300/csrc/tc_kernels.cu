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
// plus the engine's B operands; at least kTcSmemFloor per 256 threads so that
// no more CTAs share an SM than its 512 tensor-memory columns hold (each
// 128-row block takes 128 columns: two 256-thread CTAs, one 512-thread CTA)
template <int THREADS>
constexpr size_t tc_smem_floor() {
  return THREADS <= 256 ? size_t(80) * 1024 : size_t(120) * 1024;
}

// CTAs per SM the register budget aims at (as many as tensor memory holds)
template <int THREADS>
constexpr int tc_min_blocks() {
  return THREADS <= 256 ? 2 : 1;
}

// strided tiles: TC columns x L, 256 threads for L <= 512 (512 for 1024)
template <int L, TcForm F> struct TcStridedShape {
  static constexpr int P = L / 16;
  static constexpr int TC = P >= 32 ? 8 : 16;
  static constexpr int threads = P * TC;
  static constexpr size_t exch = size_t(L) * TC * sizeof(float2);
  static constexpr size_t need = exch + tc_extra_smem<F>(threads);
  static constexpr size_t smem = need > tc_smem_floor<threads>() ? need : tc_smem_floor<threads>();
};

template <int M, TcForm F> struct TcContigShape {
  typedef ContigShape<float, M, 16> CS;
  static constexpr int threads = CS::threads;
  static constexpr size_t exch = (CS::smem + 15) / 16 * 16;
  static constexpr size_t need = exch + tc_extra_smem<F>(threads);
  static constexpr size_t smem = need > tc_smem_floor<threads>() ? need : tc_smem_floor<threads>();
};

template <int L, TcForm F>
__global__ void __launch_bounds__(TcStridedShape<L, F>::threads, tc_min_blocks<TcStridedShape<L, F>::threads>())
k_strided_tc(const StridedArgs a, int* err) {
  typedef TcStridedShape<L, F> SH;
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

template <int M, TcForm F>
__global__ void __launch_bounds__(TcContigShape<M, F>::threads, tc_min_blocks<TcContigShape<M, F>::threads>())
k_zr2c_tc(const ContigArgs a, int* err) {
  typedef TcContigShape<M, F> TS;
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

template <int M, TcForm F>
__global__ void __launch_bounds__(TcContigShape<M, F>::threads, tc_min_blocks<TcContigShape<M, F>::threads>())
k_zc2r_tc(const ContigArgs a, int* err) {
  typedef TcContigShape<M, F> TS;
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

template <int L, TcForm F>
static bool run_strided_tc(const StridedArgs& a, int* err, cudaStream_t s) {
  typedef TcStridedShape<L, F> SH;
  auto k = k_strided_tc<L, F>;
  static PerDevice prepared;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  k<<<unsigned((a.ncols + SH::TC - 1) / SH::TC), SH::threads, SH::smem, s>>>(a, err);
  count_launch();
  return true;
}

template <int M, TcForm F, bool R2C>
static bool run_contig_tc(const ContigArgs& a, int* err, cudaStream_t s) {
  typedef TcContigShape<M, F> SH;
  auto k = R2C ? k_zr2c_tc<M, F> : k_zc2r_tc<M, F>;
  static PerDevice prepared;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  k<<<unsigned((a.nlines + SH::CS::TL - 1) / SH::CS::TL), SH::threads, SH::smem, s>>>(a, err);
  count_launch();
  return true;
}

bool tc_length_supported(int len, bool contig) {
  return len == 128 || len == 256 || len == 512 || (!contig && len == 1024);
}

bool launch_strided_tc(int form, int L, const StridedArgs& a, int* err, cudaStream_t s) {
#define AFG_TC_S(n)                                                                          \
  case n:                                                                                    \
    return form == 1 ? run_strided_tc<n, TcForm::TF32x3>(a, err, s) : run_strided_tc<n, TcForm::BF16x6>(a, err, s);
  switch (L) {
    AFG_TC_S(128) AFG_TC_S(256) AFG_TC_S(512) AFG_TC_S(1024)
    default: return false;
  }
#undef AFG_TC_S
}

bool launch_z_tc(int form, bool r2c, int M, const ContigArgs& a, int* err, cudaStream_t s) {
#define AFG_TC_Z(n)                                                                                \
  case n:                                                                                          \
    if (form == 1) return r2c ? run_contig_tc<n, TcForm::TF32x3, true>(a, err, s)                  \
                              : run_contig_tc<n, TcForm::TF32x3, false>(a, err, s);                \
    return r2c ? run_contig_tc<n, TcForm::BF16x6, true>(a, err, s) : run_contig_tc<n, TcForm::BF16x6, false>(a, err, s);
  switch (M) {
    AFG_TC_Z(128) AFG_TC_Z(256) AFG_TC_Z(512)
    default: return false;
  }
#undef AFG_TC_Z
}

}  // namespace afg
