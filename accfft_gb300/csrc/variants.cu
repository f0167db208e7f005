// Alternative radix plans and tile shapes of the float r2c / c2r passes, for
// the plan-time tuner (ACCFFT_MEASURE, plan.cpp).  Variant 0 is the default
// kernel of kernels.cu; here:
//   strided pass (MODE 0), L in {64, 128, 256, 512, 1024}:
//     1  half the columns per tile (TC / 2, at least 8)
//     2  the next smaller first radix (E = 16 for a default of 32, 8 for 16)
//     3  the default shape with 16-byte loads and stores: each pair of
//        neighbouring columns' threads loads two rows as float4 and swaps
//        halves by warp shuffle (launches with partial or misaligned tiles
//        run the default kernel)
//     4  (L in {512, 1024}) one persistent CTA a SM with three 64 KB column
//        tiles in flight: tensor copies (TMA) load the next two tiles while
//        the CTA transforms the current one in place in shared memory
//        (launches whose tiles are partial, straddle slabs or are not
//        16-byte aligned run the default kernel)
//   z r2c / z c2r (plain and mirror-pair mode), M in {64, 128, 256, 512}:
//     1  the other line count per CTA (z r2c: TL / 2; z c2r: TL where its
//        default is TL / 2, else TL / 2)
//     2  the next smaller first radix (with that radix's default line count)
// A variant that does not exist for a length launches nothing (false).
#include <cstdint>

#include <cuda.h>   // CUtensorMap and its encoder's enums (the encoder itself comes from the runtime)

#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace afg {

namespace {

template <int L>
constexpr int alt_e() {
  constexpr int E = LineFFT<float, L>::E;
  return E == 32 ? 16 : (E == 16 ? 8 : 0);
}
template <int L>
constexpr int half_tc() {
  constexpr int TC = StridedShape<float, L>::TC;
  return TC / 2 >= 8 ? TC / 2 : 0;
}
// the default z c2r line count (kernels.cu halves TL for M >= 256)
template <int M>
constexpr int zc2r_default_tl() {
  constexpr int TL = ContigShape<float, M>::TL;
  return M >= 256 && TL >= 2 ? TL / 2 : TL;
}
template <int M>
constexpr int zc2r_alt_tl() {
  constexpr int TL = ContigShape<float, M>::TL;
  return zc2r_default_tl<M>() == TL ? (TL / 2 >= 2 ? TL / 2 : 0) : TL;
}
template <int M>
constexpr int zr2c_alt_tl() {
  constexpr int TL = ContigShape<float, M>::TL;
  return TL / 2 >= 2 ? TL / 2 : 0;
}

template <int L, int EF, int TCF>
bool run_strided_v(const StridedArgs& a, cudaStream_t s) {
  typedef StridedShape<float, L, EF, TCF> SH;
  auto k = k_strided<float, L, 0, EF, TCF>;
  static PerDevice prepared;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  StridedArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  return launch_pass(k, unsigned((a.ncols + SH::TC - 1) / SH::TC), SH::threads, SH::smem, s, b) == cudaSuccess;
}

// The default strided tile (MODE 0) with 16-byte global accesses.  Threads c
// and c+1 (c even) of one line position t own neighbouring columns; for each
// pair of stage-0 entries (i, i+1) the even thread loads row t+i*P and the
// odd thread row t+(i+1)*P, both as (column c, column c+1), and one shuffle
// swaps the halves each needs.  The outputs leave the same way in reverse.
template <int L>
__global__ void __launch_bounds__(StridedShape<float, L>::threads, (strided_min_blocks<float, L, 0, 0>()))
k_strided_vec(const StridedArgs a) {
  typedef LineFFT<float, L> LN;
  typedef float2 V;
  constexpr int TC = StridedShape<float, L>::TC, P = LN::P, E = LN::E;
  static_assert(E % 2 == 0 && TC % 2 == 0 && LN::NS >= 2, "pairs of entries, columns and stages");
  PassScope scope(a.early_trigger);
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  const int c = threadIdx.x % TC;
  const int t = threadIdx.x / TC;
  const bool odd = (c & 1) != 0;
  const long long g0 = (long long)blockIdx.x * TC;   // whole tiles inside one slab (launcher)
  const long long slab = g0 / a.cps;
  const long long cc0 = g0 - slab * a.cps + (c & ~1);
  const V* in = static_cast<const V*>(a.in) + slab * a.in_slab + cc0;
  V* out = static_cast<V*>(a.out) + slab * a.out_slab + cc0;
  const long long il = a.in_line, ol = a.out_line;
  const float sg = a.inverse ? -1.f : 1.f;
  auto swap = [&](V x) { return make_float2(__shfl_xor_sync(0xffffffffu, x.x, 1), __shfl_xor_sync(0xffffffffu, x.y, 1)); };
  V v[E];
#pragma unroll
  for (int i = 0; i < E; i += 2) {
    const float4 q = *reinterpret_cast<const float4*>(in + (long long)(t + (odd ? i + 1 : i) * P) * il);
    const V lo = make_float2(q.x, q.y), hi = make_float2(q.z, q.w);
    const V got = swap(odd ? lo : hi);
    V x0 = odd ? got : lo;   // row t+i*P, this thread's column
    V x1 = odd ? hi : got;   // row t+(i+1)*P
    x0.y *= sg;
    x1.y *= sg;
    v[i] = x0;
    v[i + 1] = x1;
  }
  LN::stages(t, static_cast<const V*>(a.tw), [&](int p, V x) { sm[p * TC + c] = x; },
             [&](int p) { return sm[p * TC + c]; }, [] {}, v);
  // outputs: entry i = b*R + r of the last stage is frequency t + b*P + r*Ns
  constexpr int R = LN::pl.radix[LN::NS - 1];
  constexpr int Ns = plan_ns_before(LN::pl, LN::NS - 1);
#pragma unroll
  for (int i = 0; i < E; i += 2) {
    const int p0 = t + (i / R) * P + (i % R) * Ns;
    const int p1 = t + ((i + 1) / R) * P + ((i + 1) % R) * Ns;
    V y0 = v[i], y1 = v[i + 1];
    y0.y *= sg;
    y1.y *= sg;
    const V got = swap(odd ? y0 : y1);
    const float4 q = odd ? make_float4(got.x, got.y, y1.x, y1.y) : make_float4(y0.x, y0.y, got.x, got.y);
    *reinterpret_cast<float4*>(out + (long long)(odd ? p1 : p0) * ol) = q;
  }
}

template <int L>
bool run_strided_vec(const StridedArgs& a, cudaStream_t s) {
  typedef StridedShape<float, L> SH;
  constexpr int TC = SH::TC;
  const bool aligned = reinterpret_cast<uintptr_t>(a.in) % 16 == 0 && reinterpret_cast<uintptr_t>(a.out) % 16 == 0 &&
                       a.in_line % 2 == 0 && a.out_line % 2 == 0 && a.in_slab % 2 == 0 && a.out_slab % 2 == 0;
  if (!aligned || a.ncols_main > 0 || a.ncols <= 0 || a.cps % TC != 0 || a.ncols % TC != 0) return false;
  auto k = k_strided_vec<L>;
  static PerDevice prepared;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  StridedArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  return launch_pass(k, unsigned(a.ncols / TC), SH::threads, SH::smem, s, b) == cudaSuccess;
}

// ------------------------------------------------- variant 4: tensor-copy pipeline
// Tiles of TC columns x L rows of one slab (64 KB), NBUF buffers: buffer s
// holds the tile of local iteration it (it % NBUF == s), loaded by one tensor
// copy per BR rows that complete on mbarrier s (phase it / NBUF).  The CTA
// reads its stage-0 inputs from the buffer, then runs the exchanges in the
// same buffer, stores the outputs straight to global memory, and hands the
// buffer to the load of iteration it + NBUF.
template <int L>
struct PipeShape {
  static constexpr int TC = L >= 1024 ? 8 : 16;
  static constexpr int P = LineFFT<float, L>::P;
  static constexpr int threads = P * TC;
  static constexpr int NBUF = 3;
  static constexpr int BR = L < 256 ? L : 256;   // rows a tensor copy (box limit 256)
  static constexpr unsigned tile_bytes = unsigned(L) * TC * 8;
  static constexpr size_t smem = NBUF * size_t(tile_bytes) + 8 * NBUF;
  static_assert(L % BR == 0 && tile_bytes < (1u << 20), "whole boxes; mbarrier transaction count");
};

__device__ __forceinline__ uint32_t sm_addr(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ bool pipe_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// wait on phase `parity` of mbarrier `bar`, at most `limit` polls (every
// thread polls; a limit of 0 gives up at once)
__device__ __forceinline__ bool pipe_wait(uint32_t bar, uint32_t parity, unsigned limit) {
  for (unsigned k = 0; k < limit; ++k)
    if (pipe_try(bar, parity)) return true;
  return false;
}

template <int L>
__global__ void __launch_bounds__(PipeShape<L>::threads, 1)
    k_strided_pipe(const __grid_constant__ CUtensorMap tm, const StridedArgs a) {
  typedef LineFFT<float, L> LN;
  typedef PipeShape<L> SH;
  typedef float2 V;
  constexpr int TC = SH::TC, NB = SH::NBUF, E = LN::E;
  PassScope scope(a.early_trigger);
  extern __shared__ __align__(128) unsigned char smraw[];
  V* const buf0 = reinterpret_cast<V*>(smraw);
  unsigned long long* const bars = reinterpret_cast<unsigned long long*>(smraw + NB * size_t(SH::tile_bytes));
  const int c = threadIdx.x % TC, t = threadIdx.x / TC;
  const long long tps = a.cps / TC;        // tiles a slab
  const long long ntiles = a.ncols / TC;   // whole tiles (launcher)
  const float sg = a.inverse ? -1.f : 1.f;
  // thread 0: the tensor copies of `tile` into buffer s
  auto issue = [&](long long tile, int s) {
    const uint32_t bar = sm_addr(bars + s);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(SH::tile_bytes) : "memory");
    const int z = int(tile / tps), x = int((tile - (long long)z * tps) * TC);
    const uint32_t dst = sm_addr(buf0 + (size_t)s * L * TC);
#pragma unroll
    for (int r = 0; r < L; r += SH::BR)
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
              dst + uint32_t(r) * TC * 8),
          "l"(reinterpret_cast<uint64_t>(&tm)), "r"(x), "r"(r), "r"(z), "r"(bar)
          : "memory");
  };
  if (threadIdx.x == 0) {
    for (int s = 0; s < NB; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sm_addr(bars + s)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int s = 0; s < NB; ++s) {
      const long long tile = blockIdx.x + (long long)s * gridDim.x;
      if (tile < ntiles) issue(tile, s);
    }
  long long it = 0;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int s = int(it % NB);
    const bool got = pipe_wait(sm_addr(bars + s), uint32_t((it / NB) & 1), a.wait_limit);
    if (__syncthreads_or(!got)) {
      // a load did not arrive: record it, let the copies already issued
      // (iterations it .. it + NB - 1) land before the CTA's shared memory
      // goes away (a wait of its own limit: the pass limit may be tiny), and
      // leave
      for (long long j = it; j < it + NB; ++j)
        if (blockIdx.x + j * gridDim.x < ntiles) pipe_wait(sm_addr(bars + j % NB), uint32_t((j / NB) & 1), 1u << 22);
      if (threadIdx.x == 0 && a.wait_err) atomicExch(a.wait_err, 1);
      return;
    }
    V* sm = buf0 + (size_t)s * L * TC;
    const long long z = tile / tps;
    const long long col = (tile - z * tps) * TC + c;
    V* out = static_cast<V*>(a.out) + z * a.out_slab + col;
    const long long ol = a.out_line;
    V v[E];
    LN::compute(
        t, static_cast<const V*>(a.tw),
        [&](int p) {
          V x = sm[p * TC + c];
          x.y *= sg;
          return x;
        },
        [&](int p, V x) { sm[p * TC + c] = x; }, [&](int p) { return sm[p * TC + c]; }, [] { __syncthreads(); }, v);
    LN::emit(t, v, [&](int p, V x) {
      x.y *= sg;
      out[p * ol] = x;
    });
    // every access of buffer s is done and ordered before the tensor copy
    // (async proxy) that refills it with the tile of iteration it + NB
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      const long long nt = tile + (long long)NB * gridDim.x;
      if (nt < ntiles) issue(nt, s);
    }
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, looked up once through the runtime
EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return EncodeTiledFn(nullptr);
    }
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

template <int L>
bool run_strided_pipe(const StridedArgs& a, cudaStream_t s) {
  typedef PipeShape<L> SH;
  constexpr int TC = SH::TC;
  // whole tiles inside one slab, 16-byte aligned base and row / slab strides
  // (complex float elements: even strides), coordinates inside 32 bits
  if (a.ncols_main > 0 || a.ncols <= 0 || a.cps <= 0 || a.cps % TC != 0 || a.ncols % a.cps != 0) return false;
  const long long nslab = a.ncols / a.cps;
  if (reinterpret_cast<uintptr_t>(a.in) % 16 != 0 || a.in_line % 2 != 0 || (nslab > 1 && a.in_slab % 2 != 0) ||
      a.in_line <= 0 || (nslab > 1 && a.in_slab <= 0) || a.cps >= (1LL << 31) || nslab >= (1LL << 31))
    return false;
  const EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  CUtensorMap tm;
  const cuuint64_t dims[3] = {cuuint64_t(a.cps), cuuint64_t(L), cuuint64_t(nslab)};
  const cuuint64_t strides[2] = {cuuint64_t(a.in_line) * 8,
                                 cuuint64_t(nslab > 1 ? a.in_slab : a.in_line * L) * 8};
  const cuuint32_t box[3] = {cuuint32_t(TC), cuuint32_t(SH::BR), 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void*>(a.in), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  auto k = k_strided_pipe<L>;
  static PerDevice prepared, occupancy;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  const long long grid = persistent_grid(occupancy, k, SH::threads, SH::smem, a.ncols / TC);
  if (grid < 1) return false;
  StridedArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  if (launch_pass(k, unsigned(grid), SH::threads, SH::smem, s, tm, b) == cudaSuccess) return true;
  cudaGetLastError();   // a refused launch: the default kernel runs instead and reports its own errors
  return false;
}

template <int L>
bool strided_variant(int v, const StridedArgs& a, cudaStream_t s) {
  if (v == 1) {
    if constexpr (half_tc<L>() > 0) return run_strided_v<L, 0, half_tc<L>()>(a, s);
  } else if (v == 2) {
    if constexpr (alt_e<L>() > 0) return run_strided_v<L, alt_e<L>(), 0>(a, s);
  } else if (v == 3) {
    return run_strided_vec<L>(a, s);
  } else if (v == 4) {
    if constexpr (L == 512 || L == 1024) return run_strided_pipe<L>(a, s);
  }
  return false;
}

// pair mode: TL / 2 mirror pairs per CTA (as kernels.cu)
template <int TL>
unsigned contig_grid(const ContigArgs& a) {
  const long long per = a.pair_n1 > 0 ? TL / 2 : TL;
  const long long units = a.pair_n1 > 0 ? a.nlines / 2 : a.nlines;
  return unsigned((units + per - 1) / per);
}

template <bool R2C, int M, int EF, int TLF>
bool run_contig_v(const ContigArgs& a, cudaStream_t s) {
  typedef ContigShape<float, M, EF, TLF> SH;
  if (a.pair_n1 > 0 && SH::TL < 2) return false;
  void (*k)(const ContigArgs);
  if constexpr (R2C) k = k_zr2c<float, M, EF, TLF>;
  else k = k_zc2r<float, M, EF, TLF>;
  static PerDevice prepared;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  ContigArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  return launch_pass(k, contig_grid<SH::TL>(a), SH::threads, SH::smem, s, b) == cudaSuccess;
}

template <bool R2C, int M>
bool contig_variant(int v, const ContigArgs& a, cudaStream_t s) {
  if (v == 1) {
    constexpr int tl = R2C ? zr2c_alt_tl<M>() : zc2r_alt_tl<M>();
    if constexpr (tl > 0) return run_contig_v<R2C, M, 0, tl>(a, s);
  } else if (v == 2) {
    if constexpr (alt_e<M>() > 0) return run_contig_v<R2C, M, alt_e<M>(), 0>(a, s);
  }
  return false;
}

// first radix and tile width (columns or lines per CTA) of a variant
template <int L>
void strided_shape(int v, int* E, int* tile) {
  *E = *tile = 0;
  if (v == 0) {
    *E = LineFFT<float, L>::E;
    *tile = StridedShape<float, L>::TC;
  } else if (v == 1) {
    if constexpr (half_tc<L>() > 0) {
      *E = LineFFT<float, L>::E;
      *tile = half_tc<L>();
    }
  } else if (v == 2) {
    if constexpr (alt_e<L>() > 0) {
      *E = alt_e<L>();
      *tile = StridedShape<float, L, alt_e<L>()>::TC;
    }
  } else if (v == 3) {
    *E = LineFFT<float, L>::E;
    *tile = StridedShape<float, L>::TC;
  } else if (v == 4) {
    if constexpr (L == 512 || L == 1024) {
      *E = LineFFT<float, L>::E;
      *tile = PipeShape<L>::TC;
    }
  }
}
template <bool R2C, int M>
void contig_shape(int v, int* E, int* tile) {
  *E = *tile = 0;
  if (v == 0) {
    *E = LineFFT<float, M>::E;
    *tile = R2C ? ContigShape<float, M>::TL : zc2r_default_tl<M>();
  } else if (v == 1) {
    constexpr int tl = R2C ? zr2c_alt_tl<M>() : zc2r_alt_tl<M>();
    if constexpr (tl > 0) {
      *E = LineFFT<float, M>::E;
      *tile = tl;
    }
  } else if (v == 2) {
    if constexpr (alt_e<M>() > 0) {
      *E = alt_e<M>();
      *tile = ContigShape<float, M, alt_e<M>()>::TL;
    }
  }
}

}  // namespace

#define AFG_VAR_STRIDED(X) X(64) X(128) X(256) X(512) X(1024)
#define AFG_VAR_CONTIG(X) X(64) X(128) X(256) X(512)

bool launch_strided_variant_f32(int L, int v, const StridedArgs& a, cudaStream_t s) {
  switch (L) {
#define AFG_CASE(n) case n: return strided_variant<n>(v, a, s);
    AFG_VAR_STRIDED(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
}

bool launch_contig_variant_f32(bool r2c, int M, int v, const ContigArgs& a, cudaStream_t s) {
  switch (M) {
#define AFG_CASE(n) case n: return r2c ? contig_variant<true, n>(v, a, s) : contig_variant<false, n>(v, a, s);
    AFG_VAR_CONTIG(AFG_CASE)
#undef AFG_CASE
    default: return false;
  }
}

// kind: PK_STRIDED, PK_ZR2C or PK_ZC2R; E = tile = 0 when the variant does
// not exist for the length (variant 0 of a length without variants too)
void variant_shape(int kind, int L, int v, int* E, int* tile) {
  *E = *tile = 0;
  if (kind == PK_STRIDED) {
    switch (L) {
#define AFG_CASE(n) case n: strided_shape<n>(v, E, tile); break;
      AFG_VAR_STRIDED(AFG_CASE)
#undef AFG_CASE
      default: break;
    }
  } else if (kind == PK_ZR2C || kind == PK_ZC2R) {
    switch (L) {
#define AFG_CASE(n) \
  case n: kind == PK_ZR2C ? contig_shape<true, n>(v, E, tile) : contig_shape<false, n>(v, E, tile); break;
      AFG_VAR_CONTIG(AFG_CASE)
#undef AFG_CASE
      default: break;
    }
  }
}

}  // namespace afg
