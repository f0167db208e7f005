// Persistent strided pass with the next tile prefetched (float, MODE 0; the
// tuner's variant 3 of the y and x passes for lines of 512 and 1024).
//
// A column tile of the default strided kernel (16 columns x L) is loaded
// into registers, transformed and stored by a CTA that then exits; for
// 1024-point lines its 128 KB exchange buffer and 128-register threads leave
// one CTA per SM, so an SM's loads stop while it computes and stores.  Here a
// CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...: as soon as the
// threads have taken a tile from the staging buffer into registers, they
// issue cp.async copies of the CTA's next tile into that buffer, and the
// copies run while the tile is transformed and stored.  The exchange buffer
// holds half the tile's columns and every exchange runs in two rounds
// (LineFFT::stages_rounds), so staging buffer + exchange buffer fit one SM
// (1024: 128 + 64 KB, one 512-thread CTA per SM; 512: 64 + 32 KB, two
// 256-thread CTAs per SM).
//
// Eligible launches: every tile whole and inside one slab (columns per slab
// and column count multiples of 16), no Nyquist split layout.  Rows move as
// 16-byte copies when the tile base and the line stride are 16-byte aligned,
// else as 8-byte copies.
#include <cstdint>

#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace afg {

namespace {

template <int L> struct PfShape {
  typedef LineFFT<float, L> LN;
  static constexpr int P = LN::P;
  static constexpr int E = LN::E;
  static constexpr int TC = 16;            // columns per tile: 128-byte row segments
  static constexpr int XG = 2;             // exchange rounds
  static constexpr int HALF = TC / XG;     // columns in the exchange buffer
  static constexpr int threads = P * TC;
  static constexpr size_t stage_bytes = size_t(L) * TC * sizeof(float2);
  // exchange rows of HALF entries (64 B), one pad row after every 32 rows:
  // stage 0 writes rows 32 apart from neighbouring threads, which the pad
  // moves to the other half of the banks
  __host__ __device__ static constexpr int xrow(int p) { return p + (p >> 5); }
  static constexpr size_t xch_bytes = size_t(xrow(L)) * HALF * sizeof(float2);
  static constexpr size_t smem = stage_bytes + xch_bytes;
  static constexpr int min_blocks = threads <= 256 ? 2 : 1;
  static_assert((L * TC / 2) % threads == 0 && (L * TC) % threads == 0, "whole copies per thread");
};

__device__ __forceinline__ uint32_t pf_smem(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(pf_smem(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(pf_smem(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int L>
__global__ void __launch_bounds__(PfShape<L>::threads, PfShape<L>::min_blocks)
k_strided_pf(const StridedArgs a, long long ntiles, int vec16) {
  typedef PfShape<L> SH;
  typedef typename SH::LN LN;
  typedef float2 V;
  constexpr int TC = SH::TC, P = SH::P, E = SH::E, HALF = SH::HALF;
  PassScope scope(a.early_trigger);
  extern __shared__ __align__(16) unsigned char smraw[];
  V* stage = reinterpret_cast<V*>(smraw);
  V* xch = reinterpret_cast<V*>(smraw + SH::stage_bytes);
  const int c = threadIdx.x % TC;
  const int t = threadIdx.x / TC;
  const int grp = c / HALF;
  const int ch = c % HALF;
  const float sg = a.inverse ? -1.f : 1.f;
  const V* tw = static_cast<const V*>(a.tw);
  const long long il = a.in_line, ol = a.out_line;
  auto tile_in = [&](long long tile) {
    const long long g0 = tile * TC;
    const long long slab = g0 / a.cps;
    return static_cast<const V*>(a.in) + slab * a.in_slab + (g0 - slab * a.cps);
  };
  // copies of one tile into the staging buffer: element (row, col) at
  // row * TC + col
  auto prefetch = [&](long long tile) {
    const V* src = tile_in(tile);
    if (vec16) {
#pragma unroll
      for (int k = 0; k < L * TC / 2 / SH::threads; ++k) {
        const int q = threadIdx.x + k * SH::threads;
        const int row = q / (TC / 2), cp = q % (TC / 2);
        cp_async16(stage + 2 * q, src + row * il + 2 * cp);
      }
    } else {
#pragma unroll
      for (int k = 0; k < L * TC / SH::threads; ++k) {
        const int q = threadIdx.x + k * SH::threads;
        cp_async8(stage + q, src + (q / TC) * il + (q % TC));
      }
    }
    cp_async_commit();
  };
  long long tile = blockIdx.x;
  if (tile < ntiles) prefetch(tile);
  for (; tile < ntiles; tile += gridDim.x) {
    cp_async_wait_all();
    __syncthreads();   // the tile is in the staging buffer; the last tile's exchange reads are done
    V v[E];
#pragma unroll
    for (int r = 0; r < E; ++r) {
      V x = stage[(t + r * P) * TC + c];
      x.y *= sg;
      v[r] = x;
    }
    __syncthreads();   // every thread has its tile: the staging buffer is free
    const long long next = tile + gridDim.x;
    if (next < ntiles) prefetch(next);
    LN::template stages_rounds<SH::XG>(
        t, grp, tw, [&](int p, V x) { xch[SH::xrow(p) * HALF + ch] = x; },
        [&](int p) { return xch[SH::xrow(p) * HALF + ch]; }, v);
    const long long g0 = tile * TC;
    const long long slab = g0 / a.cps;
    V* out = static_cast<V*>(a.out) + slab * a.out_slab + (g0 - slab * a.cps) + c;
    LN::emit(t, v, [&](int p, V x) {
      x.y *= sg;
      out[p * ol] = x;
    });
  }
}

template <int L>
bool run_pf(const StridedArgs& a, cudaStream_t s) {
  typedef PfShape<L> SH;
  constexpr int TC = SH::TC;
  if (a.ncols_main > 0 || a.cps % TC != 0 || a.ncols % TC != 0 || a.ncols <= 0) return false;
  auto k = k_strided_pf<L>;
  static PerDevice prepared, occupancy;
  if (!prepare_smem(prepared, k, SH::smem)) return false;
  const int occ = per_device(occupancy, [&] {
    int n = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, SH::threads, SH::smem) == cudaSuccess && n > 0 ? n
                                                                                                               : -1;
  });
  int dev = 0, sms = 0;
  if (occ < 1 || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    return false;
  const long long ntiles = a.ncols / TC;
  const long long cap = (long long)sms * occ;
  const unsigned grid = unsigned(ntiles < cap ? ntiles : cap);
  // 16-byte copies: tile bases (multiples of 16 columns from a slab start)
  // and rows 16-byte aligned
  const int vec16 = (reinterpret_cast<uintptr_t>(a.in) % 16 == 0) && a.in_line % 2 == 0 && a.in_slab % 2 == 0;
  StridedArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  return launch_pass(k, grid, SH::threads, SH::smem, s, b, ntiles, vec16) == cudaSuccess;
}

}  // namespace

bool pf_length(int L) { return L == 512 || L == 1024; }

bool launch_strided_pf_f32(int L, const StridedArgs& a, cudaStream_t s) {
  switch (L) {
    case 512: return run_pf<512>(a, s);
    case 1024: return run_pf<1024>(a, s);
    default: return false;
  }
}

}  // namespace afg
