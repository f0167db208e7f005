// Strided pass of 1024-point lines over two-CTA clusters (float, MODE 0; the
// tuner's variant 3 of the y and x passes for lines of 1024).
//
// The default kernel keeps a 16-column tile of 1024 rows (128 KB) in one
// CTA: 512 threads at 128 registers and a 128 KB exchange buffer leave one
// CTA per SM, whose loads stop while it computes.  Here the two CTAs of a
// cluster share the tile by decimation in time,
//     X[k]       = E[k] + w_L^k O[k]
//     X[k + L/2] = E[k] - w_L^k O[k],   k < L/2,
// E and O the L/2-point transforms of the even and odd rows: CTA rank 0
// transforms the even rows, rank 1 the odd rows (the 512-point engine, 16
// columns, 256 threads, 64 KB), both leave their spectrum in shared memory,
// and after a cluster barrier rank 0 writes rows k < L/2 and rank 1 rows
// k >= L/2, each reading the other half from its peer's shared memory.  Two
// such CTAs fit an SM, and the row segments stay 128 bytes.
//
// In place is safe: every row a CTA reads is in its registers before the
// first cluster barrier, and the stores come after it.  The second barrier
// keeps each CTA's shared memory alive until its peer has read it.
//
// Twiddles (a.tw): w_L^k for k < L/2, then the stage table of the L/2-point
// plan (plan.cpp builds both).
#include <cooperative_groups.h>

#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace cg = cooperative_groups;

namespace afg {

namespace {

template <int L> struct C2Shape {
  static constexpr int H = L / 2;
  typedef LineFFT<float, H> LN;
  static constexpr int P = LN::P;
  static constexpr int TC = 16;              // columns per tile: 128-byte row segments
  static constexpr int threads = P * TC;
  static constexpr size_t smem = size_t(H) * TC * sizeof(float2);
  static constexpr int min_blocks = threads <= 256 ? 2 : 1;
};

template <int L>
__global__ void __launch_bounds__(C2Shape<L>::threads, C2Shape<L>::min_blocks) k_strided_c2(const StridedArgs a) {
  typedef C2Shape<L> SH;
  typedef typename SH::LN LN;
  typedef float2 V;
  constexpr int TC = SH::TC, H = SH::H;
  PassScope scope(a.early_trigger);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  const long long tile = blockIdx.x / 2;
  const int c = threadIdx.x % TC;
  const int t = threadIdx.x / TC;
  const long long g = tile * TC + c;
  const bool valid = g < a.ncols;
  const long long gs = valid ? g : 0;        // idle lanes read column 0, store nothing
  const long long slab = gs / a.cps;
  const long long cc = gs - slab * a.cps;
  const V* in = static_cast<const V*>(a.in) + slab * a.in_slab + cc + rank * a.in_line;
  V* out = static_cast<V*>(a.out) + slab * a.out_slab + cc;
  const long long il2 = 2 * a.in_line, ol = a.out_line;
  const float sg = a.inverse ? -1.f : 1.f;
  const V* comb = static_cast<const V*>(a.tw);
  const V* stage_tw = comb + H;
  auto xw = [&](int p, V x) { sm[p * TC + c] = x; };
  auto xr = [&](int p) { return sm[p * TC + c]; };
  auto ld = [&](int p) {
    V x = in[p * il2];
    x.y *= sg;
    return x;
  };
  // the half-length transform; its spectrum lands in this CTA's shared memory
  LN::template run<true, false>(t, stage_tw, ld, xw, xw, xr);
  cluster.sync();   // both halves' spectra are complete and visible to the peer
  const V* peer = cluster.map_shared_rank(sm, rank ^ 1);
#pragma unroll 4
  for (int i = 0; i < H / (SH::threads / TC); ++i) {
    const int k = t + i * (SH::threads / TC);
    const V mine = sm[k * TC + c], other = peer[k * TC + c];
    const V e = rank == 0 ? mine : other;
    const V o = rank == 0 ? other : mine;
    const V wo = c_mul(o, __ldg(comb + k));
    V x = rank == 0 ? c_add(e, wo) : c_sub(e, wo);
    x.y *= sg;
    if (valid) out[(long long)(k + rank * H) * ol] = x;
  }
  cluster.sync();   // the peer has finished reading this CTA's shared memory
}

// whether the kernel's clusters can be scheduled, checked once per device
template <int L>
int c2_check() {
  typedef C2Shape<L> SH;
  auto k = k_strided_c2<L>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SH::smem) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2, 1, 1);
  cfg.blockDim = dim3(SH::threads, 1, 1);
  cfg.dynamicSmemBytes = SH::smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess || n < 1) {
    cudaGetLastError();
    return -1;
  }
  return 1;
}

template <int L>
bool run_c2(const StridedArgs& a, cudaStream_t s) {
  typedef C2Shape<L> SH;
  if (a.ncols_main > 0 || a.ncols <= 0) return false;
  static PerDevice state;
  if (per_device(state, c2_check<L>) != 1) return false;
  const long long tiles = (a.ncols + SH::TC - 1) / SH::TC;
  StridedArgs b = a;
  b.early_trigger = pdl_mode() == 2;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(2 * tiles), 1, 1);
  cfg.blockDim = dim3(SH::threads, 1, 1);
  cfg.dynamicSmemBytes = SH::smem;
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_mode() > 0 ? 2 : 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_strided_c2<L>, b);
  count_launch();
  return e == cudaSuccess;
}

}  // namespace

bool launch_strided_c2_f32(int L, const StridedArgs& a, cudaStream_t s) {
  switch (L) {
    case 1024: return run_c2<1024>(a, s);
    default: return false;
  }
}

}  // namespace afg
