// Fused z+y slab passes: one thread-block cluster per x-slab.
//
// An r2c x-slab is [N1][N2/2+1] complex (1.05 MB at 512^3 float): too large
// for one CTA, small enough for the distributed shared memory of a cluster
// of C CTAs.  CTA c of the cluster owns rows y in [c*R, (c+1)*R) (R = N1/C)
// and columns kz in [c*W, (c+1)*W) (W = ceil((N2/2+1)/C)).
//
// forward (z r2c + y forward):
//   1. each CTA transforms its R real rows along z into its row buffer;
//   2. cluster barrier; each CTA gathers its W columns of all N1 rows from
//      the row buffers of the whole cluster (DSMEM loads) into registers;
//   3. cluster barrier (the row buffers are no longer read remotely); the y
//      transform runs with its exchanges in the CTA's own buffer and stores
//      the columns to the spectrum.
// inverse (y backward + z c2r): the mirror image, with the y results pushed
// into the owners' row buffers by DSMEM stores between two cluster barriers.
//
// HBM traffic per direction: the real field and the spectrum once each,
// instead of twice the spectrum more for a separate y pass.
#include <cooperative_groups.h>

#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace cg = cooperative_groups;

namespace afg {

template <typename T, int N1, int M, int C>
struct SlabShape {
  typedef LineFFT<T, N1> LY;
  typedef LineFFT<T, M> LZ;
  static constexpr int H2 = M + 1;
  static constexpr int R = N1 / C;
  static constexpr int W = (H2 + C - 1) / C;
  static constexpr int threads = LY::P * W;
  static constexpr int RZ = threads / LZ::P;   // rows per z batch
  static constexpr int slots = sizeof(T) == 4 ? 16 : 8;
  static constexpr int PW = LZ::E > slots ? LZ::E : slots;
  __host__ __device__ static constexpr int pad(int p) { return p + p / PW; }
  static constexpr int need = (pad(M - 1) + 1) > H2 ? (pad(M - 1) + 1) : H2;
  static constexpr int pitch = ((need + slots - 1) / slots) * slots + (LZ::P < slots ? LZ::P : 0);
  static constexpr int rb = R * pitch, ex = N1 * W;
  static constexpr size_t smem = size_t(rb > ex ? rb : ex) * sizeof(typename CT<T>::V);
  static_assert(N1 % C == 0, "rows must split evenly over the cluster");
  static_assert(RZ >= 1, "too few threads for a z row");
};

template <typename T, int N1, int M, int C>
__global__ void __launch_bounds__(SlabShape<T, N1, M, C>::threads)
k_slab_fwd(const SlabArgs a) {
  typedef SlabShape<T, N1, M, C> SH;
  typedef typename SH::LY LY;
  typedef typename SH::LZ LZ;
  typedef typename CT<T>::V V;
  constexpr int R = SH::R, W = SH::W, H2 = SH::H2, PITCH = SH::pitch, RZ = SH::RZ;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const long long slab = blockIdx.x / C;
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);
  const V* twz = static_cast<const V*>(a.tw_z);
  const V* twp = static_cast<const V*>(a.tw_post);

  // ---- 1. z r2c of the CTA's rows, RZ rows at a time
  {
    const int tz = threadIdx.x % LZ::P;
    const int gi = threadIdx.x / LZ::P;
#pragma unroll 1
    for (int r0 = 0; r0 < R; r0 += RZ) {
      const int lr = r0 + gi;
      const bool act = gi < RZ && lr < R;
      const int lrs = act ? lr : r0;
      V* row = sm + lrs * PITCH;
      const V* src = reinterpret_cast<const V*>(static_cast<const T*>(a.in) +
                                                ((slab * N1) + rank * R + lrs) * a.real_row);
      auto ld = [&](int p) { return src[p]; };
      auto xw = [&](int p, V x) { if (act) row[SH::pad(p)] = x; };
      auto xr = [&](int p) { return row[SH::pad(p)]; };
      LZ::template run<true, false>(tz, twz, ld, xw, xw, xr);
      __syncthreads();
      V xk[LZ::E];
#pragma unroll
      for (int r = 0; r < LZ::E; ++r) {
        const int k = tz + r * LZ::P;
        xk[r] = r2c_split(xr(k), xr(k == 0 ? 0 : M - k), __ldg(twp + k));
      }
      V z0 = xr(0);
      __syncthreads();
      if (act) {
#pragma unroll
        for (int r = 0; r < LZ::E; ++r) row[tz + r * LZ::P] = xk[r];
        if (tz == 0) row[M] = c_make<V>(z0.x - z0.y, T(0));
      }
      __syncthreads();
    }
  }
  cluster.sync();

  // ---- 2./3. y transform of the CTA's columns
  const int c = threadIdx.x % W, ty = threadIdx.x / W;
  const int kz = rank * W + c;
  const bool valid = kz < H2;
  const int kzs = valid ? kz : 0;
  auto ldy = [&](int p) {
    const V* owner = cluster.map_shared_rank(sm, p / R);
    return owner[(p % R) * PITCH + kzs];
  };
  auto xwy = [&](int p, V x) { sm[p * W + c] = x; };
  auto xry = [&](int p) { return sm[p * W + c]; };
  V v[LY::E];
  LY::compute(ty, static_cast<const V*>(a.tw_y), ldy, xwy, xry, [&] { cluster.sync(); }, v);
  V* out = static_cast<V*>(a.out) + slab * N1 * H2 + kzs;
  LY::emit(ty, v, [&](int p, V x) {
    if (valid) out[(long long)p * H2] = x;
  });
}

template <typename T, int N1, int M, int C>
__global__ void __launch_bounds__(SlabShape<T, N1, M, C>::threads)
k_slab_inv(const SlabArgs a) {
  typedef SlabShape<T, N1, M, C> SH;
  typedef typename SH::LY LY;
  typedef typename SH::LZ LZ;
  typedef typename CT<T>::V V;
  constexpr int R = SH::R, W = SH::W, H2 = SH::H2, PITCH = SH::pitch, RZ = SH::RZ;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const long long slab = blockIdx.x / C;
  extern __shared__ __align__(16) unsigned char smraw[];
  V* sm = reinterpret_cast<V*>(smraw);

  // ---- 1. y backward transform of the CTA's columns (conjugated forward engine)
  {
    const int c = threadIdx.x % W, ty = threadIdx.x / W;
    const int kz = rank * W + c;
    const bool valid = kz < H2;
    const int kzs = valid ? kz : 0;
    const V* in = static_cast<const V*>(a.in) + slab * N1 * H2 + kzs;
    auto ld = [&](int p) { return c_conj(in[(long long)p * H2]); };
    auto xwy = [&](int p, V x) { sm[p * W + c] = x; };
    auto xry = [&](int p) { return sm[p * W + c]; };
    V v[LY::E];
    LY::compute(ty, static_cast<const V*>(a.tw_y), ld, xwy, xry, [] {}, v);
    cluster.sync();   // every CTA is done with its exchange buffer
    LY::emit(ty, v, [&](int p, V x) {
      if (valid) {
        V* owner = cluster.map_shared_rank(sm, p / R);
        owner[(p % R) * PITCH + kz] = c_conj(x);
      }
    });
  }
  cluster.sync();   // the rows of this CTA are complete

  // ---- 2. z c2r of the CTA's rows
  const V* twz = static_cast<const V*>(a.tw_z);
  const V* twp = static_cast<const V*>(a.tw_post);
  const int tz = threadIdx.x % LZ::P;
  const int gi = threadIdx.x / LZ::P;
#pragma unroll 1
  for (int r0 = 0; r0 < R; r0 += RZ) {
    const int lr = r0 + gi;
    const bool act = gi < RZ && lr < R;
    const int lrs = act ? lr : r0;
    V* row = sm + lrs * PITCH;
    V* dst = reinterpret_cast<V*>(static_cast<T*>(a.out) + ((slab * N1) + rank * R + lrs) * a.real_row);
    auto ld = [&](int p) {
      V xk = row[p], xm = row[M - p];
      if (p == 0) { xk.y = T(0); xm.y = T(0); }
      return c_conj(c2r_merge(xk, xm, c_conj(__ldg(twp + p))));
    };
    auto xw = [&](int p, V x) { if (act) row[SH::pad(p)] = x; };
    auto xr = [&](int p) { return row[SH::pad(p)]; };
    auto st = [&](int p, V x) { x.y = -x.y; if (act) dst[p] = x; };
    V v[LZ::E];
    LZ::compute(tz, twz, ld, xw, xr, [] { __syncthreads(); }, v);
    LZ::emit(tz, v, st);
    __syncthreads();
  }
}

// ------------------------------------------------------------- launchers
namespace {

template <typename K>
bool cluster_launch(K kernel, int C, int threads, size_t smem, long long grid, const SlabArgs& a, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, 1, 1);
  cfg.blockDim = dim3((unsigned)threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, a) == cudaSuccess;
}

// whether the kernels' clusters can be scheduled, checked once per device
template <typename T, int N1, int M, int C>
struct SlabKernels {
  typedef SlabShape<T, N1, M, C> SH;
  static PerDevice state;   // 1: usable, -1: not on this device
  static int check() {
    auto kf = k_slab_fwd<T, N1, M, C>;
    auto ki = k_slab_inv<T, N1, M, C>;
    for (auto k : {kf, ki}) {
      if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SH::smem) != cudaSuccess) {
        cudaGetLastError();
        return -1;
      }
      if (C > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return -1;
      }
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(C, 1, 1);
      cfg.blockDim = dim3(SH::threads, 1, 1);
      cfg.dynamicSmemBytes = SH::smem;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = C;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess || n < 1) {
        cudaGetLastError();
        return -1;
      }
    }
    return 1;
  }
  static bool ready() { return per_device(state, check) == 1; }
  static bool launch(bool fwd, const SlabArgs& a, cudaStream_t s) {
    if (!ready()) return false;
    bool ok = fwd ? cluster_launch(k_slab_fwd<T, N1, M, C>, C, SH::threads, SH::smem, (long long)a.n0 * C, a, s)
                  : cluster_launch(k_slab_inv<T, N1, M, C>, C, SH::threads, SH::smem, (long long)a.n0 * C, a, s);
    if (ok) count_launch();
    return ok;
  }
};
template <typename T, int N1, int M, int C>
PerDevice SlabKernels<T, N1, M, C>::state;

}  // namespace

// Grids with a fused slab kernel (float): 512 x (N2 = 512) over 16-CTA
// clusters, 256 x 256 over 8, 128 x 128 over 2.
bool slab_available(bool dbl, int N1, int N2) {
  if (dbl) return false;
  if (N1 == 512 && N2 == 512) return SlabKernels<float, 512, 256, 16>::ready();
  if (N1 == 256 && N2 == 256) return SlabKernels<float, 256, 128, 8>::ready();
  if (N1 == 128 && N2 == 128) return SlabKernels<float, 128, 64, 2>::ready();
  return false;
}

bool launch_slab(bool dbl, int N1, int N2, bool forward, const SlabArgs& a, cudaStream_t s) {
  if (dbl) return false;
  if (N1 == 512 && N2 == 512) return SlabKernels<float, 512, 256, 16>::launch(forward, a, s);
  if (N1 == 256 && N2 == 256) return SlabKernels<float, 256, 128, 8>::launch(forward, a, s);
  if (N1 == 128 && N2 == 128) return SlabKernels<float, 128, 64, 2>::launch(forward, a, s);
  return false;
}

}  // namespace afg
