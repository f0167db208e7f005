// Persistent z+y passes of a full r2c (z r2c, then y) or c2r (y, then z c2r):
// one kernel whose CTAs take work items from a global counter.  A z item is
// TL rows of one x-slab, a y item TC columns of one x-slab; the y items of a
// slab need only that slab's z rows (and the backward z items only that
// slab's y columns).  Items are handed out in slab order with the dependent
// kind `lead` slabs behind, so a slab's spectrum is usually still in L2 when
// its second pass reads it: the second pass's HBM read, and one of the two
// write-backs of the spectrum, disappear.
//
// Deadlock freedom: every item an item waits for was handed out earlier, to a
// CTA that is running it, and items of the first kind wait for nothing.  The
// waits are bounded anyway (wait_limit polls of at least 128 ns; the default
// is about half a second): a wait that gives up sets the plan's error word,
// which the host reports, and its item is skipped, so nothing reads a slab
// that is only partly written and the kernel always ends.
#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace afg {

template <typename T, int M, int L> struct ZyShape {
  typedef ContigShape<T, M> ZS;
  typedef StridedShape<T, L> YS;
  static constexpr int threads = ZS::threads;
  static constexpr int TL = ZS::TL, TC = YS::TC;
  static constexpr int ZI = (L + TL - 1) / TL;          // z items per slab (N1 = L rows)
  static constexpr int YI = (M + 1 + TC - 1) / TC;      // y items per slab (M + 1 columns)
  static constexpr size_t smem = ZS::smem > YS::smem ? ZS::smem : YS::smem;
  static constexpr bool ok = ZS::threads == YS::threads;
};

// item -> (first kind?, slab, sub-tile): `lead` slabs of the first kind, then
// groups of [first kind of slab g + lead][second kind of slab g], then the
// last `lead` slabs of the second kind
__device__ __forceinline__ void zy_decode(long long item, int n0, int lead, int n_first, int n_second,
                                          bool& first, int& slab, int& sub) {
  const long long A = (long long)lead * n_first;
  const long long B = (long long)(n0 - lead) * (n_first + n_second);
  if (item < A) {
    first = true;
    slab = int(item / n_first);
    sub = int(item % n_first);
  } else if (item < A + B) {
    const long long i = item - A;
    const int g = int(i / (n_first + n_second));
    const int r = int(i % (n_first + n_second));
    if (r < n_first) {
      first = true;
      slab = lead + g;
      sub = r;
    } else {
      first = false;
      slab = g;
      sub = r - n_first;
    }
  } else {
    const long long i = item - A - B;
    first = false;
    slab = n0 - lead + int(i / n_second);
    sub = int(i % n_second);
  }
}

// thread 0 waits until `count` items of the slab are done, polling at most
// `limit` times; false (for the whole CTA) when it gave up
__device__ __forceinline__ bool zy_wait(const unsigned* done, int* err, int slab, unsigned count, unsigned limit) {
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    const volatile unsigned* d = done + slab;
    bool ok = false;
    for (unsigned it = 0; it < limit; ++it) {
      if (*d >= count) {
        ok = true;
        break;
      }
      __nanosleep(128);
    }
    if (!ok) atomicExch(err, 1);
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ void zy_signal(unsigned* done, int slab) {
  __syncthreads();   // every thread's stores of the item are issued
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(done + slab, 1u);
  }
}

// control words (zeroed per launch): [0] next item, [1 + s] items done in
// slab s; err is the plan's error word (sticky until the host reads it)
template <typename T, int M, int L, bool FWD>
__global__ void __launch_bounds__(ZyShape<T, M, L>::threads, 2)
k_zy_persistent(const ContigArgs z, const StridedArgs y, unsigned* ctl, int* err, int n0, int lead) {
  typedef ZyShape<T, M, L> SH;
  typedef typename CT<T>::V V;
  __shared__ long long s_item;
  unsigned* next = ctl;
  unsigned* done = ctl + 1;
  const int n_first = FWD ? SH::ZI : SH::YI, n_second = FWD ? SH::YI : SH::ZI;
  const long long total = (long long)n0 * (SH::ZI + SH::YI);
  const long long zslab = (long long)L;                       // z rows per slab
  const long long spec_slab = (long long)L * (M + 1);        // complex per spectrum slab
  for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(next, 1u);
    __syncthreads();
    const long long item = s_item;
    if (item >= total) break;
    bool first;
    int slab, sub;
    zy_decode(item, n0, lead, n_first, n_second, first, slab, sub);
    const bool is_z = first == FWD;
    if (is_z) {
      ContigArgs a = z;
      if (FWD) {
        a.in = static_cast<const T*>(z.in) + slab * zslab * z.in_dist;
        a.out = static_cast<V*>(z.out) + slab * zslab * z.out_dist;
        a.nlines = zslab;
        zr2c_tile<T, M>(a, sub);
        zy_signal(done, slab);
      } else if (zy_wait(done, err, slab, SH::YI, z.wait_limit)) {
        a.in = static_cast<const V*>(z.in) + slab * zslab * z.in_dist;
        a.out = static_cast<T*>(z.out) + slab * zslab * z.out_dist;
        a.nlines = zslab;
        zc2r_tile<T, M, 0, 0, true>(a, sub);
      }
    } else if (!FWD || zy_wait(done, err, slab, SH::ZI, y.wait_limit)) {
      StridedArgs a = y;
      a.in = static_cast<const V*>(y.in) + slab * spec_slab;
      a.out = static_cast<V*>(y.out) + slab * spec_slab;
      a.ncols = a.cps = M + 1;
      strided_tile<T, L, 0, 0, 0, true>(a, sub);
      if (!FWD) zy_signal(done, slab);
    }
    __syncthreads();   // shared memory and s_item are free for the next item
  }
}

template <typename T, int M, int L>
static bool run_zy(bool forward, const ContigArgs& z, const StridedArgs& y, unsigned* ctl, int* err, int n0,
                   int lead, cudaStream_t s) {
  typedef ZyShape<T, M, L> SH;
  static_assert(SH::ok, "z and y tiles of the persistent kernel have one thread count");
  auto k = forward ? k_zy_persistent<T, M, L, true> : k_zy_persistent<T, M, L, false>;
  // resident CTAs on the whole device (the grid of a persistent kernel), per
  // device and direction; -1 when the kernel cannot run there
  static PerDevice blocks[2];
  const int nb = per_device(blocks[forward ? 0 : 1], [&] {
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(SH::smem)) != cudaSuccess) return -1;
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, SH::threads, SH::smem) != cudaSuccess || per_sm < 1)
      return -1;
    return per_sm * sms;
  });
  if (nb < 1) return false;
  const long long items = (long long)n0 * (SH::ZI + SH::YI);
  const unsigned grid = unsigned(items < nb ? items : nb);
  k<<<grid, SH::threads, SH::smem, s>>>(z, y, ctl, err, n0, lead);
  count_launch();
  return true;
}

bool zy_persistent_available(bool dbl, int M, int L) {
  return !dbl && ((M == 256 && L == 512) || (M == 128 && L == 256));
}

bool launch_zy_persistent(bool dbl, bool forward, int M, int L, const ContigArgs& z, const StridedArgs& y,
                          unsigned* ctl, int* err, int n0, int lead, cudaStream_t s) {
  if (dbl) return false;
  if (M == 256 && L == 512) return run_zy<float, 256, 512>(forward, z, y, ctl, err, n0, lead, s);
  if (M == 128 && L == 256) return run_zy<float, 128, 256>(forward, z, y, ctl, err, n0, lead, s);
  return false;
}

}  // namespace afg
