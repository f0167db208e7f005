// Per-device launch preparation.  Function attributes (the dynamic
// shared-memory opt-in, cluster permissions) and occupancy results belong to
// one device, so a process that runs plans on several GPUs prepares each
// kernel once per device.  The cache is lock-free: two host threads that
// race on the first call both compute the same value and store it.
#pragma once
#include <atomic>

#include <cuda_runtime.h>

namespace afg {

struct PerDevice {
  static constexpr int kMaxDevices = 64;
  std::atomic<int> value[kMaxDevices];   // 0 = not computed yet (static storage: zero-initialised)
};

// The cached value for the current device, computing it on first use.
// `compute` returns a non-zero int (a flag, a count, or a negative failure
// code); a device index outside the cache recomputes every call.
template <class F>
inline int per_device(PerDevice& cache, F&& compute) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= PerDevice::kMaxDevices) return compute();
  int v = cache.value[dev].load(std::memory_order_acquire);
  if (v != 0) return v;
  v = compute();
  cache.value[dev].store(v, std::memory_order_release);
  return v;
}

// Opt a kernel in to more than 48 KiB of dynamic shared memory on the current
// device; true when the kernel may be launched with `smem` bytes.
template <typename K>
inline bool prepare_smem(PerDevice& cache, K kernel, size_t smem) {
  return per_device(cache, [&] {
           if (smem <= 48 * 1024) return 1;
           return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) == cudaSuccess
                      ? 1
                      : -1;
         }) == 1;
}

// CTAs of a persistent grid over `tiles` tiles: as many as fit the current
// device at once (SMs x resident CTAs of the kernel), at most `tiles`; 0 when
// the occupancy query fails
template <typename K>
inline long long persistent_grid(PerDevice& cache, K kernel, int threads, size_t smem, long long tiles) {
  const int occ = per_device(cache, [&] {
    int n = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) == cudaSuccess && n > 0 ? n : -1;
  });
  int dev = 0, sms = 0;
  if (occ < 1 || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    return 0;
  const long long cap = (long long)sms * occ;
  return tiles < cap ? tiles : cap;
}

}  // namespace afg
