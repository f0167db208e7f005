// Input scan of double-float transforms: the largest biased exponent of the
// doubles a transform reads first, from the exponent field with integer
// operations (no FP64 instruction).  The passes turn it into the exact
// power-of-two scale that keeps the transform inside float's exponent range
// (df_shift_of in df64.cuh).
#include "launch.h"

namespace afg {

namespace {

__device__ __forceinline__ unsigned exp_of(unsigned long long bits) { return unsigned(bits >> 52) & 0x7FFu; }

// contiguous doubles, grid-stride
__global__ void k_df_maxexp(const unsigned long long* __restrict__ x, long long n, int* out) {
  unsigned m = 0;
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += step) m = max(m, exp_of(__ldg(x + i)));
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, int(m));
}

// rows of `len` doubles, `stride` apart (the padded rows of an in-place r2c)
__global__ void k_df_maxexp_rows(const unsigned long long* __restrict__ x, long long rows, int len, long long stride,
                                 int* out) {
  unsigned m = 0;
  for (long long r = blockIdx.x; r < rows; r += gridDim.x)
    for (int c = threadIdx.x; c < len; c += blockDim.x) m = max(m, exp_of(__ldg(x + r * stride + c)));
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, int(m));
}

}  // namespace

bool launch_df_scan(const void* x, long long rows, long long len, long long stride, int* out, cudaStream_t s) {
  if (cudaMemsetAsync(out, 0, sizeof(int), s) != cudaSuccess) return false;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const auto* p = static_cast<const unsigned long long*>(x);
  if (stride == len || rows == 1) {
    const long long n = rows * len;
    long long blocks = (n + 255) / 256;
    if (blocks > 8LL * sms) blocks = 8LL * sms;
    if (blocks < 1) blocks = 1;
    k_df_maxexp<<<unsigned(blocks), 256, 0, s>>>(p, n, out);
  } else {
    long long blocks = rows < 8LL * sms ? rows : 8LL * sms;
    if (blocks < 1) blocks = 1;
    k_df_maxexp_rows<<<unsigned(blocks), 256, 0, s>>>(p, rows, int(len), stride, out);
  }
  count_launch();
  return cudaGetLastError() == cudaSuccess;
}

}  // namespace afg
