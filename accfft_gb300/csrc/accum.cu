// Row-wise accumulation of real fields, out[r][c] += in[r][c] for the first
// `len` entries of each of `rows` rows; the two arrays have their own row
// strides (the caller's real array, and a c2r result left in place in the
// padded rows of the plan's spectrum scratch).  The term-by-term sum of
// divergence_slow uses it, as the reference's daxpy does
// (src/operators_gpu.txx:337-446).  Grid-stride loop, HBM-bound.
#include "launch.h"

namespace afg {

namespace {

template <typename T>
__global__ void k_add_rows(T* __restrict__ out, long long out_row, const T* __restrict__ in, long long in_row,
                           long long rows, int len) {
  const long long n = rows * len;
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += step) {
    const long long r = i / len;
    const long long c = i - r * len;
    out[r * out_row + c] += in[r * in_row + c];
  }
}

}  // namespace

bool launch_add_rows(bool dbl, void* out, long long out_row, const void* in, long long in_row, long long rows,
                     int len, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long n = rows * len;
  long long blocks = (n + 255) / 256;
  if (blocks > 8LL * sms) blocks = 8LL * sms;
  if (blocks < 1) blocks = 1;
  if (dbl)
    k_add_rows<double><<<unsigned(blocks), 256, 0, s>>>(static_cast<double*>(out), out_row,
                                                        static_cast<const double*>(in), in_row, rows, len);
  else
    k_add_rows<float><<<unsigned(blocks), 256, 0, s>>>(static_cast<float*>(out), out_row,
                                                       static_cast<const float*>(in), in_row, rows, len);
  count_launch();
  return cudaGetLastError() == cudaSuccess;
}

}  // namespace afg
