// Laplacian of a float grid that allocates no device memory.
//
// Who needs it: code that may not call cudaMalloc - a plugin inside an
// application whose memory manager has reserved the whole device (a new
// allocation would fail or fragment that pool), or a latency-bound loop where
// an allocation could stall the device.  Such callers cannot create a plan
// (plans allocate twiddle tables and a spectrum buffer), so this entry point
// carries its own working memory.
//
// The first call on a device does the set-up (cudaGetSymbolAddress); make
// that first call before any stream capture.  All calls share the one array
// and it keeps the last call's contents: nothing in it has to start at zero
// (the spectrum is fully written by the first pass and the tables are
// rewritten by every call), but calls that overlap on the GPU race.
//
// Working memory: one file-scope __device__ array of kNoAllocBytes bytes
// holding the half spectrum and the twiddle tables.  Every GPU that loads this
// library keeps the array for the life of the process.  Host code never uses
// the array's name as an address (on the host it names a stand-in object):
// the device address is taken once per device with cudaGetSymbolAddress, with
// that device current, and passed to the kernels.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/accfft_gb300.h"
#include "args.h"
#include "launch.h"
#include "line_plan.h"

namespace afg {
void set_last_error(int code, const char* msg);
}

namespace {

constexpr size_t kNoAllocBytes = size_t(64) << 20;   // 64 MiB per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

int err(int code, const char* msg) {
  afg::set_last_error(code, msg);
  return code;
}

// device address of the working array on the current device (set-up on the
// first call per device)
int scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return err(ACCFFT_C_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return err(ACCFFT_C_EINVAL, "laplace_gpuf_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return err(ACCFFT_C_ECUDA, "laplace_gpuf_noalloc: cudaGetSymbolAddress failed");
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[dev];
  return ACCFFT_C_OK;
}

// exp(-2*pi*i*m/d) rounded to float, from an exactly reduced angle
float2 unit_root(long long m, long long d) {
  m %= d;
  if (m < 0) m += d;
  const long double q = 0.785398163397448309615660845819875721L;
  long long o = (8 * m) / d, r = 8 * m - o * d;
  long double a = q * (long double)r / (long double)d, b = q * (long double)(d - r) / (long double)d;
  long double c, s;
  switch (o) {
    case 0: c = cosl(a); s = sinl(a); break;
    case 1: c = sinl(b); s = cosl(b); break;
    case 2: c = -sinl(a); s = cosl(a); break;
    case 3: c = -cosl(b); s = sinl(b); break;
    case 4: c = -cosl(a); s = -sinl(a); break;
    case 5: c = -sinl(b); s = -cosl(b); break;
    case 6: c = sinl(a); s = -cosl(a); break;
    default: c = cosl(b); s = -sinl(b); break;
  }
  return make_float2((float)c, (float)-s);
}

// stage twiddles of the single-precision line plan of length L
void append_stage_table(std::vector<float2>& t, int L) {
  afg::LinePlan pl = afg::plan_for(L, false);
  size_t base = t.size();
  int n = afg::plan_tw_size(pl);
  t.resize(base + (n > 0 ? n : 1), make_float2(0.f, 0.f));
  for (int s = 1; s < pl.ns; ++s) {
    int Ns = afg::plan_ns_before(pl, s), R = pl.radix[s], off = afg::plan_tw_offset(pl, s);
    for (int r = 1; r < R; ++r)
      for (int k = 0; k < Ns; ++k) t[base + off + (size_t)(r - 1) * Ns + k] = unit_root((long long)k * r, (long long)Ns * R);
  }
  while (t.size() % 32) t.push_back(make_float2(0.f, 0.f));   // 256-byte aligned segments
}

}  // namespace

extern "C" int accfft_c_laplace_gpuf_noalloc(const int n[3], float* LA, const float* A, void* stream) {
  if (!n || !LA || !A) return err(ACCFFT_C_EINVAL, "laplace_gpuf_noalloc: NULL argument");
  const int N0 = n[0], N1 = n[1], N2 = n[2];
  if (N0 < 1 || N1 < 1 || N2 < 2 || N2 % 2) return err(ACCFFT_C_EINVAL, "laplace_gpuf_noalloc: sizes must be positive with N2 even");
  const int M = N2 / 2;
  if (!afg::length_supported(N0) || !afg::length_supported(N1) || !afg::length_supported(M))
    return err(ACCFFT_C_EUNSUPPORTED, "laplace_gpuf_noalloc: an axis length has no compiled kernels");
  if ((reinterpret_cast<uintptr_t>(LA) | reinterpret_cast<uintptr_t>(A)) % 8)
    return err(ACCFFT_C_EINVAL, "laplace_gpuf_noalloc: arrays must be 8-byte aligned");

  // twiddle tables of this grid: x, y, z (length N2/2), then the r2c split w_{N2}^k
  std::vector<float2> tab;
  const size_t ox = 0;
  append_stage_table(tab, N0);
  const size_t oy = tab.size();
  append_stage_table(tab, N1);
  const size_t oz = tab.size();
  append_stage_table(tab, M);
  const size_t op = tab.size();
  for (int k = 0; k <= M; ++k) tab.push_back(unit_root(k, N2));

  const long long H2 = M + 1;
  const size_t spec_bytes = ((size_t)N0 * N1 * H2 * sizeof(float2) + 255) / 256 * 256;
  const size_t need = spec_bytes + tab.size() * sizeof(float2);
  if (need > kNoAllocBytes) {
    char msg[256];
    snprintf(msg, sizeof msg,
             "laplace_gpuf_noalloc: a %dx%dx%d grid needs %zu bytes of working memory; this entry point holds "
             "%zu bytes (use a plan and accfft_c_laplace instead)",
             N0, N1, N2, need, kNoAllocBytes);
    return err(ACCFFT_C_EINVAL, msg);
  }

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the working array is the current device's: a stream of another device
  // would run the kernels against the wrong array
  if (s) {
    int cur = 0, sdev = 0;
    cudaError_t de = cudaGetDevice(&cur);
    if (de == cudaSuccess) de = cudaStreamGetDevice(s, &sdev);
    if (de != cudaSuccess) return err(ACCFFT_C_ECUDA, cudaGetErrorString(de));
    if (sdev != cur)
      return err(ACCFFT_C_EINVAL, "laplace_gpuf_noalloc: the stream belongs to another device than the current one");
  }
  unsigned char* base = nullptr;
  if (int rc = scratch_address(&base)) return rc;
  float2* spec = reinterpret_cast<float2*>(base);
  float2* tw = reinterpret_cast<float2*>(base + spec_bytes);
  // the spectrum is fully written by the first pass; only the tables are
  // refreshed (the previous call may have used another grid)
  cudaError_t e = cudaMemcpyAsync(tw, tab.data(), tab.size() * sizeof(float2), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return err(ACCFFT_C_ECUDA, cudaGetErrorString(e));

  afg::ContigArgs z{};
  z.in = A;
  z.out = spec;
  z.tw = tw + oz;
  z.tw_post = tw + op;
  z.nlines = (long long)N0 * N1;
  z.in_dist = N2;
  z.out_dist = H2;
  afg::StridedArgs y{};
  y.in = y.out = spec;
  y.tw = tw + oy;
  y.ncols = (long long)N0 * H2;
  y.cps = H2;
  y.in_slab = y.out_slab = (long long)N1 * H2;
  y.in_line = y.out_line = H2;
  afg::StridedArgs x{};
  x.in = x.out = spec;
  x.tw = tw + ox;
  x.ncols = x.cps = (long long)N1 * H2;
  x.in_line = x.out_line = (long long)N1 * H2;
  x.sym.kind = afg::SYM_LAPLACE;
  x.sym.n0 = N0;
  x.sym.n1 = N1;
  x.sym.n2 = N2;
  x.sym.h2 = (int)H2;
  x.sym.scale = 1.0 / ((double)N0 * N1 * N2);

  bool ok = afg::launch_zr2c(afg::PREC_F32, M, z, s);
  ok = ok && afg::launch_strided(afg::PREC_F32, N1, 0, y, s);
  ok = ok && afg::launch_strided(afg::PREC_F32, N0, 1, x, s);
  y.inverse = 1;
  ok = ok && afg::launch_strided(afg::PREC_F32, N1, 0, y, s);
  afg::ContigArgs zi = z;
  zi.in = spec;
  zi.out = LA;
  zi.in_dist = H2;
  zi.out_dist = N2;
  ok = ok && afg::launch_zc2r(afg::PREC_F32, M, zi, s);
  if (!ok) return err(ACCFFT_C_EUNSUPPORTED, "laplace_gpuf_noalloc: kernel dispatch failed");
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return err(ACCFFT_C_ECUDA, cudaGetErrorString(e));
  return ACCFFT_C_OK;
}
