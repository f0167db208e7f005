// Plan layer of the C ABI (include/accfft_gb300.h): size bookkeeping with the
// reference's semantics, twiddle tables, scratch ownership and the pass
// sequences of every transform and operator.  All device work is issued by
// the pass kernels through the launchers in launch.h; there is no host
// fallback: a size without kernels is rejected at plan time.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <array>
#include <mutex>
#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <initializer_list>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <functional>
#include <map>
#include <string>
#include <deque>
#include <tuple>
#include <vector>

#include "../../include/accfft_gb300.h"
#include "args.h"
#include "launch.h"
#include "line_plan.h"

using namespace afg;

namespace {

thread_local std::string g_err;
thread_local int g_err_code = ACCFFT_C_OK;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  g_err_code = code;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(ACCFFT_C_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

bool packed_eligible(const accfft_c_plan* p);

// polls a bounded device-side wait makes before it gives up
// (accfft_c_set_wait_limit); the default is about half a second
constexpr unsigned kDefaultWaitLimit = 1u << 22;
std::atomic<unsigned> g_wait_limit{kDefaultWaitLimit};

// exp(-2*pi*i*m/d) with exact integer octant reduction and long-double
// evaluation on [0, pi/4]
void twiddle(long long m, long long d, long double* c, long double* s) {
  m %= d;
  if (m < 0) m += d;
  const long double q = 0.785398163397448309615660845819875721L;  // pi/4
  long long o = (8 * m) / d;
  long long r = 8 * m - o * d;
  long double phi = q * (long double)r / (long double)d;
  long double psi = q * (long double)(d - r) / (long double)d;
  long double cc = 0, ss = 0;
  switch (o) {
    case 0: cc = cosl(phi); ss = sinl(phi); break;
    case 1: cc = sinl(psi); ss = cosl(psi); break;
    case 2: cc = -sinl(phi); ss = cosl(phi); break;
    case 3: cc = -cosl(psi); ss = sinl(psi); break;
    case 4: cc = -cosl(phi); ss = -sinl(phi); break;
    case 5: cc = -sinl(psi); ss = -cosl(psi); break;
    case 6: cc = sinl(phi); ss = -cosl(phi); break;
    default: cc = cosl(psi); ss = -sinl(psi); break;
  }
  *c = cc;
  *s = -ss;   // forward sign
}

// stage twiddles of a line length (layout fixed by plan_tw_offset)
// cls: 0 float, 1 double, 2 double-float (line_plan.h plan_select)
std::vector<long double> stage_table(int L, int cls, int first_radix = 0) {
  LinePlan pl = plan_select(L, cls, first_radix);
  int n = plan_tw_size(pl);
  std::vector<long double> t(2 * (size_t)(n > 0 ? n : 1), 0.0L);
  for (int s = 1; s < pl.ns; ++s) {
    int Ns = plan_ns_before(pl, s), R = pl.radix[s], off = plan_tw_offset(pl, s);
    for (int r = 1; r < R; ++r)
      for (int k = 0; k < Ns; ++k) {
        long double c, si;
        twiddle((long long)k * r, (long long)Ns * R, &c, &si);
        size_t i = (size_t)off + (size_t)(r - 1) * Ns + k;
        t[2 * i] = c;
        t[2 * i + 1] = si;
      }
  }
  return t;
}

// Radix plan of the generic kernels (gen.cu) for a line of L: the prime
// factors (at most 31), largest first, each multiplied into the first radix
// that stays at most 32 (fewer stages: each stage is a shared-memory round
// trip); false when L has a larger prime factor, exceeds 4096 or needs more
// than kGenMaxStages stages.  Lengths of one or no stage are fine.
bool gen_factor(int L, GenPlan* g) {
  if (L < 1 || L > 4096) return false;
  std::vector<int> pf;
  int m = L;
  for (int q = 2; q * q <= m; ++q)
    while (m % q == 0) {
      pf.push_back(q);
      m /= q;
    }
  if (m > 1) pf.push_back(m);
  for (int q : pf)
    if (q > 31) return false;
  std::sort(pf.begin(), pf.end(), std::greater<int>());
  std::vector<int> rad;
  for (int q : pf) {
    bool merged = false;
    for (int& r : rad)
      if (r * q <= 32) {
          r *= q;
          merged = true;
          break;
        }
    if (!merged) rad.push_back(q);
  }
  if ((int)rad.size() > kGenMaxStages) return false;
  if (g) {
    g->L = L;
    g->nst = (int)rad.size();
    int off = 0, Ns = 1;
    for (int s = 0; s < g->nst; ++s) {
      g->radix[s] = rad[s];
      g->off[s] = off;
      off += (rad[s] - 1) * Ns;
      Ns *= rad[s];
    }
  }
  return true;
}
// stage twiddles of a generic radix plan: entry (r-1)*Ns + k of stage s is
// w_{Ns*R}^{r*k}
std::vector<long double> gen_table(const GenPlan& g) {
  std::vector<long double> t;
  int Ns = 1;
  for (int s = 0; s < g.nst; ++s) {
    const int R = g.radix[s];
    for (int r = 1; r < R; ++r)
      for (int k = 0; k < Ns; ++k) {
        long double c, sn;
        twiddle((long long)r * k, (long long)Ns * R, &c, &sn);
        t.push_back(c);
        t.push_back(sn);
      }
    Ns *= R;
  }
  if (t.empty()) t.assign(2, 0.0L);
  return t;
}

// r2c split twiddles w_{2M}^k, k = 0..M
std::vector<long double> post_table(int M) {
  std::vector<long double> t(2 * (size_t)(M + 1));
  for (int k = 0; k <= M; ++k) twiddle(k, 2LL * M, &t[2 * k], &t[2 * k + 1]);
  return t;
}

constexpr unsigned XB = 1, YB = 2, ZB = 4;

}  // namespace

// one pass of a plan recorded into a batch (accfft_c_batch_record): the
// kernel kind (afg::PassKind), line length, strided mode and arguments
struct PassRecord {
  int kind = 0, L = 0, mode = 0;
  afg::StridedArgs s{};
  afg::ContigArgs c{};
};

struct accfft_c_plan {
  int kind = 0;         // 1 = r2c, 2 = c2c
  bool dbl = false;
  int n[3] = {0, 0, 0};
  bool inplace = false;
  void* data = nullptr;
  void* data_out = nullptr;
  long long alloc_max = 0;
  int device = 0;
  // device tables: x, y and z stage twiddles (z: length N2/2 for r2c, N2 for
  // c2c) and the r2c split twiddles
  void* tw_block = nullptr;
  const void* tw_x = nullptr;
  const void* tw_y = nullptr;
  const void* tw_z = nullptr;
  const void* tw_post = nullptr;
  const void* fd_tab = nullptr;   // finite-difference Laplacian eigenvalues per axis (r2c plans)
  // stage twiddles of the tuner's alternative first radix (variant 2) of the
  // x, y and z lines (float r2c plans; nullptr where the length has none)
  const void* tw_x_alt = nullptr;
  const void* tw_y_alt = nullptr;
  const void* tw_z_alt = nullptr;
  // spectrum-sized scratch (r2c plans): out-of-place c2r and operators
  void* scratch = nullptr;
  // how the z and y passes of r2c/c2r run: 0 = one kernel each over the whole
  // grid, 1 = one cluster slab kernel, 2 = slab batches alternating z and y
  // (z(b+1) on a second stream overlaps y(b); a batch's intermediate spectrum
  // is still in L2 when the next pass reads it)
  int zy_mode = 0;
  int zy_batches = 1;
  // packed pass order of full r2c / c2r transforms of device arrays
  // (accfft_c_set_pass_order): y and x passes over the real field viewed as
  // complex [N0][N1][N2/2] (rows of a multiple of 128 bytes for the usual
  // sizes) in the plan scratch, then one z pass over mirror-paired lines that
  // finishes the real transform and writes the natural spectrum in whole
  // rows; c2r runs the same passes backwards.  Out-of-place float and double
  // plans only.
  bool packed = false;
  // record mode: the plan's passes are appended here instead of launched
  std::vector<PassRecord>* recording = nullptr;
  // radix / tile variants of the float r2c / c2r passes (variants.cu), chosen
  // by timing at plan creation under ACCFFT_MEASURE: y, x, z r2c, z c2r
  int var_y = 0, var_x = 0, var_zr = 0, var_zc = 0;
  bool tuned = false;
  cudaStream_t stream2 = nullptr;
  static constexpr int kMaxBatches = 64;
  // control words of the persistent z+y kernels (1 + N0, zeroed per launch)
  unsigned* zy_ctl = nullptr;
  int zy_lead = 32;   // slabs between a slab's first and second pass (ACCFFT_GB300_ZY_LEAD)
  // pinned-host real arrays: slab batches staged through a device ring
  static constexpr int kHostBatches = 16, kHostSlots = 3;
  // slab batches per call (ACCFFT_GB300_HOST_BATCHES, 1..16).  Four measured
  // best at 512^3 with three calls in flight: 98.8 % of the host link's
  // duplex floor against 93 % for 16, whose ~230 API calls per r2c+c2r pair
  // left the enqueue thread behind on a busy host
  int host_batches = 4;
  void* hstage = nullptr;
  long long hstage_bytes = 0;
  static_assert(1 + kHostBatches + kHostSlots <= kMaxBatches + 1, "host path events fit evb");
  cudaEvent_t evb[kMaxBatches + 2] = {};
  cudaStream_t stream = 0;
  bool blocking = true;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // 3-D operators keep their spectrum in the aligned split layout in scratch:
  // main [N0][N1][M] (rows of M = N2/2 complex, 128-byte aligned) and the
  // Nyquist plane [N0][N1] (kz = N2/2) after it
  bool split = false;
  // axes (x, y, z) whose lines have no compiled kernels run the generic
  // kernels (gen.cu) with a radix plan made here; gen_any: at least one
  bool gen[3] = {false, false, false};
  bool gen_any = false;
  afg::GenPlan gp[3] = {};
  // tensor-core form (ACCFFT_C_TC_*): 0 none, 1 3xTF32, 2 split BF16
  int tc = 0;
  // device word set by a kernel whose bounded wait gave up (tensor-core
  // completion waits, the persistent z+y kernel's waits between items).  It
  // stays set until a blocking or timed call (or accfft_c_check) reads and
  // clears it; waits_used marks plans that have launched such kernels.
  int* wait_err = nullptr;
  bool waits_used = false;
  // double plan whose kernels compute in double-float (ACCFFT_C_F64_DF);
  // df_exp receives the largest biased exponent of each transform's input
  bool df = false;
  int* df_exp = nullptr;
  // per-kernel CUDA-event profiling (accfft_c_set_profiling)
  bool profile = false;
  std::vector<cudaEvent_t> pev;
  std::vector<std::pair<std::string, int>> pending;   // label, event pair index
  std::map<std::string, std::pair<long long, double>> pstats;

  long long esz() const { return dbl ? 8 : 4; }
  int prec() const { return dbl ? (df ? PREC_DF : PREC_F64) : PREC_F32; }
  int M() const { return n[2] / 2; }
  long long H2() const { return n[2] / 2 + 1; }
  // row length (reals) of the plan's real arrays
  long long rrow() const { return inplace ? 2 * H2() : n[2]; }
};

namespace {

// ----------------------------------------------------------- local sizes
// P = 1 restatement of dfft_get_local_size_t: isize = {N0, N1, tuple}
long long local_size(int N0, int N1, int tuple, int* isize, int* istart, int real_bytes) {
  isize[0] = N0;
  isize[1] = N1;
  isize[2] = tuple;
  istart[0] = istart[1] = istart[2] = 0;
  return (long long)N0 * N1 * tuple * real_bytes;
}

long long local_size_r2c(const int* n, int* isize, int* istart, int* osize, int* ostart, int rb) {
  int s0[3], s1[3], st[3];
  long long amax = 0;
  long long nt = (long long)(n[2] / 2 + 1) * 2;
  amax = std::max(amax, local_size(n[0], n[1], (int)nt, s0, st, rb));
  amax = std::max(amax, 2 * local_size(n[0], (int)(nt / 2), n[1], s1, st, rb));
  amax = std::max(amax, 2 * local_size(n[1], (int)(nt / 2), n[0], s1, st, rb));
  // single-axis y and x transforms
  amax = std::max(amax, local_size(n[0], n[2], n[1], s1, st, rb));
  amax = std::max(amax, 2 * local_size(n[0], n[2], n[1] / 2 + 1, s1, st, rb));
  amax = std::max(amax, (long long)n[1] * n[2] * n[0] * rb);
  amax = std::max(amax, 2LL * n[1] * n[2] * (n[0] / 2 + 1) * rb);
  local_size(n[0], n[1], n[2], isize, istart, rb);
  osize[0] = n[0];
  osize[1] = n[1];
  osize[2] = n[2] / 2 + 1;
  ostart[0] = ostart[1] = ostart[2] = 0;
  return amax;
}

long long local_size_c2c(const int* n, int* isize, int* istart, int* osize, int* ostart, int rb) {
  local_size(n[0], n[1], n[2], isize, istart, rb);
  for (int i = 0; i < 3; ++i) {
    osize[i] = n[i];
    ostart[i] = 0;
  }
  return 2LL * n[0] * n[1] * n[2] * rb;
}

// -------------------------------------------------------------- plan make
accfft_c_plan* make_plan(int kind, bool dbl, const int* n, void* data, void* data_out, unsigned flags = 0) {
  g_err.clear();
  g_err_code = ACCFFT_C_OK;
  if (!n) {
    fail(ACCFFT_C_EINVAL, "plan: NULL size array");
    return nullptr;
  }
  for (int i = 0; i < 3; ++i)
    if (n[i] < 1) {
      fail(ACCFFT_C_EINVAL, "plan: size n[%d]=%d must be positive", i, n[i]);
      return nullptr;
    }
  int zlen = kind == 1 ? n[2] / 2 : n[2];
  // axes without compiled kernels take the generic kernels when their length
  // factors into primes up to 31 (the real z axis of r2c plans then as a
  // whole line of N2, odd N2 included)
  bool gen[3] = {!length_supported(n[0]), !length_supported(n[1]),
                 kind == 1 ? (n[2] % 2 != 0 || !length_supported(n[2] / 2)) : !length_supported(n[2])};
  const int glen[3] = {n[0], n[1], n[2]};
  for (int i = 0; i < 3; ++i)
    if (gen[i] && !gen_factor(glen[i], nullptr)) {
      fail(ACCFFT_C_EUNSUPPORTED, "plan: no kernels for %s length %d (sizes %dx%dx%d): lengths up to 4096 whose "
           "prime factors are at most 31", i == 0 ? "x" : i == 1 ? "y" : "z", glen[i], n[0], n[1], n[2]);
      return nullptr;
    }
  const bool gen_any = gen[0] || gen[1] || gen[2];
  if (gen_any && (dbl && (flags & ACCFFT_C_F64_DF))) {
    fail(ACCFFT_C_EUNSUPPORTED, "plan: double-float plans need compiled lengths (sizes %dx%dx%d)", n[0], n[1], n[2]);
    return nullptr;
  }
  const unsigned tcf = flags & (ACCFFT_C_TC_TF32 | ACCFFT_C_TC_BF16);
  if (tcf) {
    if (tcf == (ACCFFT_C_TC_TF32 | ACCFFT_C_TC_BF16) || kind != 1 || dbl) {
      fail(ACCFFT_C_EUNSUPPORTED, "plan: tensor-core forms are float r2c plans with one of the two flags");
      return nullptr;
    }
    if (gen_any || !tc_length_supported(n[0], false) || !tc_length_supported(n[1], false) ||
        !tc_length_supported(zlen, true)) {
      fail(ACCFFT_C_EUNSUPPORTED, "plan: no tensor-core kernels for %dx%dx%d (x, y in 128..1024, N2/2 in 128..512, "
           "powers of two)", n[0], n[1], n[2]);
      return nullptr;
    }
  }
  if ((flags & ACCFFT_C_F64_DF) && !dbl) {
    fail(ACCFFT_C_EUNSUPPORTED, "plan: ACCFFT_C_F64_DF is a flag of double plans");
    return nullptr;
  }
  auto* p = new accfft_c_plan;
  p->kind = kind;
  p->tc = tcf == ACCFFT_C_TC_TF32 ? 1 : tcf == ACCFFT_C_TC_BF16 ? 2 : 0;
  for (int i = 0; i < 3; ++i) {
    p->gen[i] = gen[i];
    if (gen[i]) gen_factor(glen[i], &p->gp[i]);
  }
  p->gen_any = gen_any;
  p->df = (flags & ACCFFT_C_F64_DF) != 0;
  p->dbl = dbl;
  for (int i = 0; i < 3; ++i) p->n[i] = n[i];
  // in place when the plan-time pointers are equal (the reference's rule);
  // two NULL pointers make an out-of-place plan
  p->inplace = (data == data_out) && data != nullptr;
  p->data = data;
  p->data_out = data_out;
  int is[3], ist[3], os[3], ost[3];
  p->alloc_max = kind == 1 ? local_size_r2c(n, is, ist, os, ost, dbl ? 8 : 4)
                           : local_size_c2c(n, is, ist, os, ost, dbl ? 8 : 4);
  cudaGetDevice(&p->device);

  // twiddle tables, rounded from long double to the plan's precision
  std::vector<std::vector<long double>> tabs;
  // the tensor-core forms run every line as radix 16 first (16 x 16 x ...)
  const int er = p->tc ? 16 : 0;
  const int cls = p->df ? 2 : (dbl ? 1 : 0);
  tabs.push_back(stage_table(n[0], cls, er));
  tabs.push_back(stage_table(n[1], cls, er));
  tabs.push_back(stage_table(zlen, cls, er));
  if (kind == 1) tabs.push_back(post_table(n[2] / 2));
  // finite-difference Laplacian eigenvalues D(k) = 2 (cos(2 pi k / N) - 1) N^2
  // for |k| = 0..N/2 of each axis (x, then y, then z; the Poisson solver's
  // method 0), padded to an even count
  if (kind == 1) {
    std::vector<long double> fd;
    for (int a = 0; a < 3; ++a) {
      for (int k = 0; k <= n[a] / 2; ++k) {
        long double c, sn;
        twiddle(k, n[a], &c, &sn);
        fd.push_back(2.0L * (c - 1.0L) * (long double)n[a] * (long double)n[a]);
      }
    }
    if (fd.size() % 2) fd.push_back(0.0L);
    tabs.push_back(fd);
  }
  // float r2c plans: the stage twiddles of each axis's alternative first
  // radix (the tuner's variant 2, variants.cu: 16 for a default of 32, 8 for 16)
  const bool alt_tables = kind == 1 && cls == 0 && !p->tc;
  int alt_e[3] = {0, 0, 0};
  if (alt_tables) {
    const int lens[3] = {n[0], n[1], zlen};
    for (int a = 0; a < 3; ++a) {
      const int e = plan_select(lens[a], 0, 0).E;
      alt_e[a] = e == 32 ? 16 : (e == 16 ? 8 : 0);
      if (alt_e[a] && plan_with_e(lens[a], alt_e[a]).E == 0) alt_e[a] = 0;
      tabs.push_back(alt_e[a] ? stage_table(lens[a], 0, alt_e[a]) : std::vector<long double>(2, 0.0L));
    }
  }
  int gen_tab[3] = {-1, -1, -1};
  for (int i = 0; i < 3; ++i)
    if (p->gen[i]) {
      gen_tab[i] = (int)tabs.size();
      tabs.push_back(gen_table(p->gp[i]));
    }
  const size_t cbytes = dbl ? 16 : 8;
  std::vector<size_t> off;
  size_t total = 0;
  for (auto& t : tabs) {
    off.push_back(total);
    total += ((t.size() / 2) * cbytes + 255) / 256 * 256;
  }
  std::vector<unsigned char> host(total, 0);
  for (size_t i = 0; i < tabs.size(); ++i) {
    auto& t = tabs[i];
    for (size_t j = 0; j < t.size(); ++j) {
      if (p->df) {
        // double-float entries: the float nearest the value, then the float
        // nearest the rest
        const float hi = (float)t[j];
        const float lo = (float)(t[j] - (long double)hi);
        memcpy(&host[off[i] + j * 8], &hi, 4);
        memcpy(&host[off[i] + j * 8 + 4], &lo, 4);
      } else if (dbl) {
        double v = (double)t[j];
        memcpy(&host[off[i] + j * 8], &v, 8);
      } else {
        float v = (float)t[j];
        memcpy(&host[off[i] + j * 4], &v, 4);
      }
    }
  }
  cudaError_t e = cudaMalloc(&p->tw_block, total);
  if (e == cudaSuccess) e = cudaMemcpy(p->tw_block, host.data(), total, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && kind == 1) e = cudaMalloc(&p->scratch, (size_t)p->alloc_max);
  if (e == cudaSuccess) e = cudaMalloc(&p->wait_err, sizeof(int));
  if (e == cudaSuccess && p->df) e = cudaMalloc(&p->df_exp, 16);
  if (e == cudaSuccess) e = cudaMemset(p->wait_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaEventCreate(&p->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&p->ev1);
  if (e != cudaSuccess) {
    cuda_fail(e, "plan: device allocation");
    accfft_c_destroy_plan(p);
    return nullptr;
  }
  if (kind == 1) {
    // second stream and events for the slab-batch pipelines (host-resident
    // real arrays, see Exec::zy)
    e = cudaStreamCreateWithFlags(&p->stream2, cudaStreamNonBlocking);
    for (int b = 0; e == cudaSuccess && b < accfft_c_plan::kMaxBatches + 2; ++b)
      e = cudaEventCreateWithFlags(&p->evb[b], cudaEventDisableTiming);
    if (e != cudaSuccess) {
      cuda_fail(e, "plan: stream creation");
      accfft_c_destroy_plan(p);
      return nullptr;
    }
    // operators keep their spectrum in the split layout when its rows of M
    // complex are 128-byte aligned (M a multiple of 16 for float, 8 for double)
    const int M = n[2] / 2;
    p->split = M >= 8 && M % (dbl ? 8 : 16) == 0 && !p->gen_any;
    if (const char* hb = getenv("ACCFFT_GB300_HOST_BATCHES")) {
      const int v = atoi(hb);
      p->host_batches = v < 1 ? 1 : (v > accfft_c_plan::kHostBatches ? accfft_c_plan::kHostBatches : v);
    }
    // ACCFFT_GB300_ZY = fused | batch<n> selects an alternative z+y schedule
    // for device-resident data (both measured slower on GB300 than the
    // default whole-grid passes; kept for comparison)
    // ACCFFT_GB300_ORDER = packed | natural: the pass order of full transforms
    const char* ord = getenv("ACCFFT_GB300_ORDER");
    p->packed = packed_eligible(p) && !(ord && std::string(ord) == "natural");
    const char* env = getenv("ACCFFT_GB300_ZY");
    std::string zy = env && !p->gen_any ? env : "";
    if (zy == "fused" && slab_available(dbl, n[1], n[2])) {
      p->zy_mode = 1;
    } else if (zy == "persistent") {
      p->zy_mode = 3;
      if (const char* le = getenv("ACCFFT_GB300_ZY_LEAD")) p->zy_lead = atoi(le) > 0 ? atoi(le) : 1;
    } else if (zy.rfind("batch", 0) == 0) {
      int nb = atoi(zy.c_str() + 5);
      p->zy_mode = 2;
      p->zy_batches = nb < 1 ? 1 : nb > accfft_c_plan::kMaxBatches ? accfft_c_plan::kMaxBatches : nb;
    }
  }
  auto* base = static_cast<unsigned char*>(p->tw_block);
  p->tw_x = base + off[0];
  p->tw_y = base + off[1];
  p->tw_z = base + off[2];
  if (kind == 1) p->tw_post = base + off[3];
  if (kind == 1) p->fd_tab = base + off[4];
  for (int i = 0; i < 3; ++i)
    if (gen_tab[i] >= 0) p->gp[i].tw = base + off[(size_t)gen_tab[i]];
  if (alt_tables) {
    p->tw_x_alt = alt_e[0] ? base + off[5] : nullptr;
    p->tw_y_alt = alt_e[1] ? base + off[6] : nullptr;
    p->tw_z_alt = alt_e[2] ? base + off[7] : nullptr;
  }
  return p;
}

// ------------------------------------------------------------ execution
// Makes the plan's device current for the lifetime of a call and restores the
// caller's afterwards, so a plan works from any current device of the process.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    int cur = 0;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// The copies between pinned host arrays and the staging rings of every plan
// on a device go through one host-to-device and one device-to-host stream of
// that device, in the order the calls were made.  Each direction of the link
// then moves one transform's slab batches after another's with no gap, and
// a c2r's copies back to the host overlap the next r2c's copies in: calls on
// several plans keep both directions busy.  With a copy stream per plan, the
// copies of calls in flight on different plans shared a direction of the
// link or took turns, depending on how the copy engines served the streams
// (measured 0.70 to 0.98 of the duplex floor for the same three-plan loop on
// one GPU).  Created on first use, kept for the life of the process.
cudaStream_t host_copy_stream(int device, bool h2d) {
  static std::mutex mu;
  static cudaStream_t streams[64][2] = {};
  if (device < 0 || device >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  cudaStream_t& s = streams[device][h2d ? 0 : 1];
  if (!s) {
    DeviceGuard guard(device);
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      s = nullptr;
    }
  }
  return s;
}

// Reads and clears the plan's wait-error word once the plan's stream is idle:
// ACCFFT_C_ECUDA when a bounded device-side wait of this call, or of an
// earlier asynchronous call of the plan, gave up.
int take_wait_error(accfft_c_plan* p, const char* fn) {
  if (!p->waits_used || !p->wait_err) return ACCFFT_C_OK;
  int flag = 0;
  cudaError_t e = cudaMemcpy(&flag, p->wait_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "reading the wait-error word");
  if (!flag) return ACCFFT_C_OK;
  cudaMemset(p->wait_err, 0, sizeof(int));
  return fail(ACCFFT_C_ECUDA,
              "%s: a device-side wait gave up (%s) in this call or an earlier asynchronous call of the plan; "
              "its results are not valid",
              fn, p->tc ? "a tensor-core stage waiting for its matrix products"
                        : "the persistent z+y kernel waiting for another item, or a pipelined strided pass "
                          "waiting for its tile loads");
}

struct Exec {
  DeviceGuard guard;   // first member: constructed before anything touches the device
  accfft_c_plan* p;
  double* timer;
  int rc = ACCFFT_C_OK;
  int weight = 0;   // adjoint weighting of the z passes (ContigArgs::weight)

  Exec(accfft_c_plan* plan, double* t) : guard(plan->device), p(plan), timer(t) {
    if ((p->blocking || timer) && !p->recording) cudaEventRecord(p->ev0, p->stream);
  }
  bool ok() const { return rc == ACCFFT_C_OK; }
  // launch, or append to the batch the plan is recording into (float passes
  // with a grouped kernel only: strided modes 0 and 1, z r2c and z c2r)
  bool record(int kind, int L, int mode, const StridedArgs* sa, const ContigArgs* ca) {
    PassRecord r;
    r.kind = kind;
    r.L = L;
    r.mode = mode;
    if (sa) r.s = *sa;
    if (ca) r.c = *ca;
    const void* args = sa ? static_cast<const void*>(&r.s) : static_cast<const void*>(&r.c);
    if ((kind == PK_STRIDED && mode > 1) || grouped_tiles(kind, L, args) < 0) {
      if (ok()) rc = fail(ACCFFT_C_EUNSUPPORTED, "batch: pass of length %d has no grouped kernel "
                          "(float plain and symbol passes of lengths up to 256)", L);
      return true;
    }
    p->recording->push_back(r);
    return true;
  }
  bool go_strided(int L, int mode, const StridedArgs& a, cudaStream_t st) {
    if (p->recording) return record(PK_STRIDED, L, mode, &a, nullptr);
    return launch_strided(p->prec(), L, mode, a, st);
  }
  bool go_zr2c(int M, const ContigArgs& a, cudaStream_t st) {
    if (p->recording) return record(PK_ZR2C, M, 0, nullptr, &a);
    return launch_zr2c(p->prec(), M, a, st);
  }
  bool go_zc2r(int M, const ContigArgs& a, cudaStream_t st) {
    if (p->recording) return record(PK_ZC2R, M, 0, nullptr, &a);
    return launch_zc2r(p->prec(), M, a, st);
  }
  // kernels a batch cannot record: the call fails while the plan records
  bool not_recordable(const char* what) {
    if (!p->recording) return false;
    if (ok()) rc = fail(ACCFFT_C_EUNSUPPORTED, "batch: %s cannot be recorded into a batch", what);
    return true;
  }
  // double-float plans: the largest exponent of the transform's input (rows
  // of len doubles, stride apart), read by every pass of the transform
  void df_scan(const void* x, long long rows, long long len, long long stride) {
    if (!ok() || !p->df) return;
    if (!timed("df_scan", p->stream, [&] { return launch_df_scan(x, rows, len, stride, p->df_exp, p->stream); }))
      rc = fail(ACCFFT_C_ECUDA, "double-float input scan: launch failed");
  }
  // run one launcher; with profiling on, bracket it with CUDA events on its stream
  template <class F>
  bool timed(const char* label, cudaStream_t st, F&& launch) {
    if (!p->profile || p->recording) return launch();
    size_t k = p->pending.size();
    if (k >= 512) {   // fold before the event pool grows further
      fold_profile(p);
      k = 0;
    }
    while (p->pev.size() < 2 * (k + 1)) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return launch();
      p->pev.push_back(e);
    }
    cudaEventRecord(p->pev[2 * k], st);
    bool r = launch();
    cudaEventRecord(p->pev[2 * k + 1], st);
    p->pending.emplace_back(label, (int)k);
    return r;
  }
  static void fold_profile(accfft_c_plan* q) {
    for (auto& rec : q->pending) {
      float ms = 0;
      cudaEventSynchronize(q->pev[2 * rec.second + 1]);
      if (cudaEventElapsedTime(&ms, q->pev[2 * rec.second], q->pev[2 * rec.second + 1]) == cudaSuccess) {
        auto& st = q->pstats[rec.first];
        st.first += 1;
        st.second += ms;
      }
    }
    q->pending.clear();
  }
  void unsupported(const char* what, int L) {
    if (ok()) rc = fail(ACCFFT_C_EUNSUPPORTED, "%s: no kernel for length %d", what, L);
  }
  void strided(const void* in, void* out, const void* tw, int L, long long ncols, long long cps, long long slab,
               long long line, int inverse) {
    if (!ok()) return;
    const int axis = tw == p->tw_x ? 0 : 1;
    if (p->gen[axis]) {
      gen_strided(axis, in, out, ncols, cps, slab, line, inverse,
                  axis == 0 ? (inverse ? "x_inv" : "x") : (inverse ? "y_inv" : "y"));
      return;
    }
    StridedArgs a{};
    a.dfx = p->df_exp;
    a.in = in;
    a.out = out;
    a.tw = tw;
    a.ncols = ncols;
    a.cps = cps;
    a.in_slab = a.out_slab = slab;
    a.in_line = a.out_line = line;
    a.inverse = inverse;
    a.wait_limit = g_wait_limit.load();
    if (!p->tc && !p->recording) a.variant = tw == p->tw_x ? p->var_x : p->var_y;
    if (a.variant == 2) a.tw = tw == p->tw_x ? p->tw_x_alt : p->tw_y_alt;
    a.wait_err = p->wait_err;
    if (p->tc || a.variant == 4) p->waits_used = true;
    if (!timed(tw == p->tw_x ? (inverse ? "x_inv" : "x") : (inverse ? "y_inv" : "y"), p->stream, [&] {
          return p->tc ? launch_strided_tc(p->tc, L, a, p->wait_err, p->stream) : go_strided(L, 0, a, p->stream);
        }))
      unsupported("strided pass", L);
  }
  void strided_sym(const void* in, void* out, const void* acc, const void* tw, int L, long long ncols, long long cps,
                   long long slab, long long line, const SymArgs& sym, const char* label) {
    if (!ok()) return;
    StridedArgs a{};
    a.dfx = p->df_exp;
    a.in = in;
    a.out = out;
    a.acc = acc;
    a.tw = tw;
    a.ncols = ncols;
    a.cps = cps;
    a.in_slab = a.out_slab = slab;
    a.in_line = a.out_line = line;
    a.sym = sym;
    const int mode = acc ? 4 : 1;   // fused pass, with the accumulate input when given
    if (!timed(label, p->stream, [&] { return go_strided(L, mode, a, p->stream); }))
      unsupported("symbol pass", L);
  }
  // y pass over an [N0][N1][h] complex array, x pass over [N0][N1*h]
  // the symbol multiply of an operator that runs as r2c, symbol, c2r
  // (double-float plans, plans with generic-length axes) over the natural
  // spectrum in the plan scratch
  void sym_spectrum(void* spec, const SymArgs& s) {
    if (!ok()) return;
    const long long cols = (long long)p->n[1] * p->H2();
    if (!timed("sym", p->stream, [&] { return launch_sym_spectrum(p->dbl, spec, p->n[0], cols, s, p->stream); }))
      rc = fail(ACCFFT_C_ECUDA, "operator: symbol pass launch failed");
  }
  // lines of an axis without compiled kernels (gen.cu)
  void gen_strided(int axis, const void* in, void* out, long long ncols, long long cps, long long slab,
                   long long line, int inverse, const char* label) {
    if (!ok() || not_recordable("a pass of a length without compiled kernels")) return;
    GenArgs g{};
    g.g = p->gp[axis];
    g.in = in;
    g.out = out;
    g.nlines = ncols;
    g.cps = cps;
    g.in_slab = g.out_slab = slab;
    g.in_line = g.out_line = line;
    g.inverse = inverse;
    g.tc = gen_lines_per_cta(g.g.L, p->dbl);
    if (!timed(label, p->stream, [&] { return launch_gen(p->prec(), 0, g, p->stream); }))
      rc = fail(ACCFFT_C_ECUDA, "%s: generic pass launch failed (length %d)", label, g.g.L);
  }
  // z lines of an axis without compiled kernels: mode 1 c2c, 2 r2c, 3 c2r
  void gen_z(int mode, const void* in, void* out, long long in_dist, long long out_dist, int inverse,
             const char* label) {
    if (!ok() || not_recordable("a pass of a length without compiled kernels")) return;
    if (weight) {
      rc = fail(ACCFFT_C_EUNSUPPORTED, "%s: adjoint weighting needs compiled z lengths", label);
      return;
    }
    GenArgs g{};
    g.g = p->gp[2];
    g.in = in;
    g.out = out;
    g.nlines = (long long)p->n[0] * p->n[1];
    g.in_dist = in_dist;
    g.out_dist = out_dist;
    g.inverse = inverse;
    g.tc = gen_lines_per_cta(g.g.L, p->dbl);
    if (!timed(label, p->stream, [&] { return launch_gen(p->prec(), mode, g, p->stream); }))
      rc = fail(ACCFFT_C_ECUDA, "%s: generic pass launch failed (length %d)", label, g.g.L);
  }
  void ypass(const void* in, void* out, long long h, int inverse) {
    strided(in, out, p->tw_y, p->n[1], (long long)p->n[0] * h, h, (long long)p->n[1] * h, h, inverse);
  }
  void xpass(const void* in, void* out, long long h, int inverse) {
    long long c = (long long)p->n[1] * h;
    strided(in, out, p->tw_x, p->n[0], c, c, 0, c, inverse);
  }
  void zr2c(const void* in, void* out, long long in_row) {
    if (!ok()) return;
    if (p->gen[2]) {
      gen_z(2, in, out, in_row, p->H2(), 0, "z_r2c");
      return;
    }
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.weight = weight;
    a.in = in;
    a.out = out;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = (long long)p->n[0] * p->n[1];
    a.in_dist = in_row;
    a.out_dist = p->H2();
    a.wait_limit = g_wait_limit.load();
    if (!p->tc && !p->recording) a.variant = p->var_zr;
    if (a.variant == 2) a.tw = p->tw_z_alt;
    if (p->tc) p->waits_used = true;
    if (!timed("z_r2c", p->stream, [&] {
          return p->tc ? launch_z_tc(p->tc, true, p->M(), a, p->wait_err, p->stream)
                       : go_zr2c(p->M(), a, p->stream);
        }))
      unsupported("z r2c pass", p->M());
  }
  void zc2r(const void* in, void* out, long long out_row) {
    if (!ok()) return;
    if (p->gen[2]) {
      gen_z(3, in, out, p->H2(), out_row, 0, "z_c2r");
      return;
    }
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.weight = weight;
    a.in = in;
    a.out = out;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = (long long)p->n[0] * p->n[1];
    a.in_dist = p->H2();
    a.out_dist = out_row;
    a.wait_limit = g_wait_limit.load();
    if (!p->tc && !p->recording) a.variant = p->var_zc;
    if (a.variant == 2) a.tw = p->tw_z_alt;
    if (p->tc) p->waits_used = true;
    if (!timed("z_c2r", p->stream, [&] {
          return p->tc ? launch_z_tc(p->tc, false, p->M(), a, p->wait_err, p->stream)
                       : go_zc2r(p->M(), a, p->stream);
        }))
      unsupported("z c2r pass", p->M());
  }
  // z passes of the packed order: complex lines of M (the packed real field,
  // dense rows) taken in mirror pairs <-> the natural half spectrum
  long long mirror_pairs() const {
    const long long n0 = p->n[0], n1 = p->n[1];
    return (n0 - 1) / 2 * n1 + (1 + (n0 % 2 == 0)) * (n1 / 2 + 1);
  }
  void zr2c_pairs(const void* in, void* out) {
    if (!ok()) return;
    ContigArgs a{};
    a.in = in;
    a.out = out;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = 2 * mirror_pairs();
    a.in_dist = 2LL * p->M();
    a.out_dist = p->H2();
    a.pair_n0 = p->n[0];
    a.pair_n1 = p->n[1];
    a.variant = p->recording ? 0 : p->var_zr;
    if (a.variant == 2) a.tw = p->tw_z_alt;
    if (!timed("z_r2c", p->stream, [&] { return go_zr2c(p->M(), a, p->stream); }))
      unsupported("z r2c pass (mirror pairs)", p->M());
  }
  void zc2r_pairs(const void* in, void* out) {
    if (!ok()) return;
    ContigArgs a{};
    a.in = in;
    a.out = out;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = 2 * mirror_pairs();
    a.in_dist = p->H2();
    a.out_dist = 2LL * p->M();
    a.pair_n0 = p->n[0];
    a.pair_n1 = p->n[1];
    a.variant = p->recording ? 0 : p->var_zc;
    if (a.variant == 2) a.tw = p->tw_z_alt;
    if (!timed("z_c2r", p->stream, [&] { return go_zc2r(p->M(), a, p->stream); }))
      unsupported("z c2r pass (mirror pairs)", p->M());
  }
  // out[r][c] += in[r][c] over the plan's N0*N1 real rows
  void add_rows(void* out, long long out_row, const void* in, long long in_row, long long rows, int len) {
    if (!ok() || not_recordable("the row accumulation of divergence_slow")) return;
    if (!timed("add", p->stream, [&] { return launch_add_rows(p->dbl, out, out_row, in, in_row, rows, len, p->stream); }))
      rc = fail(ACCFFT_C_ECUDA, "row accumulation: launch failed");
  }
  // z passes and y pass restricted to slabs [s0, s0 + ns) on stream st
  // (the real side `in` / `out` points at the batch's first row)
  void zr2c_slabs(const void* in, void* out, long long in_row, long long s0, long long ns, cudaStream_t st) {
    if (!ok()) return;
    const long long N1 = p->n[1];
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.weight = weight;
    a.in = in;
    a.out = static_cast<char*>(out) + s0 * N1 * p->H2() * 2 * p->esz();
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = ns * N1;
    a.in_dist = in_row;
    a.out_dist = p->H2();
    if (!timed("z_r2c", st, [&] { return go_zr2c(p->M(), a, st); })) unsupported("z r2c pass", p->M());
  }
  void zc2r_slabs(const void* in, void* out, long long out_row, long long s0, long long ns, cudaStream_t st) {
    if (!ok()) return;
    const long long N1 = p->n[1];
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.weight = weight;
    a.in = static_cast<const char*>(in) + s0 * N1 * p->H2() * 2 * p->esz();
    a.out = out;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = ns * N1;
    a.in_dist = p->H2();
    a.out_dist = out_row;
    if (!timed("z_c2r", st, [&] { return go_zc2r(p->M(), a, st); })) unsupported("z c2r pass", p->M());
  }
  void ypass_slabs(const void* in, void* out, int inverse, long long s0, long long ns, cudaStream_t st) {
    if (!ok()) return;
    const long long N1 = p->n[1], h = p->H2();
    const long long off = s0 * N1 * h * 2 * p->esz();
    StridedArgs a{};
    a.dfx = p->df_exp;
    a.in = static_cast<const char*>(in) + off;
    a.out = static_cast<char*>(out) + off;
    a.tw = p->tw_y;
    a.ncols = ns * h;
    a.cps = h;
    a.in_slab = a.out_slab = N1 * h;
    a.in_line = a.out_line = h;
    a.inverse = inverse;
    if (!timed(inverse ? "y_inv" : "y", st, [&] { return go_strided(p->n[1], 0, a, st); }))
      unsupported("strided pass", p->n[1]);
  }
  // z r2c then y forward (forward = true), or y backward then z c2r, over
  // the whole grid of device arrays (mid: the spectrum the inverse y pass
  // writes).  Alternative schedules: the cluster slab kernel (zy_mode 1) or
  // slab batches with z and y on two streams (zy_mode 2).
  void zy(bool forward, const void* in, void* mid, void* out, long long row) {
    if (!ok()) return;
    if (p->zy_mode == 1 && weight == 0) {
      slab(forward, in, out);
      return;
    }
    if (p->zy_mode == 3 && weight == 0 && zy_persistent_available(p->dbl, p->M(), p->n[1])) {
      zy_persistent(forward, in, mid, out, row);
      return;
    }
    const long long N0 = p->n[0];
    int nb = p->zy_mode == 2 ? p->zy_batches : 1;
    if (nb > N0) nb = (int)N0;
    cudaStream_t A = p->stream, B = nb > 1 ? p->stream2 : p->stream;
    if (B != A) {
      cudaEventRecord(p->evb[0], A);
      cudaStreamWaitEvent(B, p->evb[0], 0);
    }
    for (int b = 0; b < nb; ++b) {
      const long long s0 = N0 * b / nb, s1 = N0 * (b + 1) / nb;
      // forward: z on A, y on B; inverse: y on A, z on B
      if (forward) zr2c_slabs(real_at(in, s0, row), out, row, s0, s1 - s0, A);
      else ypass_slabs(in, mid, 1, s0, s1 - s0, A);
      if (B != A) {
        cudaEventRecord(p->evb[1 + b], A);
        cudaStreamWaitEvent(B, p->evb[1 + b], 0);
      }
      if (forward) ypass_slabs(out, out, 0, s0, s1 - s0, B);
      else zc2r_slabs(mid, real_at(out, s0, row), row, s0, s1 - s0, B);
    }
    if (B != A) {
      cudaEventRecord(p->evb[nb + 1], B);
      cudaStreamWaitEvent(A, p->evb[nb + 1], 0);
    }
  }
  // z and y in one persistent kernel (zy_fused.cu); mid is the spectrum the
  // backward y pass writes and the z c2r pass reads
  void zy_persistent(bool forward, const void* in, void* mid, void* out, long long row) {
    const long long N0 = p->n[0], H = p->H2();
    const size_t ctl_bytes = size_t(1 + N0) * sizeof(unsigned);
    if (!p->zy_ctl) {
      cudaError_t e = cudaMalloc(&p->zy_ctl, ctl_bytes);
      if (e != cudaSuccess) {
        p->zy_ctl = nullptr;
        rc = cuda_fail(e, "execute: control words of the persistent z+y kernel");
        return;
      }
    }
    cudaError_t e = cudaMemsetAsync(p->zy_ctl, 0, ctl_bytes, p->stream);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "execute: clearing the persistent kernel's control words");
      return;
    }
    ContigArgs z{};
    z.dfx = p->df_exp;
    z.tw = p->tw_z;
    z.tw_post = p->tw_post;
    StridedArgs y{};
    y.dfx = p->df_exp;
    y.tw = p->tw_y;
    y.in_line = y.out_line = H;
    if (forward) {
      z.in = in;
      z.in_dist = row;
      z.out = out;
      z.out_dist = H;
      y.in = y.out = out;
    } else {
      y.in = in;
      y.out = mid;
      y.inverse = 1;
      z.in = mid;
      z.in_dist = H;
      z.out = out;
      z.out_dist = row;
    }
    z.wait_limit = y.wait_limit = g_wait_limit.load();
    p->waits_used = true;
    int lead = p->zy_lead;
    if (lead > N0) lead = int(N0);
    if (!timed(forward ? "zy_persistent" : "yz_persistent", p->stream, [&] {
          return launch_zy_persistent(p->dbl, forward, p->M(), p->n[1], z, y, p->zy_ctl, p->wait_err, int(N0), lead,
                                      p->stream);
        }))
      unsupported("persistent z+y pass", p->M());
  }
  static const void* real_at(const void* base, long long s0, long long row, long long N1, long long esz) {
    return static_cast<const char*>(base) + s0 * N1 * row * esz;
  }
  const void* real_at(const void* base, long long s0, long long row) const {
    return real_at(base, s0, row, p->n[1], p->esz());
  }
  void* real_at(void* base, long long s0, long long row) const {
    return const_cast<void*>(real_at(static_cast<const void*>(base), s0, row, p->n[1], p->esz()));
  }
  // The same z+y work when the real array lives in pinned host memory: the
  // copy engine moves slab batches between the host array and a ring of
  // kHostSlots device staging slots on the plan's second stream, while the
  // plan's stream runs the z and y kernels of the batches already staged.
  // Host-to-device and device-to-host copies use separate engines, so an
  // r2c on one plan overlaps a c2r on another.
  void zy_host(bool forward, const void* in, void* mid, void* out, long long row) {
    if (not_recordable("a pinned-host array")) return;
    if (!ok()) return;
    const long long N0 = p->n[0], N1 = p->n[1];
    const int nb = (int)std::min<long long>(N0, p->host_batches);
    const long long slab_rows = (N0 + nb - 1) / nb;                 // largest batch, in slabs
    const long long slot_bytes = slab_rows * N1 * row * p->esz();
    if (!ensure_stage(slot_bytes)) return;
    auto slot = [&](int b) { return static_cast<char*>(p->hstage) + (b % accfft_c_plan::kHostSlots) * slot_bytes; };
    cudaStream_t A = p->stream, C = host_copy_stream(p->device, forward);
    if (!C) C = p->stream2;
    cudaEvent_t* ev_start = &p->evb[0];
    cudaEvent_t* ev_copy = &p->evb[1];                               // nb events: batch b moved
    cudaEvent_t* ev_free = &p->evb[1 + accfft_c_plan::kHostBatches]; // kHostSlots: slot reusable
    cudaEventRecord(*ev_start, A);
    cudaStreamWaitEvent(C, *ev_start, 0);
    for (int b = 0; b < nb && ok(); ++b) {
      const long long s0 = N0 * b / nb, s1 = N0 * (b + 1) / nb, ns = s1 - s0;
      const size_t bytes = (size_t)(ns * N1 * row * p->esz());
      const int k = b % accfft_c_plan::kHostSlots;
      if (forward) {
        if (b >= accfft_c_plan::kHostSlots) cudaStreamWaitEvent(C, ev_free[k], 0);
        copy("h2d", C, slot(b), real_at(in, s0, row), bytes);
        cudaEventRecord(ev_copy[b], C);
        cudaStreamWaitEvent(A, ev_copy[b], 0);
        zr2c_slabs(slot(b), out, row, s0, ns, A);
        cudaEventRecord(ev_free[k], A);
        ypass_slabs(out, out, 0, s0, ns, A);
      } else {
        ypass_slabs(in, mid, 1, s0, ns, A);
        if (b >= accfft_c_plan::kHostSlots) cudaStreamWaitEvent(A, ev_free[k], 0);
        zc2r_slabs(mid, slot(b), row, s0, ns, A);
        cudaEventRecord(ev_copy[b], A);
        cudaStreamWaitEvent(C, ev_copy[b], 0);
        copy("d2h", C, real_at(out, s0, row), slot(b), bytes);
        cudaEventRecord(ev_free[k], C);
      }
    }
    // the plan's stream ends after the last copy
    cudaEventRecord(p->evb[accfft_c_plan::kMaxBatches + 1], C);
    cudaStreamWaitEvent(A, p->evb[accfft_c_plan::kMaxBatches + 1], 0);
  }
  // y pass of the packed order over ns slabs of dense rows (M complex), from
  // in_base to out_base (the first slab of each), on stream st
  void ypass_dense(const void* in_base, void* out_base, int inverse, long long ns, cudaStream_t st) {
    if (!ok()) return;
    const long long N1 = p->n[1], M = p->M();
    StridedArgs a{};
    a.in = in_base;
    a.out = out_base;
    a.tw = p->tw_y;
    a.ncols = ns * M;
    a.cps = M;
    a.in_slab = a.out_slab = N1 * M;
    a.in_line = a.out_line = M;
    a.inverse = inverse;
    a.variant = p->recording ? 0 : p->var_y;
    if (a.variant == 2) a.tw = p->tw_y_alt;
    if (!timed(inverse ? "y_inv" : "y", st, [&] { return go_strided(p->n[1], 0, a, st); }))
      unsupported("strided pass", p->n[1]);
  }
  // The packed order with the real array in pinned host memory (r2c input or
  // c2r output), moved in slab batches through the staging ring on the
  // plan's second stream, overlapped with the y passes of the batches
  // already staged; the x and z passes follow (r2c) or precede (c2r) on the
  // plan's stream.  Same kernels, so the same results as device arrays.
  void packed_host(bool forward, const void* in, void* out) {
    if (not_recordable("a pinned-host array")) return;
    if (!ok()) return;
    const long long N0 = p->n[0], N1 = p->n[1], M = p->M(), row = p->n[2];
    const int nb = (int)std::min<long long>(N0, p->host_batches);
    const long long slab_rows = (N0 + nb - 1) / nb;
    const long long slot_bytes = slab_rows * N1 * row * p->esz();
    if (!ensure_stage(slot_bytes)) return;
    auto slot = [&](int b) { return static_cast<char*>(p->hstage) + (b % accfft_c_plan::kHostSlots) * slot_bytes; };
    auto dense_at = [&](long long s0) { return static_cast<char*>(p->scratch) + s0 * N1 * M * 2 * p->esz(); };
    cudaStream_t A = p->stream, C = host_copy_stream(p->device, forward);
    if (!C) C = p->stream2;
    cudaEvent_t* ev_start = &p->evb[0];
    cudaEvent_t* ev_copy = &p->evb[1];
    cudaEvent_t* ev_free = &p->evb[1 + accfft_c_plan::kHostBatches];
    void* sc = p->scratch;
    if (!forward) {
      zc2r_pairs(in, sc);
      xpass(sc, sc, M, 1);
    }
    cudaEventRecord(*ev_start, A);
    cudaStreamWaitEvent(C, *ev_start, 0);
    for (int b = 0; b < nb && ok(); ++b) {
      const long long s0 = N0 * b / nb, s1 = N0 * (b + 1) / nb, ns = s1 - s0;
      const size_t bytes = (size_t)(ns * N1 * row * p->esz());
      const int k = b % accfft_c_plan::kHostSlots;
      if (forward) {
        if (b >= accfft_c_plan::kHostSlots) cudaStreamWaitEvent(C, ev_free[k], 0);
        copy("h2d", C, slot(b), real_at(in, s0, row), bytes);
        cudaEventRecord(ev_copy[b], C);
        cudaStreamWaitEvent(A, ev_copy[b], 0);
        ypass_dense(slot(b), dense_at(s0), 0, ns, A);
        cudaEventRecord(ev_free[k], A);
      } else {
        if (b >= accfft_c_plan::kHostSlots) cudaStreamWaitEvent(A, ev_free[k], 0);
        ypass_dense(dense_at(s0), slot(b), 1, ns, A);
        cudaEventRecord(ev_copy[b], A);
        cudaStreamWaitEvent(C, ev_copy[b], 0);
        copy("d2h", C, real_at(out, s0, row), slot(b), bytes);
        cudaEventRecord(ev_free[k], C);
      }
    }
    cudaEventRecord(p->evb[accfft_c_plan::kMaxBatches + 1], C);
    cudaStreamWaitEvent(A, p->evb[accfft_c_plan::kMaxBatches + 1], 0);
    if (forward) {
      xpass(sc, sc, M, 0);
      zr2c_pairs(sc, out);
    }
  }
  bool ensure_stage(long long slot_bytes) {
    const long long need = slot_bytes * accfft_c_plan::kHostSlots;
    if (p->hstage_bytes >= need) return true;
    // the old ring may still be in use by earlier calls on the plan's streams
    cudaStreamSynchronize(p->stream);
    cudaStreamSynchronize(p->stream2);
    if (p->hstage) cudaFree(p->hstage);
    p->hstage = nullptr;
    p->hstage_bytes = 0;
    cudaError_t e = cudaMalloc(&p->hstage, (size_t)need);
    if (e != cudaSuccess) {
      p->hstage = nullptr;
      rc = cuda_fail(e, "execute: staging buffer for host arrays");
      return false;
    }
    p->hstage_bytes = need;
    return true;
  }
  void copy(const char* label, cudaStream_t st, void* dst, const void* src, size_t bytes) {
    if (!ok()) return;
    cudaError_t e = cudaSuccess;
    timed(label, st, [&] {
      e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st);
      return true;
    });
    if (e != cudaSuccess) rc = cuda_fail(e, "execute: host copy");
  }
  void zc2c(const void* in, void* out, int inverse) {
    if (!ok() || not_recordable("a z c2c pass")) return;
    if (p->gen[2]) {
      gen_z(1, in, out, p->n[2], p->n[2], inverse, "z_c2c");
      return;
    }
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.in = in;
    a.out = out;
    a.tw = p->tw_z;
    a.nlines = (long long)p->n[0] * p->n[1];
    a.in_dist = a.out_dist = p->n[2];
    a.inverse = inverse;
    if (!timed("z_c2c", p->stream, [&] { return launch_zc2c(p->prec(), p->n[2], a, p->stream); }))
      unsupported("z c2c pass", p->n[2]);
  }
  void zsym(const void* in, void* out, const void* acc, long long row, const SymArgs& sym) {
    if (!ok() || not_recordable("a z derivative pass")) return;
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.in = in;
    a.out = out;
    a.acc = acc;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = (long long)p->n[0] * p->n[1];
    a.in_dist = a.out_dist = row;
    a.sym = sym;
    if (!timed("z_deriv", p->stream, [&] { return launch_zsym(p->prec(), p->M(), a, p->stream); }))
      unsupported("z symbol pass", p->M());
  }
  void slab(bool forward, const void* in, void* out) {
    if (!ok()) return;
    SlabArgs a{};
    a.in = in;
    a.out = out;
    a.tw_y = p->tw_y;
    a.tw_z = p->tw_z;
    a.tw_post = p->tw_post;
    a.n0 = p->n[0];
    a.real_row = p->rrow();
    if (!timed(forward ? "zy_slab" : "yz_slab", p->stream,
               [&] { return launch_slab(p->dbl, p->n[1], p->n[2], forward, a, p->stream); }))
      rc = fail(ACCFFT_C_ECUDA, "slab pass launch failed");
  }
  // single-axis real transform along x (axis 0) or y (axis 1) of an
  // unpadded [N0][N1][N2] real array (the reference's x-only / y-only
  // layouts, src/accfft_gpu.cpp:1319-1604): adjacent z columns are packed as
  // one complex column; mode 2 = r2c, 3 = c2r
  void pair_axis(int axis, int mode, const void* in, void* out) {
    if (!ok()) return;
    const long long N0 = p->n[0], N1 = p->n[1], N2 = p->n[2];
    const long long pr = N2 / 2;   // complex pairs per real row
    StridedArgs a{};
    a.dfx = p->df_exp;
    a.in = in;
    a.out = out;
    int L;
    long long real_slab, real_line, spec_slab, spec_line;
    if (axis == 1) {
      L = (int)N1;
      a.tw = p->tw_y;
      a.ncols = N0 * pr;
      a.cps = pr;
      real_slab = N1 * pr;
      real_line = pr;
      spec_slab = (N1 / 2 + 1) * N2;
      spec_line = N2;
    } else {
      L = (int)N0;
      a.tw = p->tw_x;
      a.ncols = a.cps = N1 * pr;
      real_slab = 0;
      real_line = N1 * pr;
      spec_slab = 0;
      spec_line = N1 * N2;
    }
    if (mode == 2) {
      a.in_slab = real_slab; a.in_line = real_line; a.out_slab = spec_slab; a.out_line = spec_line;
    } else {
      a.in_slab = spec_slab; a.in_line = spec_line; a.out_slab = real_slab; a.out_line = real_line;
    }
    if (!timed(axis == 0 ? "x_real" : "y_real", p->stream, [&] { return go_strided(L, mode, a, p->stream); }))
      unsupported("single-axis pass", L);
  }
  // ---- passes through the aligned intermediate layout (p->split)
  void* main_buf() const { return p->scratch; }
  void* nyq_buf() const {
    return static_cast<char*>(p->scratch) + (long long)p->n[0] * p->n[1] * p->M() * 2 * p->esz();
  }
  void zr2c_split(const void* in, long long in_row) {
    if (!ok()) return;
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.in = in;
    a.out = main_buf();
    a.nyq_out = nyq_buf();
    a.weight = weight;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = (long long)p->n[0] * p->n[1];
    a.in_dist = in_row;
    a.out_dist = p->M();
    if (!timed("z_r2c", p->stream, [&] { return go_zr2c(p->M(), a, p->stream); }))
      unsupported("z r2c pass", p->M());
  }
  void zc2r_split(void* out, long long out_row) {
    if (!ok()) return;
    ContigArgs a{};
    a.dfx = p->df_exp;
    a.in = main_buf();
    a.nyq_in = nyq_buf();
    a.out = out;
    a.weight = weight;
    a.tw = p->tw_z;
    a.tw_post = p->tw_post;
    a.nlines = (long long)p->n[0] * p->n[1];
    a.in_dist = p->M();
    a.out_dist = out_row;
    if (!timed("z_c2r", p->stream, [&] { return go_zc2r(p->M(), a, p->stream); }))
      unsupported("z c2r pass", p->M());
  }
  // y lines of the main part (aligned columns) and, as extra columns of the
  // same launch, the contiguous y lines of the Nyquist plane
  void y_split(int inverse) {
    if (!ok()) return;
    const long long N0 = p->n[0], N1 = p->n[1], M = p->M();
    StridedArgs a{};
    a.dfx = p->df_exp;
    a.in = a.out = main_buf();
    a.tw = p->tw_y;
    a.ncols_main = N0 * M;
    a.ncols = N0 * M + N0;
    a.cps = M;
    a.in_slab = a.out_slab = N1 * M;
    a.in_line = a.out_line = M;
    a.in_nyq = a.out_nyq = nyq_buf();
    a.nyq_slab = N1;
    a.nyq_line = 1;
    a.inverse = inverse;
    if (!timed(inverse ? "y_inv" : "y", p->stream, [&] { return go_strided((int)N1, 0, a, p->stream); }))
      unsupported("strided pass", (int)N1);
  }
  // fused x pass of a 3-D operator on the split layout (in place, aligned;
  // the Nyquist plane's x lines are the launch's last N1 columns)
  void x_split_sym(SymArgs sym) {
    if (!ok()) return;
    const long long N1 = p->n[1], M = p->M();
    StridedArgs a{};
    a.dfx = p->df_exp;
    a.in = a.out = main_buf();
    a.tw = p->tw_x;
    a.ncols_main = N1 * M;
    a.ncols = N1 * M + N1;
    a.cps = a.ncols_main;
    a.in_slab = a.out_slab = 0;
    a.in_line = a.out_line = N1 * M;
    a.in_nyq = a.out_nyq = nyq_buf();
    a.nyq_slab = 1;
    a.nyq_line = N1;
    sym.h2 = (int)M;
    a.sym = sym;
    if (!timed("x_sym", p->stream, [&] { return go_strided(p->n[0], 1, a, p->stream); }))
      unsupported("symbol pass", p->n[0]);
  }
  int finish() {
    if (p->recording) return rc;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess && ok()) rc = cuda_fail(e, "kernel launch");
    if (p->blocking || timer) {
      cudaEventRecord(p->ev1, p->stream);
      e = cudaEventSynchronize(p->ev1);
      if (e != cudaSuccess && ok()) rc = cuda_fail(e, "kernel execution");
      if (ok() && timer) {
        float ms = 0;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        timer[4] += ms / 1000.0;
      }
      if (ok()) rc = take_wait_error(p, "execute");
    }
    return rc;
  }
};

// plans that can run the packed pass order (exec_r2c_plan)
bool packed_eligible(const accfft_c_plan* p) {
  return p->kind == 1 && !p->inplace && !p->tc && !p->df && !p->gen_any && p->scratch != nullptr;
}

// every array is accessed as whole complex elements (8 or 16 bytes)
int check_align(const accfft_c_plan* p, const char* fn, std::initializer_list<const void*> ptrs) {
  const uintptr_t a = p->dbl ? 16 : 8;
  for (const void* q : ptrs)
    if (q && (reinterpret_cast<uintptr_t>(q) % a))
      return fail(ACCFFT_C_EINVAL, "%s: array %p is not %d-byte aligned", fn, q, (int)a);
  return ACCFFT_C_OK;
}

// 0: device (or managed) memory, 1: pinned host memory (copied through the
// staging ring, or reached by kernels over the host link), -1: memory the
// GPU cannot address
int classify(const void* q) {
  if (!q) return 0;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  if (at.type == cudaMemoryTypeHost) return 1;
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return 0;
  return -1;
}

int check_addressable(const char* fn, std::initializer_list<const void*> ptrs) {
  for (const void* q : ptrs)
    if (classify(q) < 0)
      return fail(ACCFFT_C_EINVAL, "%s: array %p is neither device memory nor pinned host memory", fn, q);
  return ACCFFT_C_OK;
}

// ---------------------------------------------------------------- tuner
// ACCFFT_MEASURE (the reference's default flag, src/accfft_gpu.cpp:341-382:
// time the candidates at plan creation and keep the fastest): a float r2c
// plan times the radix / tile variants of its y, x, z r2c and z c2r passes
// (variants.cu) on its own scratch and a temporary spectrum, in the plan's
// pass order, and keeps the fastest of each.  Choices are cached per process
// by grid and order, so plans of one grid run the same kernels.
constexpr unsigned kMeasureFlag = 2u;   // ACCFFT_MEASURE
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, std::array<int, 4>> g_tuned;

bool variant_exists(int kind, int L, int v) {
  int E = 0, t = 0;
  variant_shape(kind, L, v, &E, &t);
  return E > 0;
}

void tune_variants(accfft_c_plan* p) {
  if (p->kind != 1 || p->dbl || p->tc || p->df || !p->scratch) return;
  const int kinds[4] = {PK_STRIDED, PK_STRIDED, PK_ZR2C, PK_ZC2R};
  const int lens[4] = {p->n[1], p->n[0], p->M(), p->M()};
  bool any = false;   // nothing to choose when no pass length has a variant
  for (int w = 0; w < 4; ++w)
    for (int v = 1; v <= kMaxVariant; ++v) any = any || variant_exists(kinds[w], lens[w], v);
  if (!any) return;
  const auto key = std::make_tuple(p->n[0], p->n[1], p->n[2], p->packed ? 1 : 0);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      p->var_y = it->second[0];
      p->var_x = it->second[1];
      p->var_zr = it->second[2];
      p->var_zc = it->second[3];
      p->tuned = true;
      return;
    }
  }
  DeviceGuard guard(p->device);
  void* tmp = nullptr;
  if (cudaMalloc(&tmp, (size_t)p->alloc_max) != cudaSuccess) {
    cudaGetLastError();   // no room to tune: keep the defaults
    return;
  }
  cudaMemsetAsync(p->scratch, 0, (size_t)p->alloc_max, p->stream);
  cudaMemsetAsync(tmp, 0, (size_t)p->alloc_max, p->stream);
  const bool was_blocking = p->blocking;
  p->blocking = false;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const long long M = p->M(), h = p->packed ? M : p->H2();
  void* sc = p->scratch;
  // one pass of the given kind with the plan's current variants
  auto pass = [&](int which) {
    Exec ex(p, nullptr);
    if (which == 0) ex.ypass(sc, sc, h, 0);
    else if (which == 1) ex.xpass(sc, sc, h, 0);
    else if (which == 2) p->packed ? ex.zr2c_pairs(sc, tmp) : ex.zr2c(tmp, sc, p->n[2]);
    else p->packed ? ex.zc2r_pairs(tmp, sc) : ex.zc2r(sc, tmp, p->n[2]);
    return ex.finish();
  };
  auto ms_of = [&](int which) {
    if (pass(which) != ACCFFT_C_OK) return -1.0f;   // warm-up and launch check
    cudaEventRecord(e0, p->stream);
    for (int r = 0; r < 3; ++r) pass(which);
    cudaEventRecord(e1, p->stream);
    float ms = -1.0f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) return -1.0f;
    return ms;
  };
  int* slot[4] = {&p->var_y, &p->var_x, &p->var_zr, &p->var_zc};
  bool ok = true;
  for (int w = 0; w < 4 && ok; ++w) {
    float best = -1.0f;
    int best_v = 0;
    for (int v = 0; v <= kMaxVariant; ++v) {
      if (v > 0 && !variant_exists(kinds[w], lens[w], v)) continue;
      *slot[w] = v;
      const float t = ms_of(w);
      if (t < 0) {
        if (v == 0) ok = false;
        continue;
      }
      if (best < 0 || t < best) {
        best = t;
        best_v = v;
      }
    }
    *slot[w] = best_v;
  }
  cudaStreamSynchronize(p->stream);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(tmp);
  p->blocking = was_blocking;
  g_err.clear();
  g_err_code = ACCFFT_C_OK;
  if (!ok) {
    p->var_y = p->var_x = p->var_zr = p->var_zc = 0;
    return;
  }
  p->tuned = true;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned[key] = {p->var_y, p->var_x, p->var_zr, p->var_zc};
}

int check_plan(accfft_c_plan* p, int kind, int dbl, const char* fn) {
  g_err.clear();
  g_err_code = ACCFFT_C_OK;
  if (!p) return fail(ACCFFT_C_EINVAL, "%s: NULL plan", fn);
  if (kind && p->kind != kind)
    return fail(ACCFFT_C_ENOTBAKED, "%s: the plan was made for a %s transform", fn, p->kind == 1 ? "r2c" : "c2c");
  if (dbl >= 0 && (int)p->dbl != dbl)
    return fail(ACCFFT_C_EINVAL, "%s: precision mismatch (plan is %s)", fn, p->dbl ? "double" : "float");
  if (p->tc && strcmp(fn, "execute_r2c") && strcmp(fn, "execute_c2r") && strcmp(fn, "execute"))
    return fail(ACCFFT_C_EUNSUPPORTED, "%s: tensor-core plans run full r2c / c2r transforms only", fn);
  if (p->gen_any) {
    // axes without compiled kernels: the transforms (any xyz) and the 3-D
    // operators, which run as r2c, symbol, c2r
    static const char* const gen_ok[] = {"execute_r2c", "execute_c2r", "execute", "execute_c2c", "laplace",
                                         "biharmonic", "inv_laplace", "inv_biharmonic", "heat", "helmholtz",
                                         "poisson"};
    bool ok = false;
    for (const char* f : gen_ok) ok = ok || !strcmp(fn, f);
    if (!ok)
      return fail(ACCFFT_C_EUNSUPPORTED,
                  "%s: the plan has an axis length without compiled kernels (%dx%dx%d); such plans run the "
                  "transforms and the 3-D spectral operators only", fn, p->n[0], p->n[1], p->n[2]);
  }
  if (p->df) {
    static const char* const df_ok[] = {"execute_r2c", "execute_c2r", "execute", "execute_c2c", "laplace",
                                        "biharmonic", "inv_laplace", "inv_biharmonic", "heat", "helmholtz",
                                        "poisson"};
    bool ok = false;
    for (const char* f : df_ok) ok = ok || !strcmp(fn, f);
    if (!ok)
      return fail(ACCFFT_C_EUNSUPPORTED,
                  "%s: double-float plans run r2c, c2r and c2c transforms and the 3-D spectral operators only", fn);
  }
  return ACCFFT_C_OK;
}

// accfft_execute_gpu (src/accfft_gpu.cpp:444-623) at P = 1
int exec_r2c_plan(accfft_c_plan* p, int direction, void* in, void* out, double* timer, unsigned xyz,
                  int weight = 0) {
  if (!in) in = p->data;
  if (!out) out = p->data_out;
  if (!in || !out) return fail(ACCFFT_C_EINVAL, "execute: NULL data pointer and none given at plan time");
  if (int rc = check_align(p, "execute", {in, out})) return rc;
  if (int rc = check_addressable("execute", {in, out})) return rc;
  const bool host_in = classify(in) == 1, host_out = classify(out) == 1;
  const long long h = p->H2();
  if (p->tc) {
    if ((xyz & 7) != 7 || host_in || host_out || weight)
      return fail(ACCFFT_C_EUNSUPPORTED, "execute: tensor-core plans run full transforms (xyz = 7) of device arrays");
    if (direction != -1 && direction != 1)
      return fail(ACCFFT_C_EINVAL, "execute: direction must be -1 or +1 (got %d)", direction);
    Exec ex(p, timer);
    if (direction == -1) {
      ex.zr2c(in, out, p->rrow());
      ex.ypass(out, out, h, 0);
      ex.xpass(out, out, h, 0);
    } else {
      void* buf = p->inplace ? in : p->scratch;
      ex.xpass(in, buf, h, 1);
      ex.ypass(buf, buf, h, 1);
      ex.zc2r(buf, out, p->rrow());
    }
    return ex.finish();
  }
  if (p->df && (host_in || host_out))
    return fail(ACCFFT_C_EUNSUPPORTED, "execute: double-float plans take device arrays");
  if (p->gen_any && (host_in || host_out))
    return fail(ACCFFT_C_EUNSUPPORTED, "execute: plans with an axis length without compiled kernels take device arrays");
  if (p->packed && (xyz & 7) == 7 && weight == 0 && p->zy_mode == 0 && (direction == -1 || direction == 1)) {
    // packed order: r2c = y, x over the packed real field (in -> scratch),
    // then the mirror-pair z pass (scratch -> natural spectrum); c2r the
    // reverse.  The input array is only read.  A real array in pinned host
    // memory is staged through the device ring; other host arrays are
    // reached by the kernels over the host link.
    Exec ex(p, timer);
    const long long M = p->M();
    void* sc = p->scratch;
    if ((direction == -1 && host_in) || (direction == 1 && host_out)) {
      ex.packed_host(direction == -1, in, out);
    } else if (direction == -1) {
      ex.ypass(in, sc, M, 0);
      ex.xpass(sc, sc, M, 0);
      ex.zr2c_pairs(sc, out);
    } else {
      ex.zc2r_pairs(in, sc);
      ex.xpass(sc, sc, M, 1);
      ex.ypass(sc, out, M, 1);
    }
    return ex.finish();
  }
  Exec ex(p, timer);
  ex.weight = weight;
  const long long spec_doubles = 2LL * p->n[0] * p->n[1] * h;
  if (direction == -1 && (xyz & ZB)) ex.df_scan(in, (long long)p->n[0] * p->n[1], p->n[2], p->rrow());
  else ex.df_scan(in, 1, spec_doubles, spec_doubles);
  if (direction == -1) {
    void* work = in;   // with z skipped the reference transforms the input in place
    if ((xyz & ZB) && (xyz & YB) && !p->gen_any) {
      if (host_in) ex.zy_host(true, in, nullptr, out, p->rrow());
      else ex.zy(true, in, nullptr, out, p->rrow());
      work = out;
    } else {
      if (xyz & ZB) {
        ex.zr2c(in, out, p->rrow());
        work = out;
      }
      if (xyz & YB) ex.ypass(work, work, h, 0);
    }
    if (xyz & XB) ex.xpass(work, work, h, 0);
  } else if (direction == 1) {
    // x and y inverse passes read the input spectrum; out of place they write
    // the plan scratch so the input survives (the reference overwrites it)
    void* src = in;
    void* buf = (!(xyz & ZB) || p->inplace) ? in : p->scratch;
    if (xyz & XB) {
      ex.xpass(src, buf, h, 1);
      src = buf;
    }
    if ((xyz & YB) && (xyz & ZB) && !p->gen_any) {
      if (host_out) ex.zy_host(false, src, buf, out, p->rrow());
      else ex.zy(false, src, buf, out, p->rrow());
    } else {
      if (xyz & YB) {
        ex.ypass(src, buf, h, 1);
        src = buf;
      }
      if (xyz & ZB) ex.zc2r(src, out, p->rrow());
    }
  } else {
    return fail(ACCFFT_C_EINVAL, "execute: direction must be -1 or +1 (got %d)", direction);
  }
  return ex.finish();
}

// accfft_execute_c2c_gpu (src/accfft_gpu.cpp:943-1136) at P = 1
int exec_c2c_plan(accfft_c_plan* p, int direction, void* in, void* out, double* timer, unsigned xyz) {
  if (!in) in = p->data;
  if (!out) out = p->data_out;
  if (!in || !out) return fail(ACCFFT_C_EINVAL, "execute: NULL data pointer and none given at plan time");
  if (direction != -1 && direction != 1)
    return fail(ACCFFT_C_EINVAL, "execute: direction must be -1 or +1 (got %d)", direction);
  if (int rc = check_align(p, "execute_c2c", {in, out})) return rc;
  if (int rc = check_addressable("execute_c2c", {in, out})) return rc;
  const int inv = direction == 1;
  const long long h = p->n[2];
  Exec ex(p, timer);
  const long long cdoubles = 2LL * p->n[0] * p->n[1] * p->n[2];
  ex.df_scan(in, 1, cdoubles, cdoubles);
  // the axes are independent, so the backward transform also starts with z
  // (in -> out) and never writes its input
  void* work = in;
  if (xyz & ZB) {
    ex.zc2c(in, out, inv);
    work = out;
  }
  if (xyz & YB) ex.ypass(work, work, h, inv);
  if (xyz & XB) ex.xpass(work, work, h, inv);
  return ex.finish();
}

SymArgs make_sym(const accfft_c_plan* p, int kind, double scale, int axis_len = 0) {
  SymArgs s{};
  s.kind = kind;
  s.n0 = p->n[0];
  s.n1 = p->n[1];
  s.n2 = p->n[2];
  s.h2 = (int)p->H2();
  s.axis_len = axis_len;
  s.scale = scale;
  s.fd_tab = p->fd_tab;
  s.fd_y = p->n[0] / 2 + 1;
  s.fd_z = s.fd_y + p->n[1] / 2 + 1;
  return s;
}

// full 3-D operator: r2c (z, y) -> fused x pass (forward, symbol, inverse) ->
// inverse y -> c2r, through the plan scratch spectrum
int op3d(accfft_c_plan* p, int sym_kind, void* outr, const void* inr, double* timer, double param = 0.0) {
  if (!outr || !inr) return fail(ACCFFT_C_EINVAL, "operator: NULL array");
  if (int rc = check_align(p, "operator", {outr, inr})) return rc;
  if (int rc = check_addressable("operator", {outr, inr})) return rc;
  const long long h = p->H2();
  const double N = (double)p->n[0] * p->n[1] * p->n[2];
  Exec ex(p, timer);
  SymArgs sym = make_sym(p, sym_kind, 1.0 / N);
  sym.param = param;
  if (p->df || p->gen_any) {
    // double-float plans and plans with a generic-length axis: the plan's
    // r2c, the symbol multiply over the spectrum, the plan's c2r (in
    // double-float each transform scans its own input for the exponent its
    // passes scale by)
    if (sym_kind == SYM_POISSON_FD && p->df)
      return fail(ACCFFT_C_EUNSUPPORTED, "poisson: double-float plans take the spectral method (1) only");
    void* s = p->scratch;
    const long long spec_doubles = 2LL * p->n[0] * p->n[1] * h;
    ex.df_scan(inr, (long long)p->n[0] * p->n[1], p->n[2], p->rrow());
    ex.zr2c(inr, s, p->rrow());
    ex.ypass(s, s, h, 0);
    ex.xpass(s, s, h, 0);
    ex.sym_spectrum(s, sym);
    ex.df_scan(s, 1, spec_doubles, spec_doubles);
    ex.xpass(s, s, h, 1);
    ex.ypass(s, s, h, 1);
    ex.zc2r(s, outr, p->rrow());
    return ex.finish();
  }
  if (p->split) {
    ex.zr2c_split(inr, p->rrow());
    ex.y_split(0);
    ex.x_split_sym(sym);
    ex.y_split(1);
    ex.zc2r_split(outr, p->rrow());
    return ex.finish();
  }
  void* s = p->scratch;
  ex.zr2c(inr, s, p->rrow());
  ex.ypass(s, s, h, 0);
  long long c = (long long)p->n[1] * h;
  ex.strided_sym(s, s, nullptr, p->tw_x, p->n[0], c, c, 0, c, sym, "x_sym");
  ex.ypass(s, s, h, 1);
  ex.zc2r(s, outr, p->rrow());
  return ex.finish();
}

// one-pass single-axis derivative d/dx_axis of a real field (optionally added
// to acc).  y and x lines view pairs of adjacent reals as one complex value:
// the symbol i*w/N is Hermitian-consistent, so it maps real to real and acts
// on both members of the pair independently.
void deriv_axis(Exec& ex, accfft_c_plan* p, int axis, void* out, const void* in, const void* acc,
                double alpha = 1.0) {
  const long long rr = p->rrow();
  const int N0 = p->n[0], N1 = p->n[1], N2 = p->n[2];
  if (axis == 2) {
    ex.zsym(in, out, acc, rr, make_sym(p, SYM_DERIV1, alpha / N2, N2));
    return;
  }
  const long long cr = rr / 2;            // complex pairs per stored row
  const long long cols = N2 / 2;          // pairs holding data
  if (axis == 1) {
    ex.strided_sym(in, out, acc, p->tw_y, N1, (long long)N0 * cols, cols, (long long)N1 * cr, cr,
                   make_sym(p, SYM_DERIV1, alpha / N1, N1), "y_deriv");
  } else {
    ex.strided_sym(in, out, acc, p->tw_x, N0, (long long)N1 * cols, cols, cr, (long long)N1 * cr,
                   make_sym(p, SYM_DERIV1, alpha / N0, N0), "x_deriv");
  }
}

}  // namespace

namespace afg {
// lets other translation units of the library report through accfft_c_last_error
void set_last_error(int code, const char* msg) { fail(code, "%s", msg); }
}  // namespace afg

// ================================================================== C ABI
extern "C" {

const char* accfft_c_last_error(void) { return g_err.c_str(); }
int accfft_c_last_error_code(void) { return g_err_code; }
int accfft_c_version(void) { return 1; }
int accfft_c_length_supported(int len) { return length_supported(len) ? 1 : 0; }
int accfft_c_length_generic(int len) { return gen_factor(len, nullptr) ? 1 : 0; }
int accfft_c_line_plan(int len, int precision, int* E, int* P, int* radices) {
  if (len < 1 || precision < 0 || precision > 2 || !E || !P || !radices) return -1;
  const LinePlan pl = plan_select(len, precision, 0);
  if (pl.E == 0) return -1;
  *E = pl.E;
  *P = pl.P;
  for (int s = 0; s < pl.ns; ++s) radices[s] = pl.radix[s];
  return pl.ns;
}
unsigned long long accfft_c_kernel_launches(void) { return launch_count(); }
int accfft_c_set_pdl(int mode) {
  const int was = pdl_mode();
  if (mode >= 0) set_pdl(mode);
  return was;
}
long long accfft_c_set_wait_limit(long long polls) {
  const unsigned v = polls < 0 ? kDefaultWaitLimit : polls > 0xFFFFFFFFLL ? 0xFFFFFFFFu : unsigned(polls);
  return (long long)g_wait_limit.exchange(v);
}
int accfft_c_check(accfft_c_plan* p) {
  if (!p) return fail(ACCFFT_C_EINVAL, "check: NULL plan");
  DeviceGuard guard(p->device);
  cudaError_t e = cudaStreamSynchronize(p->stream);
  if (e != cudaSuccess) return cuda_fail(e, "check: stream synchronisation");
  return take_wait_error(p, "check");
}

long long accfft_c_dfft_get_local_size(int N0, int N1, int tuple, int isize[3], int istart[3], int real_bytes) {
  return local_size(N0, N1, tuple, isize, istart, real_bytes);
}
long long accfft_c_local_size_dft_r2c(const int n[3], int isize[3], int istart[3], int osize[3], int ostart[3],
                                      int real_bytes) {
  return local_size_r2c(n, isize, istart, osize, ostart, real_bytes);
}
long long accfft_c_local_size_dft_c2c(const int n[3], int isize[3], int istart[3], int osize[3], int ostart[3],
                                      int real_bytes) {
  return local_size_c2c(n, isize, istart, osize, ostart, real_bytes);
}

accfft_c_plan* accfft_c_plan_dft_3d_r2c_gpu(const int n[3], double* data, double* data_out, unsigned flags) {
  return make_plan(1, true, n, data, data_out, flags);
}
accfft_c_plan* accfft_c_plan_dft_3d_r2c_gpuf(const int n[3], float* data, float* data_out, unsigned flags) {
  accfft_c_plan* p = make_plan(1, false, n, data, data_out, flags);
  if (p && (flags & kMeasureFlag)) tune_variants(p);
  return p;
}
accfft_c_plan* accfft_c_plan_dft_3d_c2c_gpu(const int n[3], double* data, double* data_out, unsigned flags) {
  return make_plan(2, true, n, data, data_out, flags);
}
accfft_c_plan* accfft_c_plan_dft_3d_c2c_gpuf(const int n[3], float* data, float* data_out, unsigned flags) {
  return make_plan(2, false, n, data, data_out, flags);
}

void accfft_c_destroy_plan(accfft_c_plan* p) {
  if (!p) return;
  DeviceGuard guard(p->device);
  if (p->tw_block) cudaFree(p->tw_block);
  if (p->scratch) cudaFree(p->scratch);
  if (p->hstage) cudaFree(p->hstage);
  if (p->wait_err) cudaFree(p->wait_err);
  if (p->zy_ctl) cudaFree(p->zy_ctl);
  if (p->df_exp) cudaFree(p->df_exp);
  if (p->ev0) cudaEventDestroy(p->ev0);
  if (p->ev1) cudaEventDestroy(p->ev1);
  for (cudaEvent_t e : p->evb)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->pev) cudaEventDestroy(e);
  if (p->stream2) cudaStreamDestroy(p->stream2);
  delete p;
}

int accfft_c_plan_info(const accfft_c_plan* p, int n[3], int* kind, int* is_double, int* inplace,
                       long long* alloc_max) {
  if (!p) return fail(ACCFFT_C_EINVAL, "plan_info: NULL plan");
  if (n)
    for (int i = 0; i < 3; ++i) n[i] = p->n[i];
  if (kind) *kind = p->kind;
  if (is_double) *is_double = p->dbl;
  if (inplace) *inplace = p->inplace;
  if (alloc_max) *alloc_max = p->alloc_max;
  return ACCFFT_C_OK;
}

int accfft_c_set_profiling(accfft_c_plan* p, int on) {
  if (!p) return fail(ACCFFT_C_EINVAL, "set_profiling: NULL plan");
  p->profile = on != 0;
  return ACCFFT_C_OK;
}

int accfft_c_profile_read(accfft_c_plan* p, int max_entries, char* labels, long long* counts, double* total_ms) {
  if (!p) return fail(ACCFFT_C_EINVAL, "profile_read: NULL plan");
  DeviceGuard guard(p->device);
  Exec::fold_profile(p);
  int n = 0;
  for (auto& kv : p->pstats) {
    if (n >= max_entries) break;
    if (labels) {
      memset(labels + 32 * n, 0, 32);
      strncpy(labels + 32 * n, kv.first.c_str(), 31);
    }
    if (counts) counts[n] = kv.second.first;
    if (total_ms) total_ms[n] = kv.second.second;
    ++n;
  }
  p->pstats.clear();
  return n;
}

int accfft_c_set_zy_schedule(accfft_c_plan* p, int mode) {
  if (!p) return fail(ACCFFT_C_EINVAL, "set_zy_schedule: NULL plan");
  if (p->kind != 1) return fail(ACCFFT_C_ENOTBAKED, "set_zy_schedule: r2c plans only");
  if (mode == 0) {
    p->zy_mode = 0;
    return ACCFFT_C_OK;
  }
  if (mode == 1) {
    if (!slab_available(p->dbl, p->n[1], p->n[2]))
      return fail(ACCFFT_C_EUNSUPPORTED, "set_zy_schedule: no slab kernel for %dx%d", p->n[1], p->n[2]);
    p->zy_mode = 1;
    return ACCFFT_C_OK;
  }
  if (mode == 2) {
    if (!zy_persistent_available(p->dbl, p->M(), p->n[1]))
      return fail(ACCFFT_C_EUNSUPPORTED, "set_zy_schedule: no persistent z+y kernel for N1 = %d, N2 = %d",
                  p->n[1], p->n[2]);
    p->zy_mode = 3;
    return ACCFFT_C_OK;
  }
  return fail(ACCFFT_C_EINVAL,
              "set_zy_schedule: mode must be 0 (separate passes), 1 (cluster slab kernel) or 2 (persistent z+y kernel)");
}

int accfft_c_plan_tuning(const accfft_c_plan* p, int variant[4], int radix[4], int tile[4]) {
  if (!p) return fail(ACCFFT_C_EINVAL, "plan_tuning: NULL plan");
  const int v[4] = {p->var_y, p->var_x, p->var_zr, p->var_zc};
  const int kinds[4] = {PK_STRIDED, PK_STRIDED, PK_ZR2C, PK_ZC2R};
  const int lens[4] = {p->n[1], p->n[0], p->M(), p->M()};
  for (int w = 0; w < 4; ++w) {
    int E = 0, t = 0;
    variant_shape(kinds[w], lens[w], v[w], &E, &t);
    if (E == 0 && v[w] == 0) E = plan_select(lens[w], p->prec(), 0).E;   // no variants: the default radix
    if (variant) variant[w] = v[w];
    if (radix) radix[w] = E;
    if (tile) tile[w] = t;
  }
  return p->tuned ? 1 : 0;
}

int accfft_c_set_variants(accfft_c_plan* p, const int variant[4]) {
  if (!p || !variant) return fail(ACCFFT_C_EINVAL, "set_variants: NULL argument");
  if (p->kind != 1 || p->dbl || p->tc || p->df)
    return fail(ACCFFT_C_EUNSUPPORTED, "set_variants: float r2c plans only (CUDA-core form)");
  const int kinds[4] = {PK_STRIDED, PK_STRIDED, PK_ZR2C, PK_ZC2R};
  const int lens[4] = {p->n[1], p->n[0], p->M(), p->M()};
  for (int w = 0; w < 4; ++w)
    if (variant[w] < 0 || variant[w] > kMaxVariant ||
        (variant[w] > 0 && !variant_exists(kinds[w], lens[w], variant[w])))
      return fail(ACCFFT_C_EUNSUPPORTED, "set_variants: pass %d of length %d has no variant %d", w, lens[w], variant[w]);
  p->var_y = variant[0];
  p->var_x = variant[1];
  p->var_zr = variant[2];
  p->var_zc = variant[3];
  return ACCFFT_C_OK;
}

int accfft_c_set_pass_order(accfft_c_plan* p, int order) {
  if (!p) return fail(ACCFFT_C_EINVAL, "set_pass_order: NULL plan");
  if (order == 0) {
    p->packed = false;
    return ACCFFT_C_OK;
  }
  if (order != 1) return fail(ACCFFT_C_EINVAL, "set_pass_order: order must be 0 (natural) or 1 (packed)");
  if (!packed_eligible(p))
    return fail(ACCFFT_C_EUNSUPPORTED, "set_pass_order: the packed order needs an out-of-place float or double r2c plan with compiled lengths");
  p->packed = true;
  return ACCFFT_C_OK;
}

int accfft_c_set_stream(accfft_c_plan* p, void* stream, int blocking) {
  if (!p) return fail(ACCFFT_C_EINVAL, "set_stream: NULL plan");
  p->stream = static_cast<cudaStream_t>(stream);
  p->blocking = blocking != 0;
  return ACCFFT_C_OK;
}

#define AFG_EXEC_R2C(SFX, T, DBL)                                                                        \
  int accfft_c_execute_r2c_gpu##SFX(accfft_c_plan* p, T* in, T* out, double* timer, unsigned xyz) {     \
    int rc = check_plan(p, 1, DBL, "execute_r2c");                                                       \
    return rc ? rc : exec_r2c_plan(p, -1, in, out, timer, xyz);                                          \
  }                                                                                                      \
  int accfft_c_execute_c2r_gpu##SFX(accfft_c_plan* p, T* in, T* out, double* timer, unsigned xyz) {     \
    int rc = check_plan(p, 1, DBL, "execute_c2r");                                                       \
    return rc ? rc : exec_r2c_plan(p, 1, in, out, timer, xyz);                                           \
  }                                                                                                      \
  int accfft_c_execute_gpu##SFX(accfft_c_plan* p, int dir, T* in, T* out, double* timer, unsigned xyz) { \
    int rc = check_plan(p, 1, DBL, "execute");                                                           \
    return rc ? rc : exec_r2c_plan(p, dir, in, out, timer, xyz);                                         \
  }                                                                                                      \
  int accfft_c_execute_c2c_gpu##SFX(accfft_c_plan* p, int dir, T* in, T* out, double* timer,            \
                                    unsigned xyz) {                                                      \
    int rc = check_plan(p, 2, DBL, "execute_c2c");                                                       \
    return rc ? rc : exec_c2c_plan(p, dir, in, out, timer, xyz);                                         \
  }
AFG_EXEC_R2C(, double, 1)
AFG_EXEC_R2C(f, float, 0)
#undef AFG_EXEC_R2C

int accfft_c_execute_r2c_axis(accfft_c_plan* p, int axis, const void* in, void* out, double* timer) {
  int rc = check_plan(p, 1, -1, "execute_r2c_axis");
  if (rc) return rc;
  if (!in || !out) return fail(ACCFFT_C_EINVAL, "execute_r2c_axis: NULL array");
  if (int a = check_align(p, "execute_r2c_axis", {in, out})) return a;
  if (int a = check_addressable("execute_r2c_axis", {in, out})) return a;
  if (axis < 0 || axis > 2) return fail(ACCFFT_C_EINVAL, "execute_r2c_axis: axis must be 0, 1 or 2");
  Exec ex(p, timer);
  if (axis == 2) ex.zr2c(in, out, p->rrow());
  else ex.pair_axis(axis, 2, in, out);
  return ex.finish();
}
int accfft_c_execute_c2r_axis(accfft_c_plan* p, int axis, const void* in, void* out, double* timer) {
  int rc = check_plan(p, 1, -1, "execute_c2r_axis");
  if (rc) return rc;
  if (!in || !out) return fail(ACCFFT_C_EINVAL, "execute_c2r_axis: NULL array");
  if (int a = check_align(p, "execute_c2r_axis", {in, out})) return a;
  if (int a = check_addressable("execute_c2r_axis", {in, out})) return a;
  if (axis < 0 || axis > 2) return fail(ACCFFT_C_EINVAL, "execute_c2r_axis: axis must be 0, 1 or 2");
  Exec ex(p, timer);
  if (axis == 2) ex.zc2r(in, out, p->rrow());
  else ex.pair_axis(axis, 3, in, out);
  return ex.finish();
}

int accfft_c_laplace(accfft_c_plan* p, void* LA, const void* A, double* timer) {
  int rc = check_plan(p, 1, -1, "laplace");
  return rc ? rc : op3d(p, SYM_LAPLACE, LA, A, timer);
}
int accfft_c_biharmonic(accfft_c_plan* p, void* BA, const void* A, double* timer) {
  int rc = check_plan(p, 1, -1, "biharmonic");
  return rc ? rc : op3d(p, SYM_BIHARM, BA, A, timer);
}
int accfft_c_inv_laplace(accfft_c_plan* p, void* invLA, const void* A, double* timer) {
  int rc = check_plan(p, 1, -1, "inv_laplace");
  return rc ? rc : op3d(p, SYM_INVLAP, invLA, A, timer);
}
int accfft_c_inv_biharmonic(accfft_c_plan* p, void* invBA, const void* A, double* timer) {
  int rc = check_plan(p, 1, -1, "inv_biharmonic");
  return rc ? rc : op3d(p, SYM_INVBIHARM, invBA, A, timer);
}

int accfft_c_grad(accfft_c_plan* p, void* A_x, void* A_y, void* A_z, const void* A, unsigned xyz, double* timer) {
  int rc = check_plan(p, 1, -1, "grad");
  if (rc) return rc;
  if (!A || ((xyz & XB) && !A_x) || ((xyz & YB) && !A_y) || ((xyz & ZB) && !A_z))
    return fail(ACCFFT_C_EINVAL, "grad: NULL array for a selected component");
  if (int a = check_align(p, "grad", {A_x, A_y, A_z, A})) return a;
  if (int a = check_addressable("grad", {A_x, A_y, A_z, A})) return a;
  Exec ex(p, timer);
  if (xyz & XB) deriv_axis(ex, p, 0, A_x, A, nullptr);
  if (xyz & YB) deriv_axis(ex, p, 1, A_y, A, nullptr);
  if (xyz & ZB) deriv_axis(ex, p, 2, A_z, A, nullptr);
  return ex.finish();
}

int accfft_c_grad_slow(accfft_c_plan* p, void* A_x, void* A_y, void* A_z, const void* A, unsigned xyz,
                       double* timer) {
  int rc = check_plan(p, 1, -1, "grad_slow");
  if (rc) return rc;
  if (!A || ((xyz & XB) && !A_x) || ((xyz & YB) && !A_y) || ((xyz & ZB) && !A_z))
    return fail(ACCFFT_C_EINVAL, "grad_slow: NULL array for a selected component");
  const int kinds[3] = {SYM_GRADX, SYM_GRADY, SYM_GRADZ};
  void* outs[3] = {A_x, A_y, A_z};
  for (int j = 0; j < 3; ++j)
    if (xyz & (1u << j)) {
      rc = op3d(p, kinds[j], outs[j], A, timer);
      if (rc) return rc;
    }
  return ACCFFT_C_OK;
}

int accfft_c_divergence(accfft_c_plan* p, void* divA, const void* A_x, const void* A_y, const void* A_z,
                        double* timer) {
  int rc = check_plan(p, 1, -1, "divergence");
  if (rc) return rc;
  if (!divA || !A_x || !A_y || !A_z) return fail(ACCFFT_C_EINVAL, "divergence: NULL array");
  if (int a = check_align(p, "divergence", {divA, A_x, A_y, A_z})) return a;
  if (int a = check_addressable("divergence", {divA, A_x, A_y, A_z})) return a;
  Exec ex(p, timer);
  deriv_axis(ex, p, 0, divA, A_x, nullptr);
  deriv_axis(ex, p, 1, divA, A_y, divA);
  deriv_axis(ex, p, 2, divA, A_z, divA);
  return ex.finish();
}

// The reference's slow divergence (src/operators_gpu.txx:337-446, CPU
// src/operators.txx:1019-1119) transforms each component over two axes only:
// A_x over {x, z}, A_y over {y, z}, A_z over {z}, multiplies by i*k/(N_j N2)
// with the 3-D multipliers' filter (index N_j/2 -> 0 with integer N_j/2) and
// transforms back.  On an odd axis that filter is not Hermitian-consistent,
// and the c2r's real projection then gives a result different from the fast
// divergence, so this keeps the reference's pass structure: z r2c, one fused
// forward/multiply/inverse pass along x (or y), z c2r; the y term's c2r lands
// in the padded rows of the scratch and is added by a row kernel; the z term
// is the accumulating z derivative pass.
int accfft_c_divergence_slow(accfft_c_plan* p, void* divA, const void* A_x, const void* A_y, const void* A_z,
                             double* timer) {
  int rc = check_plan(p, 1, -1, "divergence_slow");
  if (rc) return rc;
  if (!divA || !A_x || !A_y || !A_z) return fail(ACCFFT_C_EINVAL, "divergence_slow: NULL array");
  if (int a = check_align(p, "divergence_slow", {divA, A_x, A_y, A_z})) return a;
  if (int a = check_addressable("divergence_slow", {divA, A_x, A_y, A_z})) return a;
  const long long h = p->H2(), rr = p->rrow();
  const int N0 = p->n[0], N1 = p->n[1], N2 = p->n[2];
  void* s = p->scratch;
  Exec ex(p, timer);
  // x term over {x, z}: lines along x of the half spectrum
  ex.zr2c(A_x, s, rr);
  const long long c = (long long)N1 * h;
  ex.strided_sym(s, s, nullptr, p->tw_x, N0, c, c, 0, c, make_sym(p, SYM_GRADX, 1.0 / ((double)N0 * N2)), "x_sym");
  ex.zc2r(s, divA, rr);
  // y term over {y, z}: the x multiplier's fold applied along the y lines
  ex.zr2c(A_y, s, rr);
  SymArgs sy = make_sym(p, SYM_GRADX, 1.0 / ((double)N1 * N2));
  sy.n0 = N1;
  ex.strided_sym(s, s, nullptr, p->tw_y, N1, (long long)N0 * h, h, (long long)N1 * h, h, sy, "y_sym");
  ex.zc2r(s, s, 2 * h);
  ex.add_rows(divA, rr, s, 2 * h, (long long)N0 * N1, N2);
  // z term over {z}
  deriv_axis(ex, p, 2, divA, A_z, divA);
  return ex.finish();
}

// --- adjoints (no counterpart in the reference; used by the autograd layer)
int accfft_c_r2c_adjoint(accfft_c_plan* p, const void* dX, void* du, double* timer) {
  int rc = check_plan(p, 1, -1, "r2c_adjoint");
  return rc ? rc : exec_r2c_plan(p, 1, const_cast<void*>(dX), du, timer, 7, 1);
}
int accfft_c_c2r_adjoint(accfft_c_plan* p, const void* dx, void* dY, double* timer) {
  int rc = check_plan(p, 1, -1, "c2r_adjoint");
  return rc ? rc : exec_r2c_plan(p, -1, const_cast<void*>(dx), dY, timer, 7, 2);
}
int accfft_c_grad_adjoint(accfft_c_plan* p, void* out, const void* g_x, const void* g_y, const void* g_z,
                          double* timer) {
  int rc = check_plan(p, 1, -1, "grad_adjoint");
  if (rc) return rc;
  if (!out || !g_x || !g_y || !g_z) return fail(ACCFFT_C_EINVAL, "grad_adjoint: NULL array");
  if (int a = check_align(p, "grad_adjoint", {out, g_x, g_y, g_z})) return a;
  if (int a = check_addressable("grad_adjoint", {out, g_x, g_y, g_z})) return a;
  Exec ex(p, timer);
  deriv_axis(ex, p, 0, out, g_x, nullptr, -1.0);
  deriv_axis(ex, p, 1, out, g_y, out, -1.0);
  deriv_axis(ex, p, 2, out, g_z, out, -1.0);
  return ex.finish();
}
int accfft_c_divergence_adjoint(accfft_c_plan* p, void* a_x, void* a_y, void* a_z, const void* d, double* timer) {
  int rc = check_plan(p, 1, -1, "divergence_adjoint");
  if (rc) return rc;
  if (!d || !a_x || !a_y || !a_z) return fail(ACCFFT_C_EINVAL, "divergence_adjoint: NULL array");
  if (int a = check_align(p, "divergence_adjoint", {a_x, a_y, a_z, d})) return a;
  if (int a = check_addressable("divergence_adjoint", {a_x, a_y, a_z, d})) return a;
  Exec ex(p, timer);
  deriv_axis(ex, p, 0, a_x, d, nullptr, -1.0);
  deriv_axis(ex, p, 1, a_y, d, nullptr, -1.0);
  deriv_axis(ex, p, 2, a_z, d, nullptr, -1.0);
  return ex.finish();
}

// --- spectral solvers (no GPU counterpart in the reference; the analogues of
// the Poisson filter of steps/step4/kernels.cu and the exact heat propagator
// of steps/step6/step6.cpp, on the operators' folded wave numbers)
int accfft_c_heat(accfft_c_plan* p, void* out, const void* in, double t, double* timer) {
  int rc = check_plan(p, 1, -1, "heat");
  if (rc) return rc;
  if (!(t >= 0)) return fail(ACCFFT_C_EINVAL, "heat: time must be >= 0");
  return op3d(p, SYM_HEAT, out, in, timer, t);
}
int accfft_c_helmholtz(accfft_c_plan* p, void* out, const void* in, double alpha, double* timer) {
  int rc = check_plan(p, 1, -1, "helmholtz");
  return rc ? rc : op3d(p, SYM_HELMHOLTZ, out, in, timer, alpha);
}

// steps/step4 (steps/step4/kernels.cu:24-110, steps/step4/step4_gpu.cpp:620-650):
// r2c -> Poisson filter -> c2r as one fused operator on the unit cube
int accfft_c_poisson(accfft_c_plan* p, void* phi, const void* rho, int method, double* timer) {
  int rc = check_plan(p, 1, -1, "poisson");
  if (rc) return rc;
  if (method != 0 && method != 1) return fail(ACCFFT_C_EINVAL, "poisson: method must be 0 or 1 (got %d)", method);
  return op3d(p, method == 0 ? SYM_POISSON_FD : SYM_POISSON_SPEC, phi, rho, timer);
}

}  // extern "C"

// --- batches of independent transforms (no counterpart in the reference)
// Recorded per instance, run level by level: level k holds the k-th pass of
// every instance, and each level launches one grouped kernel per (pass kind,
// line length, mode) over all its instances' tiles.
struct accfft_c_batch {
  int device = 0;
  std::deque<std::vector<PassRecord>> instances;   // a deque keeps recording plans' pointers valid
  std::vector<const accfft_c_plan*> owners;   // one instance per plan
  struct Launch {
    int kind, L, mode, ntasks;
    long long grid;
    size_t tab_off, starts_off;   // bytes into dev
  };
  std::vector<Launch> launches;
  std::vector<int> level_end;        // launches index where each level ends
  void* dev = nullptr;
  size_t dev_bytes = 0;
  bool final = false;
  int tasks = 0;
  // Launch i waits only for the launches of the level before it that hold
  // one of its instances (deps[i]), so no level waits for the whole of the
  // level before: an instance's next pass starts once its own pass is done.
  // The launches run on kBranches streams forked from the caller's stream
  // and joined at the end (created by finalize; one event per launch).
  static constexpr int kBranches = 8;
  cudaStream_t branch[kBranches] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[kBranches] = {};
  std::vector<int> branch_of;             // branch of each launch
  std::vector<std::vector<int>> deps;     // launches each launch waits for
  std::vector<cudaEvent_t> done;          // recorded after each launch
};

extern "C" {

accfft_c_batch* accfft_c_batch_create(void) {
  auto* b = new accfft_c_batch;
  cudaGetDevice(&b->device);
  return b;
}

void accfft_c_batch_destroy(accfft_c_batch* b) {
  if (!b) return;
  DeviceGuard guard(b->device);
  if (b->dev) cudaFree(b->dev);
  for (int j = 0; j < accfft_c_batch::kBranches; ++j) {
    if (b->branch[j]) cudaStreamDestroy(b->branch[j]);
    if (b->join[j]) cudaEventDestroy(b->join[j]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  for (cudaEvent_t e : b->done)
    if (e) cudaEventDestroy(e);
  delete b;
}

int accfft_c_batch_record(accfft_c_batch* b, accfft_c_plan* p, int on) {
  g_err.clear();
  g_err_code = ACCFFT_C_OK;
  if (!b || !p) return fail(ACCFFT_C_EINVAL, "batch_record: NULL batch or plan");
  if (!on) {
    if (!p->recording) return fail(ACCFFT_C_EINVAL, "batch_record: the plan is not recording");
    p->recording = nullptr;
    return ACCFFT_C_OK;
  }
  if (b->final) return fail(ACCFFT_C_EINVAL, "batch_record: the batch is finalised");
  if (p->recording) return fail(ACCFFT_C_EINVAL, "batch_record: the plan is already recording");
  if (p->kind != 1 || p->dbl || p->tc || p->zy_mode != 0)
    return fail(ACCFFT_C_EUNSUPPORTED, "batch_record: batches take float r2c plans with the default z+y schedule");
  if (p->device != b->device) return fail(ACCFFT_C_EINVAL, "batch_record: plan and batch on different devices");
  for (const accfft_c_plan* q : b->owners)
    if (q == p) return fail(ACCFFT_C_EINVAL, "batch_record: a plan holds one instance of a batch (its scratch is shared)");
  b->owners.push_back(p);
  b->instances.emplace_back();
  p->recording = &b->instances.back();
  return ACCFFT_C_OK;
}

int accfft_c_batch_finalize(accfft_c_batch* b) {
  g_err.clear();
  g_err_code = ACCFFT_C_OK;
  if (!b) return fail(ACCFFT_C_EINVAL, "batch_finalize: NULL batch");
  if (b->final) return ACCFFT_C_OK;
  for (const accfft_c_plan* q : b->owners)
    if (q->recording) return fail(ACCFFT_C_EINVAL, "batch_finalize: a plan is still recording");
  size_t levels = 0;
  for (auto& v : b->instances) levels = std::max(levels, v.size());
  std::vector<unsigned char> host;
  std::vector<int> prev_launch(b->instances.size(), -1);   // each instance's launch at the level before
  auto align = [&](size_t a) { host.resize((host.size() + a - 1) / a * a); };
  b->tasks = 0;
  for (size_t lv = 0; lv < levels; ++lv) {
    // the level's tasks, grouped by (kind, length, mode) in first-seen order
    std::vector<std::pair<std::tuple<int, int, int>, std::vector<const PassRecord*>>> groups;
    std::vector<std::vector<int>> members;   // instance indices of each group
    int inst = 0;
    for (auto& v : b->instances) {
      const int me = inst++;
      if (lv >= v.size()) continue;
      const PassRecord& r = v[lv];
      auto key = std::make_tuple(r.kind, r.L, r.mode);
      auto it = std::find_if(groups.begin(), groups.end(), [&](auto& g) { return g.first == key; });
      if (it == groups.end()) {
        groups.push_back({key, {}});
        members.push_back({});
        it = groups.end() - 1;
      }
      it->second.push_back(&r);
      members[it - groups.begin()].push_back(me);
    }
    std::vector<int> this_launch(b->instances.size(), -1);
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      auto& g = groups[gi];
      std::vector<int> dep;
      for (int m : members[gi]) {
        if (prev_launch[m] >= 0 && std::find(dep.begin(), dep.end(), prev_launch[m]) == dep.end())
          dep.push_back(prev_launch[m]);
        this_launch[m] = (int)b->launches.size();
      }
      b->deps.push_back(dep);
      accfft_c_batch::Launch ln{};
      std::tie(ln.kind, ln.L, ln.mode) = g.first;
      ln.ntasks = (int)g.second.size();
      const bool str = ln.kind == PK_STRIDED;
      const size_t rec = str ? sizeof(StridedArgs) : sizeof(ContigArgs);
      align(256);
      ln.tab_off = host.size();
      host.resize(host.size() + rec * g.second.size());
      std::vector<long long> starts;
      long long grid = 0;
      for (size_t k = 0; k < g.second.size(); ++k) {
        const PassRecord* r = g.second[k];
        const void* args = str ? static_cast<const void*>(&r->s) : static_cast<const void*>(&r->c);
        memcpy(&host[ln.tab_off + k * rec], args, rec);
        const long long t = grouped_tiles(ln.kind, ln.L, args);
        if (t < 0) return fail(ACCFFT_C_EUNSUPPORTED, "batch_finalize: no grouped kernel for length %d", ln.L);
        starts.push_back(grid);
        grid += t;
      }
      if (grid >= (1LL << 31)) return fail(ACCFFT_C_EOVERFLOW, "batch_finalize: a level needs more than 2^31 CTAs");
      ln.grid = grid;
      align(16);
      ln.starts_off = host.size();
      host.resize(host.size() + starts.size() * sizeof(long long));
      memcpy(&host[ln.starts_off], starts.data(), starts.size() * sizeof(long long));
      b->launches.push_back(ln);
      b->tasks += ln.ntasks;
    }
    for (size_t m = 0; m < this_launch.size(); ++m)
      if (this_launch[m] >= 0) prev_launch[m] = this_launch[m];
    b->level_end.push_back((int)b->launches.size());
  }
  // branches: within a level, the largest grid first onto the branch with the
  // fewest CTAs so far
  b->branch_of.assign(b->launches.size(), 0);
  for (size_t lv = 0, first = 0; lv < b->level_end.size(); first = (size_t)b->level_end[lv++]) {
    const size_t last = (size_t)b->level_end[lv];
    std::vector<size_t> order;
    for (size_t i = first; i < last; ++i) order.push_back(i);
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return b->launches[x].grid > b->launches[y].grid; });
    long long load[accfft_c_batch::kBranches] = {};
    for (size_t i : order) {
      int j = (int)(std::min_element(load, load + accfft_c_batch::kBranches) - load);
      b->branch_of[i] = j;
      load[j] += b->launches[i].grid;
    }
  }
  DeviceGuard guard(b->device);
  for (int j = 0; j < accfft_c_batch::kBranches; ++j) {
    cudaError_t e = cudaStreamCreateWithFlags(&b->branch[j], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[j], cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "batch_finalize: branch streams");
  }
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
    return cuda_fail(cudaGetLastError(), "batch_finalize: fork event");
  b->done.assign(b->launches.size(), nullptr);
  for (auto& e : b->done)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      return cuda_fail(cudaGetLastError(), "batch_finalize: launch events");
  if (!host.empty()) {
    cudaError_t e = cudaMalloc(&b->dev, host.size());
    if (e == cudaSuccess) e = cudaMemcpy(b->dev, host.data(), host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "batch_finalize: descriptor tables");
    b->dev_bytes = host.size();
  }
  b->final = true;
  return ACCFFT_C_OK;
}

int accfft_c_batch_run(accfft_c_batch* b, void* stream) {
  g_err.clear();
  g_err_code = ACCFFT_C_OK;
  if (!b) return fail(ACCFFT_C_EINVAL, "batch_run: NULL batch");
  if (!b->final) return fail(ACCFFT_C_ENOTBAKED, "batch_run: finalise the batch first");
  DeviceGuard guard(b->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto* base = static_cast<unsigned char*>(b->dev);
  auto go = [&](const accfft_c_batch::Launch& ln, cudaStream_t s) {
    return launch_grouped(ln.kind, ln.L, ln.mode, base + ln.tab_off,
                          reinterpret_cast<const long long*>(base + ln.starts_off), ln.ntasks, ln.grid, s);
  };
  // fork every branch from the caller's stream; each launch waits for the
  // launches holding its instances' previous passes; join at the end
  cudaEventRecord(b->fork, st);
  for (int j = 0; j < accfft_c_batch::kBranches; ++j) cudaStreamWaitEvent(b->branch[j], b->fork, 0);
  for (size_t i = 0; i < b->launches.size(); ++i) {
    cudaStream_t s = b->branch[b->branch_of[i]];
    for (int d : b->deps[i])
      if (b->branch_of[(size_t)d] != b->branch_of[i]) cudaStreamWaitEvent(s, b->done[(size_t)d], 0);
    if (!go(b->launches[i], s)) {
      for (int j = 0; j < accfft_c_batch::kBranches; ++j) {
        cudaEventRecord(b->join[j], b->branch[j]);
        cudaStreamWaitEvent(st, b->join[j], 0);
      }
      return fail(ACCFFT_C_ECUDA, "batch_run: grouped launch of length %d failed", b->launches[i].L);
    }
    cudaEventRecord(b->done[i], s);
  }
  for (int j = 0; j < accfft_c_batch::kBranches; ++j) {
    cudaEventRecord(b->join[j], b->branch[j]);
    cudaStreamWaitEvent(st, b->join[j], 0);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ACCFFT_C_OK : cuda_fail(e, "batch_run");
}

int accfft_c_batch_info(const accfft_c_batch* b, int* instances, int* levels, int* launches, int* tasks) {
  if (!b) return fail(ACCFFT_C_EINVAL, "batch_info: NULL batch");
  if (instances) *instances = (int)b->instances.size();
  if (levels) *levels = (int)b->level_end.size();
  if (launches) *launches = (int)b->launches.size();
  if (tasks) *tasks = b->tasks;
  return ACCFFT_C_OK;
}

}  // extern "C"

