// Line FFTs of lengths without compiled kernels (float and double plans).
//
// The compiled passes (kernels.cu) fix the line length, radix plan and tile
// shape at compile time for the lengths of AFG_LENGTHS_*; any other length
// whose prime factors are at most 31 runs here, from a radix plan chosen at
// plan creation (gen_factor: radices up to 32), with
// TC lines per CTA held in shared memory and the Stockham stages run
// between two shared-memory buffers (stage s of radix R reads x[j + r*L/R],
// multiplies by w_{Ns*R}^{(j%Ns)*r} and writes y[(j/Ns)*Ns*R + j%Ns + r*Ns],
// the R-point DFT in registers from the same codelets as the compiled
// engine).  These kernels make every such grid run; they are not tuned.
//
// Four kernels:
//   k_gen_strided      c2c along strided lines (y and x passes)
//   k_gen_contig<0>    c2c along contiguous lines (z pass of c2c plans)
//   k_gen_contig<1>    real lines of L -> L/2+1 complex (z pass of r2c plans,
//                      odd L included: two real lines as one complex line)
//   k_gen_contig<2>    L/2+1 complex -> real lines of L (the Hermitian
//                      completion, imaginary parts of kz = 0 and L/2 dropped;
//                      two lines per complex line)
// Inverse transforms conjugate on the way in and out.
#include "launch.h"
#include "passes.cuh"
#include "per_device.h"

namespace afg {

namespace {

constexpr int kGenThreads = 256;
// global loads a thread issues before it stores any of them to shared
// memory: a loop of runtime length that stored each value as it arrived
// would wait out one memory latency per entry
constexpr int kGenBatch = 8;

// entry p of line c of a shared-memory buffer sits at p*ps + c*cs: strided
// passes interleave the lines (ps = lines per CTA, cs = 1: the global loads
// run along the lines' common rows), contiguous passes keep them apart
// (ps = 1, cs = L: the global loads and the stages run along a line)
template <typename T, int R>
__device__ __forceinline__ void gen_stage(const typename CT<T>::V* __restrict__ in, typename CT<T>::V* __restrict__ out,
                                          const typename CT<T>::V* __restrict__ tw, int L, int Ns, int ps, int cs,
                                          int c, int j0, int jstep) {
  typedef typename CT<T>::V V;
  const int nb = L / R;
  // j / Ns as a high product (exact for j, Ns < 2^16): magic = ceil(2^32 / Ns)
  const unsigned magic = Ns > 1 ? 0xFFFFFFFFu / unsigned(Ns) + 1u : 0u;
  for (int j = j0; j < nb; j += jstep) {
    const int q = Ns > 1 ? int(__umulhi(unsigned(j), magic)) : j;
    const int k = j - q * Ns;
    V v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[(j + r * nb) * ps + c * cs];
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = c_mul(v[r], ld_tw(tw + (r - 1) * Ns + k));
    Dft<R, 1>::run(v);
    const int base = q * Ns * R + k;
#pragma unroll
    for (int o = 0; o < R; ++o) out[(base + o * Ns) * ps + c * cs] = v[o];
  }
}

// every stage over the CTA's tc lines (layout as gen_stage; interleaved:
// lines interleaved, thread c = tid % tc; else lines apart, consecutive
// threads on consecutive butterflies of one line); returns the buffer
// holding the result
template <typename T>
__device__ typename CT<T>::V* gen_fft(typename CT<T>::V* a, typename CT<T>::V* b, const GenPlan& g, int tc,
                                      bool interleaved) {
  typedef typename CT<T>::V V;
  const int per = kGenThreads / tc;   // threads per line
  const int c = interleaved ? threadIdx.x % tc : threadIdx.x / per;
  const int j0 = interleaved ? threadIdx.x / tc : threadIdx.x % per;
  const int jstep = per;
  const int ps = interleaved ? tc : 1, cs = interleaved ? 1 : g.L;
  const V* tw = static_cast<const V*>(g.tw);
  int Ns = 1;
  for (int s = 0; s < g.nst; ++s) {
    const V* t = tw + g.off[s];
    switch (g.radix[s]) {
#define AFG_GEN_R(R) \
  case R: gen_stage<T, R>(a, b, t, g.L, Ns, ps, cs, c, j0, jstep); break;
      AFG_GEN_R(2) AFG_GEN_R(3) AFG_GEN_R(4) AFG_GEN_R(5) AFG_GEN_R(6) AFG_GEN_R(7) AFG_GEN_R(8) AFG_GEN_R(9)
      AFG_GEN_R(10) AFG_GEN_R(11) AFG_GEN_R(12) AFG_GEN_R(13) AFG_GEN_R(14) AFG_GEN_R(15) AFG_GEN_R(16)
      AFG_GEN_R(17) AFG_GEN_R(18) AFG_GEN_R(19) AFG_GEN_R(20) AFG_GEN_R(21) AFG_GEN_R(22) AFG_GEN_R(23)
      AFG_GEN_R(24) AFG_GEN_R(25) AFG_GEN_R(26) AFG_GEN_R(27) AFG_GEN_R(28) AFG_GEN_R(29) AFG_GEN_R(30)
      AFG_GEN_R(31) AFG_GEN_R(32)
#undef AFG_GEN_R
      default: break;   // gen_factor produces no other radix
    }
    __syncthreads();
    V* x = a;
    a = b;
    b = x;
    Ns *= g.radix[s];
  }
  return a;
}

template <typename T>
__global__ void __launch_bounds__(kGenThreads) k_gen_strided(const GenArgs ga) {
  typedef typename CT<T>::V V;
  PassScope scope(ga.early_trigger);
  extern __shared__ __align__(16) unsigned char smraw[];
  const int L = ga.g.L, tc = ga.tc;
  V* a = reinterpret_cast<V*>(smraw);
  V* b = a + (size_t)L * tc;
  const T sg = ga.inverse ? T(-1) : T(1);
  // this thread's column is fixed (the CTA size is a multiple of tc): its
  // slab and offset are worked out once; it visits rows p0, p0 + pstep, ...
  const int c = threadIdx.x % tc, p0 = threadIdx.x / tc, pstep = kGenThreads / tc;
  const long long col = (long long)blockIdx.x * tc + c;
  const bool valid = col < ga.nlines;
  const long long slab = valid ? col / ga.cps : 0;
  const long long cc = valid ? col - slab * ga.cps : 0;
  const V* in = static_cast<const V*>(ga.in) + slab * ga.in_slab + cc;
  for (int p = p0; p < L; p += kGenBatch * pstep) {
    V x[kGenBatch];
#pragma unroll
    for (int u = 0; u < kGenBatch; ++u) {
      const int q = p + u * pstep;
      x[u] = c_make<V>(T(0), T(0));
      if (valid && q < L) x[u] = in[(long long)q * ga.in_line];
    }
#pragma unroll
    for (int u = 0; u < kGenBatch; ++u) {
      const int q = p + u * pstep;
      x[u].y *= sg;
      if (q < L) a[q * tc + c] = x[u];
    }
  }
  __syncthreads();
  const V* res = gen_fft<T>(a, b, ga.g, tc, true);
  V* out = static_cast<V*>(ga.out) + slab * ga.out_slab + cc;
  if (valid) {
    for (int p = p0; p < L; p += pstep) {
      V x = res[p * tc + c];
      x.y *= sg;
      out[(long long)p * ga.out_line] = x;
    }
  }
}

// contiguous lines: MODE 0 c2c; MODE 1 r2c and MODE 2 c2r hold two real
// lines in each complex slot (line 2c as the real part, 2c+1 as the
// imaginary part: half the line transforms), so a CTA of tc slots covers
// 2*tc real lines
template <typename T, int MODE>
__global__ void __launch_bounds__(kGenThreads) k_gen_contig(const GenArgs ga) {
  typedef typename CT<T>::V V;
  PassScope scope(ga.early_trigger);
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int LPS = MODE == 0 ? 1 : 2;   // lines per slot
  const int L = ga.g.L, tc = ga.tc, H = L / 2 + 1, n = L * tc;
  V* a = reinterpret_cast<V*>(smraw);
  V* b = a + (size_t)n;
  const long long l0 = (long long)blockIdx.x * tc * LPS;
  const long long d = ga.in_dist;
  const T sg = ga.inverse ? T(-1) : T(1);
  // entry e = c*L + p of the slots: slot c, position p (c = e / L as a high
  // product, exact for e < 2^16: L*tc is at most 6144; L = 1 is the real z
  // axis of N2 = 1)
  const unsigned magic = L > 1 ? 0xFFFFFFFFu / unsigned(L) + 1u : 0u;
  // load, consecutive threads along p, kGenBatch entries (of each line) in
  // flight a thread
  for (int e0 = threadIdx.x; e0 < n; e0 += kGenBatch * kGenThreads) {
    V x0[kGenBatch], x1[kGenBatch];
#pragma unroll
    for (int u = 0; u < kGenBatch; ++u) {
      const int e = e0 + u * kGenThreads;
      const int c = L > 1 ? int(__umulhi(unsigned(e), magic)) : e, p = e - c * L;
      const long long l = l0 + (long long)c * LPS;
      x0[u] = x1[u] = c_make<V>(T(0), T(0));
      if (e >= n) continue;
      if constexpr (MODE == 0) {
        if (l < ga.nlines) x0[u] = static_cast<const V*>(ga.in)[l * d + p];
      } else if constexpr (MODE == 1) {
        const T* r = static_cast<const T*>(ga.in) + l * d + p;
        if (l < ga.nlines) x0[u].x = r[0];
        if (l + 1 < ga.nlines) x1[u].x = r[d];
      } else {
        // entry p of each line's full spectrum comes from its half at
        // min(p, L - p) (the Hermitian completion, below)
        const V* h = static_cast<const V*>(ga.in) + l * d + (p < H ? p : L - p);
        if (l < ga.nlines) x0[u] = h[0];
        if (l + 1 < ga.nlines) x1[u] = h[d];
      }
    }
#pragma unroll
    for (int u = 0; u < kGenBatch; ++u) {
      const int e = e0 + u * kGenThreads;
      if (e >= n) break;
      V x = x0[u];
      if constexpr (MODE == 0) {
        x.y *= sg;
      } else if constexpr (MODE == 1) {
        x.y = x1[u].x;
      } else {
        // spectra A (line 2c) and B (line 2c+1): imaginary parts of DC and
        // Nyquist dropped, the mirrored half conjugated; the slot holds
        // conj(A + iB) for the forward engine
        const int c = L > 1 ? int(__umulhi(unsigned(e), magic)) : e, p = e - c * L;
        V A = x0[u], B = x1[u];
        if (p == 0 || 2 * p == L) A.y = B.y = T(0);
        if (p >= H) {
          A.y = -A.y;
          B.y = -B.y;
        }
        x = c_make<V>(A.x - B.y, -(A.y + B.x));
      }
      a[e] = x;
    }
  }
  __syncthreads();
  const V* res = gen_fft<T>(a, b, ga.g, tc, false);
  const long long od = ga.out_dist;
  if constexpr (MODE == 1) {
    // X = A + iB: A[k] = (X[k] + conj X[L-k]) / 2, B[k] = (X[k] - conj X[L-k]) / 2i
    const unsigned mh = H > 1 ? 0xFFFFFFFFu / unsigned(H) + 1u : 0u;
    for (int e = threadIdx.x; e < H * tc; e += kGenThreads) {
      const int c = H > 1 ? int(__umulhi(unsigned(e), mh)) : e, k = e - c * H;
      const long long l = l0 + 2LL * c;
      if (l >= ga.nlines) continue;
      const V X = res[c * L + k], Y = res[c * L + (k == 0 ? 0 : L - k)];
      V* o = static_cast<V*>(ga.out) + l * od + k;
      o[0] = c_make<V>(T(0.5) * (X.x + Y.x), T(0.5) * (X.y - Y.y));
      if (l + 1 < ga.nlines) o[od] = c_make<V>(T(0.5) * (X.y + Y.y), T(-0.5) * (X.x - Y.x));
    }
  } else {
    for (int e = threadIdx.x; e < n; e += kGenThreads) {
      const int c = L > 1 ? int(__umulhi(unsigned(e), magic)) : e, p = e - c * L;
      const long long l = l0 + (long long)c * LPS;
      if (l >= ga.nlines) continue;
      V x = res[e];
      if constexpr (MODE == 0) {
        x.y *= sg;
        static_cast<V*>(ga.out)[l * od + p] = x;
      } else {
        // the forward engine gave conj(a + ib): line 2c is a, line 2c+1 is b
        T* o = static_cast<T*>(ga.out) + l * od + p;
        o[0] = x.x;
        if (l + 1 < ga.nlines) o[od] = -x.y;
      }
    }
  }
}

// lines_per_slot: 2 for the paired real kernels
template <typename T, typename K>
bool gen_launch(K kernel, const GenArgs& g, cudaStream_t s, int lines_per_slot = 1) {
  typedef typename CT<T>::V V;
  const size_t smem = 2 * (size_t)g.g.L * g.tc * sizeof(V);
  // the shared-memory opt-in belongs to the current device and the sizes
  // differ between lengths: set it on every launch above the default (cheap)
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
    return false;
  GenArgs b = g;
  b.early_trigger = pdl_mode() == 2;
  const long long per = (long long)g.tc * lines_per_slot;
  const long long grid = (g.nlines + per - 1) / per;
  return launch_pass(kernel, unsigned(grid), kGenThreads, smem, s, b) == cudaSuccess;
}

}  // namespace

// lines of L per CTA for the generic kernels: as many as fit 96 KB of
// shared memory (two buffers), at most 16, at least 1
int gen_lines_per_cta(int L, bool dbl) {
  const size_t per = 2 * (size_t)L * (dbl ? 16 : 8);
  int tc = 16;
  while (tc > 1 && per * tc > 96 * 1024) tc /= 2;
  return tc;
}

bool launch_gen(int prec, int mode, const GenArgs& g, cudaStream_t s) {
  // mode: 0 strided c2c, 1 contiguous c2c, 2 r2c, 3 c2r
  if (prec == PREC_F32) {
    switch (mode) {
      case 0: return gen_launch<float>(k_gen_strided<float>, g, s);
      case 1: return gen_launch<float>(k_gen_contig<float, 0>, g, s);
      case 2: return gen_launch<float>(k_gen_contig<float, 1>, g, s, 2);
      case 3: return gen_launch<float>(k_gen_contig<float, 2>, g, s, 2);
    }
  } else if (prec == PREC_F64) {
    switch (mode) {
      case 0: return gen_launch<double>(k_gen_strided<double>, g, s);
      case 1: return gen_launch<double>(k_gen_contig<double, 0>, g, s);
      case 2: return gen_launch<double>(k_gen_contig<double, 1>, g, s, 2);
      case 3: return gen_launch<double>(k_gen_contig<double, 2>, g, s, 2);
    }
  }
  return false;
}

}  // namespace afg
